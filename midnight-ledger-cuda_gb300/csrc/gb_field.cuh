// Montgomery arithmetic for the two BLS12-381 fields, written for sm_103a.
//
//   fp_t : base field Fp, 381-bit modulus, 12 x 32-bit limbs, R = 2^384
//   fr_t : scalar field Fr, 255-bit modulus, 8 x 32-bit limbs, R = 2^256
//
// The memory image of each type is byte-identical to blst's 64-bit-limb
// Montgomery representation (blst_fp / blst_fr), which is what the reference
// FFI passes across the boundary (midnight-sppark-msm/src/lib.rs:17-36,
// vendor/midnight-curves-0.3.1/src/bls12_381/fq.rs:25-29): little-endian
// limbs, Montgomery form, every stored value fully reduced into [0, m).
//
// Multiplication is CIOS Montgomery multiplication.  On the device each
// multiply-accumulate row is one inline-PTX carry chain (mad.lo.cc /
// madc.hi.cc on 32-bit limbs) in a single asm statement, with the partial
// products split into an even-limb row and an odd-limb row; a portable C
// version of the same algorithm is kept for host builds of this header, which
// the CPU test suite uses to check the limb logic against the oracle without
// a GPU.
#pragma once

#include <stdint.h>

#include <utility>

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#define GB_D __device__ __forceinline__
// operations off the hot loops (point doubling, full addition, conversions).
// With the Fp product out of line they inline cheaply; GB_COLD_NOINLINE keeps
// them as calls.
#if defined(GB_COLD_NOINLINE)
#define GB_COLD inline __host__ __device__ __noinline__
#else
#define GB_COLD __host__ __device__ __forceinline__
#endif
#else
#define GB_HD inline
#define GB_D inline
#define GB_COLD inline
#endif

#include "gb_fp_sqr.cuh"

namespace gb {

struct FpCfg {
    static constexpr int N = 12;
    static constexpr uint32_t INV = 0xfffcfffdu;  // -p^-1 mod 2^32
    static constexpr uint32_t M0 = 0xffffaaabu, M1 = 0xb9feffffu, M2 = 0xb153ffffu, M3 = 0x1eabfffeu,
                              M4 = 0xf6b0f624u, M5 = 0x6730d2a0u, M6 = 0xf38512bfu, M7 = 0x64774b84u,
                              M8 = 0x434bacd7u, M9 = 0x4b1ba7b6u, M10 = 0x397fe69au, M11 = 0x1a0111eau;
    GB_HD static uint32_t mod(int i)
    {
        constexpr uint32_t P[12] = {0xffffaaabu, 0xb9feffffu, 0xb153ffffu, 0x1eabfffeu,
                                    0xf6b0f624u, 0x6730d2a0u, 0xf38512bfu, 0x64774b84u,
                                    0x434bacd7u, 0x4b1ba7b6u, 0x397fe69au, 0x1a0111eau};
        return P[i];
    }
    GB_HD static uint32_t one(int i)
    {
        constexpr uint32_t O[12] = {0x0002fffdu, 0x76090000u, 0xc40c0002u, 0xebf4000bu,
                                    0x53c758bau, 0x5f489857u, 0x70525745u, 0x77ce5853u,
                                    0xa256ec6du, 0x5c071a97u, 0xfa80e493u, 0x15f65ec3u};
        return O[i];
    }
    GB_HD static uint32_t r2(int i)
    {
        constexpr uint32_t R2[12] = {0x1c341746u, 0xf4df1f34u, 0x09d104f1u, 0x0a76e6a6u,
                                     0x4c95b6d5u, 0x8de5476cu, 0x939d83c0u, 0x67eb88a9u,
                                     0xb519952du, 0x9a793e85u, 0x92cae3aau, 0x11988fe5u};
        return R2[i];
    }
};

struct FrCfg {
    static constexpr int N = 8;
    static constexpr uint32_t INV = 0xffffffffu;  // -r^-1 mod 2^32
    static constexpr uint32_t M0 = 0x00000001u, M1 = 0xffffffffu, M2 = 0xfffe5bfeu, M3 = 0x53bda402u,
                              M4 = 0x09a1d805u, M5 = 0x3339d808u, M6 = 0x299d7d48u, M7 = 0x73eda753u;
    GB_HD static uint32_t mod(int i)
    {
        constexpr uint32_t P[8] = {0x00000001u, 0xffffffffu, 0xfffe5bfeu, 0x53bda402u,
                                   0x09a1d805u, 0x3339d808u, 0x299d7d48u, 0x73eda753u};
        return P[i];
    }
    GB_HD static uint32_t one(int i)
    {
        constexpr uint32_t O[8] = {0xfffffffeu, 0x00000001u, 0x00034802u, 0x5884b7fau,
                                   0xecbc4ff5u, 0x998c4fefu, 0xacc5056fu, 0x1824b159u};
        return O[i];
    }
    GB_HD static uint32_t r2(int i)
    {
        constexpr uint32_t R2[8] = {0xf3f29c6du, 0xc999e990u, 0x87925c23u, 0x2b6cedcbu,
                                    0x7254398fu, 0x05d31496u, 0x9f59ff11u, 0x0748d9d9u};
        return R2[i];
    }
};

// ---------------------------------------------------------------------------
// Multi-limb primitives.  Device versions use PTX carry flags; host versions
// use 64-bit intermediates.  Both compute the same function.
// ---------------------------------------------------------------------------

// out = a + b over N limbs; returns the carry out.  Plain C with 64-bit
// intermediates: the compiler owns the carry propagation.
template <int N>
GB_HD uint32_t mp_add(uint32_t *out, const uint32_t *a, const uint32_t *b)
{
    uint64_t c = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        uint64_t v = (uint64_t)a[i] + b[i] + c;
        out[i] = (uint32_t)v;
        c = v >> 32;
    }
    return (uint32_t)c;
}

// out = a - b over N limbs; returns the borrow (1 if a < b).
template <int N>
GB_HD uint32_t mp_sub(uint32_t *out, const uint32_t *a, const uint32_t *b)
{
    uint64_t br = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        uint64_t v = (uint64_t)a[i] - b[i] - br;
        out[i] = (uint32_t)v;
        br = (v >> 32) & 1;
    }
    return (uint32_t)br;
}

#if defined(__CUDA_ARCH__)
// acc[0..N] += sum_k x[k] * y * 2^(64k) over 32-bit limbs: the low half of
// x[k]*y lands on limb 2k, the high half on limb 2k+1, one carry chain,
// final carry into acc[N].  The whole chain is ONE asm statement that starts
// without a carry-in and ends by absorbing its carry, so no carry crosses a
// statement boundary and the compiler may freely interleave independent
// chains (the statements are deliberately not volatile).
GB_D void row_mac12(uint32_t *acc, uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3, uint32_t x4,
                    uint32_t x5, uint32_t y)
{
    asm(
        "mad.lo.cc.u32 %0, %13, %19, %0;\n\t"
        "madc.hi.cc.u32 %1, %13, %19, %1;\n\t"
        "madc.lo.cc.u32 %2, %14, %19, %2;\n\t"
        "madc.hi.cc.u32 %3, %14, %19, %3;\n\t"
        "madc.lo.cc.u32 %4, %15, %19, %4;\n\t"
        "madc.hi.cc.u32 %5, %15, %19, %5;\n\t"
        "madc.lo.cc.u32 %6, %16, %19, %6;\n\t"
        "madc.hi.cc.u32 %7, %16, %19, %7;\n\t"
        "madc.lo.cc.u32 %8, %17, %19, %8;\n\t"
        "madc.hi.cc.u32 %9, %17, %19, %9;\n\t"
        "madc.lo.cc.u32 %10, %18, %19, %10;\n\t"
        "madc.hi.cc.u32 %11, %18, %19, %11;\n\t"
        "addc.u32 %12, %12, 0;"
        : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]),
          "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
        : "r"(x0), "r"(x1), "r"(x2), "r"(x3), "r"(x4), "r"(x5), "r"(y));
}

GB_D void row_mac8(uint32_t *acc, uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3, uint32_t y)
{
    asm(
        "mad.lo.cc.u32 %0, %9, %13, %0;\n\t"
        "madc.hi.cc.u32 %1, %9, %13, %1;\n\t"
        "madc.lo.cc.u32 %2, %10, %13, %2;\n\t"
        "madc.hi.cc.u32 %3, %10, %13, %3;\n\t"
        "madc.lo.cc.u32 %4, %11, %13, %4;\n\t"
        "madc.hi.cc.u32 %5, %11, %13, %5;\n\t"
        "madc.lo.cc.u32 %6, %12, %13, %6;\n\t"
        "madc.hi.cc.u32 %7, %12, %13, %7;\n\t"
        "addc.u32 %8, %8, 0;"
        : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]),
          "+r"(acc[7]), "+r"(acc[8])
        : "r"(x0), "r"(x1), "r"(x2), "r"(x3), "r"(y));
}

// acc += modulus * m, modulus limbs as immediates (no registers held for them)
#define GB_ROW12_IMM(acc, x0, x1, x2, x3, x4, x5, y)                                                    \
    asm("mad.lo.cc.u32 %0, %13, %14, %0;\n\t"                                                         \
        "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"                                                        \
        "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"                                                        \
        "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"                                                        \
        "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"                                                        \
        "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"                                                        \
        "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"                                                        \
        "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"                                                        \
        "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"                                                        \
        "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"                                                        \
        "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"                                                      \
        "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"                                                      \
        "addc.u32 %12, %12, 0;"                                                                         \
        : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]),          \
          "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]),        \
          "+r"(acc[12])                                                                                 \
        : "r"(y), "n"(x0), "n"(x1), "n"(x2), "n"(x3), "n"(x4), "n"(x5))

#define GB_ROW8_IMM(acc, x0, x1, x2, x3, y)                                                             \
    asm("mad.lo.cc.u32 %0, %9, %10, %0;\n\t"                                                          \
        "madc.hi.cc.u32 %1, %9, %10, %1;\n\t"                                                         \
        "madc.lo.cc.u32 %2, %9, %11, %2;\n\t"                                                         \
        "madc.hi.cc.u32 %3, %9, %11, %3;\n\t"                                                         \
        "madc.lo.cc.u32 %4, %9, %12, %4;\n\t"                                                         \
        "madc.hi.cc.u32 %5, %9, %12, %5;\n\t"                                                         \
        "madc.lo.cc.u32 %6, %9, %13, %6;\n\t"                                                         \
        "madc.hi.cc.u32 %7, %9, %13, %7;\n\t"                                                         \
        "addc.u32 %8, %8, 0;"                                                                           \
        : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]),          \
          "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])                                                      \
        : "r"(y), "n"(x0), "n"(x1), "n"(x2), "n"(x3))

template <class Cfg>
GB_D void row_mac_mod(uint32_t *acc, int parity, uint32_t m);

template <>
GB_D void row_mac_mod<FpCfg>(uint32_t *acc, int parity, uint32_t m)
{
    typedef FpCfg C;
    if (parity == 0) GB_ROW12_IMM(acc, C::M0, C::M2, C::M4, C::M6, C::M8, C::M10, m);
    else GB_ROW12_IMM(acc, C::M1, C::M3, C::M5, C::M7, C::M9, C::M11, m);
}

template <>
GB_D void row_mac_mod<FrCfg>(uint32_t *acc, int parity, uint32_t m)
{
    typedef FrCfg C;
    // r's two lowest limbs are 1 and 2^32 - 1: m * 1 = m and m (2^32 - 1)
    // = (m - [m != 0]) 2^32 + (-m mod 2^32), so those two products of the
    // row are additions (measured on GB300: Fr products 7% faster, the
    // 16 x 2^20 NTT 3.61 -> 3.55 ms)
    if (parity == 0) {
        asm("add.cc.u32 %0, %0, %9;\n\t"
            "addc.cc.u32 %1, %1, 0;\n\t"
            "madc.lo.cc.u32 %2, %9, %10, %2;\n\t"
            "madc.hi.cc.u32 %3, %9, %10, %3;\n\t"
            "madc.lo.cc.u32 %4, %9, %11, %4;\n\t"
            "madc.hi.cc.u32 %5, %9, %11, %5;\n\t"
            "madc.lo.cc.u32 %6, %9, %12, %6;\n\t"
            "madc.hi.cc.u32 %7, %9, %12, %7;\n\t"
            "addc.u32 %8, %8, 0;"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]),
              "+r"(acc[7]), "+r"(acc[8])
            : "r"(m), "n"(C::M2), "n"(C::M4), "n"(C::M6));
    } else {
        const uint32_t lo = 0u - m, hi = m - (m != 0u);
        asm("add.cc.u32 %0, %0, %10;\n\t"
            "addc.cc.u32 %1, %1, %11;\n\t"
            "madc.lo.cc.u32 %2, %9, %12, %2;\n\t"
            "madc.hi.cc.u32 %3, %9, %12, %3;\n\t"
            "madc.lo.cc.u32 %4, %9, %13, %4;\n\t"
            "madc.hi.cc.u32 %5, %9, %13, %5;\n\t"
            "madc.lo.cc.u32 %6, %9, %14, %6;\n\t"
            "madc.hi.cc.u32 %7, %9, %14, %7;\n\t"
            "addc.u32 %8, %8, 0;"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]),
              "+r"(acc[7]), "+r"(acc[8])
            : "r"(m), "r"(lo), "r"(hi), "n"(C::M3), "n"(C::M5), "n"(C::M7));
    }
}

// even[0..N-1] = even[1..N] + odd[0..N-1], even[N] = odd[N] + carry: the
// division by 2^32 that ends each CIOS step, as one carry chain
GB_D void fold12(uint32_t *e, const uint32_t *o)
{
    asm("add.cc.u32 %0, %1, %13;\n\t"
        "addc.cc.u32 %1, %2, %14;\n\t"
        "addc.cc.u32 %2, %3, %15;\n\t"
        "addc.cc.u32 %3, %4, %16;\n\t"
        "addc.cc.u32 %4, %5, %17;\n\t"
        "addc.cc.u32 %5, %6, %18;\n\t"
        "addc.cc.u32 %6, %7, %19;\n\t"
        "addc.cc.u32 %7, %8, %20;\n\t"
        "addc.cc.u32 %8, %9, %21;\n\t"
        "addc.cc.u32 %9, %10, %22;\n\t"
        "addc.cc.u32 %10, %11, %23;\n\t"
        "addc.cc.u32 %11, %12, %24;\n\t"
        "addc.u32 %12, %25, 0;"
        : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]),
          "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "+r"(e[12])
        : "r"(o[0]), "r"(o[1]), "r"(o[2]), "r"(o[3]), "r"(o[4]), "r"(o[5]), "r"(o[6]), "r"(o[7]), "r"(o[8]),
          "r"(o[9]), "r"(o[10]), "r"(o[11]), "r"(o[12]));
}

GB_D void fold8(uint32_t *e, const uint32_t *o)
{
    asm("add.cc.u32 %0, %1, %9;\n\t"
        "addc.cc.u32 %1, %2, %10;\n\t"
        "addc.cc.u32 %2, %3, %11;\n\t"
        "addc.cc.u32 %3, %4, %12;\n\t"
        "addc.cc.u32 %4, %5, %13;\n\t"
        "addc.cc.u32 %5, %6, %14;\n\t"
        "addc.cc.u32 %6, %7, %15;\n\t"
        "addc.cc.u32 %7, %8, %16;\n\t"
        "addc.u32 %8, %17, 0;"
        : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]),
          "+r"(e[8])
        : "r"(o[0]), "r"(o[1]), "r"(o[2]), "r"(o[3]), "r"(o[4]), "r"(o[5]), "r"(o[6]), "r"(o[7]), "r"(o[8]));
}

template <int N>
GB_D void fold(uint32_t *e, const uint32_t *o);
template <>
GB_D void fold<12>(uint32_t *e, const uint32_t *o) { fold12(e, o); }
template <>
GB_D void fold<8>(uint32_t *e, const uint32_t *o) { fold8(e, o); }

// acc += x * y where x is given by its even (parity 0) or odd (parity 1)
// limbs: x[parity + 2k] for k < N/2
template <int N>
GB_D void row_mac(uint32_t *acc, const uint32_t *x, int parity, uint32_t y);

template <>
GB_D void row_mac<12>(uint32_t *acc, const uint32_t *x, int parity, uint32_t y)
{
    if (parity == 0) row_mac12(acc, x[0], x[2], x[4], x[6], x[8], x[10], y);
    else row_mac12(acc, x[1], x[3], x[5], x[7], x[9], x[11], y);
}

template <>
GB_D void row_mac<8>(uint32_t *acc, const uint32_t *x, int parity, uint32_t y)
{
    if (parity == 0) row_mac8(acc, x[0], x[2], x[4], x[6], y);
    else row_mac8(acc, x[1], x[3], x[5], x[7], y);
}

// Device modular addition and subtraction as explicit carry chains (one
// instruction per limb and chain); measured on GB300 against the 64-bit
// C form, they make the NTT 14% and the MSM 2% faster.  GB_ADD_C selects the
// C form.
template <class Cfg>
GB_D void mod_add_dev(uint32_t *r, const uint32_t *a, const uint32_t *b);
template <class Cfg>
GB_D void mod_sub_dev(uint32_t *r, const uint32_t *a, const uint32_t *b);

// a + b mod m for a, b < m: one carry chain for the sum, one borrow chain
// subtracting the modulus (immediates), then a select
template <>
GB_D void mod_add_dev<FpCfg>(uint32_t *r, const uint32_t *a, const uint32_t *b)
{
    typedef FpCfg C;
    uint32_t s[12], t[12], c, br;
    asm("add.cc.u32 %0, %13, %25;\n\t"
        "addc.cc.u32 %1, %14, %26;\n\t"
        "addc.cc.u32 %2, %15, %27;\n\t"
        "addc.cc.u32 %3, %16, %28;\n\t"
        "addc.cc.u32 %4, %17, %29;\n\t"
        "addc.cc.u32 %5, %18, %30;\n\t"
        "addc.cc.u32 %6, %19, %31;\n\t"
        "addc.cc.u32 %7, %20, %32;\n\t"
        "addc.cc.u32 %8, %21, %33;\n\t"
        "addc.cc.u32 %9, %22, %34;\n\t"
        "addc.cc.u32 %10, %23, %35;\n\t"
        "addc.cc.u32 %11, %24, %36;\n\t"
        "addc.u32 %12, 0, 0;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11]), "=r"(c)
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]));
    asm("sub.cc.u32 %0, %13, %26;\n\t"
        "subc.cc.u32 %1, %14, %27;\n\t"
        "subc.cc.u32 %2, %15, %28;\n\t"
        "subc.cc.u32 %3, %16, %29;\n\t"
        "subc.cc.u32 %4, %17, %30;\n\t"
        "subc.cc.u32 %5, %18, %31;\n\t"
        "subc.cc.u32 %6, %19, %32;\n\t"
        "subc.cc.u32 %7, %20, %33;\n\t"
        "subc.cc.u32 %8, %21, %34;\n\t"
        "subc.cc.u32 %9, %22, %35;\n\t"
        "subc.cc.u32 %10, %23, %36;\n\t"
        "subc.cc.u32 %11, %24, %37;\n\t"
        "subc.u32 %12, %25, 0;"
        : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7]), "=r"(t[8]), "=r"(t[9]), "=r"(t[10]), "=r"(t[11]), "=r"(br)
        : "r"(s[0]), "r"(s[1]), "r"(s[2]), "r"(s[3]), "r"(s[4]), "r"(s[5]), "r"(s[6]), "r"(s[7]), "r"(s[8]), "r"(s[9]), "r"(s[10]), "r"(s[11]), "r"(c), "n"(C::M0), "n"(C::M1), "n"(C::M2), "n"(C::M3), "n"(C::M4), "n"(C::M5), "n"(C::M6), "n"(C::M7), "n"(C::M8), "n"(C::M9), "n"(C::M10), "n"(C::M11));
    // br = 0: s + c * 2^384 >= m, keep s - m
#pragma unroll
    for (int i = 0; i < 12; i++) r[i] = br ? s[i] : t[i];
}

// a - b mod m for a, b < m
template <>
GB_D void mod_sub_dev<FpCfg>(uint32_t *r, const uint32_t *a, const uint32_t *b)
{
    typedef FpCfg C;
    uint32_t d[12], t[12], br;
    asm("sub.cc.u32 %0, %13, %25;\n\t"
        "subc.cc.u32 %1, %14, %26;\n\t"
        "subc.cc.u32 %2, %15, %27;\n\t"
        "subc.cc.u32 %3, %16, %28;\n\t"
        "subc.cc.u32 %4, %17, %29;\n\t"
        "subc.cc.u32 %5, %18, %30;\n\t"
        "subc.cc.u32 %6, %19, %31;\n\t"
        "subc.cc.u32 %7, %20, %32;\n\t"
        "subc.cc.u32 %8, %21, %33;\n\t"
        "subc.cc.u32 %9, %22, %34;\n\t"
        "subc.cc.u32 %10, %23, %35;\n\t"
        "subc.cc.u32 %11, %24, %36;\n\t"
        "subc.u32 %12, 0, 0;"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]), "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(br)
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]));
    asm("add.cc.u32 %0, %12, %24;\n\t"
        "addc.cc.u32 %1, %13, %25;\n\t"
        "addc.cc.u32 %2, %14, %26;\n\t"
        "addc.cc.u32 %3, %15, %27;\n\t"
        "addc.cc.u32 %4, %16, %28;\n\t"
        "addc.cc.u32 %5, %17, %29;\n\t"
        "addc.cc.u32 %6, %18, %30;\n\t"
        "addc.cc.u32 %7, %19, %31;\n\t"
        "addc.cc.u32 %8, %20, %32;\n\t"
        "addc.cc.u32 %9, %21, %33;\n\t"
        "addc.cc.u32 %10, %22, %34;\n\t"
        "addc.u32 %11, %23, %35;\n\t"
        : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7]), "=r"(t[8]), "=r"(t[9]), "=r"(t[10]), "=r"(t[11])
        : "r"(d[0]), "r"(d[1]), "r"(d[2]), "r"(d[3]), "r"(d[4]), "r"(d[5]), "r"(d[6]), "r"(d[7]), "r"(d[8]), "r"(d[9]), "r"(d[10]), "r"(d[11]), "n"(C::M0), "n"(C::M1), "n"(C::M2), "n"(C::M3), "n"(C::M4), "n"(C::M5), "n"(C::M6), "n"(C::M7), "n"(C::M8), "n"(C::M9), "n"(C::M10), "n"(C::M11));
#pragma unroll
    for (int i = 0; i < 12; i++) r[i] = br ? t[i] : d[i];
}

// a + b mod m for a, b < m: one carry chain for the sum, one borrow chain
// subtracting the modulus (immediates), then a select
template <>
GB_D void mod_add_dev<FrCfg>(uint32_t *r, const uint32_t *a, const uint32_t *b)
{
    typedef FrCfg C;
    uint32_t s[8], t[8], c, br;
    asm("add.cc.u32 %0, %9, %17;\n\t"
        "addc.cc.u32 %1, %10, %18;\n\t"
        "addc.cc.u32 %2, %11, %19;\n\t"
        "addc.cc.u32 %3, %12, %20;\n\t"
        "addc.cc.u32 %4, %13, %21;\n\t"
        "addc.cc.u32 %5, %14, %22;\n\t"
        "addc.cc.u32 %6, %15, %23;\n\t"
        "addc.cc.u32 %7, %16, %24;\n\t"
        "addc.u32 %8, 0, 0;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(c)
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
    asm("sub.cc.u32 %0, %9, %18;\n\t"
        "subc.cc.u32 %1, %10, %19;\n\t"
        "subc.cc.u32 %2, %11, %20;\n\t"
        "subc.cc.u32 %3, %12, %21;\n\t"
        "subc.cc.u32 %4, %13, %22;\n\t"
        "subc.cc.u32 %5, %14, %23;\n\t"
        "subc.cc.u32 %6, %15, %24;\n\t"
        "subc.cc.u32 %7, %16, %25;\n\t"
        "subc.u32 %8, %17, 0;"
        : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7]), "=r"(br)
        : "r"(s[0]), "r"(s[1]), "r"(s[2]), "r"(s[3]), "r"(s[4]), "r"(s[5]), "r"(s[6]), "r"(s[7]), "r"(c), "n"(C::M0), "n"(C::M1), "n"(C::M2), "n"(C::M3), "n"(C::M4), "n"(C::M5), "n"(C::M6), "n"(C::M7));
    // br = 0: s + c * 2^256 >= m, keep s - m
#pragma unroll
    for (int i = 0; i < 8; i++) r[i] = br ? s[i] : t[i];
}

// a - b mod m for a, b < m
template <>
GB_D void mod_sub_dev<FrCfg>(uint32_t *r, const uint32_t *a, const uint32_t *b)
{
    typedef FrCfg C;
    uint32_t d[8], t[8], br;
    asm("sub.cc.u32 %0, %9, %17;\n\t"
        "subc.cc.u32 %1, %10, %18;\n\t"
        "subc.cc.u32 %2, %11, %19;\n\t"
        "subc.cc.u32 %3, %12, %20;\n\t"
        "subc.cc.u32 %4, %13, %21;\n\t"
        "subc.cc.u32 %5, %14, %22;\n\t"
        "subc.cc.u32 %6, %15, %23;\n\t"
        "subc.cc.u32 %7, %16, %24;\n\t"
        "subc.u32 %8, 0, 0;"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]), "=r"(br)
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
    asm("add.cc.u32 %0, %8, %16;\n\t"
        "addc.cc.u32 %1, %9, %17;\n\t"
        "addc.cc.u32 %2, %10, %18;\n\t"
        "addc.cc.u32 %3, %11, %19;\n\t"
        "addc.cc.u32 %4, %12, %20;\n\t"
        "addc.cc.u32 %5, %13, %21;\n\t"
        "addc.cc.u32 %6, %14, %22;\n\t"
        "addc.u32 %7, %15, %23;\n\t"
        : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7])
        : "r"(d[0]), "r"(d[1]), "r"(d[2]), "r"(d[3]), "r"(d[4]), "r"(d[5]), "r"(d[6]), "r"(d[7]), "n"(C::M0), "n"(C::M1), "n"(C::M2), "n"(C::M3), "n"(C::M4), "n"(C::M5), "n"(C::M6), "n"(C::M7));
#pragma unroll
    for (int i = 0; i < 8; i++) r[i] = br ? t[i] : d[i];
}

#endif

template <class Cfg>
struct mont_t {
    static constexpr int N = Cfg::N;
    uint32_t v[N];

    GB_HD static mont_t zero()
    {
        mont_t r;
#pragma unroll
        for (int i = 0; i < N; i++) r.v[i] = 0;
        return r;
    }
    GB_HD static mont_t one()
    {
        mont_t r;
#pragma unroll
        for (int i = 0; i < N; i++) r.v[i] = Cfg::one(i);
        return r;
    }
    GB_HD static mont_t modulus()
    {
        mont_t r;
#pragma unroll
        for (int i = 0; i < N; i++) r.v[i] = Cfg::mod(i);
        return r;
    }
    GB_HD bool is_zero() const
    {
        uint32_t x = 0;
#pragma unroll
        for (int i = 0; i < N; i++) x |= v[i];
        return x == 0;
    }
    GB_HD bool operator==(const mont_t &o) const
    {
        uint32_t x = 0;
#pragma unroll
        for (int i = 0; i < N; i++) x |= v[i] ^ o.v[i];
        return x == 0;
    }
    GB_HD bool operator!=(const mont_t &o) const { return !(*this == o); }

    // conditional subtraction of the modulus: r = a >= m ? a - m : a,
    // for a < 2m.  `carry` is an extra top bit of a.
    GB_HD static void reduce_once(uint32_t *a, uint32_t carry)
    {
        uint32_t t[N], m[N];
#pragma unroll
        for (int i = 0; i < N; i++) m[i] = Cfg::mod(i);
        uint32_t br = mp_sub<N>(t, a, m);
        // keep t when a >= m, i.e. carry set or no borrow
        bool take = carry || !br;
#pragma unroll
        for (int i = 0; i < N; i++) a[i] = take ? t[i] : a[i];
    }

    GB_HD friend mont_t operator+(const mont_t &a, const mont_t &b)
    {
        mont_t r;
#if defined(__CUDA_ARCH__) && !defined(GB_ADD_C)
        mod_add_dev<Cfg>(r.v, a.v, b.v);
        return r;
#endif
        uint32_t c = mp_add<N>(r.v, a.v, b.v);
        reduce_once(r.v, c);
        return r;
    }
    GB_HD friend mont_t operator-(const mont_t &a, const mont_t &b)
    {
        mont_t r;
#if defined(__CUDA_ARCH__) && !defined(GB_ADD_C)
        mod_sub_dev<Cfg>(r.v, a.v, b.v);
        return r;
#endif
        uint32_t br = mp_sub<N>(r.v, a.v, b.v);
        if (br) {
            uint32_t m[N];
#pragma unroll
            for (int i = 0; i < N; i++) m[i] = Cfg::mod(i);
            mp_add<N>(r.v, r.v, m);
        }
        return r;
    }
    GB_HD mont_t operator-() const
    {
        if (is_zero()) return *this;
        mont_t r, m = modulus();
        mp_sub<N>(r.v, m.v, v);
        return r;
    }
    GB_HD mont_t dbl() const { return *this + *this; }
    GB_HD mont_t &operator+=(const mont_t &o) { return *this = *this + o; }
    GB_HD mont_t &operator-=(const mont_t &o) { return *this = *this - o; }

    // Montgomery product a * b * 2^(-32N) mod m (CIOS), fully reduced.
    GB_HD friend mont_t operator*(const mont_t &a, const mont_t &b)
    {
#if defined(__CUDA_ARCH__) && !defined(GB_FP_MUL_INLINE)
        if constexpr (N == 12) return mul_by_value(a, b);
#endif
        mont_t r;
        mont_mul(r.v, a.v, b.v);
        return r;
    }
#if defined(__CUDA_ARCH__) && !defined(GB_FP_MUL_INLINE)
    static __device__ __noinline__ mont_t mul_by_value(mont_t a, mont_t b);
#endif
    GB_HD mont_t &operator*=(const mont_t &o) { return *this = *this * o; }
    GB_HD mont_t sqr() const
    {
#if defined(__CUDA_ARCH__) && !defined(GB_FP_MUL_INLINE) && !defined(GB_FP_SQR_OFF)
        if constexpr (N == 12) return sqr_by_value(*this);
#endif
        return *this * *this;
    }
#if defined(__CUDA_ARCH__) && !defined(GB_FP_MUL_INLINE)
    static __device__ __noinline__ mont_t sqr_by_value(mont_t a);
#endif

    GB_HD static void mont_mul(uint32_t *out, const uint32_t *a, const uint32_t *b);

    GB_HD mont_t to_mont() const
    {
        mont_t r2;
#pragma unroll
        for (int i = 0; i < N; i++) r2.v[i] = Cfg::r2(i);
        return *this * r2;
    }
    GB_HD mont_t from_mont() const
    {
        mont_t o = zero();
        o.v[0] = 1;
        return *this * o;
    }
    // this^(m-2): Fermat inverse; zero maps to zero
    GB_COLD mont_t inverse() const
    {
        uint32_t e[N], two[N];
#pragma unroll
        for (int i = 0; i < N; i++) { e[i] = Cfg::mod(i); two[i] = 0; }
        two[0] = 2;
        mp_sub<N>(e, e, two);
        mont_t acc = one();
        for (int i = 32 * N - 1; i >= 0; i--) {
            acc = acc.sqr();
            if ((e[i >> 5] >> (i & 31)) & 1u) acc = acc * *this;
        }
        return acc;
    }
    // this^-1 by the binary extended Euclidean algorithm (Stein's binary
    // GCD carrying the Bezout coefficient, Knuth TAOCP vol. 2, 4.5.2 and
    // exercise 4.5.2-39); zero maps to zero.  With u = this, v = m and
    // x1 a = u, x2 a = v (mod m) held throughout, halvings and subtractions
    // bring u or v to 1 in at most 2 log2(m) steps.  The Montgomery form is
    // restored by two products with R^2 (the plain inverse of aR is
    // a^-1 R^-1).  Its dependent chain is short next to the 300-odd products
    // of a Fermat inversion, so a single thread inverts much sooner; its
    // data-dependent branches suit one inversion per tile, not one per
    // thread of a warp.
    GB_COLD mont_t inverse_binary() const
    {
        if (is_zero()) return *this;
        uint32_t u[N], w[N], x1[N], x2[N], m[N];
#pragma unroll
        for (int i = 0; i < N; i++) {
            u[i] = v[i];
            w[i] = m[i] = Cfg::mod(i);
            x1[i] = x2[i] = 0;
        }
        x1[0] = 1;
        auto is_one = [](const uint32_t *a) {
            uint32_t x = a[0] ^ 1u;
            for (int i = 1; i < N; i++) x |= a[i];
            return x == 0;
        };
        // a /= 2 with an extra top bit
        auto half = [](uint32_t *a, uint32_t top) {
            for (int i = 0; i < N - 1; i++) a[i] = (a[i] >> 1) | (a[i + 1] << 31);
            a[N - 1] = (a[N - 1] >> 1) | (top << 31);
        };
        // x / 2 mod m (m odd, x < m)
        auto half_mod = [&](uint32_t *x) {
            uint32_t top = 0;
            if (x[0] & 1u) top = mp_add<N>(x, x, m);
            half(x, top);
        };
        // x = x - y mod m (x, y < m)
        auto sub_mod = [&](uint32_t *x, const uint32_t *y) {
            if (mp_sub<N>(x, x, y)) mp_add<N>(x, x, m);
        };
        while (!is_one(u) && !is_one(w)) {
            while (!(u[0] & 1u)) {
                half(u, 0);
                half_mod(x1);
            }
            while (!(w[0] & 1u)) {
                half(w, 0);
                half_mod(x2);
            }
            uint32_t d[N];
            if (!mp_sub<N>(d, u, w)) {  // u >= w
                for (int i = 0; i < N; i++) u[i] = d[i];
                sub_mod(x1, x2);
            } else {
                mp_sub<N>(w, w, u);
                sub_mod(x2, x1);
            }
        }
        mont_t r, r2;
        const uint32_t *res = is_one(u) ? x1 : x2;
        for (int i = 0; i < N; i++) {
            r.v[i] = res[i];
            r2.v[i] = Cfg::r2(i);
        }
        return (r * r2) * r2;
    }
    // this^e for a 64-bit exponent
    GB_COLD mont_t pow_u64(uint64_t e) const
    {
        mont_t acc = one(), base = *this;
        while (e) {
            if (e & 1) acc = acc * base;
            base = base.sqr();
            e >>= 1;
        }
        return acc;
    }
};

#if defined(__CUDA_ARCH__)
// Device CIOS: for each limb b[i], accumulate a*b[i] and m*p into the running
// sum held as two rows, `even` (products of even-indexed limbs) and `odd`
// (products of odd-indexed limbs, stored one limb lower), so each row is a
// single uninterrupted carry chain; the rows are folded once per iteration
// while dividing by 2^32.
template <class Cfg>
GB_D void mont_step(uint32_t *even, uint32_t *odd, const uint32_t *a, uint32_t bi)
{
    constexpr int N = Cfg::N;
    row_mac<N>(even, a, 0, bi);
    // the odd row starts from zero each step: its limbs are plain products
    // (no overlaps, so no carries) -- independent multiplies that can issue
    // alongside the even row's carry chain
#pragma unroll
    for (int k = 0; k < N / 2; k++) {
        odd[2 * k] = a[2 * k + 1] * bi;
        odd[2 * k + 1] = __umulhi(a[2 * k + 1], bi);
    }
    odd[N] = 0;
    // value = even + odd * 2^32; the Montgomery step makes even[0] zero
    const uint32_t m = even[0] * Cfg::INV;
    row_mac_mod<Cfg>(even, 0, m);
    row_mac_mod<Cfg>(odd, 1, m);
    // value / 2^32 = even[1..N] + odd[0..N]
    fold<N>(even, odd);
}

// REDUCE = false skips the final conditional subtraction: the result is
// then below m + a*b/R, i.e. below 2m whenever a*b < m*R
template <class Cfg, bool REDUCE = true>
GB_D void mont_mul_device(uint32_t *out, const uint32_t *a, const uint32_t *b)
{
    constexpr int N = Cfg::N;
    uint32_t even[N + 1], odd[N + 1];
#pragma unroll
    for (int i = 0; i < N + 1; i++) even[i] = 0;
#if defined(GB_MUL_ROLLED)
    // rolled outer loop: b's limbs are shifted down each step, so the code
    // of one product stays a few hundred instructions (instruction-cache
    // friendly when many products are inlined into one kernel)
    uint32_t bb[N];
#pragma unroll
    for (int i = 0; i < N; i++) bb[i] = b[i];
#pragma unroll 1
    for (int i = 0; i < N; i++) {
        const uint32_t bi = bb[0];
#pragma unroll
        for (int j = 0; j + 1 < N; j++) bb[j] = bb[j + 1];
        mont_step<Cfg>(even, odd, a, bi);
    }
#else
#pragma unroll
    for (int i = 0; i < N; i++) mont_step<Cfg>(even, odd, a, b[i]);
#endif
    // even[0..N] < 2m; final conditional subtraction
    if (REDUCE) mont_t<Cfg>::reduce_once(even, even[N]);
#pragma unroll
    for (int i = 0; i < N; i++) out[i] = even[i];
}
#endif

// Out-of-line products.  A point addition inlines ten Fp products; fully
// unrolled, that is ~100 KB of code per addition and the MSM kernels then
// stall on instruction fetch.  One out-of-line copy per module (called ten
// times) keeps the footprint small: measured on GB300, the 2^20 MSM
// accumulation runs 18% faster this way, despite the call overhead.  The
// product is called by value from operator* (below); fp_mul_call serves the
// pointer interface.
// GB_FP_MUL_INLINE / GB_FR_MUL_CALL select the other forms for measurement.
#if defined(__CUDA_ARCH__) && !defined(GB_FP_MUL_INLINE)
#define GB_FP_MUL_CALL 1
static __device__ __noinline__ void fp_mul_call(uint32_t *out, const uint32_t *a, const uint32_t *b)
{
    mont_mul_device<FpCfg>(out, a, b);
}
#endif
#if defined(__CUDA_ARCH__) && defined(GB_FR_MUL_CALL)
static __device__ __noinline__ void fr_mul_call(uint32_t *out, const uint32_t *a, const uint32_t *b)
{
    mont_mul_device<FrCfg>(out, a, b);
}
#endif

#if defined(__CUDA_ARCH__) && !defined(GB_FP_MUL_INLINE)
// the out-of-line product with operands and result passed by value, so they
// stay in registers across the call (a pointer interface would put them on
// the stack)
template <class Cfg>
__device__ __noinline__ mont_t<Cfg> mont_t<Cfg>::mul_by_value(mont_t<Cfg> a, mont_t<Cfg> b)
{
    mont_t<Cfg> r;
    mont_mul_device<Cfg>(r.v, a.v, b.v);
    return r;
}
#endif

#if defined(__CUDA_ARCH__)
// Fp Montgomery squaring: CIOS whose step i adds a_i times (a_i at word i,
// then the words of 2 * sum_{j>i} a_j 2^(32 j)), so every cross product
// a_i a_j is computed once, doubled: the a*a rows take 84 products instead
// of 144 (the Montgomery rows are unchanged), 234 multiply-adds in all
// against 300.  A step's multiplicand is below 2a < 2p, so the running sum
// stays below 3p < 2^384 and the result below 2p, as in the product (the
// rows are restated word by word and checked against a^2 R^-1 mod p in
// tests/test_fp_sqr_rows.py).  Measured on GB300: the 2^20 MSM's
// accumulation 3 % faster.  GB_FP_SQR_OFF selects the product form.
template <int I>
GB_D void sqr_step_fp(uint32_t *even, uint32_t *odd, const uint32_t *a, const uint32_t *d)
{
    typedef FpCfg C;
    constexpr int J0 = (I + 1) & ~1;  // first even word at or above I
    // multiplicand word j of step I: 0 below I, a_I at I, 2 a_{I+1} (without
    // a_I's top bit) at I + 1, the words of 2a above
    auto y = [&](int j) -> uint32_t {
        return j < I ? 0u : j == I ? a[I] : j == I + 1 ? (a[(I + 1) % 12] << 1) : d[j % 12];
    };
    uint32_t ye[6];
#pragma unroll
    for (int k = 0; k < 6; k++) ye[k] = J0 + 2 * k < 12 ? y(J0 + 2 * k) : 0u;
    if constexpr (J0 < 12) sqr_row12<J0>(even, ye, a[I]);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const int j = 2 * k + 1;
        const uint32_t yj = y(j);
        odd[2 * k] = j < I ? 0u : yj * a[I];
        odd[2 * k + 1] = j < I ? 0u : __umulhi(yj, a[I]);
    }
    odd[12] = 0;
    const uint32_t m = even[0] * C::INV;
    row_mac_mod<C>(even, 0, m);
    row_mac_mod<C>(odd, 1, m);
    fold<12>(even, odd);
}

template <int... I>
GB_D void sqr_steps_fp(uint32_t *even, uint32_t *odd, const uint32_t *a, const uint32_t *d,
                       std::integer_sequence<int, I...>)
{
    (sqr_step_fp<I>(even, odd, a, d), ...);
}

GB_D void mont_sqr_fp_device(uint32_t *out, const uint32_t *a)
{
    uint32_t d[12], even[13], odd[13];
    d[0] = a[0] << 1;
#pragma unroll
    for (int j = 1; j < 12; j++) d[j] = (a[j] << 1) | (a[j - 1] >> 31);
#pragma unroll
    for (int i = 0; i < 13; i++) even[i] = 0;
    sqr_steps_fp(even, odd, a, d, std::make_integer_sequence<int, 12>{});
    mont_t<FpCfg>::reduce_once(even, even[12]);
#pragma unroll
    for (int i = 0; i < 12; i++) out[i] = even[i];
}
#endif

#if defined(__CUDA_ARCH__) && !defined(GB_FP_MUL_INLINE)
template <class Cfg>
__device__ __noinline__ mont_t<Cfg> mont_t<Cfg>::sqr_by_value(mont_t<Cfg> a)
{
    mont_t<Cfg> r;
    if constexpr (Cfg::N == 12) mont_sqr_fp_device(r.v, a.v);
    else mont_mul_device<Cfg>(r.v, a.v, a.v);
    return r;
}
#endif

template <class Cfg>
GB_HD void mont_t<Cfg>::mont_mul(uint32_t *out, const uint32_t *a, const uint32_t *b)
{
#if defined(__CUDA_ARCH__) && defined(GB_FP_MUL_CALL)
    if constexpr (Cfg::N == 12) {
        fp_mul_call(out, a, b);
        return;
    }
#endif
#if defined(__CUDA_ARCH__) && defined(GB_FR_MUL_CALL)
    if constexpr (Cfg::N == 8) {
        fr_mul_call(out, a, b);
        return;
    }
#endif
#if defined(__CUDA_ARCH__) && !defined(GB_PORTABLE_MUL)
    mont_mul_device<Cfg>(out, a, b);
#else
    uint32_t t[N + 2];
#pragma unroll
    for (int i = 0; i < N + 2; i++) t[i] = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        uint64_t c = 0;
#pragma unroll
        for (int j = 0; j < N; j++) {
            uint64_t v = (uint64_t)a[j] * b[i] + t[j] + c;
            t[j] = (uint32_t)v;
            c = v >> 32;
        }
        uint64_t v = (uint64_t)t[N] + c;
        t[N] = (uint32_t)v;
        t[N + 1] = (uint32_t)(v >> 32);
        uint32_t m = t[0] * Cfg::INV;
        v = (uint64_t)m * Cfg::mod(0) + t[0];
        c = v >> 32;
#pragma unroll
        for (int j = 1; j < N; j++) {
            v = (uint64_t)m * Cfg::mod(j) + t[j] + c;
            t[j - 1] = (uint32_t)v;
            c = v >> 32;
        }
        v = (uint64_t)t[N] + c;
        t[N - 1] = (uint32_t)v;
        t[N] = t[N + 1] + (uint32_t)(v >> 32);
    }
    reduce_once(t, t[N]);
#pragma unroll
    for (int i = 0; i < N; i++) out[i] = t[i];
#endif
}

using fp_t = mont_t<FpCfg>;
using fr_t = mont_t<FrCfg>;

// Two independent Fp products in one out-of-line call.  The two CIOS chains
// are independent straight-line code, so they interleave and a pair costs
// little more than one product's latency; latency-bound kernels (bucket
// reduction, fix-up, trees), whose warps each run one dependent chain of
// point operations, issue their products in pairs through this.
struct fp_pair {
    fp_t a, b;
};
#if defined(__CUDACC__)
static __device__ __noinline__ fp_pair fp_mul2(fp_t a0, fp_t b0, fp_t a1, fp_t b1)
{
    fp_pair r;
#if defined(__CUDA_ARCH__)
    mont_mul_device<FpCfg>(r.a.v, a0.v, b0.v);
    mont_mul_device<FpCfg>(r.b.v, a1.v, b1.v);
#endif
    return r;
}
#endif

}  // namespace gb
