// Fr NTT / inverse NTT / coset LDE for sm_103a and the NTT entry points of
// the C ABI (midnight-sppark-msm/src/bls12_381_g1_msm.cu:2542-2602,
// 3447-3556, 6488-6502 and the device-vector variants 2604-3440).
//
// Transform: decimation-in-frequency radix-2 stages executed in passes of up
// to 10 stages each; a pass loads 2^g elements that interact in those stages
// into shared memory, runs the g butterfly stages there and writes back.  The
// DIF output is in bit-reversed order; a final pass permutes it to natural
// order and applies the optional scale (1/n for the inverse).  Twiddles
// w^j, j < n/2, are tabulated once per (log_n, direction) and kept resident.
// Within a pass, either each thread runs one radix-2 butterfly per stage
// (a barrier per stage), or each thread holds 4 or 8 elements and runs 2 or 3
// stages in registers between exchanges through shared memory.
#include <atomic>
#include <cstdlib>
#include <map>
#include <string>
#include <mutex>
#include <algorithm>
#include <tuple>
#include <vector>

#include "gb_ntt.cuh"

namespace gb {

static constexpr int kPassBits = 10;

// CTAs per SM the staged passes are compiled for (their register budget)
#ifndef GB_NTT_MIN_BLOCKS
#define GB_NTT_MIN_BLOCKS 3
#endif

// ---------------------------------------------------------------- host math
fr_t host_fr_from_u64(uint64_t v)
{
    fr_t a = fr_t::zero();
    a.v[0] = (uint32_t)v;
    a.v[1] = (uint32_t)(v >> 32);
    return a.to_mont();
}

fr_t host_fr_inverse(const fr_t &a) { return a.inverse(); }

fr_t host_omega(uint32_t log_n, bool inverse)
{
    // ROOT_OF_UNITY (fq.rs:70), Montgomery limbs as u32
    fr_t w;
    const uint32_t root[8] = {0x5f0e466au, 0xb9b58d8cu, 0x1819d7ecu, 0x5b1b4c80u,
                              0x52a31e64u, 0x0af53ae3u, 0x19e9b27bu, 0x5bf3addau};
    for (int i = 0; i < 8; i++) w.v[i] = root[i];
    for (uint32_t i = log_n; i < 32; i++) w = w.sqr();
    return inverse ? w.inverse() : w;
}

// ---------------------------------------------------------------- kernels

__global__ void twiddle_kernel(fr_t *tw, size_t half, fr_t w)
{
    size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= half) return;
    tw[x] = w.pow_u64(x);
}

// One DIF pass over stages s_hi .. s_hi-g+1.  Block b covers the 2^g
// elements i = hi * 2^(s_hi+1) + t * 2^s_lo + lo, t < 2^g.
__global__ void ntt_dif_pass_kernel(fr_t *data, uint32_t log_n, int s_hi, int g, const fr_t *__restrict__ tw)
{
    extern __shared__ fr_t sm[];
    const int s_lo = s_hi - g + 1;
    const size_t n = (size_t)1 << log_n;
    fr_t *d = data + (size_t)blockIdx.y * n;
    const size_t b = blockIdx.x;
    const size_t lo = b & (((size_t)1 << s_lo) - 1);
    const size_t hi = b >> s_lo;
    const size_t base = (hi << (s_hi + 1)) + lo;
    const uint32_t cnt = 1u << g;
    for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) sm[t] = d[base + ((size_t)t << s_lo)];
    __syncthreads();
    for (int s = s_hi; s >= s_lo; s--) {
        const uint32_t h = 1u << (s - s_lo);
        for (uint32_t u = threadIdx.x; u < cnt / 2; u += blockDim.x) {
            uint32_t t0 = (u / h) * 2 * h + (u % h);
            uint32_t t1 = t0 + h;
            size_t j = ((size_t)(t0 % h) << s_lo) + lo;  // i mod 2^s
            fr_t a = sm[t0], c = sm[t1];
            sm[t0] = a + c;
            fr_t diff = a - c;
            if (j) diff = diff * tw[j << (log_n - 1 - s)];
            sm[t1] = diff;
        }
        __syncthreads();
    }
    for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) d[base + ((size_t)t << s_lo)] = sm[t];
}

// The same pass with E = 2^EL elements per thread: the pass's g stages run
// in groups of up to EL (radix-E steps).  For a group over local bits
// [B, B + R), thread u holds the E elements whose local index has, outside
// those bits, the value (u << (EL - R)) | (k >> R), and k & (2^R - 1) inside
// them; it runs the group's R stages in registers, and the block exchanges
// through shared memory between groups.  Needs g >= EL (2^g / E threads).
// Shared memory is padded with one element per 8 (position t + t/8) so the
// strided gathers of the low groups spread over all banks.
__device__ __forceinline__ uint32_t ntt_pad(uint32_t t) { return t + (t >> 3); }

template <int EL, int R>
__device__ __forceinline__ void ntt_reg_group(fr_t *sm, uint32_t u, int B, int s_lo, size_t lo, uint32_t log_n,
                                              const fr_t *__restrict__ tw)
{
    constexpr int E = 1 << EL;
    uint32_t tl[E];
    fr_t x[E];
#pragma unroll
    for (int k = 0; k < E; k++) {
        const uint32_t rest = (u << (EL - R)) | ((uint32_t)k >> R);
        const uint32_t klo = (uint32_t)k & ((1u << R) - 1);
        tl[k] = (rest & ((1u << B) - 1)) | (klo << B) | ((rest >> B) << (B + R));
        x[k] = sm[ntt_pad(tl[k])];
    }
#pragma unroll
    for (int st = 0; st < R; st++) {
        const int p = B + R - 1 - st;  // local bit of this stage
        const int sidx = s_lo + p;     // global stage
        const int hk = 1 << (R - 1 - st);
#pragma unroll
        for (int k = 0; k < E; k++) {
            if ((k & hk) == 0) {
                const int k1 = k + hk;
                const size_t j = ((size_t)(tl[k] & ((1u << p) - 1)) << s_lo) + lo;
                const fr_t a = x[k], c = x[k1];
                x[k] = a + c;
                fr_t diff = a - c;
                if (j) diff = diff * tw[j << (log_n - 1 - sidx)];
                x[k1] = diff;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < E; k++) sm[ntt_pad(tl[k])] = x[k];
}

template <int EL>
__global__ void ntt_dif_pass_reg_kernel(fr_t *data, uint32_t log_n, int s_hi, int g, const fr_t *__restrict__ tw)
{
    extern __shared__ fr_t sm[];
    const int s_lo = s_hi - g + 1;
    const size_t n = (size_t)1 << log_n;
    fr_t *d = data + (size_t)blockIdx.y * n;
    const size_t b = blockIdx.x;
    const size_t lo = b & (((size_t)1 << s_lo) - 1);
    const size_t hi = b >> s_lo;
    const size_t base = (hi << (s_hi + 1)) + lo;
    const uint32_t cnt = 1u << g;
    for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) sm[ntt_pad(t)] = d[base + ((size_t)t << s_lo)];
    __syncthreads();
    int top = g;  // local bits still to process: [0, top)
    while (top > 0) {
        if (top >= EL) {
            ntt_reg_group<EL, EL>(sm, threadIdx.x, top - EL, s_lo, lo, log_n, tw);
            top -= EL;
        } else if (EL == 3 && top == 2) {
            ntt_reg_group<EL, (EL == 3 ? 2 : 1)>(sm, threadIdx.x, 0, s_lo, lo, log_n, tw);
            top = 0;
        } else {
            ntt_reg_group<EL, 1>(sm, threadIdx.x, 0, s_lo, lo, log_n, tw);
            top = 0;
        }
        __syncthreads();
    }
    for (uint32_t t = threadIdx.x; t < cnt; t += blockDim.x) d[base + ((size_t)t << s_lo)] = sm[ntt_pad(t)];
}

// ---------------------------------------------------------------- staged passes
// The pass with its twiddles staged in shared memory.  A CTA holds Q = 2^q
// sub-blocks of 2^g elements (Q * 2^g <= 1024) and its own contiguous chunk
// of the pass's twiddle table, which one thread copies in with a TMA bulk
// copy (cp.async.bulk + mbarrier) while the block gathers the data.
//
// Pass twiddle table: for a pass over global stages s_lo .. s_lo+g-1, chunk
// lo (lo < 2^s_lo, the sub-block's offset below the pass) has 2^g entries;
// entry m = 2^p + t' (t' < 2^p) is the twiddle of local stage p for the
// butterflies whose local index is t' mod 2^p:
//     w^(((t' << s_lo) + lo) << (log_n - 1 - s_lo - p))
// (entry 0 is unused).  A pass with s_lo = 0 has the single chunk lo = 0.
//
// Shared memory is addressed in 16-byte chunks.  Element t of a sub-block
// occupies chunks 2t and 2t+1 of its 128-byte row r = t/4, permuted inside
// the row by r ^ (r >> 1) ^ (r >> 2) ^ (r >> 4) and, for the data, by a
// twist of the sub-block number, so that the gathers of every radix-2^R
// group (the remainder group first, at the top bits), the twiddle reads and
// the strided global loads are free of bank conflicts for g >= 5 (the last
// pass's bit-reversed reads keep a few).  The global
// twiddle table is stored in the same permuted order, so the bulk copy
// lands it ready to use.
__host__ __device__ __forceinline__ uint32_t ntt_swz_row(uint32_t r) { return (r ^ (r >> 1) ^ (r >> 2) ^ (r >> 4)) & 7u; }
__host__ __device__ __forceinline__ uint32_t ntt_twist(uint32_t q) { return (q & 1u) | ((q & 2u) << 1) | ((q & 4u) >> 1); }
__host__ __device__ __forceinline__ uint32_t ntt_chunk(uint32_t t, uint32_t h, uint32_t x)
{
    const uint32_t r = t >> 2;
    return (r << 3) | ((((t & 3u) << 1) | h) ^ ntt_swz_row(r) ^ x);
}

__device__ __forceinline__ fr_t ntt_ld(const uint4 *s, uint32_t t, uint32_t x)
{
    const uint4 a = s[ntt_chunk(t, 0, x)], b = s[ntt_chunk(t, 1, x)];
    fr_t r;
    r.v[0] = a.x, r.v[1] = a.y, r.v[2] = a.z, r.v[3] = a.w;
    r.v[4] = b.x, r.v[5] = b.y, r.v[6] = b.z, r.v[7] = b.w;
    return r;
}

__device__ __forceinline__ void ntt_st(uint4 *s, uint32_t t, uint32_t x, const fr_t &v)
{
    s[ntt_chunk(t, 0, x)] = make_uint4(v.v[0], v.v[1], v.v[2], v.v[3]);
    s[ntt_chunk(t, 1, x)] = make_uint4(v.v[4], v.v[5], v.v[6], v.v[7]);
}

// Butterfly arithmetic of the staged passes.  The values between stages and
// passes are kept in [0, 2r) (Harvey's lazy butterflies): a product x * w
// with x < 2r and a twiddle w < r is below 2r without the Montgomery
// product's final subtraction, and sums and differences are reduced mod 2r;
// the last pass reduces its outputs to [0, r).  Measured on GB300 this makes
// the transform 7% faster than reducing every result; GB_NTT_EAGER selects
// the fully reduced form.
#if !defined(GB_NTT_EAGER)
__device__ __forceinline__ fr_t bfly_add(const fr_t &a, const fr_t &b)
{
    fr_t r;
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
        : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]), "r"(a.v[7]),
          "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]), "r"(b.v[6]), "r"(b.v[7]));
    // 2r = 0xe7db4ea6 533afa90 6673b010 1343b00a a77b4805 fffcb7fd fffffffe 00000002
    asm("sub.cc.u32 %0, %9, 0x00000002;\n\t"
        "subc.cc.u32 %1, %10, 0xfffffffe;\n\t"
        "subc.cc.u32 %2, %11, 0xfffcb7fd;\n\t"
        "subc.cc.u32 %3, %12, 0xa77b4805;\n\t"
        "subc.cc.u32 %4, %13, 0x1343b00a;\n\t"
        "subc.cc.u32 %5, %14, 0x6673b010;\n\t"
        "subc.cc.u32 %6, %15, 0x533afa90;\n\t"
        "subc.cc.u32 %7, %16, 0xe7db4ea6;\n\t"
        "subc.u32 %8, %17, 0;"
        : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7]), "=r"(br)
        : "r"(s[0]), "r"(s[1]), "r"(s[2]), "r"(s[3]), "r"(s[4]), "r"(s[5]), "r"(s[6]), "r"(s[7]), "r"(c));
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = br ? s[i] : t[i];
    return r;
}

__device__ __forceinline__ fr_t bfly_sub(const fr_t &a, const fr_t &b)
{
    fr_t r;
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
        : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]), "r"(a.v[7]),
          "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]), "r"(b.v[6]), "r"(b.v[7]));
    asm("add.cc.u32 %0, %8, 0x00000002;\n\t"
        "addc.cc.u32 %1, %9, 0xfffffffe;\n\t"
        "addc.cc.u32 %2, %10, 0xfffcb7fd;\n\t"
        "addc.cc.u32 %3, %11, 0xa77b4805;\n\t"
        "addc.cc.u32 %4, %12, 0x1343b00a;\n\t"
        "addc.cc.u32 %5, %13, 0x6673b010;\n\t"
        "addc.cc.u32 %6, %14, 0x533afa90;\n\t"
        "addc.u32 %7, %15, 0xe7db4ea6;"
        : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7])
        : "r"(d[0]), "r"(d[1]), "r"(d[2]), "r"(d[3]), "r"(d[4]), "r"(d[5]), "r"(d[6]), "r"(d[7]));
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = br ? t[i] : d[i];
    return r;
}

__device__ __forceinline__ fr_t bfly_mul(const fr_t &x, const fr_t &w)
{
    fr_t r;
#if defined(__CUDA_ARCH__)
    mont_mul_device<FrCfg, false>(r.v, x.v, w.v);
#endif
    return r;
}

// [0, 2r) -> [0, r)
__device__ __forceinline__ fr_t bfly_out(fr_t v)
{
    fr_t::reduce_once(v.v, 0);
    return v;
}
#else
__device__ __forceinline__ fr_t bfly_add(const fr_t &a, const fr_t &b) { return a + b; }
__device__ __forceinline__ fr_t bfly_sub(const fr_t &a, const fr_t &b) { return a - b; }
__device__ __forceinline__ fr_t bfly_mul(const fr_t &x, const fr_t &w) { return x * w; }
__device__ __forceinline__ fr_t bfly_out(fr_t v) { return v; }
#endif

// chunk(t, h, x) = lin(t) ^ h ^ x, with lin linear over GF(2) in the bits
// of t: addresses of elements whose indices differ in known bits are found
// by XOR-ing precomputed images of those bits.
__device__ __forceinline__ uint32_t ntt_lin(uint32_t t)
{
    const uint32_t r = t >> 2;
    return (r << 3) | (((t & 3u) << 1) ^ ntt_swz_row(r));
}

__device__ __forceinline__ fr_t ntt_ld_c(const uint4 *s, uint32_t c)
{
    const uint4 a = s[c], b = s[c ^ 1u];
    fr_t r;
    r.v[0] = a.x, r.v[1] = a.y, r.v[2] = a.z, r.v[3] = a.w;
    r.v[4] = b.x, r.v[5] = b.y, r.v[6] = b.z, r.v[7] = b.w;
    return r;
}

__device__ __forceinline__ void ntt_st_c(uint4 *s, uint32_t c, const fr_t &v)
{
    s[c] = make_uint4(v.v[0], v.v[1], v.v[2], v.v[3]);
    s[c ^ 1u] = make_uint4(v.v[4], v.v[5], v.v[6], v.v[7]);
}

// One radix-2^R group over local bits [B, B + R) of a sub-block; thread u
// (within the sub-block) holds E = 2^EL elements, which need B >= EL - R.
// Element k of the thread has local index
//     tl[k] = tl[0] ^ (k >> R) ^ ((k mod 2^R) << B)
// (the bits of k >> R sit below B), so its chunk address is lin(tl[0]) XOR
// images of single bits.  The butterflies of one stage that share a twiddle
// (same local index mod 2^p) read it once.
template <int EL, int R>
__device__ __forceinline__ void ntt_tw_group(uint4 *sd, const uint4 *stw, uint32_t u, int B, uint32_t twist,
                                             bool lo_zero)
{
    constexpr int E = 1 << EL;
    const uint32_t rest0 = u << (EL - R);
    const uint32_t tl0 = (rest0 & ((1u << B) - 1)) | ((rest0 >> B) << (B + R));
    const uint32_t base = ntt_lin(tl0) ^ twist;
    uint32_t img_b[R];  // lin(1 << (B + j))
#pragma unroll
    for (int j = 0; j < R; j++) img_b[j] = ntt_lin(1u << (B + j));
    // lin of the bits k >> R (below B): constants
    auto img_lo = [](uint32_t v) { return ntt_lin(v); };
    uint32_t off[E];
    fr_t x[E];
#pragma unroll
    for (int k = 0; k < E; k++) {
        uint32_t o = img_lo((uint32_t)k >> R);
#pragma unroll
        for (int j = 0; j < R; j++)
            if ((k >> j) & 1) o ^= img_b[j];
        off[k] = o;
        x[k] = ntt_ld_c(sd, base ^ o);
    }
#pragma unroll
    for (int st = 0; st < R; st++) {
        const int p = B + R - 1 - st;  // local bit of this stage
        const int lh = R - 1 - st, hk = 1 << lh;
        // twiddle entry of key (kl, kr): m = 2^p ^ (tl0 mod 2^p) ^ kr ^ (kl << B)
        const uint32_t tp0 = tl0 & ((1u << p) - 1);
        const uint32_t tbase = ntt_lin((1u << p) ^ tp0);
        fr_t w[E / 2];
        bool one[E / 2];
#pragma unroll
        for (int key = 0; key < (hk << (EL - R)); key++) {
            const uint32_t kl = (uint32_t)key & (hk - 1), kr = (uint32_t)key >> lh;
            uint32_t o = img_lo(kr);
#pragma unroll
            for (int j = 0; j < lh; j++)
                if ((kl >> j) & 1) o ^= img_b[j];
            one[key] = lo_zero && (tp0 | kr | kl) == 0;
            w[key] = ntt_ld_c(stw, tbase ^ o);
        }
#pragma unroll
        for (int k = 0; k < E; k++) {
            if ((k & hk) == 0) {
                const int k1 = k + hk;
                const int key = (k & (hk - 1)) | ((k >> R) << lh);
                const fr_t a = x[k], c = x[k1];
                x[k] = bfly_add(a, c);
                fr_t diff = bfly_sub(a, c);
                if (!one[key]) diff = bfly_mul(diff, w[key]);
                x[k1] = diff;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < E; k++) ntt_st_c(sd, base ^ off[k], x[k]);
}

// Spin limits of the twiddle copy's waits.  The first wait gives up after
// the launch's `spins` polls (kWaitSpins unless a test lowers it), counts a
// timeout in the call's status word and skips the butterflies; the CTA then
// waits again, up to kDrainSpins polls, for the copy still in flight, so
// that it does not leave while the copy can still write its shared memory.
// The copy's source lies inside the pass's twiddle table and its size is
// that of the CTA's chunk (at most 2^10 entries of 32 bytes), so in a
// working GPU it lands within microseconds.
static constexpr unsigned kWaitSpins = 1u << 24;
static constexpr unsigned kDrainSpins = 1u << 26;

// bounded wait on the phase of an mbarrier with the given parity; true when
// the phase completed
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, unsigned spins)
{
    for (unsigned i = 0; i < spins; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Factors by position i (natural order) of a transform, applied by the last
// pass to its outputs or by a fused first pass to its inputs:
//   on == 1: f[i mod 3] (the ZETA coset distribution times a scale);
//   on == 2: pw_hi[i >> lo_bits] * pw_lo[i mod 2^lo_bits] (powers of a
//            coset shift from two tables, any scale folded into pw_hi);
//   on == 0: none.
struct ntt_factors {
    fr_t f[3];
    int on;
    const fr_t *pw_lo = nullptr, *pw_hi = nullptr;
    uint32_t lo_bits = 0;
};

__device__ __forceinline__ fr_t ntt_factor(const ntt_factors &fac, size_t i)
{
    fr_t f;
    if (fac.on == 2) {
        const fr_t lo = fac.pw_lo[i & (((size_t)1 << fac.lo_bits) - 1)];
        const fr_t hi = fac.pw_hi[i >> fac.lo_bits];
        f = hi * lo;
    } else {
        const uint32_t c = (uint32_t)(i % 3);
#pragma unroll
        for (int w = 0; w < 8; w++) f.v[w] = c == 0 ? fac.f[0].v[w] : c == 1 ? fac.f[1].v[w] : fac.f[2].v[w];
    }
    return f;
}

// The input of a fused first pass: `count` polynomials of in_len values
// each at src (values past in_len read as zero: the zero padding of a coset
// LDE), each value multiplied by fac's factor of its position when fac.on.
struct ntt_input {
    const fr_t *src;
    size_t in_len;
    ntt_factors fac;
};

__device__ __forceinline__ uint32_t brev_bits(uint32_t x, int bits) { return bits ? __brev(x) >> (32 - bits) : 0u; }

// One staged pass.  src and dst may alias (in place) except in the LAST
// pass, which reads the DIF order from src and writes natural order to dst.
//
// Grid, for a pass with s_lo > 0: CTA c covers sub-blocks (c / count) * Q ..
// + Q - 1 of transform c % count, so CTAs sharing a twiddle chunk run
// together.  For s_lo = 0 the batch is one run of count * 2^(log_n - g)
// sub-blocks and CTA c covers run positions c * Q .. c * Q + Q - 1 (those
// past the end are skipped).  In the LAST pass run position F of transform
// F / NB (NB = 2^(log_n - g) sub-blocks per transform) is the sub-block whose
// outputs land in column F mod NB of the natural order, i.e. sub-block
// bitrev(F mod NB): element t of it is output bitrev(t) * NB + (F mod NB),
// so the Q sub-blocks of a CTA write Q adjacent outputs per row.
//
// ntt_tw_piece runs the part of a pass that CTA `cta` of the per-pass grid
// covers; it returns false (for every thread) when the twiddle copy did not
// land.  QUEUE selects the form that the persistent work-queue kernel runs:
// the block may be wider than the piece (the extra threads sit out the
// butterfly groups), the sources are read through L2 because other CTAs of
// the same launch wrote them, and the mbarrier completes one phase per piece.
// LOADF selects the fused first pass of a coset LDE or coset transform: the
// sub-blocks are gathered from `in` (see ntt_input) instead of src; it needs
// s_lo > 0, i.e. a transform of two or more passes.  A twiddle copy that
// does not land within `spins` polls is counted in *status.
template <int EL, bool LAST, bool QUEUE, bool LOADF = false>
__device__ __forceinline__ bool ntt_tw_piece(const fr_t *src, fr_t *dst, uint32_t log_n, int s_hi, int g, int q,
                                             size_t count, const fr_t *__restrict__ twt, const ntt_factors &fac,
                                             size_t cta, uint4 *smem, uint32_t mbar, uint32_t parity, int &copy_ok,
                                             uint32_t *status, unsigned spins, const ntt_input &in = ntt_input{})
{
    const int s_lo = s_hi - g + 1;
    const uint32_t sub = 1u << g, Q = 1u << q, nd = Q << g;
    const size_t n = (size_t)1 << log_n;
    const uint32_t tw_entries = s_lo > 0 ? nd : sub;
    uint4 *sd = smem;
    uint4 *stw = smem + 2 * (size_t)nd;
    const int nb_log = (int)log_n - g;                 // log2 sub-blocks per transform
    const size_t total = count << nb_log;              // sub-blocks in the batch
    const bool q_fast = !LAST || nb_log >= q;          // LAST: Q adjacent columns of one transform

    size_t poly = 0, b0 = 0;
    const fr_t *twsrc = twt;
    if (s_lo > 0) {
        poly = cta % count;
        b0 = (size_t)(cta / count) << q;
        twsrc = twt + ((b0 & (((size_t)1 << s_lo) - 1)) << g);
    } else {
        b0 = cta << q;
    }

    if (threadIdx.x == 0) {
        // the previous piece's generic reads of the twiddle buffer are done
        // (barrier); order them before the async-proxy write
        if (QUEUE) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const uint32_t bytes = tw_entries * (uint32_t)sizeof(fr_t);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                (uint32_t)__cvta_generic_to_shared(stw)),
            "l"(twsrc), "r"(bytes), "r"(mbar)
            : "memory");
    }

    // gather the sub-blocks into shared memory
    for (uint32_t idx = threadIdx.x; idx < nd; idx += blockDim.x) {
        uint32_t qq, t;
        size_t addr;
        bool valid = true;
        if (s_lo > 0) {
            qq = idx & (Q - 1);
            t = idx >> q;
            const size_t b = b0 + qq;
            addr = poly * n + ((b >> s_lo) << (s_hi + 1)) + (b & (((size_t)1 << s_lo) - 1)) + ((size_t)t << s_lo);
        } else {
            qq = idx >> g;
            t = idx & (sub - 1);
            const size_t F = b0 + qq;
            valid = F < total;
            if (LAST) {
                const size_t col = F & (((size_t)1 << nb_log) - 1);
                addr = ((F >> nb_log) << log_n) + ((size_t)brev_bits((uint32_t)col, nb_log) << g) + t;
            } else {
                addr = (F << g) + t;
            }
        }
        fr_t v = fr_t::zero();
        if (LOADF) {
            // first pass: s_hi = log_n - 1, so the position is addr - poly * n
            const size_t i = addr - poly * n;
            if (i < in.in_len) {
                v = in.src[poly * in.in_len + i];
                if (in.fac.on) v = v * ntt_factor(in.fac, i);
            }
        } else if (valid) {
            if (QUEUE) {
                const uint4 *p = reinterpret_cast<const uint4 *>(src + addr);
                const uint4 lo = __ldcg(p), hi = __ldcg(p + 1);
                v.v[0] = lo.x, v.v[1] = lo.y, v.v[2] = lo.z, v.v[3] = lo.w;
                v.v[4] = hi.x, v.v[5] = hi.y, v.v[6] = hi.z, v.v[7] = hi.w;
            } else {
                v = src[addr];
            }
        }
        ntt_st(sd + 2 * (size_t)qq * sub, t, ntt_twist(qq & 7u), v);
    }
    if (threadIdx.x == 0) {
        bool ok = mbar_wait(mbar, parity, spins);
        if (!ok) {
            if (status) atomicAdd(status, 1u);
            mbar_wait(mbar, parity, kDrainSpins);  // let the copy in flight land before the CTA goes on
        }
        copy_ok = ok;
    }
    __syncthreads();
    if (!copy_ok) return false;

    // radix-2^EL groups; the remainder group first, at the top bits
    {
        const uint32_t per_sub = sub >> EL;  // threads per sub-block; nd >> EL threads take part
        const bool part = !QUEUE || threadIdx.x < (nd >> EL);
        const uint32_t qq = part ? threadIdx.x / per_sub : 0, ul = threadIdx.x % per_sub;
        uint4 *sdq = sd + 2 * (size_t)qq * sub;
        const uint4 *stq = stw + (s_lo > 0 ? 2 * (size_t)qq * sub : 0);
        const uint32_t twist = ntt_twist(qq & 7u);
        const bool lo_zero = s_lo == 0 || (((b0 + qq) & (((size_t)1 << s_lo) - 1)) == 0);
        int top = g;
        const int rem = g % EL;
        if (rem) {
            if (!part) {
            } else if (EL == 3 && rem == 2) {
                ntt_tw_group<EL, (EL == 3 ? 2 : 1)>(sdq, stq, ul, g - rem, twist, lo_zero);
            } else {
                ntt_tw_group<EL, 1>(sdq, stq, ul, g - rem, twist, lo_zero);
            }
            top -= rem;
            __syncthreads();
        }
        while (top > 0) {
            if (part) ntt_tw_group<EL, EL>(sdq, stq, ul, top - EL, twist, lo_zero);
            top -= EL;
            __syncthreads();
        }
    }

    // write back
    for (uint32_t idx = threadIdx.x; idx < nd; idx += blockDim.x) {
        uint32_t qq, t;
        size_t addr;
        if (s_lo > 0) {
            qq = idx & (Q - 1);
            t = idx >> q;
            const size_t b = b0 + qq;
            addr = poly * n + ((b >> s_lo) << (s_hi + 1)) + (b & (((size_t)1 << s_lo) - 1)) + ((size_t)t << s_lo);
        } else if (!LAST) {
            qq = idx >> g;
            t = idx & (sub - 1);
            if (b0 + qq >= total) continue;
            addr = ((b0 + qq) << g) + t;
        } else {
            uint32_t r;  // output row
            if (q_fast) {
                qq = idx & (Q - 1);
                r = idx >> q;
            } else {
                qq = idx >> g;
                r = idx & (sub - 1);
            }
            const size_t F = b0 + qq;
            if (F >= total) continue;
            t = brev_bits(r, g);
            const size_t col = F & (((size_t)1 << nb_log) - 1);
            const size_t i_nat = ((size_t)r << nb_log) + col;
            addr = ((F >> nb_log) << log_n) + i_nat;
            fr_t v = ntt_ld(sd + 2 * (size_t)qq * sub, t, ntt_twist(qq & 7u));
            // x * f with x < 2r, f < r is fully reduced by the product
            if (!fac.on) v = bfly_out(v);
            else v = v * ntt_factor(fac, i_nat);
            dst[addr] = v;
            continue;
        }
        dst[addr] = ntt_ld(sd + 2 * (size_t)qq * sub, t, ntt_twist(qq & 7u));
    }
    return true;
}

template <int EL, bool LAST, bool LOADF = false>
__global__ void __launch_bounds__(1024 >> EL, GB_NTT_MIN_BLOCKS)
    ntt_dif_pass_tw_kernel(const fr_t *src, fr_t *dst, uint32_t log_n, int s_hi, int g, int q, size_t count,
                           const fr_t *__restrict__ twt, ntt_factors fac, ntt_input in, uint32_t *status,
                           unsigned spins)
{
    extern __shared__ uint4 smem[];
    __shared__ uint64_t mbar_store;
    __shared__ int copy_ok;
    const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(&mbar_store);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    ntt_tw_piece<EL, LAST, false, LOADF>(src, dst, log_n, s_hi, g, q, count, twt, fac, blockIdx.x, smem, mbar, 0,
                                         copy_ok, status, spins, in);
}

// ---------------------------------------------------------------- work queue
// A ragged batch of transforms (different sizes) in one persistent launch.
// The host lists every piece of every pass of every transform as a work item,
// all first-pass pieces first, then all second-pass pieces, and so on.  Each
// CTA takes the next item from a device counter; a piece of pass p > 0 waits
// until all pieces of pass p - 1 of its transform are done (a per-(transform,
// pass) completion counter).  Items are taken in list order, so an item only
// ever waits for items taken earlier by CTAs that are running, and those wait
// only for items taken before them: the launch cannot deadlock whatever the
// number of resident CTAs.  Every wait is bounded; a wait that runs out, or a
// twiddle copy that does not land, raises the abort flag, which ends the
// launch early and is reported to the host.
struct ntt_qpass {
    const fr_t *src;
    fr_t *dst;
    const fr_t *tw;
    uint32_t pieces;
    int s_hi, g, q;
};

struct ntt_qjob {
    ntt_qpass pass[3];
    ntt_factors fac;
    uint32_t log_n, npass, counter;  // counter: index of pass 0's completion counter
};

// control words of one launch: next item, abort flag, then the completion
// counters (zeroed before the launch)
enum { NTT_Q_NEXT = 0, NTT_Q_ABORT = 1, NTT_Q_COUNTERS = 2 };
static constexpr unsigned kQueueSpins = 1u << 22;
static constexpr uint32_t kQueuePieceBits = 24;

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <int EL>
__global__ void __launch_bounds__(1024 >> EL, GB_NTT_MIN_BLOCKS)
    ntt_queue_kernel(const ntt_qjob *__restrict__ jobs, const uint2 *__restrict__ items, uint32_t n_items,
                     uint32_t *ctl, uint32_t *status, unsigned spins)
{
    extern __shared__ uint4 smem[];
    __shared__ uint64_t mbar_store;
    __shared__ int copy_ok;
    __shared__ uint32_t cur;
    __shared__ int go;
    const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(&mbar_store);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    uint32_t parity = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t it = atomicAdd(&ctl[NTT_Q_NEXT], 1u);
            int ok = it < n_items && !ld_acquire_u32(&ctl[NTT_Q_ABORT]);
            if (ok) {
                const uint2 w = items[it];
                const uint32_t pass = w.y >> kQueuePieceBits;
                if (pass > 0) {
                    const ntt_qjob &J = jobs[w.x];
                    const uint32_t need = J.pass[pass - 1].pieces;
                    const uint32_t *c = &ctl[NTT_Q_COUNTERS + J.counter + pass - 1];
                    unsigned i = 0;
                    for (; i < kQueueSpins; i++) {
                        if (ld_acquire_u32(c) >= need) break;
                        if (ld_acquire_u32(&ctl[NTT_Q_ABORT])) {
                            ok = 0;
                            break;
                        }
                        __nanosleep(64);
                    }
                    if (i == kQueueSpins) {
                        atomicAdd(&status[1], 1u);
                        atomicExch(&ctl[NTT_Q_ABORT], 1u);
                        ok = 0;
                    }
                }
            }
            cur = it;
            go = ok;
        }
        __syncthreads();
        if (!go) break;
        const uint2 w = items[cur];
        const uint32_t pass = w.y >> kQueuePieceBits, piece = w.y & ((1u << kQueuePieceBits) - 1);
        const ntt_qjob &J = jobs[w.x];
        const ntt_qpass &P = J.pass[pass];
        bool ok;
        if (pass + 1 == J.npass) {
            ok = ntt_tw_piece<EL, true, true>(P.src, P.dst, J.log_n, P.s_hi, P.g, P.q, 1, P.tw, J.fac, piece, smem,
                                              mbar, parity, copy_ok, status, spins);
        } else {
            const ntt_factors none{{fr_t::one(), fr_t::one(), fr_t::one()}, 0};
            ok = ntt_tw_piece<EL, false, true>(P.src, P.dst, J.log_n, P.s_hi, P.g, P.q, 1, P.tw, none, piece, smem,
                                               mbar, parity, copy_ok, status, spins);
        }
        parity ^= 1u;
        __syncthreads();  // every store of the piece is issued
        if (threadIdx.x == 0) {
            if (!ok) atomicExch(&ctl[NTT_Q_ABORT], 1u);
            __threadfence();
            atomicAdd(&ctl[NTT_Q_COUNTERS + J.counter + pass], 1u);
        }
        if (!ok) break;
    }
}

// pass twiddle table entries from the base table tw[e] = w^e (e < n/2),
// written in the permuted chunk order (see above)
__global__ void pass_twiddle_kernel(fr_t *out, const fr_t *__restrict__ tw, uint32_t log_n, int s_lo, int g,
                                    size_t chunks)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t sub = (size_t)1 << g;
    if (i >= chunks * sub) return;
    const size_t lo = i >> g;
    const uint32_t m = (uint32_t)(i & (sub - 1));
    fr_t v = fr_t::one();
    if (m) {
        const int p = 31 - __clz(m);
        const size_t tp = m - (1u << p);
        const size_t e = ((tp << s_lo) + lo) << (log_n - 1 - s_lo - p);
        v = tw[e];
    }
    uint4 *o = reinterpret_cast<uint4 *>(out + (lo << g));
    o[ntt_chunk(m, 0, 0)] = make_uint4(v.v[0], v.v[1], v.v[2], v.v[3]);
    o[ntt_chunk(m, 1, 0)] = make_uint4(v.v[4], v.v[5], v.v[6], v.v[7]);
}

__device__ __forceinline__ size_t bitrev_n(size_t x, uint32_t bits)
{
    return (size_t)(__brevll((unsigned long long)x) >> (64 - bits));
}

// bit-reversal permutation (in place, by swapping) and optional scaling
__global__ void bitrev_scale_kernel(fr_t *data, uint32_t log_n, bool do_scale, fr_t scale)
{
    const size_t n = (size_t)1 << log_n;
    fr_t *d = data + (size_t)blockIdx.y * n;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t r = log_n ? bitrev_n(i, log_n) : 0;
    if (i < r) {
        fr_t a = d[i], c = d[r];
        if (do_scale) { a = a * scale; c = c * scale; }
        d[i] = c;
        d[r] = a;
    } else if (i == r && do_scale) {
        d[i] = d[i] * scale;
    }
}

__global__ void mul_assign_kernel(fr_t *d, fr_t k, size_t len)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) d[i] = d[i] * k;
}

__global__ void mul_assign_zeta_kernel(fr_t *d, fr_t first, fr_t second, size_t len, size_t period_len)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    size_t c = (i % period_len) % 3;
    if (c == 1) d[i] = d[i] * first;
    else if (c == 2) d[i] = d[i] * second;
}

__global__ void mul_assign_repeating_kernel(fr_t *d, const fr_t *__restrict__ f, size_t flen, size_t len)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) d[i] = d[i] * f[i % flen];
}

__global__ void scale_zeta_kernel(fr_t *d, fr_t scale, fr_t first, fr_t second, size_t len, size_t period_len)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    fr_t v = d[i] * scale;
    size_t c = (i % period_len) % 3;
    if (c == 1) v = v * first;
    else if (c == 2) v = v * second;
    d[i] = v;
}

// d[i] *= f[(i mod period_len) mod 3]
__global__ void mul_period3_kernel(fr_t *d, fr_t f0, fr_t f1, fr_t f2, size_t len, size_t period_len)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    const size_t c = (i % period_len) % 3;
    d[i] = d[i] * (c == 0 ? f0 : c == 1 ? f1 : f2);
}

__global__ void c2e_prepare_kernel(fr_t *out, const fr_t *__restrict__ in, fr_t first, fr_t second,
                                   size_t input_len, size_t output_len, size_t count)
{
    size_t f = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= output_len * count) return;
    size_t li = f % output_len, p = f / output_len;
    if (li >= input_len) {
        out[f] = fr_t::zero();
        return;
    }
    fr_t v = in[p * input_len + li];
    size_t c = li % 3;
    if (c == 1) v = v * first;
    else if (c == 2) v = v * second;
    out[f] = v;
}

// d[i] *= fac's factor of position i mod period_len (mode 1 or 2)
__global__ void mul_factors_kernel(fr_t *d, ntt_factors fac, size_t len, size_t period_len)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    d[i] = d[i] * ntt_factor(fac, i % period_len);
}

// out[p][i] = i < in_len ? in[p][i] * factor(i) : 0 for count polynomials of
// out_len values (the padded input of an unfused coset LDE); in may equal out
// when in_len == out_len
__global__ void c2e_factors_kernel(fr_t *out, const fr_t *in, ntt_factors fac, size_t input_len, size_t output_len,
                                   size_t count)
{
    const size_t f = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= output_len * count) return;
    const size_t li = f % output_len, p = f / output_len;
    fr_t v = fr_t::zero();
    if (li < input_len) {
        v = in[p * input_len + li];
        if (fac.on) v = v * ntt_factor(fac, li);
    }
    out[f] = v;
}

// out[j] = scale * base^j
__global__ void powers_table_kernel(fr_t *out, fr_t base, fr_t scale, size_t len)
{
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < len) out[j] = scale * base.pow_u64(j);
}

// ---------------------------------------------------------------- host side

// The first twiddle wait's poll limit for every launch; a test lowers it
// through gb_ntt_wait_limit_set to make the wait run out on purpose (the
// copy then still lands within the drain wait, see kDrainSpins).
static std::atomic<long long> g_wait_spins_override{-1};
static unsigned wait_spins()
{
    const long long v = g_wait_spins_override.load(std::memory_order_relaxed);
    return v < 0 ? kWaitSpins : (unsigned)v;
}

// The calling lane's wait-status words (see lane_status_device), which the
// kernels of an NTT call add to when a bounded wait runs out.
struct ntt_status {
    uint32_t *p;
    ntt_status() : p(lane_status_device()) {}
    uint32_t *ptr() const { return p; }
};

namespace {
std::mutex g_tw_mu;
std::map<std::tuple<int, uint32_t, bool>, fr_t *> g_tw;

const fr_t *twiddles(uint32_t log_n, bool inverse, cudaStream_t s)
{
    int dev = current_device();
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto key = std::make_tuple(dev, log_n, inverse);
    auto it = g_tw.find(key);
    if (it != g_tw.end()) return it->second;
    size_t half = log_n ? ((size_t)1 << (log_n - 1)) : 1;
    fr_t *tw = nullptr;
    GB_CUDA_OK(cudaMalloc(&tw, half * sizeof(fr_t)));
    twiddle_kernel<<<blocks_for(half, 256), 256, 0, s>>>(tw, half, host_omega(log_n, inverse));
    GB_CHECK_LAUNCH();
    GB_CUDA_OK(cudaStreamSynchronize(s));
    g_tw[key] = tw;
    return tw;
}

void set_ntt_smem()
{
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(ntt_dif_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (1 << kPassBits) * (int)sizeof(fr_t));
        cudaFuncSetAttribute(ntt_dif_pass_reg_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (1 << kPassBits) / 8 * 9 * (int)sizeof(fr_t));
        cudaFuncSetAttribute(ntt_dif_pass_reg_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (1 << kPassBits) / 8 * 9 * (int)sizeof(fr_t));
        const int staged = 2 * (1 << kPassBits) * (int)sizeof(fr_t);
        cudaFuncSetAttribute(ntt_dif_pass_tw_kernel<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged);
        cudaFuncSetAttribute(ntt_dif_pass_tw_kernel<3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged);
        cudaFuncSetAttribute(ntt_dif_pass_tw_kernel<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged);
        cudaFuncSetAttribute(ntt_dif_pass_tw_kernel<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged);
        cudaFuncSetAttribute(ntt_dif_pass_tw_kernel<2, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             staged);
        cudaFuncSetAttribute(ntt_dif_pass_tw_kernel<3, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             staged);
        cudaFuncSetAttribute(ntt_queue_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, staged);
    });
}

static int sm_count()
{
    static int n = 0;
    if (!n) GB_CUDA_OK(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, current_device()));
    return n;
}

// (s_hi, g) of each pass: ceil(log_n / 10) passes of near-equal size, the
// larger ones first
std::vector<std::pair<int, int>> pass_split(uint32_t log_n)
{
    std::vector<std::pair<int, int>> out;
    const int L = (int)log_n, P = (L + kPassBits - 1) / kPassBits;
    int s_hi = L - 1;
    for (int i = 0; i < P; i++) {
        const int g = L / P + (i < L % P ? 1 : 0);
        out.emplace_back(s_hi, g);
        s_hi -= g;
    }
    return out;
}

std::map<std::tuple<int, uint32_t, bool, int>, fr_t *> g_pass_tw;

// the pass twiddle table of the pass with top stage s_hi (cached per device)
const fr_t *pass_twiddles(uint32_t log_n, bool inverse, int s_hi, int g, const fr_t *tw, cudaStream_t s)
{
    int dev = current_device();
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto key = std::make_tuple(dev, log_n, inverse, s_hi);
    auto it = g_pass_tw.find(key);
    if (it != g_pass_tw.end()) return it->second;
    const int s_lo = s_hi - g + 1;
    const size_t chunks = s_lo > 0 ? (size_t)1 << s_lo : 1;
    const size_t entries = chunks << g;
    fr_t *t = nullptr;
    GB_CUDA_OK(cudaMalloc(&t, entries * sizeof(fr_t)));
    pass_twiddle_kernel<<<blocks_for(entries, 256), 256, 0, s>>>(t, tw, log_n, s_lo, g, chunks);
    GB_CHECK_LAUNCH();
    GB_CUDA_OK(cudaStreamSynchronize(s));
    g_pass_tw[key] = t;
    return t;
}
}  // namespace

// The staged-twiddle transform (variants 4 and 5: 4 or 8 elements per
// thread), natural order out with the output factors applied.  With two or
// more passes the first pass writes to a scratch buffer, the middle ones work
// there in place and the last one writes natural order back to d, so no
// separate bit-reversal pass is needed; a single pass works in place.  With
// `in` (two or more passes only) the first pass gathers its inputs from
// in->src instead of d (zero padding and input factors, see ntt_input), so d
// is written but never read.
static void ntt_staged(fr_t *d, uint32_t log_n, size_t count, bool inverse, const fr_t *tw, int el,
                       const ntt_factors &fac, uint32_t *status, cudaStream_t s, const ntt_input *in = nullptr)
{
    const auto passes = pass_split(log_n);
    const size_t P = passes.size();
    if (in && P < 2) throw cuda_error(-1, "fused NTT input needs two or more passes");
    dev_buf<fr_t> tmp(P > 1 ? count << log_n : 0, s);
    const ntt_factors none{{fr_t::one(), fr_t::one(), fr_t::one()}, 0};
    const ntt_input no_in{nullptr, 0, none};
    const unsigned spins = wait_spins();
    for (size_t i = 0; i < P; i++) {
        const int s_hi = passes[i].first, g = passes[i].second;
        const int s_lo = s_hi - g + 1;
        const bool last = i + 1 == P;
        const fr_t *src = i == 0 ? d : tmp.get();
        fr_t *dst = last ? d : tmp.get();
        const fr_t *tab = pass_twiddles(log_n, inverse, s_hi, g, tw, s);
        int q = kPassBits - g;
        size_t ctas;
        auto ctas_for = [&](int qq) {
            const size_t total = count << (log_n - g);
            return s_lo > 0 ? total >> qq : (total + ((size_t)1 << qq) - 1) >> qq;
        };
        if (s_lo > 0) {
            q = std::min(q, s_lo);
        } else {
            const size_t total = count << (log_n - g);
            while (q > 0 && ((size_t)1 << (q - 1)) >= total) q--;
        }
        // small transforms: fewer sub-blocks per CTA until there are two
        // CTAs per SM (a single 2^16 transform is otherwise 64 CTAs)
        while (q > 0 && ctas_for(q) < 2 * (size_t)sm_count()) q--;
        ctas = ctas_for(q);
        const uint32_t nd = 1u << (g + q);
        const uint32_t tw_entries = s_lo > 0 ? nd : 1u << g;
        const size_t smem = ((size_t)nd + tw_entries) * sizeof(fr_t);
        const unsigned threads = nd >> el;
        const bool fused = in && i == 0;
        const ntt_input &pin = fused ? *in : no_in;
        if (el == 3) {
            if (last)
                ntt_dif_pass_tw_kernel<3, true><<<(unsigned)ctas, threads, smem, s>>>(
                    src, dst, log_n, s_hi, g, q, count, tab, fac, pin, status, spins);
            else if (fused)
                ntt_dif_pass_tw_kernel<3, false, true><<<(unsigned)ctas, threads, smem, s>>>(
                    src, dst, log_n, s_hi, g, q, count, tab, none, pin, status, spins);
            else
                ntt_dif_pass_tw_kernel<3, false><<<(unsigned)ctas, threads, smem, s>>>(
                    src, dst, log_n, s_hi, g, q, count, tab, none, pin, status, spins);
        } else {
            if (last)
                ntt_dif_pass_tw_kernel<2, true><<<(unsigned)ctas, threads, smem, s>>>(
                    src, dst, log_n, s_hi, g, q, count, tab, fac, pin, status, spins);
            else if (fused)
                ntt_dif_pass_tw_kernel<2, false, true><<<(unsigned)ctas, threads, smem, s>>>(
                    src, dst, log_n, s_hi, g, q, count, tab, none, pin, status, spins);
            else
                ntt_dif_pass_tw_kernel<2, false><<<(unsigned)ctas, threads, smem, s>>>(
                    src, dst, log_n, s_hi, g, q, count, tab, none, pin, status, spins);
        }
        GB_CHECK_LAUNCH();
    }
}

// A ragged batch: transform j is the 2^log_ns[j] values at d + offsets[j],
// with the output factors fac[j], in one launch of the work-queue kernel
// (staged passes, 4 elements per thread).  Transforms with two or more
// passes run through a scratch copy as ntt_staged does; every size needs
// log_ns[j] >= 3.  Returns the number of launches (0 or 1).
static int ntt_ragged(fr_t *d, const size_t *offsets, const uint32_t *log_ns, const ntt_factors *fac, size_t count,
                      bool inverse, uint32_t *status, cudaStream_t s)
{
    set_ntt_smem();
    std::vector<ntt_qjob> jobs(count);
    size_t tmp_len = 0;
    uint32_t counters = 0;
    for (size_t j = 0; j < count; j++)
        if (pass_split(log_ns[j]).size() > 1) tmp_len += (size_t)1 << log_ns[j];
    dev_buf<fr_t> tmp(tmp_len, s);
    size_t tmp_off = 0, max_passes = 0;
    for (size_t j = 0; j < count; j++) {
        const uint32_t log_n = log_ns[j];
        const auto passes = pass_split(log_n);
        const size_t P = passes.size();
        if (P > 3) throw cuda_error((int)cudaErrorInvalidValue, "ragged NTT size above 2^30");
        const fr_t *tw = twiddles(log_n, inverse, s);
        fr_t *dj = d + offsets[j];
        fr_t *tj = P > 1 ? tmp.get() + tmp_off : nullptr;
        if (P > 1) tmp_off += (size_t)1 << log_n;
        ntt_qjob &J = jobs[j];
        J.fac = fac[j];
        J.log_n = log_n;
        J.npass = (uint32_t)P;
        J.counter = counters;
        counters += (uint32_t)P;
        max_passes = std::max(max_passes, P);
        for (size_t i = 0; i < P; i++) {
            const int s_hi = passes[i].first, g = passes[i].second, s_lo = s_hi - g + 1;
            const bool last = i + 1 == P;
            int q = kPassBits - g;
            size_t pieces;
            if (s_lo > 0) {
                q = std::min(q, s_lo);
                pieces = ((size_t)1 << (log_n - g)) >> q;
            } else {
                const size_t total = (size_t)1 << (log_n - g);
                while (q > 0 && ((size_t)1 << (q - 1)) >= total) q--;
                pieces = (total + ((size_t)1 << q) - 1) >> q;
            }
            if (pieces >= ((size_t)1 << kQueuePieceBits))
                throw cuda_error((int)cudaErrorInvalidValue, "ragged NTT piece index overflow");
            ntt_qpass &Pp = J.pass[i];
            Pp.src = P == 1 || i == 0 ? dj : tj;
            Pp.dst = P == 1 || last ? dj : tj;
            Pp.tw = pass_twiddles(log_n, inverse, s_hi, g, tw, s);
            Pp.pieces = (uint32_t)pieces;
            Pp.s_hi = s_hi;
            Pp.g = g;
            Pp.q = q;
        }
    }
    std::vector<uint2> items;
    for (size_t p = 0; p < max_passes; p++)
        for (size_t j = 0; j < count; j++)
            if (p < jobs[j].npass)
                for (uint32_t c = 0; c < jobs[j].pass[p].pieces; c++)
                    items.push_back(make_uint2((uint32_t)j, ((uint32_t)p << kQueuePieceBits) | c));
    if (items.empty()) return 0;
    if (items.size() > 0xffffffffull) throw cuda_error((int)cudaErrorInvalidValue, "ragged NTT item overflow");
    dev_buf<ntt_qjob> djobs(count, s);
    dev_buf<uint2> ditems(items.size(), s);
    dev_buf<uint32_t> ctl(NTT_Q_COUNTERS + counters, s);
    h2d(djobs, jobs.data(), count * sizeof(ntt_qjob), s);
    h2d(ditems, items.data(), items.size() * sizeof(uint2), s);
    GB_CUDA_OK(cudaMemsetAsync(ctl, 0, (NTT_Q_COUNTERS + counters) * sizeof(uint32_t), s));
    const unsigned threads = 1024 >> 2;
    const size_t smem = 2 * ((size_t)1 << kPassBits) * sizeof(fr_t);
    int per_sm = 0, sms = 0, dev = current_device();
    GB_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ntt_queue_kernel<2>, threads, smem));
    GB_CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t grid = std::min(items.size(), (size_t)std::max(per_sm, 1) * (size_t)sms);
    ntt_queue_kernel<2><<<(unsigned)grid, threads, smem, s>>>(djobs, ditems, (uint32_t)items.size(), ctl, status,
                                                              wait_spins());
    GB_CHECK_LAUNCH();
    return 1;
}

// the DIF passes of `count` transforms in place; el = log2(elements per
// thread) of the register-blocked pass (1 = one butterfly per thread)
static void ntt_passes(fr_t *d, uint32_t log_n, size_t count, const fr_t *tw, int el, cudaStream_t s)
{
    const size_t n = (size_t)1 << log_n;
    int s_hi = (int)log_n - 1;
    while (s_hi >= 0) {
        int g = s_hi + 1 < kPassBits ? s_hi + 1 : kPassBits;
        uint32_t cnt = 1u << g;
        dim3 grid((unsigned)(n >> g), (unsigned)count);
        if (g >= 3 && el == 3) {
            ntt_dif_pass_reg_kernel<3><<<grid, cnt / 8, cnt / 8 * 9 * sizeof(fr_t), s>>>(d, log_n, s_hi, g, tw);
        } else if (g >= 3 && el == 2) {
            ntt_dif_pass_reg_kernel<2><<<grid, cnt / 4, cnt / 8 * 9 * sizeof(fr_t), s>>>(d, log_n, s_hi, g, tw);
        } else {
            unsigned threads = cnt / 2 < 512 ? (cnt / 2 ? cnt / 2 : 1) : 512;
            ntt_dif_pass_kernel<<<grid, threads, cnt * sizeof(fr_t), s>>>(d, log_n, s_hi, g, tw);
        }
        GB_CHECK_LAUNCH();
        s_hi -= g;
    }
}

// The whole transform of `count` polynomials with variant v, natural order
// out, then out[i] *= fac.f[(i mod n) mod 3] when fac.on.  Variants: 1 = one
// radix-2 butterfly per thread, 2 / 3 = 4 / 8 elements per thread with
// twiddles read from the global table (these three in place, followed by a
// bit-reversal pass and a factor pass), 4 / 5 = 4 / 8 elements per thread with
// the pass's twiddles staged in shared memory (fused as above).
static void ntt_transform(fr_t *d, uint32_t log_n, size_t count, bool inverse, const fr_t *tw, int v,
                          const ntt_factors &fac, uint32_t *status, cudaStream_t s)
{
    const size_t n = (size_t)1 << log_n;
    if (v >= 4 && log_n >= 3) {
        ntt_staged(d, log_n, count, inverse, tw, v == 5 ? 3 : 2, fac, status, s);
        return;
    }
    if (log_n > 0) ntt_passes(d, log_n, count, tw, v >= 4 ? 2 : v, s);
    dim3 grid(blocks_for(n, 256), (unsigned)count);
    bitrev_scale_kernel<<<grid, 256, 0, s>>>(d, log_n, false, fr_t::one());
    GB_CHECK_LAUNCH();
    if (fac.on == 1) {
        mul_period3_kernel<<<blocks_for(n * count, 256), 256, 0, s>>>(d, fac.f[0], fac.f[1], fac.f[2], n * count, n);
        GB_CHECK_LAUNCH();
    } else if (fac.on == 2) {
        mul_factors_kernel<<<blocks_for(n * count, 256), 256, 0, s>>>(d, fac, n * count, n);
        GB_CHECK_LAUNCH();
    }
}

static int g_variant_forced = 0;

// Variant: the staged-twiddle passes with 4 elements per thread, unless
// GB_NTT_VARIANT (1..5) or gb_ntt_variant_set overrides; with the autotuner
// on, each size times the five variants once on a scratch copy of one
// transform.
static int ntt_variant(fr_t *d, uint32_t log_n, bool inverse, const fr_t *tw, uint32_t *status, cudaStream_t s)
{
    static const int v_env = [] {
        const char *e = getenv("GB_NTT_VARIANT");
        return e && e[0] >= '1' && e[0] <= '5' ? e[0] - '0' : 0;
    }();
    if (g_variant_forced) return g_variant_forced;
    if (v_env) return v_env;
    int v = log_n >= 3 ? 4 : 1;
    if (!autotune_enabled() || log_n < 10) return v;
    const std::string key = "ntt:2^" + std::to_string(log_n);
    if (autotune_lookup(key, &v)) return v;
    const size_t n = (size_t)1 << log_n;
    dev_buf<fr_t> scratch(n, s);
    const ntt_factors none{{fr_t::one(), fr_t::one(), fr_t::one()}, 0};
    float best = 1e30f;
    for (int cand = 1; cand <= 5; cand++) {
        GB_CUDA_OK(cudaMemcpyAsync(scratch.get(), d, n * sizeof(fr_t), cudaMemcpyDeviceToDevice, s));
        float ms = time_on_stream(s, [&] { ntt_transform(scratch, log_n, 1, inverse, tw, cand, none, status, s); });
        if (ms < best) {
            best = ms;
            v = cand;
        }
    }
    autotune_store(key, v);
    return v;
}

static void ntt_apply(fr_t *d, uint32_t log_n, size_t count, bool inverse, const ntt_factors &fac, uint32_t *status,
                      cudaStream_t s)
{
    if (count == 0) return;
    set_ntt_smem();
    const fr_t *tw = log_n ? twiddles(log_n, inverse, s) : nullptr;
    const int v = log_n ? ntt_variant(d, log_n, inverse, tw, status, s) : 1;
    ntt_transform(d, log_n, count, inverse, tw, v, fac, status, s);
}

void ntt_inplace(fr_t *d, uint32_t log_n, size_t count, bool inverse, const fr_t *scale, uint32_t *status,
                 cudaStream_t s)
{
    ntt_factors fac{{fr_t::one(), fr_t::one(), fr_t::one()}, 0};
    if (scale) fac = ntt_factors{{*scale, *scale, *scale}, 1};
    ntt_apply(d, log_n, count, inverse, fac, status, s);
}

// Forward transforms of `count` polynomials of in_len values at src (count
// x in_len), zero-padded to 2^log_n, with infac's factor applied to input i:
// out (count x 2^log_n) = NTT(pad(src[i] * factor(i))), then the output
// factors `outfac`.  With the staged passes and two or more passes the
// padding and the input factors are fused into the first pass's gather (no
// padded copy is written or read); otherwise a prepare kernel writes the
// padded, scaled input to out first.  src and out may be the same buffer
// only when in_len = 2^log_n.
static void ntt_padded(fr_t *out, const fr_t *src, size_t in_len, size_t count, uint32_t log_n,
                       const ntt_factors &infac, const ntt_factors &outfac, uint32_t *status, cudaStream_t s)
{
    if (count == 0) return;
    set_ntt_smem();
    const size_t n = (size_t)1 << log_n;
    const fr_t *tw = log_n ? twiddles(log_n, false, s) : nullptr;
    const int v = log_n ? ntt_variant(out, log_n, false, tw, status, s) : 1;
    if (v >= 4 && pass_split(log_n).size() >= 2) {
        const ntt_input in{src, in_len, infac};
        ntt_staged(out, log_n, count, false, tw, v == 5 ? 3 : 2, outfac, status, s, &in);
        return;
    }
    c2e_factors_kernel<<<blocks_for(n * count, 256), 256, 0, s>>>(out, src, infac, in_len, n, count);
    GB_CHECK_LAUNCH();
    if (log_n) ntt_transform(out, log_n, count, false, tw, v, outfac, status, s);
}

// The two power tables of mode-2 factors for positions below `len`:
// factor(i) = scale * shift^i = pw_hi[i >> lo_bits] * pw_lo[i mod 2^lo_bits]
// with lo_bits = ceil(bits(len - 1) / 2).  Cached per (device, shift,
// scale, lo_bits); built on stream s the first time.
namespace {
std::mutex g_pw_mu;
std::map<std::string, std::pair<fr_t *, fr_t *>> g_pw;
}  // namespace

static ntt_factors power_factors(const fr_t &shift, const fr_t &scale, size_t len, cudaStream_t s)
{
    uint32_t bits = 0;
    while (bits < 63 && ((size_t)1 << bits) < len) bits++;
    const uint32_t lo_bits = (bits + 1) / 2;
    const size_t n_lo = (size_t)1 << lo_bits, n_hi = (size_t)1 << (bits - lo_bits);
    std::string key((const char *)&shift, sizeof(fr_t));
    key.append((const char *)&scale, sizeof(fr_t));
    key += ":" + std::to_string(current_device()) + ":" + std::to_string(lo_bits) + ":" + std::to_string(n_hi);
    ntt_factors f{{fr_t::one(), fr_t::one(), fr_t::one()}, 2};
    f.lo_bits = lo_bits;
    std::lock_guard<std::mutex> lk(g_pw_mu);
    auto it = g_pw.find(key);
    if (it == g_pw.end()) {
        fr_t *lo = nullptr, *hi = nullptr;
        GB_CUDA_OK(cudaMalloc(&lo, n_lo * sizeof(fr_t)));
        GB_CUDA_OK(cudaMalloc(&hi, n_hi * sizeof(fr_t)));
        fr_t step = shift;  // shift^(2^lo_bits)
        for (uint32_t b = 0; b < lo_bits; b++) step = step.sqr();
        powers_table_kernel<<<blocks_for(n_lo, 256), 256, 0, s>>>(lo, shift, fr_t::one(), n_lo);
        GB_CHECK_LAUNCH();
        powers_table_kernel<<<blocks_for(n_hi, 256), 256, 0, s>>>(hi, step, scale, n_hi);
        GB_CHECK_LAUNCH();
        GB_CUDA_OK(cudaStreamSynchronize(s));
        it = g_pw.emplace(key, std::make_pair(lo, hi)).first;
    }
    f.pw_lo = it->second.first;
    f.pw_hi = it->second.second;
    return f;
}

void launch_mul_assign(fr_t *d, const fr_t &k, size_t len, cudaStream_t s)
{
    if (!len) return;
    mul_assign_kernel<<<blocks_for(len, 256), 256, 0, s>>>(d, k, len);
    GB_CHECK_LAUNCH();
}

void launch_mul_assign_zeta(fr_t *d, const fr_t &first, const fr_t &second, size_t len, size_t period_len,
                            cudaStream_t s)
{
    if (!len) return;
    mul_assign_zeta_kernel<<<blocks_for(len, 256), 256, 0, s>>>(d, first, second, len, period_len);
    GB_CHECK_LAUNCH();
}

void launch_mul_assign_repeating(fr_t *d, const fr_t *factors, size_t factor_len, size_t len, cudaStream_t s)
{
    if (!len) return;
    mul_assign_repeating_kernel<<<blocks_for(len, 256), 256, 0, s>>>(d, factors, factor_len, len);
    GB_CHECK_LAUNCH();
}

void launch_scale_zeta(fr_t *d, const fr_t &scale, const fr_t &first, const fr_t &second, size_t len,
                       size_t period_len, cudaStream_t s)
{
    if (!len) return;
    scale_zeta_kernel<<<blocks_for(len, 256), 256, 0, s>>>(d, scale, first, second, len, period_len);
    GB_CHECK_LAUNCH();
}

void launch_coeff_to_extended_prepare(fr_t *out, const fr_t *in, const fr_t &first, const fr_t &second,
                                      size_t input_len, size_t output_len, size_t count, cudaStream_t s)
{
    size_t total = output_len * count;
    if (!total) return;
    c2e_prepare_kernel<<<blocks_for(total, 256), 256, 0, s>>>(out, in, first, second, input_len, output_len,
                                                             count);
    GB_CHECK_LAUNCH();
}

// reference NTT semantics: inverse includes 1/n
static void ntt_ref(fr_t *d, uint32_t log_n, size_t count, bool inverse, uint32_t *status, cudaStream_t s)
{
    if (inverse) {
        fr_t ninv = host_fr_inverse(host_fr_from_u64((uint64_t)1 << log_n));
        ntt_inplace(d, log_n, count, true, &ninv, status, s);
    } else {
        ntt_inplace(d, log_n, count, false, nullptr, status, s);
    }
}

// ntt_ref, then out[i] *= scale * [1, first, second][(i mod n) mod 3] (the
// reference's NTT followed by its scale-and-ZETA pass), with the factors
// applied by the transform's last pass
static void ntt_ref_zeta(fr_t *d, uint32_t log_n, size_t count, bool inverse, const fr_t &scale, const fr_t &first,
                         const fr_t &second, uint32_t *status, cudaStream_t s)
{
    fr_t sc = scale;
    if (inverse) sc = sc * host_fr_inverse(host_fr_from_u64((uint64_t)1 << log_n));
    const ntt_factors fac{{sc, sc * first, sc * second}, 1};
    ntt_apply(d, log_n, count, inverse, fac, status, s);
}

// coeff_to_extended (ZETA coset, domain.rs:325-339): count polynomials of
// input_len coefficients -> evaluations on the 2^ext_log_n extended coset,
// the distribution a_i [1, first, second][i mod 3] and the zero padding
// fused into the first NTT pass
static void c2e_zeta(fr_t *out, const fr_t *in, size_t input_len, size_t count, uint32_t ext_log_n,
                     const fr_t &first, const fr_t &second, uint32_t *status, cudaStream_t s)
{
    const ntt_factors infac{{fr_t::one(), first, second}, 1};
    const ntt_factors none{{fr_t::one(), fr_t::one(), fr_t::one()}, 0};
    ntt_padded(out, in, input_len, count, ext_log_n, infac, none, status, s);
}

// the same with the powers of a coset shift: a_i shift^i, zero padding,
// forward NTT (evaluations on shift * <w_ext>)
static void c2e_coset(fr_t *out, const fr_t *in, size_t input_len, size_t count, uint32_t ext_log_n,
                      const fr_t &shift, uint32_t *status, cudaStream_t s)
{
    const ntt_factors infac = power_factors(shift, fr_t::one(), input_len, s);
    const ntt_factors none{{fr_t::one(), fr_t::one(), fr_t::one()}, 0};
    ntt_padded(out, in, input_len, count, ext_log_n, infac, none, status, s);
}

// sppark's coset NTT (NTT::Base with Type::coset, NN order;
// vendor/sppark-0.1.15/sppark/ntt/ntt.cuh:196-209) in place on count
// polynomials: forward NTT(a_i shift^i), the powers applied by the first
// pass; inverse iNTT(a)_i shift^-i (the iNTT includes 1/n), the powers and
// 1/n applied by the last pass
static void ntt_coset(fr_t *d, uint32_t log_n, size_t count, bool inverse, const fr_t &shift, uint32_t *status,
                      cudaStream_t s)
{
    const size_t n = (size_t)1 << log_n;
    if (!inverse) {
        c2e_coset(d, d, n, count, log_n, shift, status, s);
        return;
    }
    const fr_t ninv = host_fr_inverse(host_fr_from_u64((uint64_t)n));
    const ntt_factors outfac = power_factors(host_fr_inverse(shift), ninv, n, s);
    ntt_apply(d, log_n, count, true, outfac, status, s);
}

}  // namespace gb

using namespace gb;

extern "C" {

// bls12_381_g1_msm.cu:6488-6502 (sppark NTT::Base, NN order)
RustError midnight_sppark_bls12_381_fr_ntt(RawFr *values_raw, uint32_t log_n, bool inverse)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    GB_ENTRY_BEGIN
    if (log_n > 31) return make_error((int)cudaErrorInvalidValue, "NTT size too large");
    if (!values) return make_error((int)cudaErrorInvalidValue, "null NTT values");
    size_t n = (size_t)1 << log_n;
    cudaStream_t s = lane_stream();
    ntt_status st;
    dev_buf<fr_t> d(n, s);
    h2d(d, values, n * sizeof(fr_t), s);
    ntt_ref(d, log_n, 1, inverse, st.ptr(), s);
    d2h(values, d, n * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3447-3495
RustError midnight_sppark_bls12_381_fr_ntt_zeta(RawFr *values_raw, uint32_t log_n, bool inverse, RawFr scale_raw, RawFr first_raw, RawFr second_raw)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    const fr_t scale = gb::from_raw(scale_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (log_n == 0) return ok();
    GB_ENTRY_BEGIN
    if (log_n > 31 || !values) return make_error((int)cudaErrorInvalidValue, "invalid NTT arguments");
    size_t n = (size_t)1 << log_n;
    cudaStream_t s = lane_stream();
    ntt_status st;
    dev_buf<fr_t> d(n, s);
    h2d(d, values, n * sizeof(fr_t), s);
    ntt_ref_zeta(d, log_n, 1, inverse, scale, first, second, st.ptr(), s);
    d2h(values, d, n * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3497-3556
RustError midnight_sppark_bls12_381_fr_divide_ntt_zeta(RawFr *values_raw, uint32_t log_n, const RawFr *factors_raw, size_t factor_len, RawFr scale_raw, RawFr first_raw, RawFr second_raw)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    const fr_t *factors = reinterpret_cast<const fr_t *>(factors_raw);
    const fr_t scale = gb::from_raw(scale_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (log_n == 0 || factor_len == 0) return ok();
    GB_ENTRY_BEGIN
    if (log_n > 31 || !values || !factors) return make_error((int)cudaErrorInvalidValue, "invalid NTT arguments");
    size_t n = (size_t)1 << log_n;
    cudaStream_t s = lane_stream();
    ntt_status st;
    dev_buf<fr_t> d(n, s), f(factor_len, s);
    h2d(d, values, n * sizeof(fr_t), s);
    h2d(f, factors, factor_len * sizeof(fr_t), s);
    launch_mul_assign_repeating(d, f, factor_len, n, s);
    ntt_ref_zeta(d, log_n, 1, true, scale, first, second, st.ptr(), s);
    d2h(values, d, n * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:2542-2602
RustError midnight_sppark_bls12_381_fr_coeff_to_extended_batch(RawFr *out_raw, const RawFr *inputs_raw, size_t input_len, size_t count, uint32_t extended_log_n, RawFr first_raw, RawFr second_raw)
{
    fr_t *out = reinterpret_cast<fr_t *>(out_raw);
    const fr_t *inputs = reinterpret_cast<const fr_t *>(inputs_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (input_len == 0 || count == 0) return ok();
    GB_ENTRY_BEGIN
    if (extended_log_n > 31) return make_error((int)cudaErrorInvalidValue, "extended domain too large");
    size_t output_len = (size_t)1 << extended_log_n;
    if (input_len > output_len) return make_error(-1, "input length exceeds extended domain length");
    if (!out || !inputs) return make_error((int)cudaErrorInvalidValue, "null coeff_to_extended buffers");
    cudaStream_t s = lane_stream();
    ntt_status st;
    dev_buf<fr_t> din(input_len * count, s), dout(output_len * count, s);
    h2d(din, inputs, input_len * count * sizeof(fr_t), s);
    c2e_zeta(dout, din, input_len, count, extended_log_n, first, second, st.ptr(), s);
    d2h(out, dout, output_len * count * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:2604-2660: result left resident in a new device vector
RustError midnight_sppark_bls12_381_fr_device_coeff_to_extended_batch(void **out, const RawFr *inputs_raw, size_t input_len, size_t count, uint32_t extended_log_n, RawFr first_raw, RawFr second_raw)
{
    const fr_t *inputs = reinterpret_cast<const fr_t *>(inputs_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (!out) return make_error((int)cudaErrorInvalidValue, "null device vector output");
    *out = nullptr;
    if (input_len == 0 || count == 0 || !inputs)
        return make_error((int)cudaErrorInvalidValue, "invalid resident coeff_to_extended arguments");
    GB_ENTRY_BEGIN
    if (extended_log_n > 31) return make_error((int)cudaErrorInvalidValue, "extended domain too large");
    size_t output_len = (size_t)1 << extended_log_n;
    if (input_len > output_len) return make_error(-1, "input length exceeds extended domain length");
    cudaStream_t s = lane_stream();
    ntt_status st;
    dev_buf<fr_t> din(input_len * count, s);
    h2d(din, inputs, input_len * count * sizeof(fr_t), s);
    fr_device_vec *v = device_vec_new(output_len * count, s);
    try {
        c2e_zeta(v->values, din, input_len, count, extended_log_n, first, second, st.ptr(), s);
        lane_check();
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:2662-2740: source polynomials already resident
RustError midnight_sppark_bls12_381_fr_device_coeff_to_extended_from_device_batch(void **out, const void *source, size_t input_len, size_t count, uint32_t extended_log_n, RawFr first_raw, RawFr second_raw)
{
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (!out) return make_error((int)cudaErrorInvalidValue, "null device vector output");
    *out = nullptr;
    if (!source || input_len == 0 || count == 0)
        return make_error((int)cudaErrorInvalidValue, "invalid resident coeff_to_extended arguments");
    GB_ENTRY_BEGIN
    auto *src = reinterpret_cast<const fr_device_vec *>(source);
    if (src->len < input_len * count) return make_error((int)cudaErrorInvalidValue, "source device vector too short");
    if (extended_log_n > 31) return make_error((int)cudaErrorInvalidValue, "extended domain too large");
    size_t output_len = (size_t)1 << extended_log_n;
    if (input_len > output_len) return make_error(-1, "input length exceeds extended domain length");
    cudaStream_t s = lane_stream();
    device_vec_wait(src, s);
    ntt_status st;
    fr_device_vec *v = device_vec_new(output_len * count, s);
    try {
        c2e_zeta(v->values, src->values, input_len, count, extended_log_n, first, second, st.ptr(), s);
        lane_check();
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3280-3329
RustError midnight_sppark_bls12_381_fr_device_vec_ntt_zeta(void *device_vec, uint32_t log_n, bool inverse, RawFr scale_raw, RawFr first_raw, RawFr second_raw)
{
    const fr_t scale = gb::from_raw(scale_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (!device_vec) return make_error((int)cudaErrorInvalidValue, "null device vector");
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<fr_device_vec *>(device_vec);
    size_t n = (size_t)1 << log_n;
    if (log_n > 31 || v->len != n) return make_error((int)cudaErrorInvalidValue, "resident NTT length mismatch");
    // a single value is returned unscaled, as the reference does (.cu:3296-3298)
    if (log_n == 0) return ok();
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    ntt_status st;
    ntt_ref_zeta(v->values, log_n, 1, inverse, scale, first, second, st.ptr(), s);
    lane_check();
    device_vec_mark_ready(v, s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3331-3380
RustError midnight_sppark_bls12_381_fr_device_vec_ntt_zeta_batch(void *device_vec, uint32_t log_n, size_t count, bool inverse, RawFr scale_raw, RawFr first_raw, RawFr second_raw)
{
    const fr_t scale = gb::from_raw(scale_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (!device_vec || count == 0) return make_error((int)cudaErrorInvalidValue, "invalid resident NTT batch arguments");
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<fr_device_vec *>(device_vec);
    if (log_n > 31) return make_error((int)cudaErrorInvalidValue, "resident NTT batch size overflow");
    size_t n = (size_t)1 << log_n;
    if (count > SIZE_MAX / n) return make_error((int)cudaErrorInvalidValue, "resident NTT batch size overflow");
    if (v->len != n * count) return make_error((int)cudaErrorInvalidValue, "resident NTT batch length mismatch");
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    ntt_status st;
    ntt_ref_zeta(v->values, log_n, count, inverse, scale, first, second, st.ptr(), s);
    lane_check();
    device_vec_mark_ready(v, s);
    return ok();
    GB_ENTRY_END
}

// Ragged batch in one persistent launch (no reference counterpart: the
// reference runs one transform per call or a batch of equal sizes).
RustError gb_fr_device_vec_ntt_ragged(void *device_vec, const size_t *offsets, const uint32_t *log_ns, size_t count,
                                      bool inverse, RawFr scale_raw, RawFr first_raw, RawFr second_raw)
{
    const fr_t scale = gb::from_raw(scale_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (!device_vec || (count && (!offsets || !log_ns)))
        return make_error((int)cudaErrorInvalidValue, "invalid ragged NTT arguments");
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<fr_device_vec *>(device_vec);
    std::vector<std::pair<size_t, size_t>> ranges;
    for (size_t j = 0; j < count; j++) {
        if (log_ns[j] > 30) return make_error((int)cudaErrorInvalidValue, "ragged NTT size above 2^30");
        const size_t n = (size_t)1 << log_ns[j];
        if (offsets[j] > v->len || n > v->len - offsets[j])
            return make_error((int)cudaErrorInvalidValue, "ragged NTT polynomial outside the device vector");
        ranges.emplace_back(offsets[j], n);
    }
    std::sort(ranges.begin(), ranges.end());
    for (size_t j = 1; j < ranges.size(); j++)
        if (ranges[j - 1].first + ranges[j - 1].second > ranges[j].first)
            return make_error((int)cudaErrorInvalidValue, "ragged NTT polynomials overlap");
    if (count == 0) return ok();
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    ntt_status st;
    std::vector<size_t> q_off;
    std::vector<uint32_t> q_log;
    std::vector<ntt_factors> q_fac;
    for (size_t j = 0; j < count; j++) {
        if (log_ns[j] == 0) continue;  // one value: unchanged, as a single call leaves it
        if (log_ns[j] < 3) {
            // 2 or 4 values: the plain path
            ntt_ref_zeta(v->values + offsets[j], log_ns[j], 1, inverse, scale, first, second, st.ptr(), s);
            continue;
        }
        fr_t sc = scale;
        if (inverse) sc = sc * host_fr_inverse(host_fr_from_u64((uint64_t)1 << log_ns[j]));
        q_off.push_back(offsets[j]);
        q_log.push_back(log_ns[j]);
        q_fac.push_back(ntt_factors{{sc, sc * first, sc * second}, 1});
    }
    ntt_ragged(v->values, q_off.data(), q_log.data(), q_fac.data(), q_off.size(), inverse, st.ptr(), s);
    lane_check();
    device_vec_mark_ready(v, s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3382-3440
RustError midnight_sppark_bls12_381_fr_device_vec_divide_ntt_zeta(void *device_vec, uint32_t log_n, const RawFr *factors_raw, size_t factor_len, RawFr scale_raw, RawFr first_raw, RawFr second_raw)
{
    const fr_t *factors = reinterpret_cast<const fr_t *>(factors_raw);
    const fr_t scale = gb::from_raw(scale_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (!device_vec || !factors || factor_len == 0)
        return make_error((int)cudaErrorInvalidValue, "invalid resident divide NTT arguments");
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<fr_device_vec *>(device_vec);
    size_t n = (size_t)1 << log_n;
    if (log_n > 31 || v->len != n) return make_error((int)cudaErrorInvalidValue, "resident NTT length mismatch");
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    ntt_status st;
    dev_buf<fr_t> f(factor_len, s);
    h2d(f, factors, factor_len * sizeof(fr_t), s);
    launch_mul_assign_repeating(v->values, f, factor_len, n, s);
    ntt_ref_zeta(v->values, log_n, 1, true, scale, first, second, st.ptr(), s);
    lane_check();
    device_vec_mark_ready(v, s);
    return ok();
    GB_ENTRY_END
}

// Forces the NTT pass variant (1..5; see ntt_transform), or 0 for the default
// or autotuned choice.  Process-wide.
void gb_ntt_variant_set(int variant) { g_variant_forced = variant >= 1 && variant <= 5 ? variant : 0; }

// Bounded waits (twiddle copies and work-queue waits) of NTT work that ran
// out since the last read, process-wide; the calling lane is synchronised
// first so its own pending work is counted.  Each was (or, on another lane,
// will be) reported as cudaErrorLaunchTimeout by its lane's next
// synchronising call.  The count is reset by the read.
RustError gb_ntt_wait_timeouts(uint32_t *out)
{
    if (!out) return make_error((int)cudaErrorInvalidValue, "null output");
    GB_ENTRY_BEGIN
    try {
        lane_sync(lane_stream());
    } catch (const cuda_error &e) {
        if (e.code() != (int)cudaErrorLaunchTimeout) throw;
    }
    const unsigned long long v = lane_timeouts_take();
    *out = v > 0xffffffffull ? 0xffffffffu : (uint32_t)v;
    return ok();
    GB_ENTRY_END
}

// Test hook: the poll limit of the first twiddle-copy wait of every staged
// NTT pass launched from now on (process-wide); negative restores the
// default.  0 makes the wait give up at once, so the call reports
// cudaErrorLaunchTimeout; the copy still lands within the CTA's second,
// longer wait before the CTA moves on.
void gb_ntt_wait_limit_set(int64_t spins)
{
    g_wait_spins_override.store(spins < 0 ? -1 : (spins > 0xffffffffll ? 0xffffffffll : spins));
}

// ---- coset by the powers of a shift (sppark's coset NTT and LDE form)

// coefficients -> evaluations on the coset shift * <w_ext> of the 2^ext_log_n
// domain, for count polynomials of input_len coefficients (host buffers):
// out[p][j] = sum_i in[p][i] (shift w_ext^j)^i.  The reference's sppark
// distributes the coset generator's powers in its LDE
// (vendor/sppark-0.1.15/sppark/ntt/ntt.cuh:283-338, kernels.cu:155-230);
// here the powers and the zero padding are applied by the first NTT pass.
RustError gb_fr_coeff_to_extended_coset_batch(RawFr *out_raw, const RawFr *inputs_raw, size_t input_len,
                                              size_t count, uint32_t extended_log_n, RawFr shift_raw)
{
    fr_t *out = reinterpret_cast<fr_t *>(out_raw);
    const fr_t *inputs = reinterpret_cast<const fr_t *>(inputs_raw);
    const fr_t shift = gb::from_raw(shift_raw);
    if (input_len == 0 || count == 0) return ok();
    GB_ENTRY_BEGIN
    if (extended_log_n > 31) return make_error((int)cudaErrorInvalidValue, "extended domain too large");
    const size_t output_len = (size_t)1 << extended_log_n;
    if (input_len > output_len) return make_error(-1, "input length exceeds extended domain length");
    if (!out || !inputs) return make_error((int)cudaErrorInvalidValue, "null coset LDE buffers");
    cudaStream_t s = lane_stream();
    ntt_status st;
    dev_buf<fr_t> din(input_len * count, s), dout(output_len * count, s);
    h2d(din, inputs, input_len * count * sizeof(fr_t), s);
    c2e_coset(dout, din, input_len, count, extended_log_n, shift, st.ptr(), s);
    d2h(out, dout, output_len * count * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// The same from resident coefficients (count polynomials of input_len values
// at the start of `source`) into a new resident device vector of count x
// 2^extended_log_n evaluations.
RustError gb_fr_device_coeff_to_extended_coset_batch(void **out, const void *source, size_t input_len, size_t count,
                                                     uint32_t extended_log_n, RawFr shift_raw)
{
    const fr_t shift = gb::from_raw(shift_raw);
    if (!out) return make_error((int)cudaErrorInvalidValue, "null device vector output");
    *out = nullptr;
    if (!source || input_len == 0 || count == 0)
        return make_error((int)cudaErrorInvalidValue, "invalid resident coset LDE arguments");
    GB_ENTRY_BEGIN
    auto *src = reinterpret_cast<const fr_device_vec *>(source);
    if (count > SIZE_MAX / input_len || src->len < input_len * count)
        return make_error((int)cudaErrorInvalidValue, "source device vector too short");
    if (extended_log_n > 31) return make_error((int)cudaErrorInvalidValue, "extended domain too large");
    const size_t output_len = (size_t)1 << extended_log_n;
    if (input_len > output_len) return make_error(-1, "input length exceeds extended domain length");
    cudaStream_t s = lane_stream();
    device_vec_wait(src, s);
    ntt_status st;
    fr_device_vec *v = device_vec_new(output_len * count, s);
    try {
        c2e_coset(v->values, src->values, input_len, count, extended_log_n, shift, st.ptr(), s);
        lane_check();
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// sppark's coset NTT (NTT::Base with Type::coset, natural order in and out;
// vendor/sppark-0.1.15/sppark/ntt/ntt.cuh:196-209) in place on count
// resident polynomials of 2^log_n values: forward NTT(a_i shift^i), inverse
// iNTT(a)_i shift^-i, the iNTT including 1/n.
RustError gb_fr_device_vec_ntt_coset_batch(void *device_vec, uint32_t log_n, size_t count, bool inverse,
                                           RawFr shift_raw)
{
    const fr_t shift = gb::from_raw(shift_raw);
    if (!device_vec || count == 0) return make_error((int)cudaErrorInvalidValue, "invalid resident coset NTT arguments");
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<fr_device_vec *>(device_vec);
    if (log_n > 31) return make_error((int)cudaErrorInvalidValue, "resident coset NTT size overflow");
    const size_t n = (size_t)1 << log_n;
    if (count > SIZE_MAX / n || v->len != n * count)
        return make_error((int)cudaErrorInvalidValue, "resident coset NTT length mismatch");
    if (shift.is_zero()) return make_error((int)cudaErrorInvalidValue, "zero coset shift");
    if (log_n == 0) return ok();
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    ntt_status st;
    ntt_coset(v->values, log_n, count, inverse, shift, st.ptr(), s);
    lane_check();
    device_vec_mark_ready(v, s);
    return ok();
    GB_ENTRY_END
}

// The same on one host polynomial (sppark NTT::Base(..., Type::coset)).
RustError gb_fr_ntt_coset(RawFr *values_raw, uint32_t log_n, bool inverse, RawFr shift_raw)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    const fr_t shift = gb::from_raw(shift_raw);
    if (log_n == 0) return ok();
    GB_ENTRY_BEGIN
    if (log_n > 31 || !values) return make_error((int)cudaErrorInvalidValue, "invalid coset NTT arguments");
    if (shift.is_zero()) return make_error((int)cudaErrorInvalidValue, "zero coset shift");
    const size_t n = (size_t)1 << log_n;
    cudaStream_t s = lane_stream();
    ntt_status st;
    dev_buf<fr_t> d(n, s);
    h2d(d, values, n * sizeof(fr_t), s);
    ntt_coset(d, log_n, 1, inverse, shift, st.ptr(), s);
    d2h(values, d, n * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// sppark's NTT::LDE (vendor/sppark-0.1.15/sppark/ntt/ntt.cuh:283-342): the
// 2^lg_domain_size evaluations at `in` -> the 2^(lg_domain_size +
// lg_blowup) evaluations at `out` of the same polynomial on the coset of the
// multiplicative generator 7 (group_gen, parameters/bls12_381.h:11; fq.rs
// GENERATOR): inverse NTT, then the coset LDE.  Natural order throughout.
RustError gb_fr_lde_coset(RawFr *out_raw, const RawFr *in_raw, uint32_t lg_domain_size, uint32_t lg_blowup)
{
    fr_t *out = reinterpret_cast<fr_t *>(out_raw);
    const fr_t *in = reinterpret_cast<const fr_t *>(in_raw);
    GB_ENTRY_BEGIN
    if (lg_domain_size + lg_blowup > 31 || !out || !in)
        return make_error((int)cudaErrorInvalidValue, "invalid LDE arguments");
    const size_t n = (size_t)1 << lg_domain_size, N = n << lg_blowup;
    cudaStream_t s = lane_stream();
    ntt_status st;
    dev_buf<fr_t> d(n, s), e(N, s);
    h2d(d, in, n * sizeof(fr_t), s);
    if (lg_domain_size) ntt_ref(d, lg_domain_size, 1, true, st.ptr(), s);
    c2e_coset(e, d, n, 1, lg_domain_size + lg_blowup, host_fr_from_u64(7), st.ptr(), s);
    d2h(out, e, N * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

}  // extern "C"
