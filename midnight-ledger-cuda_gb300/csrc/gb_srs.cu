// KZG structured reference string on the device:
//   * g_to_lagrange: g_lagrange = iFFT(g) * n^-1 over G1 points
//     (vendor/midnight-proofs-0.8.1/src/utils/arithmetic.rs:34-50), used when
//     an SRS is loaded or downsized (params.rs:60-77);
//   * setup from a known tau: g_i = [tau^i] G and
//     g_lagrange_i = [(tau^n - 1)/n * w^i / (tau - w^i)] G
//     (params.rs:79-129 unsafe_setup).
//
// The group FFT runs one radix-2 decimation-in-frequency stage per launch
// over XYZZ points; a butterfly is (a, b) -> (a + b, [w^j](a - b)) with a
// double-and-add scalar multiplication; a final pass scales by n^-1, converts
// to affine and applies the bit-reversal permutation.
#include <vector>

#include "gb_ntt.cuh"
#include "gb_vec.cuh"

namespace gb {

const affine_t *generator_table(cudaStream_t s);
void generator_mul_device(affine_t *d_out, const fr_t *d_scalars, size_t n, cudaStream_t s);

// [k] P for a canonical 255-bit scalar (8 x u32 limbs), double-and-add
__device__ xyzz_t xyzz_mul_scalar(const xyzz_t &p, const fr_t &canonical)
{
    xyzz_t acc = xyzz_t::inf();
    int top = 255;
    while (top >= 0 && !((canonical.v[top >> 5] >> (top & 31)) & 1u)) top--;
    for (int i = top; i >= 0; i--) {
        acc = acc.dbl();
        if ((canonical.v[i >> 5] >> (i & 31)) & 1u) acc.add(p);
    }
    return acc;
}

__global__ void affine_to_xyzz_kernel(const affine_t *__restrict__ in, xyzz_t *__restrict__ out, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = xyzz_t::from_affine(in[i]);
}

// one DIF stage s (half size 2^s) of the group FFT; tw[j] = w^j canonical
__global__ void g1_dif_stage_kernel(xyzz_t *d, uint32_t log_n, int s, const fr_t *__restrict__ tw_canon)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t half = (size_t)1 << (log_n - 1);
    if (t >= half) return;
    size_t m = (size_t)1 << s;
    size_t i0 = (t / m) * 2 * m + (t % m), i1 = i0 + m;
    size_t j = t % m;
    xyzz_t a = d[i0], b = d[i1];
    xyzz_t sum = a;
    sum.add(b);
    xyzz_t diff = a;
    diff.add(b.neg());
    if (j) diff = xyzz_mul_scalar(diff, tw_canon[j << (log_n - 1 - s)]);
    d[i0] = sum;
    d[i1] = diff;
}

__device__ __forceinline__ size_t brev(size_t x, uint32_t bits)
{
    return bits ? (size_t)(__brevll((unsigned long long)x) >> (64 - bits)) : 0;
}

// out[i] = affine([n_inv] d[bitrev(i)])
__global__ void g1_finish_kernel(const xyzz_t *__restrict__ d, uint32_t log_n, fr_t ninv_canon,
                                 affine_t *__restrict__ out)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t n = (size_t)1 << log_n;
    if (i >= n) return;
    xyzz_t p = xyzz_mul_scalar(d[brev(i, log_n)], ninv_canon);
    out[i] = p.to_affine();
}

__global__ void to_canonical_kernel(fr_t *d, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = d[i].from_mont();
}

// lagrange scalars: num[i] = (tau^n - 1)/n * w^i, den[i] = tau - w^i
__global__ void lagrange_terms_kernel(const fr_t *__restrict__ wpow, fr_t tau, fr_t mult, size_t n,
                                      fr_t *__restrict__ num, fr_t *__restrict__ den)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    num[i] = mult * wpow[i];
    den[i] = tau - wpow[i];
}

static void g_to_lagrange_device(affine_t *d_out, const affine_t *d_in, uint32_t log_n, cudaStream_t s)
{
    const size_t n = (size_t)1 << log_n;
    dev_buf<xyzz_t> pts(n, s);
    affine_to_xyzz_kernel<<<blocks_for(n, 256), 256, 0, s>>>(d_in, pts, n);
    GB_CHECK_LAUNCH();
    if (log_n) {
        // canonical twiddles of w^-1: w^-j for j < n/2
        size_t half = n / 2;
        dev_buf<fr_t> tw(half, s);
        omega_powers(tw, host_omega(log_n, true), half, s);
        to_canonical_kernel<<<blocks_for(half, 256), 256, 0, s>>>(tw, half);
        GB_CHECK_LAUNCH();
        for (int st = (int)log_n - 1; st >= 0; st--) {
            g1_dif_stage_kernel<<<blocks_for(half, 128), 128, 0, s>>>(pts, log_n, st, tw);
            GB_CHECK_LAUNCH();
        }
    }
    fr_t ninv = host_fr_inverse(host_fr_from_u64((uint64_t)n)).from_mont();
    g1_finish_kernel<<<blocks_for(n, 128), 128, 0, s>>>(pts, log_n, ninv, d_out);
    GB_CHECK_LAUNCH();
}

}  // namespace gb

using namespace gb;

// ---------------------------------------------------------------------------
// Host-side Jacobian -> affine conversion of MSM results (blst's
// p1_to_affine, which the reference's Rust callers apply to every
// commitment before it is hashed into the transcript): 6 x 64-bit limbs,
// Montgomery products with 128-bit intermediates, one binary-GCD inverse
// per batch (Montgomery's trick).  Variable time: commitments are public.
namespace hostfp {

typedef unsigned __int128 u128;
struct fp64 {
    uint64_t l[6];
};

static const fp64 kP = {{0xb9feffffffffaaabull, 0x1eabfffeb153ffffull, 0x6730d2a0f6b0f624ull, 0x64774b84f38512bfull,
                         0x4b1ba7b6434bacd7ull, 0x1a0111ea397fe69aull}};
static const uint64_t kN0 = 0x89f3fffcfffcfffdull;  // -p^-1 mod 2^64
static const fp64 kOne = {{0x760900000002fffdull, 0xebf4000bc40c0002ull, 0x5f48985753c758baull, 0x77ce585370525745ull,
                           0x5c071a97a256ec6dull, 0x15f65ec3fa80e493ull}};  // R mod p
// R^3 mod p (R = 2^384): a Montgomery product with it takes the plain
// inverse of a Montgomery value zR to the Montgomery form of 1/z
static const fp64 kR3 = {{0xed48ac6bd94ca1e0ull, 0x315f831e03a7adf8ull, 0x9a53352a615e29ddull, 0x34c04e5e921e1761ull,
                          0x2512d43565724728ull, 0x0aa6346091755d4dull}};

static bool is_zero(const fp64 &a)
{
    uint64_t t = 0;
    for (int i = 0; i < 6; i++) t |= a.l[i];
    return t == 0;
}

static bool geq(const fp64 &a, const fp64 &b)
{
    for (int i = 5; i >= 0; i--)
        if (a.l[i] != b.l[i]) return a.l[i] > b.l[i];
    return true;
}

static void sub_in(fp64 &a, const fp64 &b)
{
    uint64_t borrow = 0;
    for (int i = 0; i < 6; i++) {
        const u128 d = (u128)a.l[i] - b.l[i] - borrow;
        a.l[i] = (uint64_t)d;
        borrow = (uint64_t)(d >> 64) & 1;
    }
}

static void add_in(fp64 &a, const fp64 &b)
{
    uint64_t carry = 0;
    for (int i = 0; i < 6; i++) {
        const u128 t = (u128)a.l[i] + b.l[i] + carry;
        a.l[i] = (uint64_t)t;
        carry = (uint64_t)(t >> 64);
    }
}

static void shr1(fp64 &a)
{
    for (int i = 0; i < 5; i++) a.l[i] = (a.l[i] >> 1) | (a.l[i + 1] << 63);
    a.l[5] >>= 1;
}

// x / 2 mod p for x < p (x + p < 2^382: no carry out of six limbs)
static void half_mod(fp64 &x)
{
    if (x.l[0] & 1) add_in(x, kP);
    shr1(x);
}

// a - b mod p for a, b < p
static void sub_mod(fp64 &a, const fp64 &b)
{
    if (geq(a, b)) {
        sub_in(a, b);
    } else {
        add_in(a, kP);
        sub_in(a, b);
    }
}

static void reduce(fp64 &a)
{
    while (geq(a, kP)) sub_in(a, kP);
}

// a b R^-1 mod p (CIOS), inputs < p, result < p
static fp64 mont_mul(const fp64 &a, const fp64 &b)
{
    uint64_t t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 6; i++) {
        uint64_t carry = 0;
        for (int j = 0; j < 6; j++) {
            const u128 x = (u128)a.l[j] * b.l[i] + t[j] + carry;
            t[j] = (uint64_t)x;
            carry = (uint64_t)(x >> 64);
        }
        u128 x = (u128)t[6] + carry;
        t[6] = (uint64_t)x;
        t[7] = (uint64_t)(x >> 64);
        const uint64_t m = t[0] * kN0;
        x = (u128)m * kP.l[0] + t[0];
        carry = (uint64_t)(x >> 64);
        for (int j = 1; j < 6; j++) {
            x = (u128)m * kP.l[j] + t[j] + carry;
            t[j - 1] = (uint64_t)x;
            carry = (uint64_t)(x >> 64);
        }
        x = (u128)t[6] + carry;
        t[5] = (uint64_t)x;
        t[6] = t[7] + (uint64_t)(x >> 64);
    }
    fp64 r;
    for (int i = 0; i < 6; i++) r.l[i] = t[i];
    if (t[6] || geq(r, kP)) sub_in(r, kP);
    return r;
}

// a^-1 mod p for 0 < a < p (binary extended Euclid: x1 a = u, x2 a = v)
static fp64 inverse(const fp64 &a)
{
    fp64 u = a, v = kP, x1 = {{1, 0, 0, 0, 0, 0}}, x2 = {{0, 0, 0, 0, 0, 0}};
    auto is_one = [&](const fp64 &w) {
        for (int i = 1; i < 6; i++)
            if (w.l[i]) return false;
        return w.l[0] == 1;
    };
    while (!is_one(u) && !is_one(v)) {
        while (!(u.l[0] & 1)) {
            shr1(u);
            half_mod(x1);
        }
        while (!(v.l[0] & 1)) {
            shr1(v);
            half_mod(x2);
        }
        if (geq(u, v)) {
            sub_in(u, v);
            sub_mod(x1, x2);
        } else {
            sub_in(v, u);
            sub_mod(x2, x1);
        }
    }
    return is_one(u) ? x1 : x2;
}

}  // namespace hostfp

extern "C" {

// g_lagrange = iFFT(g) * n^-1 (arithmetic.rs:34-50); host buffers of 2^k points
RustError gb_g1_to_lagrange(RawG1Affine *out_raw, const RawG1Affine *g_raw, uint32_t k)
{
    if (k > 28) return make_error((int)cudaErrorInvalidValue, "g_to_lagrange: k too large");
    if (!out_raw || !g_raw) return make_error((int)cudaErrorInvalidValue, "null point buffers");
    GB_ENTRY_BEGIN
    const size_t n = (size_t)1 << k;
    cudaStream_t s = lane_stream();
    dev_buf<affine_t> din(n, s), dout(n, s);
    h2d(din, g_raw, n * sizeof(affine_t), s);
    g_to_lagrange_device(dout, din, k, s);
    d2h(out_raw, dout, n * sizeof(affine_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// SRS for a known tau (params.rs:79-129): g[i] = [tau^i] G,
// g_lagrange[i] = [(tau^n - 1)/n * w^i / (tau - w^i)] G; either output may be NULL
RustError gb_kzg_setup(RawG1Affine *g_out, RawG1Affine *g_lagrange_out, RawFr tau_raw, uint32_t k)
{
    if (k > 28) return make_error((int)cudaErrorInvalidValue, "kzg setup: k too large");
    GB_ENTRY_BEGIN
    const size_t n = (size_t)1 << k;
    const fr_t tau = from_raw(tau_raw);
    cudaStream_t s = lane_stream();
    dev_buf<fr_t> sc(n, s);
    dev_buf<affine_t> pts(n, s);
    if (g_out) {
        omega_powers(sc, tau, n, s);  // tau^i
        generator_mul_device(pts, sc, n, s);
        d2h(g_out, pts, n * sizeof(affine_t), s);
    }
    if (g_lagrange_out) {
        dev_buf<fr_t> wp(n, s), num(n, s);
        omega_powers(wp, host_omega(k, false), n, s);
        fr_t taun = tau.pow_u64((uint64_t)n);
        fr_t mult = (taun - fr_t::one()) * host_fr_inverse(host_fr_from_u64((uint64_t)n));
        lagrange_terms_kernel<<<blocks_for(n, 256), 256, 0, s>>>(wp, tau, mult, n, num, sc);
        GB_CHECK_LAUNCH();
        batch_invert(sc, sc, n, num, s);  // num / den
        generator_mul_device(pts, sc, n, s);
        d2h(g_lagrange_out, pts, n * sizeof(affine_t), s);
    }
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// Jacobian points (Montgomery, as the MSM entry points return them) to
// affine Montgomery coordinates; the point at infinity (Z = 0) becomes all
// zeros, the reference's RawG1Affine convention for it.  Host only: no
// device memory or stream is touched.  out and in may not overlap.
RustError gb_g1_jacobian_to_affine_batch(RawG1Affine *out_raw, const RawG1Projective *in_raw, size_t n)
{
    if (n && (!out_raw || !in_raw)) return make_error((int)cudaErrorInvalidValue, "invalid point conversion arguments");
    GB_ENTRY_BEGIN
    using namespace hostfp;
    static_assert(sizeof(RawG1Projective) == 18 * sizeof(uint64_t), "projective layout");
    static_assert(sizeof(RawG1Affine) == 12 * sizeof(uint64_t), "affine layout");
    const uint64_t *in = reinterpret_cast<const uint64_t *>(in_raw);
    uint64_t *out = reinterpret_cast<uint64_t *>(out_raw);
    std::vector<fp64> z(n), prefix(n);
    fp64 acc = kOne;  // running product of the nonzero z, Montgomery form
    for (size_t i = 0; i < n; i++) {
        for (int k = 0; k < 6; k++) z[i].l[k] = in[18 * i + 12 + k];
        reduce(z[i]);
        prefix[i] = acc;
        if (!is_zero(z[i])) acc = mont_mul(acc, z[i]);
    }
    // acc holds P R for the product P of the nonzero z: its plain inverse is
    // 1 / (P R), and the Montgomery product with R^3 gives R / P, the
    // Montgomery form of 1 / P
    fp64 inv = mont_mul(inverse(acc), kR3);
    for (size_t i = n; i-- > 0;) {
        uint64_t *o = out + 12 * i;
        if (is_zero(z[i])) {
            for (int k = 0; k < 12; k++) o[k] = 0;
            continue;
        }
        const fp64 zi = mont_mul(inv, prefix[i]);
        inv = mont_mul(inv, z[i]);
        fp64 x, y;
        for (int k = 0; k < 6; k++) {
            x.l[k] = in[18 * i + k];
            y.l[k] = in[18 * i + 6 + k];
        }
        reduce(x);
        reduce(y);
        const fp64 zi2 = mont_mul(zi, zi);
        const fp64 ax = mont_mul(x, zi2), ay = mont_mul(y, mont_mul(zi2, zi));
        for (int k = 0; k < 6; k++) {
            o[k] = ax.l[k];
            o[6 + k] = ay.l[k];
        }
    }
    return ok();
    GB_ENTRY_END
}

}  // extern "C"
