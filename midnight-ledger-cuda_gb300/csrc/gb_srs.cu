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

}  // extern "C"
