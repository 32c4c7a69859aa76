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
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "gb_ntt.cuh"

namespace gb {

static constexpr int kPassBits = 10;

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

// ---------------------------------------------------------------- host side

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
    });
}
}  // namespace

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

// Pass variant: 4 elements per thread (radix-4 register steps) from 2^18 up,
// where it is fastest on GB300; below that the radix-2 pass with up to 512
// threads keeps more warps resident.  GB_NTT_ELEMS_LOG (1, 2, 3) overrides;
// with the autotuner on, each size times the three variants once on a
// scratch copy of one transform.
static int ntt_variant(fr_t *d, uint32_t log_n, const fr_t *tw, cudaStream_t s)
{
    static const int el_env = [] {
        const char *e = getenv("GB_NTT_ELEMS_LOG");
        return e && (e[0] == '1' || e[0] == '2' || e[0] == '3') ? e[0] - '0' : 0;
    }();
    if (el_env) return el_env;
    int el = log_n >= 18 ? 2 : 1;
    if (!autotune_enabled() || log_n < 10) return el;
    const std::string key = "ntt:2^" + std::to_string(log_n);
    if (autotune_lookup(key, &el)) return el;
    const size_t n = (size_t)1 << log_n;
    dev_buf<fr_t> scratch(n, s);
    float best = 1e30f;
    for (int cand = 1; cand <= 3; cand++) {
        GB_CUDA_OK(cudaMemcpyAsync(scratch.get(), d, n * sizeof(fr_t), cudaMemcpyDeviceToDevice, s));
        float ms = time_on_stream(s, [&] { ntt_passes(scratch, log_n, 1, tw, cand, s); });
        if (ms < best) {
            best = ms;
            el = cand;
        }
    }
    autotune_store(key, el);
    return el;
}

void ntt_inplace(fr_t *d, uint32_t log_n, size_t count, bool inverse, const fr_t *scale, cudaStream_t s)
{
    if (count == 0) return;
    const size_t n = (size_t)1 << log_n;
    if (log_n > 0) {
        set_ntt_smem();
        const fr_t *tw = twiddles(log_n, inverse, s);
        ntt_passes(d, log_n, count, tw, ntt_variant(d, log_n, tw, s), s);
    }
    dim3 grid(blocks_for(n, 256), (unsigned)count);
    bitrev_scale_kernel<<<grid, 256, 0, s>>>(d, log_n, scale != nullptr, scale ? *scale : fr_t::one());
    GB_CHECK_LAUNCH();
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
static void ntt_ref(fr_t *d, uint32_t log_n, size_t count, bool inverse, cudaStream_t s)
{
    if (inverse) {
        fr_t ninv = host_fr_inverse(host_fr_from_u64((uint64_t)1 << log_n));
        ntt_inplace(d, log_n, count, true, &ninv, s);
    } else {
        ntt_inplace(d, log_n, count, false, nullptr, s);
    }
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
    dev_buf<fr_t> d(n, s);
    h2d(d, values, n * sizeof(fr_t), s);
    ntt_ref(d, log_n, 1, inverse, s);
    d2h(values, d, n * sizeof(fr_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
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
    dev_buf<fr_t> d(n, s);
    h2d(d, values, n * sizeof(fr_t), s);
    ntt_ref(d, log_n, 1, inverse, s);
    launch_scale_zeta(d, scale, first, second, n, n, s);
    d2h(values, d, n * sizeof(fr_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
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
    dev_buf<fr_t> d(n, s), f(factor_len, s);
    h2d(d, values, n * sizeof(fr_t), s);
    h2d(f, factors, factor_len * sizeof(fr_t), s);
    launch_mul_assign_repeating(d, f, factor_len, n, s);
    ntt_ref(d, log_n, 1, true, s);
    launch_scale_zeta(d, scale, first, second, n, n, s);
    d2h(values, d, n * sizeof(fr_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
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
    dev_buf<fr_t> din(input_len * count, s), dout(output_len * count, s);
    h2d(din, inputs, input_len * count * sizeof(fr_t), s);
    launch_coeff_to_extended_prepare(dout, din, first, second, input_len, output_len, count, s);
    ntt_ref(dout, extended_log_n, count, false, s);
    d2h(out, dout, output_len * count * sizeof(fr_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
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
    dev_buf<fr_t> din(input_len * count, s);
    h2d(din, inputs, input_len * count * sizeof(fr_t), s);
    fr_device_vec *v = device_vec_new(output_len * count, s);
    try {
        launch_coeff_to_extended_prepare(v->values, din, first, second, input_len, output_len, count, s);
        ntt_ref(v->values, extended_log_n, count, false, s);
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
    fr_device_vec *v = device_vec_new(output_len * count, s);
    try {
        launch_coeff_to_extended_prepare(v->values, src->values, first, second, input_len, output_len, count, s);
        ntt_ref(v->values, extended_log_n, count, false, s);
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
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    ntt_ref(v->values, log_n, 1, inverse, s);
    launch_scale_zeta(v->values, scale, first, second, n, n, s);
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
    ntt_ref(v->values, log_n, count, inverse, s);
    launch_scale_zeta(v->values, scale, first, second, n * count, n, s);
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
    dev_buf<fr_t> f(factor_len, s);
    h2d(f, factors, factor_len * sizeof(fr_t), s);
    launch_mul_assign_repeating(v->values, f, factor_len, n, s);
    ntt_ref(v->values, log_n, 1, true, s);
    launch_scale_zeta(v->values, scale, first, second, n, n, s);
    device_vec_mark_ready(v, s);
    return ok();
    GB_ENTRY_END
}

}  // extern "C"
