// Fixed-base G1 scalar multiplication by the generator ([s_i] G, affine out)
// and the integer multiply-add peak probe.
//
// [s]G is what an SRS needs (g_i = [tau^i] G, params.rs:38-129) and what the
// synthetic MSM inputs need (bases [r_i] G).  The generator table holds
// d * 2^(8w) G for w < 32, d < 256 (786 KB, built once per device on the
// device), so one [s]G costs at most 32 mixed additions and one inversion.
#include <algorithm>

#include <mutex>

#include "gb_runtime.cuh"

namespace gb {

// The generator is supplied by the host in canonical form and converted here
// (keeps the constant in one readable place: the canonical hex of the
// BLS12-381 G1 generator).
__global__ void gen_table_bases_kernel(affine_t gen_canonical, xyzz_t *bases)
{
    // thread w: 2^(8w) G
    int w = threadIdx.x;
    if (w >= 32) return;
    affine_t g;
    g.x = gen_canonical.x.to_mont();
    g.y = gen_canonical.y.to_mont();
    xyzz_t acc = xyzz_t::from_affine(g);
    for (int k = 0; k < 8 * w; k++) acc = acc.dbl();
    bases[w] = acc;
}

__global__ void gen_table_fill_kernel(const xyzz_t *bases, affine_t *table)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 32 * 256) return;
    int w = t >> 8, d = t & 255;
    xyzz_t p = xyzz_mul_small(bases[w], (uint32_t)d);
    table[t] = p.to_affine();
}

__global__ void generator_mul_kernel(const fr_t *__restrict__ scalars, size_t n, const affine_t *__restrict__ table,
                                     affine_t *__restrict__ out)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fr_t s = scalars[i].from_mont();
    xyzz_t acc = xyzz_t::inf();
    for (int w = 0; w < 32; w++) {
        uint32_t d = (s.v[w >> 2] >> (8 * (w & 3))) & 0xffu;
        if (d) acc.add_affine(table[w * 256 + d], false);
    }
    out[i] = acc.to_affine();
}

static affine_t host_generator_canonical()
{
    // x, y of the BLS12-381 G1 generator, canonical little-endian u32 limbs
    static const char *X = "17f1d3a73197d7942695638c4fa9ac0fc3688c4f9774b905a14e3a3f171bac586c55e83ff97a1aeffb3af00adb22c6bb";
    static const char *Y = "08b3f481e3aaa0f1a09e30ed741d8ae4fcf5e095d5d00af600db18cb2c04b3edd03cc744a2888ae40caa232946c5e7e1";
    affine_t g;
    auto parse = [](const char *hex, fp_t &out) {
        for (int i = 0; i < 12; i++) out.v[i] = 0;
        size_t len = strlen(hex);
        for (size_t k = 0; k < len; k++) {
            char ch = hex[len - 1 - k];
            uint32_t v = (ch >= '0' && ch <= '9') ? (uint32_t)(ch - '0') : (uint32_t)(ch - 'a' + 10);
            out.v[k / 8] |= v << (4 * (k % 8));
        }
    };
    parse(X, g.x);
    parse(Y, g.y);
    return g;
}

namespace {
std::mutex g_gen_mu;
affine_t *g_gen_table[64];
}  // namespace

const affine_t *generator_table(cudaStream_t s)
{
    int dev = current_device();
    std::lock_guard<std::mutex> lk(g_gen_mu);
    if (g_gen_table[dev]) return g_gen_table[dev];
    affine_t *table = nullptr;
    xyzz_t *bases = nullptr;
    GB_CUDA_OK(cudaMalloc(&table, 32 * 256 * sizeof(affine_t)));
    GB_CUDA_OK(cudaMalloc(&bases, 32 * sizeof(xyzz_t)));
    gen_table_bases_kernel<<<1, 32, 0, s>>>(host_generator_canonical(), bases);
    GB_CHECK_LAUNCH();
    gen_table_fill_kernel<<<32, 256, 0, s>>>(bases, table);
    GB_CHECK_LAUNCH();
    lane_sync(s);
    cudaFree(bases);
    g_gen_table[dev] = table;
    return table;
}

void generator_mul_device(affine_t *d_out, const fr_t *d_scalars, size_t n, cudaStream_t s)
{
    if (!n) return;
    const affine_t *t = generator_table(s);
    generator_mul_kernel<<<blocks_for(n, 128), 128, 0, s>>>(d_scalars, n, t, d_out);
    GB_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- peak probe
// Throughput of 32x32->64 multiply-adds, the unit in which the hot path's
// algorithmic work is counted (one Fp Montgomery product = 2*12^2 + 12 = 300
// of them, one Fr product = 2*8^2 + 8 = 136).  A multiply-add is one 64-bit
// product: a mad.lo / madc.hi instruction pair, or one mad.wide.  Two
// instruction forms are timed and the fastest configuration is the peak:
//   * mad.wide.u32 chains: acc = lo32(acc) * y + acc, 8 chains per thread;
//   * carry-chained rows as in a CIOS Montgomery step: a 12-limb operand
//     times a multiplier, as an even-limb and an odd-limb row of 6 products
//     each (mad.lo.cc / madc.hi.cc), on SETS independent accumulators per
//     thread; each accumulator's next multiplier derives from its own result.
// Every product depends on a value produced inside the loop, so no form can
// be hoisted or strength-reduced; results are folded into `sink`.
__global__ void peak_wide_kernel(uint32_t y, int iters, unsigned long long *sink)
{
    uint64_t acc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) acc[k] = (uint64_t)(threadIdx.x * 8u + k + 1u) * 0x9E3779B97F4A7C15ull;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < 8; k++)
            asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(acc[k]) : "r"((uint32_t)acc[k]), "r"(y));
    }
    uint64_t r = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) r ^= acc[k];
    if (r == 0x123456789ull) atomicAdd(sink, r);
}

template <int SETS>
__global__ void peak_row_kernel(uint32_t y, int iters, unsigned long long *sink)
{
    uint32_t e[SETS][13], o[SETS][13], a[12], bi[SETS];
#pragma unroll
    for (int k = 0; k < 12; k++) a[k] = (threadIdx.x + 1u) * 0x9E3779B9u + (uint32_t)k;
#pragma unroll
    for (int q = 0; q < SETS; q++) {
#pragma unroll
        for (int k = 0; k < 13; k++) {
            e[q][k] = (uint32_t)(k + 13 * q);
            o[q][k] = (uint32_t)(3 * k + q);
        }
        bi[q] = y ^ (threadIdx.x * (uint32_t)(q + 1));
    }
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int q = 0; q < SETS; q++) {
            row_mac12(e[q], a[0], a[2], a[4], a[6], a[8], a[10], bi[q]);
            row_mac12(o[q], a[1], a[3], a[5], a[7], a[9], a[11], bi[q]);
            bi[q] = e[q][0] ^ o[q][12];
        }
    }
    uint32_t r = 0;
#pragma unroll
    for (int q = 0; q < SETS; q++)
#pragma unroll
        for (int k = 0; k < 13; k++) r ^= e[q][k] ^ o[q][k];
    if (r == 0x1234567u) atomicAdd(sink, (unsigned long long)r);
}

}  // namespace gb

using namespace gb;

extern "C" {

// out[i] = affine([scalars[i]] G); host buffers.  Used to build SRS bases.
RustError gb_g1_generator_mul(RawG1Affine *out_raw, const RawFr *scalars_raw, size_t n)
{
    affine_t *out = reinterpret_cast<affine_t *>(out_raw);
    const fr_t *scalars = reinterpret_cast<const fr_t *>(scalars_raw);
    if (n == 0) return ok();
    if (!out || !scalars) return make_error((int)cudaErrorInvalidValue, "invalid generator mul arguments");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    dev_buf<fr_t> ds(n, s);
    dev_buf<affine_t> dout(n, s);
    h2d(ds, scalars, n * sizeof(fr_t), s);
    generator_mul_device(dout, ds, n, s);
    d2h(out, dout, n * sizeof(affine_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// Device-pointer variant (both pointers are device memory), async on the lane.
RustError gb_g1_generator_mul_device(RawG1Affine *d_out_raw, const RawFr *d_scalars_raw, size_t n)
{
    affine_t *d_out = reinterpret_cast<affine_t *>(d_out_raw);
    const fr_t *d_scalars = reinterpret_cast<const fr_t *>(d_scalars_raw);
    if (n == 0) return ok();
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    generator_mul_device(d_out, d_scalars, n, s);
    return ok();
    GB_ENTRY_END
}

// Multiply-add throughput of one probe form (whole device, 32x32->64
// products per second): form 0 = mad.wide chains, forms 1..3 = carry-chained
// rows with 1, 2 or 4 independent accumulator sets per thread.
RustError gb_imad_probe(int form, double *out_per_sec)
{
    if (!out_per_sec || form < 0 || form > 3) return make_error((int)cudaErrorInvalidValue, "invalid probe form");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    int dev = current_device(), sms = 0;
    GB_CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    unsigned long long *sink = nullptr;
    GB_CUDA_OK(cudaMallocAsync((void **)&sink, sizeof(*sink), s));
    const int threads = 256, blocks = sms * 8, iters = 2048;
    const double per_iter = form == 0 ? 8.0 : 12.0 * (1 << (form - 1));
    cudaEvent_t e0, e1;
    GB_CUDA_OK(cudaEventCreate(&e0));
    GB_CUDA_OK(cudaEventCreate(&e1));
    double best = 0;
    for (int rep = 0; rep < 3; rep++) {  // the first run warms up
        GB_CUDA_OK(cudaEventRecord(e0, s));
        if (form == 0) peak_wide_kernel<<<blocks, threads, 0, s>>>(0x9E3779B9u, iters, sink);
        else if (form == 1) peak_row_kernel<1><<<blocks, threads, 0, s>>>(0x9E3779B9u, iters, sink);
        else if (form == 2) peak_row_kernel<2><<<blocks, threads, 0, s>>>(0x9E3779B9u, iters, sink);
        else peak_row_kernel<4><<<blocks, threads, 0, s>>>(0x9E3779B9u, iters, sink);
        GB_CHECK_LAUNCH();
        GB_CUDA_OK(cudaEventRecord(e1, s));
        GB_CUDA_OK(cudaEventSynchronize(e1));
        float ms = 0;
        GB_CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
        if (rep) best = std::max(best, (double)blocks * threads * iters * per_iter / (ms * 1e-3));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(sink, s);
    *out_per_sec = best;
    return ok();
    GB_ENTRY_END
}

// Measured multiply-add peak: the fastest of the probe forms.
RustError gb_imad_peak(double *out_per_sec)
{
    if (!out_per_sec) return make_error((int)cudaErrorInvalidValue, "null output");
    double best = 0;
    for (int form = 0; form < 4; form++) {
        double r = 0;
        RustError e = gb_imad_probe(form, &r);
        if (e.code) return e;
        best = std::max(best, r);
    }
    *out_per_sec = best;
    return ok();
}

}  // extern "C"
