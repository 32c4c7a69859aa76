// BLS12-381 G1 multiexp (Pippenger) for sm_103a, and the MSM entry points
// of the C ABI (midnight-sppark-msm/src/bls12_381_g1_msm.cu:6164-6486).
//
// Pipeline for one MSM of n (scalar, base) pairs with window c:
//   1. recode     : Montgomery -> canonical, signed c-bit digits per window
//                   (digit in [-2^(c-1), 2^(c-1)], carry into the next window)
//   2. histogram  : per-block shared-memory counts of bucket keys
//   3. column scan: per-key prefix over blocks + per-key totals
//   4. key scan   : exclusive scan of totals -> bucket start offsets
//   5. scatter    : (bucket, point) pairs placed in bucket order
//   6. accumulate : each thread sums L consecutive sorted entries into XYZZ
//                   accumulators (fixed work per thread), writing finished
//                   buckets directly and chunk-edge partials aside
//   7. fix-up     : buckets spanning chunks add their partials
//   8. reduce     : sum_k (k+1) * B_k per window by segmented running sums,
//                   then a tree over segments, then the window combination.
//
// Two modes share this pipeline.  "Plain" mode keys buckets by
// (window, digit) and combines windows by Horner's rule.  "Precomputed" mode
// (MSM contexts, whose bases are fixed) stores 2^(c*j) * P_i for every window
// j at context creation, so all windows feed ONE set of 2^(c-1) buckets and
// no window combination is needed.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "gb_runtime.cuh"

namespace gb {

static constexpr uint32_t kZeroDigit = 0xffffffffu;
static constexpr int kMaxWindowBits = 16;  // 2^15 u32 counters = 128 KB smem

struct msm_plan {
    int c;             // window bits
    int nwin;          // windows: floor(255 / c) + 1 -> nwin * c >= 256
    bool precomputed;  // bases hold 2^(c*j) P_i for every window j
    size_t n;          // points
    uint32_t K;        // buckets per segment = 2^(c-1)
    uint32_t nseg;     // segments: nwin (plain) or 1 (precomputed)
    uint32_t G;        // total buckets = nseg * K
    size_t seglen;     // digits per segment
    uint32_t bps;      // sort blocks per segment
    size_t per_block;  // digits per sort block
    uint32_t L;        // sorted entries per accumulate thread
    uint32_t S;        // reduction sub-segments per segment
    int acc_variant;   // accumulate kernel instantiation (0: 256x1, 1: 256x2, 2: 128x3);
                       // GB_MSM_ACC_VARIANT overrides the default for tuning runs
};

static int default_acc_variant()
{
    const char *e = getenv("GB_MSM_ACC_VARIANT");
    if (e && e[0] >= '0' && e[0] <= '2') return e[0] - '0';
    return 1;  // 256 threads, 2 blocks per SM: the fastest on GB300 at n = 2^20
}

static int windows_for(int c) { return 255 / c + 1; }

static msm_plan make_plan(size_t n, int c, bool precomputed)
{
    msm_plan p;
    p.c = c;
    p.nwin = windows_for(c);
    p.precomputed = precomputed;
    p.n = n;
    p.K = 1u << (c - 1);
    p.nseg = precomputed ? 1 : (uint32_t)p.nwin;
    p.G = p.nseg * p.K;
    p.seglen = precomputed ? n * (size_t)p.nwin : n;
    size_t total = n * (size_t)p.nwin;
    // aim for ~4 sort blocks per SM-pair over all segments, >= 4096 digits each
    size_t target_blocks = 608;
    size_t per = (total + target_blocks - 1) / target_blocks;
    per = std::max<size_t>(per, 4096);
    per = std::min<size_t>(per, (size_t)1 << 16);
    p.bps = (uint32_t)((p.seglen + per - 1) / per);
    p.per_block = (p.seglen + p.bps - 1) / p.bps;
    // accumulate chunk: about 2 expected entries per bucket, 8..64
    double avg = (double)total / (double)p.G;
    uint32_t L = (uint32_t)std::max(8.0, std::min(64.0, avg * 0.5));
    p.L = L;
    uint32_t S = std::min<uint32_t>(p.K, precomputed ? 8192u : 256u);
    p.S = S;
    p.acc_variant = default_acc_variant();
    return p;
}

// Window size: minimise mixed additions plus bucket-reduction additions.
static int choose_window(size_t n, bool precomputed)
{
    if (n <= 1) return 8;
    int best = 8;
    double best_cost = 1e300;
    for (int c = 8; c <= kMaxWindowBits; c++) {
        double w = windows_for(c);
        double adds = (double)n * w;
        double red = (precomputed ? 1.0 : w) * std::ldexp(1.0, c) * 1.4;
        double cost = adds + red;
        if (cost < best_cost) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

__device__ __forceinline__ affine_t load_affine(const affine_t *pts, uint32_t idx)
{
    const uint4 *src = reinterpret_cast<const uint4 *>(pts + idx);
    affine_t r;
    uint4 *dst = reinterpret_cast<uint4 *>(&r);
#pragma unroll
    for (int i = 0; i < 6; i++) dst[i] = __ldg(src + i);
    return r;
}

// 1. recode: digits[j * n + i] = key | sign << 31, or kZeroDigit
__global__ void msm_recode_kernel(const fr_t *__restrict__ scalars, size_t n, int c, int nwin,
                                  uint32_t key_stride, uint32_t *__restrict__ digits)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fr_t s = scalars[i];
    s = s.from_mont();
    const uint32_t half = 1u << (c - 1);
    const uint32_t mask = (1u << c) - 1;
    uint32_t carry = 0;
    for (int j = 0; j < nwin; j++) {
        int bit = j * c;
        int limb = bit >> 5, off = bit & 31;
        uint32_t lo = limb < 8 ? s.v[limb] : 0;
        uint32_t hi = limb + 1 < 8 ? s.v[limb + 1] : 0;
        uint32_t raw = (uint32_t)((((uint64_t)hi << 32) | lo) >> off) & mask;
        raw += carry;
        uint32_t out;
        if (raw == 0) {
            carry = 0;
            out = kZeroDigit;
        } else if (raw <= half) {
            carry = 0;
            out = (raw - 1) + (uint32_t)j * key_stride;
        } else {
            carry = 1;
            uint32_t mag = (1u << c) - raw;  // digit = raw - 2^c < 0
            out = mag == 0 ? kZeroDigit : (((mag - 1) + (uint32_t)j * key_stride) | 0x80000000u);
        }
        digits[(size_t)j * n + i] = out;
    }
}

// 2. per-block histograms: hist[b][k] for block b of segment (b / bps)
__global__ void msm_hist_kernel(const uint32_t *__restrict__ digits, size_t seglen, uint32_t bps,
                                size_t per_block, uint32_t K, uint32_t *__restrict__ hist)
{
    extern __shared__ uint32_t sh[];
    const uint32_t b = blockIdx.x;
    const uint32_t seg = b / bps, within = b % bps;
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) sh[k] = 0;
    __syncthreads();
    size_t lo = (size_t)within * per_block;
    size_t hi = std::min(lo + per_block, seglen);
    const uint32_t *d = digits + (size_t)seg * seglen;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        uint32_t v = d[i];
        if (v != kZeroDigit) atomicAdd(&sh[(v & 0x7fffffffu) & (K - 1)], 1u);
    }
    __syncthreads();
    uint32_t *out = hist + (size_t)b * K;
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) out[k] = sh[k];
}

// 3. per global key g = seg*K + k: exclusive prefix over the segment's
//    blocks (in place in hist) and the total into counts[g]
__global__ void msm_colscan_kernel(uint32_t *__restrict__ hist, uint32_t bps, uint32_t K,
                                   uint32_t G, uint32_t *__restrict__ counts)
{
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    uint32_t seg = g / K, k = g % K;
    uint32_t run = 0;
    uint32_t *col = hist + (size_t)seg * bps * K + k;
    uint32_t w = 0;
    // batches of 16 independent loads keep the column walk off the latency path
    for (; w + 16 <= bps; w += 16) {
        uint32_t v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) v[u] = col[(size_t)(w + u) * K];
#pragma unroll
        for (int u = 0; u < 16; u++) {
            col[(size_t)(w + u) * K] = run;
            run += v[u];
        }
    }
    for (; w < bps; w++) {
        uint32_t v = col[(size_t)w * K];
        col[(size_t)w * K] = run;
        run += v;
    }
    counts[g] = run;
}

// 4. exclusive scan of counts[0..G) into starts[0..G], starts[G] = total.
//    One block; each thread scans a contiguous run.
__global__ void msm_keyscan_kernel(const uint32_t *__restrict__ counts, uint32_t G,
                                   uint32_t *__restrict__ starts)
{
    __shared__ uint32_t part[1024];
    const uint32_t T = blockDim.x;
    const uint32_t per = (G + T - 1) / T;
    const uint32_t lo = threadIdx.x * per;
    const uint32_t hi = min(lo + per, G);
    uint32_t sum = 0;
    for (uint32_t i = lo; i < hi; i++) sum += counts[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    // Hillis-Steele inclusive scan over the per-thread sums
    for (uint32_t off = 1; off < T; off <<= 1) {
        uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (uint32_t i = lo; i < hi; i++) {
        starts[i] = run;
        run += counts[i];
    }
    if (threadIdx.x == T - 1) starts[G] = part[T - 1];
}

// 5. scatter into bucket order: sorted[pos] = point_ref | sign << 31
__global__ void msm_scatter_kernel(const uint32_t *__restrict__ digits, size_t n, size_t seglen,
                                   uint32_t bps, size_t per_block, uint32_t K, int precomputed,
                                   const uint32_t *__restrict__ hist, const uint32_t *__restrict__ starts,
                                   uint32_t *__restrict__ sorted)
{
    extern __shared__ uint32_t cursor[];
    const uint32_t b = blockIdx.x;
    const uint32_t seg = b / bps, within = b % bps;
    const uint32_t *h = hist + (size_t)b * K;
    const uint32_t *st = starts + (size_t)seg * K;
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) cursor[k] = st[k] + h[k];
    __syncthreads();
    size_t lo = (size_t)within * per_block;
    size_t hi = std::min(lo + per_block, seglen);
    const uint32_t *d = digits + (size_t)seg * seglen;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        uint32_t v = d[i];
        if (v == kZeroDigit) continue;
        uint32_t k = (v & 0x7fffffffu) & (K - 1);
        uint32_t pos = atomicAdd(&cursor[k], 1u);
        // point reference: precomputed mode indexes the (window, point) table,
        // which is laid out exactly like the digit array; plain mode uses the
        // point index within the window.
        uint32_t ref = precomputed ? (uint32_t)i : (uint32_t)(i % n);
        sorted[pos] = ref | (v & 0x80000000u);
    }
}

// 6. accumulate L sorted entries per thread.  Instantiated for several
//    (block size, min blocks per SM) pairs: the register cap trades
//    occupancy against spills, and the plan picks one.
template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) msm_accumulate_kernel(
    const uint32_t *__restrict__ sorted, const uint32_t *__restrict__ starts, uint32_t G, uint32_t L,
    size_t nchunks, const affine_t *__restrict__ points, xyzz_t *__restrict__ buckets,
    xyzz_t *__restrict__ head, xyzz_t *__restrict__ tail)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nchunks) return;
    const uint32_t T = starts[G];
    const uint64_t lo = (uint64_t)t * L;
    if (lo >= T) return;
    const uint64_t hi = min((uint64_t)T, lo + L);
    // largest g with starts[g] <= lo; starts[G] = T > lo
    uint32_t a = 0, b = G;
    while (b - a > 1) {
        uint32_t mid = (a + b) >> 1;
        if (starts[mid] <= lo) a = mid;
        else b = mid;
    }
    uint32_t g = a;
    uint32_t gend = starts[g + 1];
    bool started_here = starts[g] >= lo;
    bool open = false;
    xyzz_t acc = xyzz_t::inf();
    for (uint64_t pos = lo; pos < hi; pos++) {
        uint32_t ref = sorted[pos];
        affine_t p = load_affine(points, ref & 0x7fffffffu);
        acc.add_affine(p, (ref >> 31) != 0);
        open = true;
        if (pos + 1 == gend) {
            if (started_here) buckets[g] = acc;
            else head[t] = acc;
            acc = xyzz_t::inf();
            open = false;
            started_here = true;
            g++;
            while (g < G && starts[g + 1] == starts[g]) g++;
            gend = g < G ? starts[g + 1] : T;
        }
    }
    if (open) tail[t] = acc;
}

// 7. buckets spanning several chunks; empty buckets become infinity
__global__ void msm_fixup_kernel(const uint32_t *__restrict__ starts, uint32_t G, uint32_t L,
                                 const xyzz_t *__restrict__ head, const xyzz_t *__restrict__ tail,
                                 xyzz_t *__restrict__ buckets)
{
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    uint32_t s = starts[g], e = starts[g + 1];
    if (s == e) {
        buckets[g] = xyzz_t::inf();
        return;
    }
    uint32_t cs = s / L, ce = (e - 1) / L;
    if (cs == ce) return;
    xyzz_t acc = tail[cs];
    for (uint32_t c = cs + 1; c < ce; c++) acc.add(tail[c]);
    acc.add(head[ce]);
    buckets[g] = acc;
}

// 8a. per (segment, sub-segment): U = sum_{k in sub} (k+1) B_k
__global__ void msm_reduce_partial_kernel(const xyzz_t *__restrict__ buckets, uint32_t K, uint32_t S,
                                          uint32_t nseg, xyzz_t *__restrict__ partial)
{
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nseg * S) return;
    uint32_t seg = t / S, s = t % S;
    uint32_t m = K / S;
    uint32_t k0 = s * m;
    const xyzz_t *B = buckets + (size_t)seg * K;
    xyzz_t run = xyzz_t::inf(), sum = xyzz_t::inf();
    for (uint32_t k = k0 + m; k-- > k0;) {
        run.add(B[k]);
        sum.add(run);
    }
    if (k0) sum.add(xyzz_mul_small(run, k0));
    partial[t] = sum;
}

// 8b. tree sum: out[seg * gridDim.x + b] = sum of the 512-element slice b of
//     in[seg * n .. seg * n + n), one block of 256 threads per slice
__global__ void __launch_bounds__(256) xyzz_tree_sum_kernel(const xyzz_t *__restrict__ in, uint32_t n,
                                                            xyzz_t *__restrict__ out)
{
    __shared__ xyzz_t sh[256];
    const uint32_t seg = blockIdx.y;
    const xyzz_t *src = in + (size_t)seg * n;
    uint32_t i0 = blockIdx.x * 512 + threadIdx.x, i1 = i0 + 256;
    xyzz_t acc = i0 < n ? src[i0] : xyzz_t::inf();
    if (i1 < n) acc.add(src[i1]);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            xyzz_t v = sh[threadIdx.x];
            v.add(sh[threadIdx.x + off]);
            sh[threadIdx.x] = v;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)seg * gridDim.x + blockIdx.x] = sh[0];
}

// 8c. combine windows (Horner) and emit a Jacobian point
__global__ void msm_combine_kernel(const xyzz_t *__restrict__ seg_sum, uint32_t nseg, int c,
                                   jacobian_t *__restrict__ out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    xyzz_t acc = xyzz_t::inf();
    for (int w = (int)nseg - 1; w >= 0; w--) {
        if (w != (int)nseg - 1)
            for (int k = 0; k < c; k++) acc = acc.dbl();
        acc.add(seg_sum[w]);
    }
    *out = acc.to_jacobian();
}

// precompute: table[j * n + i] = 2^(c*j) P_i
__global__ void msm_precompute_kernel(affine_t *table, size_t n, int c, int nwin)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    affine_t p = table[i];
    xyzz_t acc = xyzz_t::from_affine(p);
    for (int j = 1; j < nwin; j++) {
        for (int k = 0; k < c; k++) acc = acc.dbl();
        table[(size_t)j * n + i] = acc.to_affine();
    }
}

// scrambled scalars: out[i] = in[i] + mask[i mod mask_len]
__global__ void add_mask_kernel(fr_t *__restrict__ out, const fr_t *__restrict__ in, const fr_t *__restrict__ mask,
                                size_t mask_len, size_t len)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) out[i] = in[i] + mask[i % mask_len];
}

// ---------------------------------------------------------------------------
// host engine
// ---------------------------------------------------------------------------

struct msm_workspace {
    dev_buf<uint32_t> digits, hist, counts, starts, sorted;
    dev_buf<xyzz_t> buckets, head, tail, partial, segsum;
};

static void set_smem_attrs()
{
    static std::once_flag once;
    std::call_once(once, [] {
        int bytes = (1 << (kMaxWindowBits - 1)) * 4;
        cudaFuncSetAttribute(msm_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cudaFuncSetAttribute(msm_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    });
}

// Run one MSM over device-resident scalars; result written to d_out (device).
static void msm_run(const msm_plan &p, const affine_t *d_points, const fr_t *d_scalars,
                    jacobian_t *d_out, cudaStream_t s)
{
    set_smem_attrs();
    if (p.n == 0) {
        xyzz_t inf = xyzz_t::inf();
        jacobian_t j = inf.to_jacobian();
        GB_CUDA_OK(cudaMemcpyAsync(d_out, &j, sizeof(j), cudaMemcpyHostToDevice, s));
        GB_CUDA_OK(cudaStreamSynchronize(s));
        return;
    }
    const size_t total = p.n * (size_t)p.nwin;
    const uint32_t nblocks = p.nseg * p.bps;
    const size_t nchunks = (total + p.L - 1) / p.L;
    msm_workspace w;
    w.digits = dev_buf<uint32_t>(total, s);
    w.hist = dev_buf<uint32_t>((size_t)nblocks * p.K, s);
    w.counts = dev_buf<uint32_t>(p.G, s);
    w.starts = dev_buf<uint32_t>(p.G + 1, s);
    w.sorted = dev_buf<uint32_t>(total, s);
    w.buckets = dev_buf<xyzz_t>(p.G, s);
    w.head = dev_buf<xyzz_t>(nchunks, s);
    w.tail = dev_buf<xyzz_t>(nchunks, s);
    w.partial = dev_buf<xyzz_t>((size_t)p.nseg * p.S, s);
    w.segsum = dev_buf<xyzz_t>(p.nseg, s);

    int tok_all = timed_begin(s);
    msm_recode_kernel<<<blocks_for(p.n, 256), 256, 0, s>>>(d_scalars, p.n, p.c, p.nwin,
                                                           p.precomputed ? 0u : p.K, w.digits);
    GB_CHECK_LAUNCH();
    size_t smem = (size_t)p.K * 4;
    msm_hist_kernel<<<nblocks, 1024, smem, s>>>(w.digits, p.seglen, p.bps, p.per_block, p.K, w.hist);
    GB_CHECK_LAUNCH();
    msm_colscan_kernel<<<blocks_for(p.G, 256), 256, 0, s>>>(w.hist, p.bps, p.K, p.G, w.counts);
    GB_CHECK_LAUNCH();
    msm_keyscan_kernel<<<1, 1024, 0, s>>>(w.counts, p.G, w.starts);
    GB_CHECK_LAUNCH();
    msm_scatter_kernel<<<nblocks, 1024, smem, s>>>(w.digits, p.n, p.seglen, p.bps, p.per_block, p.K,
                                                   p.precomputed ? 1 : 0, w.hist, w.starts, w.sorted);
    GB_CHECK_LAUNCH();
    int tok = timed_begin(s);
    if (p.acc_variant == 1) {
        msm_accumulate_kernel<256, 2><<<blocks_for(nchunks, 256), 256, 0, s>>>(
            w.sorted, w.starts, p.G, p.L, nchunks, d_points, w.buckets, w.head, w.tail);
    } else if (p.acc_variant == 2) {
        msm_accumulate_kernel<128, 3><<<blocks_for(nchunks, 128), 128, 0, s>>>(
            w.sorted, w.starts, p.G, p.L, nchunks, d_points, w.buckets, w.head, w.tail);
    } else {
        msm_accumulate_kernel<256, 1><<<blocks_for(nchunks, 256), 256, 0, s>>>(
            w.sorted, w.starts, p.G, p.L, nchunks, d_points, w.buckets, w.head, w.tail);
    }
    GB_CHECK_LAUNCH();
    timed_end(tok, s, GB_SLOT_MSM_ACCUMULATE);
    msm_fixup_kernel<<<blocks_for(p.G, 128), 128, 0, s>>>(w.starts, p.G, p.L, w.head, w.tail, w.buckets);
    GB_CHECK_LAUNCH();
    msm_reduce_partial_kernel<<<blocks_for((size_t)p.nseg * p.S, 128), 128, 0, s>>>(
        w.buckets, p.K, p.S, p.nseg, w.partial);
    GB_CHECK_LAUNCH();
    // tree-sum each segment's S partials down to one point
    {
        const xyzz_t *src = w.partial;
        uint32_t len = p.S;
        dev_buf<xyzz_t> tmp_a, tmp_b;
        bool use_a = true;
        while (len > 1) {
            uint32_t blocks = (len + 511) / 512;
            dev_buf<xyzz_t> &dst = use_a ? tmp_a : tmp_b;
            dst = dev_buf<xyzz_t>((size_t)p.nseg * blocks, s);
            xyzz_tree_sum_kernel<<<dim3(blocks, p.nseg), 256, 0, s>>>(src, len, dst);
            GB_CHECK_LAUNCH();
            src = dst;
            len = blocks;
            use_a = !use_a;
        }
        GB_CUDA_OK(cudaMemcpyAsync(w.segsum, src, (size_t)p.nseg * sizeof(xyzz_t), cudaMemcpyDeviceToDevice, s));
    }
    msm_combine_kernel<<<1, 32, 0, s>>>(w.segsum, p.nseg, p.c, d_out);
    GB_CHECK_LAUNCH();
    timed_end(tok_all, s, GB_SLOT_MSM_TOTAL);
}

}  // namespace gb

// ---------------------------------------------------------------------------
// context + C ABI
// ---------------------------------------------------------------------------

namespace gb {

struct msm_context_t {
    int device = 0;
    size_t npoints = 0;
    RawMsmConfig config{};
    int c = 0;
    int nwin = 0;
    affine_t *table = nullptr;  // [nwin][npoints]: 2^(c*j) P_i
    cudaStream_t owner = nullptr;
    std::mutex mu;
};

static RawMsmConfig default_config(size_t npoints)
{
    uint32_t k = 0;
    size_t cap = npoints > 1 ? npoints - 1 : 0;
    while (cap) { k++; cap >>= 1; }
    RawMsmConfig c{k, 100000, 32768, 0, 3, 2, 1, 4, 0, 3};
    return c;
}

// Same acceptance rules as the reference (bls12_381_g1_msm.cu:90-110), with
// the window range widened to what this engine supports (0 = automatic).
static bool valid_config(const RawMsmConfig &c)
{
    return c.domain_k <= 31 && c.min_msm_scalars >= 1 && c.unfiltered_min_scalars >= 1 &&
           (c.window_bits == 0 || (c.window_bits >= 8 && c.window_bits <= 18)) &&
           c.sort_grid_divisor >= 1 && c.sort_grid_divisor <= 8 && c.sort_window_lanes >= 1 &&
           c.sort_window_lanes <= 4 &&
           (c.integration_blocks == 1 || c.integration_blocks == 2 || c.integration_blocks == 4 ||
            c.integration_blocks == 8 || c.integration_blocks == 16) &&
           c.batch_lanes >= 1 && c.batch_lanes <= 16 && c.reuse_event <= 1 && c.device_reduce <= 3;
}

static int plan_window(size_t n, bool precomputed, uint32_t requested)
{
    if (requested) return std::min<int>((int)requested, kMaxWindowBits);
    return choose_window(n, precomputed);
}

// Plain MSM of host bases + host scalars (one call, nothing resident).
static void msm_host_plain(jacobian_t *out, const affine_t *points, const fr_t *scalars, size_t n,
                           size_t nmsms)
{
    cudaStream_t s = lane_stream();
    dev_buf<affine_t> d_points(n, s);
    dev_buf<fr_t> d_scalars(n, s);
    dev_buf<jacobian_t> d_out(std::max<size_t>(nmsms, 1), s);
    h2d(d_points, points, n * sizeof(affine_t), s);
    msm_plan p = make_plan(n, plan_window(n, false, 0), false);
    for (size_t m = 0; m < nmsms; m++) {
        h2d(d_scalars, scalars + m * n, n * sizeof(fr_t), s);
        msm_run(p, d_points, d_scalars, d_out.get() + m, s);
    }
    d2h(out, d_out, nmsms * sizeof(jacobian_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
}

static void context_run_device(msm_context_t *ctx, jacobian_t *out_host, const fr_t *d_scalars,
                               size_t npoints, size_t nmsms, cudaStream_t s)
{
    dev_buf<jacobian_t> d_out(std::max<size_t>(nmsms, 1), s);
    msm_plan p = make_plan(npoints, ctx->c, true);
    // the table is laid out [window][ctx->npoints]; a shorter MSM over the
    // first npoints bases needs the same per-window stride, so index through
    // a plan whose point count is the context's and whose scalars beyond
    // npoints are absent: run with n = npoints over a strided view.
    if (npoints != ctx->npoints) {
        // Use the plain (non-precomputed) engine over window 0 of the table.
        msm_plan q = make_plan(npoints, plan_window(npoints, false, 0), false);
        for (size_t m = 0; m < nmsms; m++) msm_run(q, ctx->table, d_scalars + m * npoints, d_out.get() + m, s);
    } else {
        for (size_t m = 0; m < nmsms; m++) msm_run(p, ctx->table, d_scalars + m * npoints, d_out.get() + m, s);
    }
    d2h(out_host, d_out, nmsms * sizeof(jacobian_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
    timed_collect();
}

}  // namespace gb

using namespace gb;

extern "C" {

// bls12_381_g1_msm.cu:6164-6200
RustError midnight_sppark_bls12_381_g1_msm(RawG1Projective *out_raw, const RawG1Affine *points_raw, const RawFr *scalars_raw, size_t len)
{
    jacobian_t *out = reinterpret_cast<jacobian_t *>(out_raw);
    const affine_t *points = reinterpret_cast<const affine_t *>(points_raw);
    const fr_t *scalars = reinterpret_cast<const fr_t *>(scalars_raw);
    GB_ENTRY_BEGIN
    if (!out || (len && (!points || !scalars)))
        return make_error((int)cudaErrorInvalidValue, "invalid BLS12-381 G1 MSM arguments");
    msm_host_plain(out, points, scalars, len, 1);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:6202-6245; scalars laid out [nmsms][npoints]
RustError midnight_sppark_bls12_381_g1_msm_batch(RawG1Projective *out_raw, const RawG1Affine *points_raw, const RawFr *scalars_raw, size_t npoints, size_t nmsms)
{
    jacobian_t *out = reinterpret_cast<jacobian_t *>(out_raw);
    const affine_t *points = reinterpret_cast<const affine_t *>(points_raw);
    const fr_t *scalars = reinterpret_cast<const fr_t *>(scalars_raw);
    GB_ENTRY_BEGIN
    if (nmsms == 0) return ok();
    if (!out || (npoints && (!points || !scalars)))
        return make_error((int)cudaErrorInvalidValue, "invalid BLS12-381 G1 MSM batch arguments");
    msm_host_plain(out, points, scalars, npoints, nmsms);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:6247-6267: uploads the bases once and precomputes the
// per-window shifted copies used by every later context call.
RustError midnight_sppark_bls12_381_g1_msm_context_create_with_config(void **out, const RawG1Affine *points_raw, size_t npoints, RawMsmConfig config)
{
    const affine_t *points = reinterpret_cast<const affine_t *>(points_raw);
    if (!out) return make_error((int)cudaErrorInvalidValue, "null context output");
    *out = nullptr;
    if (!valid_config(config)) return make_error((int)cudaErrorInvalidValue, "invalid BLS12-381 MSM config");
    if (npoints && !points) return make_error((int)cudaErrorInvalidValue, "null MSM bases");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto *ctx = new msm_context_t();
    ctx->device = current_device();
    ctx->npoints = npoints;
    ctx->config = config;
    ctx->owner = s;
    ctx->c = plan_window(npoints, true, config.window_bits);
    ctx->nwin = windows_for(ctx->c);
    try {
        size_t total = npoints * (size_t)ctx->nwin;
        if (total) {
            GB_CUDA_OK(cudaMalloc(&ctx->table, total * sizeof(affine_t)));
            h2d(ctx->table, points, npoints * sizeof(affine_t), s);
            msm_precompute_kernel<<<blocks_for(npoints, 128), 128, 0, s>>>(ctx->table, npoints, ctx->c,
                                                                           ctx->nwin);
            GB_CHECK_LAUNCH();
        }
        GB_CUDA_OK(cudaStreamSynchronize(s));
    } catch (...) {
        if (ctx->table) cudaFree(ctx->table);
        delete ctx;
        throw;
    }
    *out = ctx;
    return ok();
    GB_ENTRY_END
}

RustError midnight_sppark_bls12_381_g1_msm_context_create(void **out, const RawG1Affine *points_raw, size_t npoints)
{
    return midnight_sppark_bls12_381_g1_msm_context_create_with_config(out, points_raw, npoints,
                                                                       default_config(npoints));
}

void midnight_sppark_bls12_381_g1_msm_context_free(void *context)
{
    auto *ctx = reinterpret_cast<msm_context_t *>(context);
    if (!ctx) return;
    cudaStreamSynchronize(ctx->owner);
    if (ctx->table) cudaFree(ctx->table);
    delete ctx;
}

// bls12_381_g1_msm.cu:6288-6308: host scalars against resident bases
RustError midnight_sppark_bls12_381_g1_msm_context_batch(RawG1Projective *out_raw, void *context, const RawFr *scalars_raw, size_t npoints, size_t nmsms)
{
    jacobian_t *out = reinterpret_cast<jacobian_t *>(out_raw);
    const fr_t *scalars = reinterpret_cast<const fr_t *>(scalars_raw);
    if (!context) return make_error(-1, "null BLS12-381 G1 MSM context");
    GB_ENTRY_BEGIN
    auto *ctx = reinterpret_cast<msm_context_t *>(context);
    if (nmsms == 0) return ok();
    if (!out || (npoints && !scalars)) return make_error((int)cudaErrorInvalidValue, "invalid MSM batch arguments");
    if (npoints > ctx->npoints) return make_error((int)cudaErrorInvalidValue, "more scalars than context bases");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t s = lane_stream();
    dev_buf<fr_t> d_scalars(npoints * nmsms, s);
    h2d(d_scalars, scalars, npoints * nmsms * sizeof(fr_t), s);
    context_run_device(ctx, out, d_scalars, npoints, nmsms, s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:6310-6344: resident scalars (device vector)
RustError midnight_sppark_bls12_381_g1_msm_context_device_batch(RawG1Projective *out_raw, void *context, const void *device_vec, size_t scalar_offset, size_t npoints, size_t nmsms)
{
    jacobian_t *out = reinterpret_cast<jacobian_t *>(out_raw);
    if (!context || !device_vec || (nmsms != 0 && !out))
        return make_error(-1, "invalid resident BLS12-381 G1 MSM arguments");
    GB_ENTRY_BEGIN
    auto *ctx = reinterpret_cast<msm_context_t *>(context);
    auto *dv = reinterpret_cast<const fr_device_vec *>(device_vec);
    if (npoints != 0 && nmsms > (SIZE_MAX - scalar_offset) / npoints)
        return make_error((int)cudaErrorInvalidValue, "resident MSM range overflow");
    if (scalar_offset + npoints * nmsms > dv->len)
        return make_error((int)cudaErrorInvalidValue, "resident MSM range exceeds device vector");
    if (npoints > ctx->npoints) return make_error((int)cudaErrorInvalidValue, "more scalars than context bases");
    if (nmsms == 0) return ok();
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t s = lane_stream();
    device_vec_wait(dv, s);
    context_run_device(ctx, out, dv->values + scalar_offset, npoints, nmsms, s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:6346-6377: ragged slices of one device vector
RustError midnight_sppark_bls12_381_g1_msm_context_device_ragged(RawG1Projective *out_raw, void *context, const void *device_vec, const RawMsmSlice *slices, size_t count)
{
    jacobian_t *out = reinterpret_cast<jacobian_t *>(out_raw);
    if (!context || !device_vec || (count != 0 && (!out || !slices)))
        return make_error(-1, "invalid ragged resident BLS12-381 G1 MSM arguments");
    if (count == 0) return ok();
    GB_ENTRY_BEGIN
    auto *ctx = reinterpret_cast<msm_context_t *>(context);
    auto *dv = reinterpret_cast<const fr_device_vec *>(device_vec);
    for (size_t i = 0; i < count; i++) {
        const RawMsmSlice &sl = slices[i];
        if (sl.scalar_offset > dv->len || sl.len > dv->len - sl.scalar_offset)
            return make_error((int)cudaErrorInvalidValue, "ragged MSM slice exceeds device vector");
        if (sl.point_offset > ctx->npoints || sl.len > ctx->npoints - sl.point_offset)
            return make_error((int)cudaErrorInvalidValue, "ragged MSM slice exceeds context bases");
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t s = lane_stream();
    device_vec_wait(dv, s);
    dev_buf<jacobian_t> d_out(count, s);
    for (size_t i = 0; i < count; i++) {
        const RawMsmSlice &sl = slices[i];
        if (sl.point_offset == 0 && sl.len == ctx->npoints) {
            msm_plan p = make_plan(sl.len, ctx->c, true);
            msm_run(p, ctx->table, dv->values + sl.scalar_offset, d_out.get() + i, s);
        } else {
            msm_plan q = make_plan(sl.len, plan_window(sl.len, false, 0), false);
            msm_run(q, ctx->table + sl.point_offset, dv->values + sl.scalar_offset, d_out.get() + i, s);
        }
    }
    d2h(out, d_out, count * sizeof(jacobian_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:6426-6486: MSM of (scalars + mask) for each batch
// entry; the caller subtracts its precomputed MSM(mask, bases)
// (midnight-sppark-msm/src/lib.rs:3302-3354).
RustError midnight_sppark_bls12_381_g1_msm_context_device_scrambled_batch(RawG1Projective *out_raw, void *context,
                                                                          const void *device_vec,
                                                                          size_t scalar_offset, size_t npoints,
                                                                          size_t nmsms, const void *mask_device_vec)
{
    jacobian_t *out = reinterpret_cast<jacobian_t *>(out_raw);
    if (!context || !device_vec || !mask_device_vec || (nmsms != 0 && !out))
        return make_error(-1, "invalid scrambled resident BLS12-381 G1 MSM arguments");
    GB_ENTRY_BEGIN
    auto *ctx = reinterpret_cast<msm_context_t *>(context);
    auto *dv = reinterpret_cast<const fr_device_vec *>(device_vec);
    auto *mv = reinterpret_cast<const fr_device_vec *>(mask_device_vec);
    if (mv->len != npoints) return make_error((int)cudaErrorInvalidValue, "resident MSM scramble mask length mismatch");
    if (npoints != 0 && nmsms > (SIZE_MAX - scalar_offset) / npoints)
        return make_error((int)cudaErrorInvalidValue, "scrambled resident MSM range overflow");
    const size_t count = npoints * nmsms;
    if (scalar_offset + count > dv->len)
        return make_error((int)cudaErrorInvalidValue, "scrambled resident MSM range exceeds device vector");
    if (npoints > ctx->npoints) return make_error((int)cudaErrorInvalidValue, "more scalars than context bases");
    if (count == 0) return ok();
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t s = lane_stream();
    device_vec_wait(dv, s);
    device_vec_wait(mv, s);
    dev_buf<fr_t> masked(count, s);
    add_mask_kernel<<<blocks_for(count, 256), 256, 0, s>>>(masked, dv->values + scalar_offset, mv->values, npoints,
                                                           count);
    GB_CHECK_LAUNCH();
    context_run_device(ctx, out, masked, npoints, nmsms, s);
    return ok();
    GB_ENTRY_END
}

}  // extern "C"
