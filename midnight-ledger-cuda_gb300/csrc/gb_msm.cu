// BLS12-381 G1 multiexp (Pippenger) for sm_103a, and the MSM entry points
// of the C ABI (midnight-sppark-msm/src/bls12_381_g1_msm.cu:6164-6486).
//
// One engine serves every entry point: a BATCH of MSMs (one or many, of
// uneven sizes) goes through each pipeline stage in a single launch.
//   1. recode     : Montgomery -> canonical, signed c-bit digits per window
//                   (digit in [-2^(c-1), 2^(c-1)], carry into the next window)
//   2. histogram  : per-block shared-memory counts of bucket keys
//   3. column scan: per-key prefix over the blocks of its segment + totals
//   4. key scan   : exclusive scan of totals -> bucket start offsets
//   5. scatter    : (bucket, point) pairs placed in bucket order
//   6. accumulate : each thread sums L consecutive sorted entries into XYZZ
//                   accumulators (fixed work per thread whatever the bucket
//                   sizes), writing finished buckets directly and chunk-edge
//                   partials aside
//   7. fix-up     : buckets spanning chunks add their partials
//   8. reduce     : sum_k (k+1) B_k per segment by segmented running sums and
//                   a tree, then per MSM the window combination.
//
// A "segment" owns 2^(c-1) buckets.  Two modes:
//   * precomputed (MSM contexts, whose bases are fixed): context creation
//     stores 2^(c*j) P_i for every window j, so each MSM is ONE segment and
//     needs no window combination;
//   * plain (bases passed per call): each (MSM, window) is a segment and the
//     windows are combined by Horner's rule.
// Both decode a digit's point as point_base + (d / n) * stride + d % n.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <atomic>
#include <tuple>
#include <set>
#include <mutex>
#include <initializer_list>
#include <vector>

#include "gb_runtime.cuh"

namespace gb {

static constexpr uint32_t kZeroDigit = 0xffffffffu;
static constexpr int kMaxWindowBits = 16;  // 2^15 u32 counters = 128 KB smem

static int windows_for(int c) { return 255 / c + 1; }

// Window size: minimise mixed additions plus bucket-reduction additions,
// over the sizes whose top window keeps at least 5 of the scalar's 255 bits
// (8, 10, 13, 16).  With fewer, nearly every point's top digit falls in a
// handful of buckets, which then span thousands of accumulation chunks.
static int choose_window(size_t n, bool precomputed)
{
    if (n <= 1) return 8;
    int best = 8;
    double best_cost = 1e300;
    for (int c = 8; c <= kMaxWindowBits; c++) {
        if (255 % c < 5) continue;
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

static int default_acc_variant()
{
    const char *e = getenv("GB_MSM_ACC_VARIANT");
    if (e && e[0] >= '0' && e[0] <= '2') return e[0] - '0';
    return 1;  // 256 threads, 2 blocks per SM: the fastest on GB300 at n = 2^20
}

// one MSM of a batch (host view)
struct msm_item {
    const fr_t *scalars;  // device pointer, n values
    size_t n;
    size_t point_base;    // first base of this MSM in table row 0
};

// per-segment and per-sort-block descriptors (device view)
struct seg_desc {
    uint64_t digit_off;   // first digit of the segment
    uint32_t len;         // digits in the segment
    uint32_t n;           // points of the segment's MSM (digit d -> window d / n, point d % n)
    uint64_t point_base;  // base index of the MSM's first point in table row 0
    uint32_t blk0, nblk;  // sort blocks of the segment
};
struct blk_desc {
    uint32_t seg;
    uint32_t lo, hi;      // digit range within the segment
};
struct item_desc {
    const fr_t *scalars;
    uint64_t point_prefix;  // sum of n over earlier items (thread -> item map)
    uint64_t digit_base;    // digits of the item start here: [window][n]
    uint32_t n;
};

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

// The canonical value of a Montgomery-form scalar s < r (s R^-1 mod r):
// Montgomery reduction alone (the product by 1 without its a * b rows),
// 8 steps of t = (t + m r) / 2^32 with m = -t0 (r's lowest limb is 1).  The
// result is below r for s < r, and the final subtraction covers s < R.
// The scalar is read with two 16-byte loads when it is 16-byte aligned.
__device__ __forceinline__ fr_t scalar_canonical(const fr_t *p)
{
    fr_t a;
    if (((uintptr_t)p & 15u) == 0) {
        const uint4 lo = __ldg(reinterpret_cast<const uint4 *>(p)), hi = __ldg(reinterpret_cast<const uint4 *>(p) + 1);
        a.v[0] = lo.x, a.v[1] = lo.y, a.v[2] = lo.z, a.v[3] = lo.w;
        a.v[4] = hi.x, a.v[5] = hi.y, a.v[6] = hi.z, a.v[7] = hi.w;
    } else {
        a = *p;
    }
    uint32_t t[9];
#pragma unroll
    for (int i = 0; i < 8; i++) t[i] = a.v[i];
    t[8] = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint32_t m = 0u - t[0];
        uint64_t c = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint64_t v = (uint64_t)m * FrCfg::mod(j) + t[j] + c;
            t[j] = (uint32_t)v;
            c = v >> 32;
        }
        const uint64_t top = (uint64_t)t[8] + c;
#pragma unroll
        for (int j = 0; j < 7; j++) t[j] = t[j + 1];
        t[7] = (uint32_t)top;
        t[8] = (uint32_t)(top >> 32);
    }
    fr_t r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = t[i];
    fr_t::reduce_once(r.v, t[8]);
    return r;
}

// 1. recode: for item m, point i, window j: digits[base_m + j * n_m + i] =
//    (|digit| - 1) | sign << 31, or kZeroDigit.  One instance per window
//    size, so the windows unroll and the scalar's limbs stay in registers
//    (with the window a run-time value they were indexed in local memory).
template <int C>
__global__ void msm_recode_kernel(const item_desc *__restrict__ items, uint32_t nitems, uint64_t total,
                                  uint32_t *__restrict__ digits)
{
    constexpr int NWIN = 255 / C + 1;
    constexpr uint32_t half = 1u << (C - 1);
    constexpr uint32_t mask = (1u << C) - 1;
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    uint32_t lo = 0, hi = nitems;  // last item with point_prefix <= t
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (items[mid].point_prefix <= t) lo = mid;
        else hi = mid;
    }
    const item_desc it = items[lo];
    const uint64_t i = t - it.point_prefix;
    const fr_t s = scalar_canonical(it.scalars + i);
    uint32_t carry = 0;
    uint32_t *out = digits + it.digit_base + i;
#pragma unroll
    for (int j = 0; j < NWIN; j++) {
        const int bit = j * C;
        const int limb = bit >> 5, off = bit & 31;
        const uint32_t l0 = limb < 8 ? s.v[limb < 8 ? limb : 7] : 0;
        const uint32_t l1 = limb + 1 < 8 ? s.v[limb + 1 < 8 ? limb + 1 : 7] : 0;
        uint32_t raw = (uint32_t)((((uint64_t)l1 << 32) | l0) >> off) & mask;
        raw += carry;
        uint32_t d;
        if (raw == 0) {
            carry = 0;
            d = kZeroDigit;
        } else if (raw <= half) {
            carry = 0;
            d = raw - 1;
        } else {
            carry = 1;
            const uint32_t mag = (1u << C) - raw;  // digit = raw - 2^c < 0
            d = mag == 0 ? kZeroDigit : ((mag - 1) | 0x80000000u);
        }
        out[(uint64_t)j * it.n] = d;
    }
}

static void launch_recode(const item_desc *items, uint32_t nitems, uint64_t total, int c, uint32_t *digits,
                          cudaStream_t s)
{
    const unsigned grid = (unsigned)((total + 255) / 256);
    switch (c) {
    case 8: msm_recode_kernel<8><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    case 9: msm_recode_kernel<9><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    case 10: msm_recode_kernel<10><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    case 11: msm_recode_kernel<11><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    case 12: msm_recode_kernel<12><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    case 13: msm_recode_kernel<13><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    case 14: msm_recode_kernel<14><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    case 15: msm_recode_kernel<15><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    case 16: msm_recode_kernel<16><<<grid, 256, 0, s>>>(items, nitems, total, digits); break;
    default: throw cuda_error((int)cudaErrorInvalidValue, "MSM window size outside 8..16");
    }
    GB_CHECK_LAUNCH();
}

// 2. per-block histograms: hist[b][k]
__global__ void msm_hist_kernel(const uint32_t *__restrict__ digits, const seg_desc *__restrict__ segs,
                                const blk_desc *__restrict__ blks, uint32_t K, uint32_t *__restrict__ hist)
{
    extern __shared__ uint32_t sh[];
    const blk_desc bd = blks[blockIdx.x];
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) sh[k] = 0;
    __syncthreads();
    const uint32_t *d = digits + segs[bd.seg].digit_off;
    for (uint32_t i = bd.lo + threadIdx.x; i < bd.hi; i += blockDim.x) {
        uint32_t v = d[i];
        if (v != kZeroDigit) atomicAdd(&sh[v & (K - 1)], 1u);
    }
    __syncthreads();
    uint32_t *out = hist + (size_t)blockIdx.x * K;
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) out[k] = sh[k];
}

// 3. per global key g = seg * K + k: exclusive prefix over the segment's
//    blocks (in place in hist) and the total into counts[g]
__global__ void msm_colscan_kernel(uint32_t *__restrict__ hist, const seg_desc *__restrict__ segs, uint32_t K,
                                   uint32_t G, uint32_t *__restrict__ counts)
{
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    const seg_desc sd = segs[g / K];
    const uint32_t k = g % K;
    uint32_t run = 0;
    uint32_t *col = hist + (size_t)sd.blk0 * K + k;
    uint32_t w = 0;
    // batches of 16 independent loads keep the column walk off the latency path
    for (; w + 16 <= sd.nblk; w += 16) {
        uint32_t v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) v[u] = col[(size_t)(w + u) * K];
#pragma unroll
        for (int u = 0; u < 16; u++) {
            col[(size_t)(w + u) * K] = run;
            run += v[u];
        }
    }
    for (; w < sd.nblk; w++) {
        uint32_t v = col[(size_t)w * K];
        col[(size_t)w * K] = run;
        run += v;
    }
    counts[g] = run;
}

// 4. exclusive scan of counts[0..G) into starts[0..G], starts[G] = total:
//    tile sums, a one-block scan of the tile sums, then the tiles themselves
static constexpr uint32_t kScanTileU32 = 4096;

__global__ void u32_tile_sum_kernel(const uint32_t *__restrict__ in, uint32_t n, uint32_t *__restrict__ sums)
{
    __shared__ uint32_t sh[256];
    uint32_t base = blockIdx.x * kScanTileU32;
    uint32_t s = 0;
    for (uint32_t i = base + threadIdx.x; i < min(base + kScanTileU32, n); i += 256) s += in[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = 128; off; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = sh[0];
}

// exclusive scan in place of up to 1024 * 64 values with one block
__global__ void u32_small_scan_kernel(uint32_t *__restrict__ v, uint32_t n)
{
    __shared__ uint32_t part[1024];
    const uint32_t T = blockDim.x;
    const uint32_t per = (n + T - 1) / T;
    const uint32_t lo = threadIdx.x * per, hi = min(lo + per, n);
    uint32_t s = 0;
    for (uint32_t i = lo; i < hi; i++) s += v[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = 1; off < T; off <<= 1) {
        uint32_t x = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (uint32_t i = lo; i < hi; i++) {
        uint32_t x = v[i];
        v[i] = run;
        run += x;
    }
}

// out[i] = tile prefix + exclusive prefix within the tile
__global__ void u32_tile_scan_kernel(const uint32_t *__restrict__ in, uint32_t n, const uint32_t *__restrict__ tile_pre,
                                     uint32_t *__restrict__ out)
{
    __shared__ uint32_t part[256];
    const uint32_t base = blockIdx.x * kScanTileU32;
    const uint32_t per = kScanTileU32 / 256;
    const uint32_t lo = base + threadIdx.x * per;
    uint32_t s = 0;
    for (uint32_t i = lo; i < min(lo + per, n); i++) s += in[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = 1; off < 256; off <<= 1) {
        uint32_t x = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    uint32_t run = tile_pre[blockIdx.x] + (threadIdx.x ? part[threadIdx.x - 1] : 0);
    for (uint32_t i = lo; i < min(lo + per, n); i++) {
        out[i] = run;
        run += in[i];
    }
}

// 5. scatter into bucket order: sorted[pos] = point_ref | sign << 31
__global__ void msm_scatter_kernel(const uint32_t *__restrict__ digits, const seg_desc *__restrict__ segs,
                                   const blk_desc *__restrict__ blks, uint32_t K, uint64_t stride,
                                   const uint32_t *__restrict__ hist, const uint32_t *__restrict__ starts,
                                   uint32_t *__restrict__ sorted)
{
    extern __shared__ uint32_t cursor[];
    const blk_desc bd = blks[blockIdx.x];
    const seg_desc sd = segs[bd.seg];
    const uint32_t *h = hist + (size_t)blockIdx.x * K;
    const uint32_t *st = starts + (size_t)bd.seg * K;
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) cursor[k] = st[k] + h[k];
    __syncthreads();
    const uint32_t *d = digits + sd.digit_off;
    for (uint32_t i = bd.lo + threadIdx.x; i < bd.hi; i += blockDim.x) {
        uint32_t v = d[i];
        if (v == kZeroDigit) continue;
        uint32_t pos = atomicAdd(&cursor[v & (K - 1)], 1u);
        uint64_t ref = sd.point_base + (uint64_t)(i / sd.n) * stride + (i % sd.n);
        sorted[pos] = (uint32_t)ref | (v & 0x80000000u);
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

// 7. buckets spanning several chunks; empty buckets become infinity.  A
//    bucket spanning up to kShortSpan chunks is summed by its own thread;
//    longer ones (skewed digit distributions: a sparse top window,
//    structured scalars) are appended to `longs` for msm_fixup_long_kernel.
static constexpr uint32_t kShortSpan = 32;

__global__ void msm_fixup_kernel(const uint32_t *__restrict__ starts, uint32_t G, uint32_t L,
                                 const xyzz_t *__restrict__ head, const xyzz_t *__restrict__ tail,
                                 xyzz_t *__restrict__ buckets, uint32_t *__restrict__ longs,
                                 uint32_t *__restrict__ nlong)
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
    if (ce - cs > kShortSpan) {
        longs[atomicAdd(nlong, 1u)] = g;
        return;
    }
    xyzz_t acc = tail[cs];
    for (uint32_t c = cs + 1; c < ce; c++) acc.GB_ADD_LAT(tail[c]);
    acc.GB_ADD_LAT(head[ce]);
    buckets[g] = acc;
}

// 7b. long buckets, one block each (grid-stride over the list): every
//     thread sums a strided share of the bucket's chunk partials, then a
//     shared-memory tree adds the 256 shares
__global__ void __launch_bounds__(256) msm_fixup_long_kernel(const uint32_t *__restrict__ starts, uint32_t L,
                                                            const xyzz_t *__restrict__ head,
                                                            const xyzz_t *__restrict__ tail,
                                                            const uint32_t *__restrict__ longs,
                                                            const uint32_t *__restrict__ nlong,
                                                            xyzz_t *__restrict__ buckets)
{
    __shared__ xyzz_t sh[256];
    const uint32_t count = *nlong;
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        const uint32_t g = longs[i];
        const uint32_t cs = starts[g] / L, ce = (starts[g + 1] - 1) / L;
        // partials: tail[cs], tail[cs+1 .. ce-1], head[ce]
        xyzz_t acc = xyzz_t::inf();
        for (uint32_t c = cs + threadIdx.x; c <= ce; c += blockDim.x) acc.GB_ADD_LAT(c == ce ? head[c] : tail[c]);
        sh[threadIdx.x] = acc;
        __syncthreads();
        for (uint32_t off = 128; off > 0; off >>= 1) {
            if (threadIdx.x < off) {
                xyzz_t v = sh[threadIdx.x];
                v.GB_ADD_LAT(sh[threadIdx.x + off]);
                sh[threadIdx.x] = v;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) buckets[g] = sh[0];
        __syncthreads();
    }
}

// 8a. per (segment, sub-segment): U = sum_{k in sub} (k+1) B_k; then each
//     aligned group of min(S, 128) sub-segments of a block is summed in
//     shared memory, so `partial` holds nseg * S / group points
__global__ void __launch_bounds__(128) msm_reduce_partial_kernel(const xyzz_t *__restrict__ buckets, uint32_t K,
                                                                 uint32_t S, uint32_t nseg,
                                                                 xyzz_t *__restrict__ partial)
{
    __shared__ xyzz_t sh[128];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    xyzz_t sum = xyzz_t::inf();
    if (t < nseg * S) {
        uint32_t seg = t / S, s = t % S;
        uint32_t m = K / S;
        uint32_t k0 = s * m;
        const xyzz_t *B = buckets + (size_t)seg * K;
        xyzz_t run = xyzz_t::inf();
        for (uint32_t k = k0 + m; k-- > k0;) {
            run.GB_ADD_LAT(B[k]);
            sum.GB_ADD_LAT(run);
        }
        if (k0) sum.GB_ADD_LAT(xyzz_mul_small(run, k0));
    }
    sh[threadIdx.x] = sum;
    __syncthreads();
    const uint32_t group = S < 128 ? S : 128;
    for (uint32_t off = group / 2; off > 0; off >>= 1) {
        if ((threadIdx.x & (group - 1)) < off) {
            xyzz_t v = sh[threadIdx.x];
            v.GB_ADD_LAT(sh[threadIdx.x + off]);
            sh[threadIdx.x] = v;
        }
        __syncthreads();
    }
    if ((threadIdx.x & (group - 1)) == 0 && t < nseg * S) partial[t / group] = sh[threadIdx.x];
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
    if (i1 < n) acc.GB_ADD_LAT(src[i1]);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            xyzz_t v = sh[threadIdx.x];
            v.GB_ADD_LAT(sh[threadIdx.x + off]);
            sh[threadIdx.x] = v;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)seg * gridDim.x + blockIdx.x] = sh[0];
}

// ---------------------------------------------------------------------------
// Cooperative point arithmetic for the latency-bound reduction.  The bucket
// reduction is a few chains of dependent XYZZ operations per segment, run on
// few warps, so its time is the latency of one operation times the chain
// length.  Here a group of 8 lanes (a quarter warp) runs one chain: the
// products of a point operation that do not depend on each other are
// computed by different lanes at the same time, with the operands and
// results in the group's shared-memory slots.  An addition is then 4 product
// levels deep (instead of 14 products in sequence) and a doubling 3 (instead
// of 10).  Every decision (infinity, equal or opposite points) reads shared
// values after a group barrier, so the 8 lanes always take the same path.
static constexpr uint32_t kCoopLanes = 8;
static constexpr uint32_t kCoopGroups = 16;  // groups per 128-thread block
static constexpr uint64_t kCoopMaxBuckets = 8u << 15;  // cooperative reduction up to 8 x 2^15 buckets
// groups of the cooperative reduction over a batch: 2^15 buckets a segment,
// then fewer buckets (a shorter chain per group, so the groups' contention
// for the SMs' issue slots weighs more)
static constexpr uint64_t kCoopGroupBudget = 6144;
static constexpr uint64_t kCoopGroupBudgetSmall = 2048;
static constexpr uint32_t kCoopFixupMaxBuckets = 1u << 14;  // cooperative fix-up up to 2^14 buckets in all
// slots of a group: RUN, SUM, OPD (operand), RES (4 each: X, Y, ZZ, ZZZ),
// then 12 temporaries
enum { CO_RUN = 0, CO_SUM = 4, CO_OPD = 8, CO_RES = 12, CO_TMP = 16, CO_SLOTS = 28 };

struct coop_t {
    fp_t *s;        // the group's slots
    uint32_t lane;  // 0..7
    uint32_t mask;  // the group's lanes in the warp
    __device__ void sync() const { __syncwarp(mask); }
};

__device__ __forceinline__ void coop_set_inf(const coop_t &c, int a)
{
    if (c.lane == 0) {
        const xyzz_t z = xyzz_t::inf();
        c.s[a] = z.x, c.s[a + 1] = z.y, c.s[a + 2] = z.zz, c.s[a + 3] = z.zzz;
    }
    c.sync();
}

// 4 slots (48 words) from src to dst, 6 words per lane
__device__ __forceinline__ void coop_copy(const coop_t &c, fp_t *dst, const fp_t *src)
{
    const uint2 *f = reinterpret_cast<const uint2 *>(src);
    uint2 *t = reinterpret_cast<uint2 *>(dst);
    const uint2 a = f[c.lane * 3], b = f[c.lane * 3 + 1], d = f[c.lane * 3 + 2];
    c.sync();
    t[c.lane * 3] = a, t[c.lane * 3 + 1] = b, t[c.lane * 3 + 2] = d;
    c.sync();
}

__device__ __forceinline__ void coop_load(const coop_t &c, int a, const xyzz_t *g)
{
    const uint2 *f = reinterpret_cast<const uint2 *>(g);
    uint2 *t = reinterpret_cast<uint2 *>(c.s + a);
    t[c.lane * 3] = f[c.lane * 3], t[c.lane * 3 + 1] = f[c.lane * 3 + 1], t[c.lane * 3 + 2] = f[c.lane * 3 + 2];
    c.sync();
}

__device__ __forceinline__ void coop_store(const coop_t &c, int a, xyzz_t *g)
{
    const uint2 *f = reinterpret_cast<const uint2 *>(c.s + a);
    uint2 *t = reinterpret_cast<uint2 *>(g);
    t[c.lane * 3] = f[c.lane * 3], t[c.lane * 3 + 1] = f[c.lane * 3 + 1], t[c.lane * 3 + 2] = f[c.lane * 3 + 2];
}

// One level of products: lane l < n computes s[xi[l]] * s[yi[l]] into
// s[oi[l]].  All lanes run the same call with their own operands, so the
// products of a level run side by side (a product per lane per branch would
// run them one after another).  Operands are read before any result is
// written.
//
// The slot indices of lane l sit in bits 5l .. 5l + 4 of x, y and o.
__device__ __forceinline__ uint32_t coop_pack(std::initializer_list<int> v)
{
    uint32_t r = 0, sh = 0;
    for (int i : v) r |= (uint32_t)i << sh, sh += 5;
    return r;
}

__device__ __forceinline__ void coop_level(const coop_t &c, uint32_t n, uint32_t x, uint32_t y, uint32_t o)
{
    const uint32_t sh = 5u * (c.lane < n ? c.lane : 0u);
    const fp_t a = c.s[(x >> sh) & 31u], b = c.s[(y >> sh) & 31u];
    const fp_t r = a * b;
    c.sync();
    if (c.lane < n) c.s[(o >> sh) & 31u] = r;
    c.sync();
}

// The same with squares: lane l < n computes s[xi[l]]^2 into s[oi[l]] (the
// squaring takes 234 multiply-adds where the product takes 300)
__device__ __forceinline__ void coop_level_sqr(const coop_t &c, uint32_t n, uint32_t x, uint32_t o)
{
    const uint32_t sh = 5u * (c.lane < n ? c.lane : 0u);
    const fp_t r = c.s[(x >> sh) & 31u].sqr();
    c.sync();
    if (c.lane < n) c.s[(o >> sh) & 31u] = r;
    c.sync();
}

// a = 2 a (dbl-2008-s-1, the products of xyzz_t::dbl in three levels)
__device__ void coop_dbl(const coop_t &c, int a)
{
    fp_t *s = c.s;
    if (s[a + 2].is_zero()) return;
    enum { U = CO_TMP, V, XX, M, W, S, MM, D, T0, T1 };
    {
        const fp_t u = s[a + 1].dbl();
        if (u.is_zero()) {
            coop_set_inf(c, a);
            return;
        }
        c.sync();
        if (c.lane == 0) s[U] = u;
        c.sync();
    }
    {
        coop_level_sqr(c, 2, coop_pack({U, a}), coop_pack({V, XX}));  // V = U^2, XX = X^2
    }
    if (c.lane == 0) s[M] = s[XX].dbl() + s[XX];
    c.sync();
    {
        // W = U V, S = X V, ZZ3 = V ZZ, MM = M^2
        coop_level(c, 4, coop_pack({U, a, V, M}), coop_pack({V, V, a + 2, M}), coop_pack({W, S, a + 2, MM}));
    }
    const fp_t X3 = s[MM] - s[S].dbl();
    if (c.lane == 0) s[D] = s[S] - X3;
    c.sync();
    {
        // M (S - X3), W Y, ZZZ3 = W ZZZ
        coop_level(c, 3, coop_pack({M, W, W}), coop_pack({D, a + 1, a + 3}), coop_pack({T0, T1, a + 3}));
    }
    if (c.lane == 0) {
        s[a] = X3;
        s[a + 1] = s[T0] - s[T1];
    }
    c.sync();
}

// a += q (add-2008-s, the products of xyzz_t::add in four levels); q's
// slots are left unchanged
__device__ void coop_add(const coop_t &c, int a, int q)
{
    fp_t *s = c.s;
    if (s[q + 2].is_zero()) return;
    if (s[a + 2].is_zero()) {
        coop_copy(c, s + a, s + q);
        return;
    }
    enum { U1 = CO_TMP, U2, S1, S2, Z12, W12, P, R, PP, RR, PPP, QQ };
    {
        // U1 = X1 ZZ2, U2 = X2 ZZ1, S1 = Y1 ZZZ2, S2 = Y2 ZZZ1, ZZ1 ZZ2, ZZZ1 ZZZ2
        coop_level(c, 6, coop_pack({a, q, a + 1, q + 1, a + 2, a + 3}), coop_pack({q + 2, a + 2, q + 3, a + 3, q + 2, q + 3}), coop_pack({U1, U2, S1, S2, Z12, W12}));
    }
    {
        const fp_t p = s[U2] - s[U1];
        const fp_t r = s[S2] - s[S1];
        if (p.is_zero()) {
            if (r.is_zero()) coop_dbl(c, a);
            else coop_set_inf(c, a);
            return;
        }
        c.sync();
        if (c.lane == 0) s[P] = p;
        if (c.lane == 1) s[R] = r;
        c.sync();
    }
    {
        coop_level_sqr(c, 2, coop_pack({P, R}), coop_pack({PP, RR}));  // PP = P^2, RR = R^2
    }
    {
        // PPP = P PP, Q = U1 PP, ZZ3 = ZZ1 ZZ2 PP
        coop_level(c, 3, coop_pack({P, U1, Z12}), coop_pack({PP, PP, PP}), coop_pack({PPP, QQ, a + 2}));
    }
    const fp_t X3 = s[RR] - s[PPP] - s[QQ].dbl();
    if (c.lane == 0) s[U2] = s[QQ] - X3;  // U2 is free from here on
    c.sync();
    {
        // R (Q - X3) -> S2, S1 PPP -> U1, ZZZ3 = ZZZ1 ZZZ2 PPP
        coop_level(c, 3, coop_pack({R, S1, W12}), coop_pack({U2, PPP, PPP}), coop_pack({S2, U1, a + 3}));
    }
    if (c.lane == 0) {
        s[a] = X3;
        s[a + 1] = s[S2] - s[U1];
    }
    c.sync();
}

// the 16 groups of a block add their SUM slots into group 0's (4 levels)
__device__ void coop_block_tree(fp_t *sh, const coop_t &c, uint32_t grp)
{
    for (uint32_t off = kCoopGroups / 2; off > 0; off >>= 1) {
        __syncthreads();
        if (grp < off) {
            coop_copy(c, c.s + CO_OPD, sh + (size_t)(grp + off) * CO_SLOTS + CO_SUM);
            coop_add(c, CO_SUM, CO_OPD);
        }
    }
}

// 7'. msm_fixup_kernel with one 8-lane group per bucket: the partials of a
//     bucket spanning several chunks are added by cooperative additions.
//     The kernel's time is the longest span's chain (bucket sizes vary), so
//     the shorter cooperative additions shorten it most where there are few
//     buckets and short chunks (proof-size MSMs).
__global__ void __launch_bounds__(128) msm_fixup_coop_kernel(const uint32_t *__restrict__ starts, uint32_t G,
                                                             uint32_t L, const xyzz_t *__restrict__ head,
                                                             const xyzz_t *__restrict__ tail,
                                                             xyzz_t *__restrict__ buckets,
                                                             uint32_t *__restrict__ longs,
                                                             uint32_t *__restrict__ nlong)
{
    __shared__ __align__(16) fp_t sh[kCoopGroups * CO_SLOTS];
    const uint32_t grp = threadIdx.x / kCoopLanes;
    const coop_t c{sh + (size_t)grp * CO_SLOTS, threadIdx.x % kCoopLanes, 0xffu << (threadIdx.x & 24u)};
    const uint32_t g = blockIdx.x * kCoopGroups + grp;
    if (g >= G) return;  // whole groups leave together; no block barrier follows
    const uint32_t s = starts[g], e = starts[g + 1];
    if (s == e) {
        coop_set_inf(c, CO_SUM);
        coop_store(c, CO_SUM, buckets + g);
        return;
    }
    const uint32_t cs = s / L, ce = (e - 1) / L;
    if (cs == ce) return;
    if (ce - cs > kShortSpan) {
        if (c.lane == 0) longs[atomicAdd(nlong, 1u)] = g;
        return;
    }
    coop_load(c, CO_SUM, tail + cs);
    for (uint32_t k = cs + 1; k <= ce; k++) {
        c.sync();
        coop_load(c, CO_OPD, k == ce ? head + k : tail + k);
        coop_add(c, CO_SUM, CO_OPD);
    }
    coop_store(c, CO_SUM, buckets + g);
}

// 8a'. msm_reduce_partial_kernel with one 8-lane group per (segment,
//      sub-segment) and the block's 16 groups summed at the end: `partial`
//      holds nseg * S / 16 points.  S is a power of two >= 16.
__global__ void __launch_bounds__(128) msm_reduce_coop_kernel(const xyzz_t *__restrict__ buckets, uint32_t K,
                                                              uint32_t S, xyzz_t *__restrict__ partial)
{
    __shared__ __align__(16) fp_t sh[kCoopGroups * CO_SLOTS];
    const uint32_t grp = threadIdx.x / kCoopLanes;
    const coop_t c{sh + (size_t)grp * CO_SLOTS, threadIdx.x % kCoopLanes, 0xffu << (threadIdx.x & 24u)};
    const uint32_t gid = blockIdx.x * kCoopGroups + grp;
    const uint32_t seg = gid / S, sub = gid % S, m = K / S, k0 = sub * m;
    const xyzz_t *B = buckets + (size_t)seg * K;
    coop_set_inf(c, CO_RUN);
    coop_set_inf(c, CO_SUM);
    for (uint32_t k = k0 + m; k-- > k0;) {
        coop_load(c, CO_OPD, B + k);
        coop_add(c, CO_RUN, CO_OPD);  // run += B[k]
        coop_add(c, CO_SUM, CO_RUN);  // sum += run
    }
    if (k0) {
        // sum += k0 * run, double-and-add from the top bit
        coop_copy(c, c.s + CO_RES, c.s + CO_RUN);
        int top = 31;
        while (!((k0 >> top) & 1u)) top--;
        for (int i = top - 1; i >= 0; i--) {
            coop_dbl(c, CO_RES);
            if ((k0 >> i) & 1u) coop_add(c, CO_RES, CO_RUN);
        }
        coop_add(c, CO_SUM, CO_RES);
    }
    coop_block_tree(sh, c, grp);
    if (grp == 0) coop_store(c, CO_SUM, partial + blockIdx.x);
}

// 8b'. tree sum with groups: out[seg * gridDim.x + b] = sum of the 32-element
//      slice b of in[seg * n .. seg * n + n)
__global__ void __launch_bounds__(128) xyzz_tree_sum_coop_kernel(const xyzz_t *__restrict__ in, uint32_t n,
                                                                 xyzz_t *__restrict__ out)
{
    __shared__ __align__(16) fp_t sh[kCoopGroups * CO_SLOTS];
    const uint32_t grp = threadIdx.x / kCoopLanes;
    const coop_t c{sh + (size_t)grp * CO_SLOTS, threadIdx.x % kCoopLanes, 0xffu << (threadIdx.x & 24u)};
    const xyzz_t *src = in + (size_t)blockIdx.y * n;
    const uint32_t i0 = blockIdx.x * 2 * kCoopGroups + grp, i1 = i0 + kCoopGroups;
    if (i0 < n) coop_load(c, CO_SUM, src + i0);
    else coop_set_inf(c, CO_SUM);
    if (i1 < n) {
        coop_load(c, CO_OPD, src + i1);
        coop_add(c, CO_SUM, CO_OPD);
    }
    coop_block_tree(sh, c, grp);
    if (grp == 0) coop_store(c, CO_SUM, out + (size_t)blockIdx.y * gridDim.x + blockIdx.x);
}

// 8c. per MSM: combine its window segments (Horner) and emit a Jacobian point
__global__ void msm_combine_kernel(const xyzz_t *__restrict__ seg_sum, uint32_t nitems, uint32_t segs_per_item,
                                   int c, jacobian_t *__restrict__ out)
{
    uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nitems) return;
    const xyzz_t *ss = seg_sum + (size_t)m * segs_per_item;
    xyzz_t acc = xyzz_t::inf();
    for (int w = (int)segs_per_item - 1; w >= 0; w--) {
        if (w != (int)segs_per_item - 1)
            for (int k = 0; k < c; k++) acc = acc.GB_DBL_LAT();
        acc.GB_ADD_LAT(ss[w]);
    }
    out[m] = acc.to_jacobian();
}

// 8c'. msm_combine_kernel with one 8-lane group per MSM (16 MSMs a block):
//       the Horner chain of a plain MSM is (windows - 1) * c doublings long
__global__ void __launch_bounds__(128) msm_combine_coop_kernel(const xyzz_t *__restrict__ seg_sum, uint32_t nitems,
                                                               uint32_t segs_per_item, int c,
                                                               jacobian_t *__restrict__ out)
{
    __shared__ __align__(16) fp_t sh[kCoopGroups * CO_SLOTS];
    const uint32_t grp = threadIdx.x / kCoopLanes;
    const coop_t cp{sh + (size_t)grp * CO_SLOTS, threadIdx.x % kCoopLanes, 0xffu << (threadIdx.x & 24u)};
    const uint32_t m = blockIdx.x * kCoopGroups + grp;
    if (m >= nitems) return;  // whole groups leave together; no block barrier follows
    const xyzz_t *ss = seg_sum + (size_t)m * segs_per_item;
    coop_set_inf(cp, CO_SUM);
    for (int w = (int)segs_per_item - 1; w >= 0; w--) {
        if (w != (int)segs_per_item - 1)
            for (int k = 0; k < c; k++) coop_dbl(cp, CO_SUM);
        coop_load(cp, CO_OPD, ss + w);
        coop_add(cp, CO_SUM, CO_OPD);
    }
    if (cp.lane == 0) {
        xyzz_t acc;
        acc.x = cp.s[CO_SUM], acc.y = cp.s[CO_SUM + 1], acc.zz = cp.s[CO_SUM + 2], acc.zzz = cp.s[CO_SUM + 3];
        out[m] = acc.to_jacobian();
    }
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

static void set_smem_attrs()
{
    static std::once_flag once;
    std::call_once(once, [] {
        int bytes = (1 << (kMaxWindowBits - 1)) * 4;
        cudaFuncSetAttribute(msm_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cudaFuncSetAttribute(msm_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    });
}

// Exclusive scan of n u32 counts into out[0..n], out[n] = total (device).
static void u32_exclusive_scan(const uint32_t *in, uint32_t n, uint32_t *out, cudaStream_t s)
{
    uint32_t tiles = (n + kScanTileU32 - 1) / kScanTileU32;
    if (tiles > 1024 * 64) throw cuda_error((int)cudaErrorInvalidValue, "MSM bucket count too large");
    dev_buf<uint32_t> sums(tiles + 1, s);
    u32_tile_sum_kernel<<<tiles, 256, 0, s>>>(in, n, sums);
    GB_CHECK_LAUNCH();
    // total = sum of tile sums: scan tiles+1 values whose last is 0
    GB_CUDA_OK(cudaMemsetAsync(sums.get() + tiles, 0, sizeof(uint32_t), s));
    u32_small_scan_kernel<<<1, 1024, 0, s>>>(sums, tiles + 1);
    GB_CHECK_LAUNCH();
    // sums[tiles] now holds the grand total; pass it through device memory
    u32_tile_scan_kernel<<<tiles, 256, 0, s>>>(in, n, sums, out);
    GB_CHECK_LAUNCH();
    GB_CUDA_OK(cudaMemcpyAsync(out + n, sums.get() + tiles, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
}

// Entries per accumulation thread: about half a bucket (8..64), then set so
// that the chunks fill whole waves of resident accumulation blocks (a 2^16
// MSM's 65536 chunks of 16 fill 84 % of one wave on 152 SMs; chunks of 14
// fill 96 %; a 2^20 MSM's 3.4 waves of 64 become 3 of 72).
static uint32_t chunk_length(uint64_t digits, double avg, uint32_t G, int variant)
{
    uint32_t L = (uint32_t)std::max(8.0, std::min(64.0, avg * 0.5));
    static int per_sm[3] = {0, 0, 0}, sms = 0;
    const int v = variant < 0 || variant > 2 ? 1 : variant;
    if (!per_sm[v]) {
        int dev = current_device(), b = 0;
        GB_CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (v == 1) GB_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, msm_accumulate_kernel<256, 2>, 256, 0));
        else if (v == 2) GB_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, msm_accumulate_kernel<128, 3>, 128, 0));
        else GB_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, msm_accumulate_kernel<256, 1>, 256, 0));
        per_sm[v] = std::max(1, b) * (v == 2 ? 128 : 256);
    }
    const uint64_t wave = (uint64_t)sms * (uint64_t)per_sm[v];  // chunks resident at once
    if (!wave || !digits) return L;
    // whole waves, rounded down (longer chunks: shorter fix-up chains) when
    // there are several, up when there is less than one
    const uint64_t waves = std::max<uint64_t>(1, digits / ((uint64_t)L * wave));
    const uint64_t L2 = (digits + waves * wave - 1) / (waves * wave);
    if (L2 >= 8 && L2 <= 2 * (uint64_t)L) return (uint32_t)L2;
    if (L2 >= 8) return L;
    // Less than one wave of 8-digit chunks (small MSMs): the accumulation
    // takes about L dependent additions per thread and the fix-up about
    // avg / L (the chunks a bucket spans; cooperative groups up to
    // kCoopFixupMaxBuckets buckets, single threads, ~1.6x slower, beyond),
    // so L ~ sqrt(avg x their latency ratio); and at least 3 digits per
    // resident chunk slot, where the additions start to queue on the
    // multiply-add pipe.  Measured on GB300 (one MSM, resident bases):
    // 2^10 points 0.65 -> 0.41 ms, 2^12 0.50 -> 0.45 ms, 2^14 0.97 -> 0.59 ms.
    const double ratio = G <= kCoopFixupMaxBuckets ? 0.8 : 1.3;
    const uint64_t by_latency = (uint64_t)std::lround(std::sqrt(avg * ratio));
    const uint64_t by_load = (3 * digits + wave - 1) / wave;
    return (uint32_t)std::min<uint64_t>(L, std::max<uint64_t>(4, std::max(by_latency, by_load)));
}

// The host half of a batch: its descriptors and launch sizes.
struct batch_plan {
    int c = 0, nwin = 0, variant = 1;
    bool precomputed = false, coop_reduce = false;
    size_t stride = 0;
    uint32_t nitems = 0, K = 0, segs_per_item = 0, nseg = 0, G = 0, nblocks = 0, L = 0, S = 0, S_coop = 0;
    uint64_t points_total = 0, digits_total = 0, nchunks = 0;
    std::vector<item_desc> idesc;
    std::vector<seg_desc> sdesc;
    std::vector<blk_desc> bdesc;
};

static batch_plan plan_batch(const std::vector<msm_item> &items, int c, bool precomputed, size_t stride)
{
    batch_plan P;
    const uint32_t nitems = (uint32_t)items.size();
    P.nitems = nitems;
    if (!nitems) return P;
    const int nwin = windows_for(c);
    const uint32_t K = 1u << (c - 1);
    const uint32_t segs_per_item = precomputed ? 1u : (uint32_t)nwin;
    const uint32_t nseg = nitems * segs_per_item;
    const uint64_t G64 = (uint64_t)nseg * K;
    if (G64 >= 0x7fffffffull) throw cuda_error((int)cudaErrorInvalidValue, "MSM batch too large");
    const uint32_t G = (uint32_t)G64;

    // items, segments, sort blocks
    std::vector<item_desc> idesc(nitems);
    std::vector<seg_desc> sdesc(nseg);
    uint64_t points_total = 0, digits_total = 0;
    for (uint32_t m = 0; m < nitems; m++) {
        const msm_item &it = items[m];
        if (it.n >= 0x7fffffffull / (uint64_t)nwin) throw cuda_error((int)cudaErrorInvalidValue, "MSM too large");
        idesc[m] = item_desc{it.scalars, points_total, digits_total, (uint32_t)it.n};
        for (uint32_t j = 0; j < segs_per_item; j++) {
            seg_desc &sd = sdesc[m * segs_per_item + j];
            sd.digit_off = digits_total + (precomputed ? 0 : (uint64_t)j * it.n);
            sd.len = (uint32_t)(precomputed ? it.n * nwin : it.n);
            sd.n = (uint32_t)std::max<size_t>(it.n, 1);
            sd.point_base = it.point_base;
        }
        points_total += it.n;
        digits_total += (uint64_t)it.n * nwin;
    }
    if (points_total + stride * (uint64_t)nwin >= 0x80000000ull && precomputed)
        throw cuda_error((int)cudaErrorInvalidValue, "MSM table too large for 31-bit point references");
    // ~4 sort blocks per SM pair over the whole batch, 4096..65536 digits
    // each, and at least K (2K from 2^23 digits): every block writes and the
    // column scan and scatter read a K-entry histogram, so blocks far
    // shorter than K move more histogram than digits (measured on GB300: the
    // sort of a 2^18-point MSM 0.192 -> 0.098 ms, of three 2^16-point MSMs
    // 0.183 -> 0.093 ms, of a 2^20-point MSM 0.387 -> 0.311 ms)
    const uint64_t per_min = std::max<uint64_t>(4096, (uint64_t)K << (digits_total >= (1u << 23) ? 1 : 0));
    uint64_t per = std::max<uint64_t>(per_min, std::min<uint64_t>(65536, (digits_total + 607) / 608));
    std::vector<blk_desc> bdesc;
    for (uint32_t sidx = 0; sidx < nseg; sidx++) {
        seg_desc &sd = sdesc[sidx];
        sd.blk0 = (uint32_t)bdesc.size();
        uint32_t nb = (uint32_t)std::max<uint64_t>(1, (sd.len + per - 1) / per);
        uint32_t chunk = (sd.len + nb - 1) / std::max<uint32_t>(nb, 1);
        for (uint32_t b = 0; b < nb; b++) {
            uint32_t lo = b * chunk, hi = std::min(sd.len, lo + chunk);
            bdesc.push_back(blk_desc{sidx, lo, std::max(lo, hi)});
        }
        sd.nblk = nb;
    }
    const uint32_t nblocks = (uint32_t)bdesc.size();
    const double avg = (double)digits_total / (double)G;
    const int variant = default_acc_variant();
    const uint32_t L = chunk_length(digits_total, avg, G, variant);
    // reduction sub-segments: ~64K threads over the batch, 32..8192 per segment
    uint32_t S = 32;
    while (S < 8192 && (uint64_t)S * 2 * nseg <= 65536) S *= 2;
    S = std::min<uint32_t>(K, S);
    // Few buckets in all (a single MSM or a small batch): the reduction is a
    // chain per sub-segment, run by cooperative 8-lane groups.  More groups
    // shorten the running sums, but each adds a double-and-add, and the
    // groups share the SMs' issue slots: one operation took about 5 us up to
    // 2048 groups, 6.5 us at 4096, 9 us at 6144 and 11 us at 8192 (GB300).
    // Measured best: at most 6144 groups over the batch with 2^15 buckets a
    // segment (4096 groups for one MSM, 6144 for three), 2048 with 2^12
    // (three 2^14-point MSMs 0.274 -> 0.225 ms).  Many buckets (large
    // batches): the one-thread-per-chain kernel keeps the multiply-add pipe
    // busier.
    const bool coop_reduce = (uint64_t)nseg * K <= kCoopMaxBuckets && K >= kCoopGroups;
    const uint64_t budget = K >= (1u << 15) ? kCoopGroupBudget : kCoopGroupBudgetSmall;
    uint32_t S_coop = kCoopGroups;
    while (S_coop < K && (uint64_t)S_coop * 2 * nseg <= budget) S_coop *= 2;
    const uint64_t nchunks = std::max<uint64_t>(1, (digits_total + L - 1) / L);

    P.c = c;
    P.nwin = nwin;
    P.variant = variant;
    P.precomputed = precomputed;
    P.coop_reduce = coop_reduce;
    P.stride = stride;
    P.K = K;
    P.segs_per_item = segs_per_item;
    P.nseg = nseg;
    P.G = G;
    P.nblocks = nblocks;
    P.L = L;
    P.S = S;
    P.S_coop = S_coop;
    P.points_total = points_total;
    P.digits_total = digits_total;
    P.nchunks = nchunks;
    P.idesc = std::move(idesc);
    P.sdesc = std::move(sdesc);
    P.bdesc = std::move(bdesc);
    return P;
}

// The device half: every launch of the batch, its scratch allocated and
// freed in stream order on s, the descriptors already in device memory.
// Queues device work only (no host synchronisation, no copy from host
// memory), so a CUDA graph can capture it.
static void run_planned(const batch_plan &P, const item_desc *d_items, const seg_desc *d_segs,
                        const blk_desc *d_blks, const affine_t *points, jacobian_t *d_out, cudaStream_t s)
{
    const int c = P.c, variant = P.variant;
    const bool precomputed = P.precomputed, coop_reduce = P.coop_reduce;
    const size_t stride = P.stride;
    const uint32_t nitems = P.nitems, K = P.K, segs_per_item = P.segs_per_item, nseg = P.nseg, G = P.G;
    const uint32_t nblocks = P.nblocks, L = P.L, S = P.S, S_coop = P.S_coop;
    const uint64_t points_total = P.points_total, digits_total = P.digits_total, nchunks = P.nchunks;
    (void)precomputed;
    dev_buf<uint32_t> digits(std::max<uint64_t>(digits_total, 1), s), sorted(std::max<uint64_t>(digits_total, 1), s);
    dev_buf<uint32_t> hist((size_t)nblocks * K, s), counts(G, s), starts((size_t)G + 1, s);
    dev_buf<xyzz_t> buckets(G, s), head(nchunks, s), tail(nchunks, s);
    dev_buf<xyzz_t> partial((size_t)nseg * (coop_reduce ? S_coop / kCoopGroups : S), s), segsum(nseg, s);

    int tok_all = timed_begin(s);
    int tok_sort = timed_begin(s);
    if (points_total) {
        launch_recode(d_items, nitems, points_total, c, digits, s);
    }
    const size_t smem = (size_t)K * 4;
    msm_hist_kernel<<<nblocks, 1024, smem, s>>>(digits, d_segs, d_blks, K, hist);
    GB_CHECK_LAUNCH();
    msm_colscan_kernel<<<blocks_for(G, 256), 256, 0, s>>>(hist, d_segs, K, G, counts);
    GB_CHECK_LAUNCH();
    u32_exclusive_scan(counts, G, starts, s);
    msm_scatter_kernel<<<nblocks, 1024, smem, s>>>(digits, d_segs, d_blks, K, precomputed ? stride : 0, hist,
                                                   starts, sorted);
    GB_CHECK_LAUNCH();
    timed_end(tok_sort, s, GB_SLOT_MSM_SORT);
    int tok = timed_begin(s);
    if (variant == 1) {
        msm_accumulate_kernel<256, 2><<<(unsigned)((nchunks + 255) / 256), 256, 0, s>>>(
            sorted, starts, G, L, nchunks, points, buckets, head, tail);
    } else if (variant == 2) {
        msm_accumulate_kernel<128, 3><<<(unsigned)((nchunks + 127) / 128), 128, 0, s>>>(
            sorted, starts, G, L, nchunks, points, buckets, head, tail);
    } else {
        msm_accumulate_kernel<256, 1><<<(unsigned)((nchunks + 255) / 256), 256, 0, s>>>(
            sorted, starts, G, L, nchunks, points, buckets, head, tail);
    }
    GB_CHECK_LAUNCH();
    timed_end(tok, s, GB_SLOT_MSM_ACCUMULATE);
    int tok_fix = timed_begin(s);
    {
        dev_buf<uint32_t> longs(G, s), nlong(1, s);
        GB_CUDA_OK(cudaMemsetAsync(nlong.get(), 0, sizeof(uint32_t), s));
        // few buckets: cooperative groups shorten the longest chain (measured
        // on GB300: 2^12 points, 4096 buckets 0.121 -> 0.051 ms; 3 x 4096
        // buckets 0.108 -> 0.071 ms); 2^15 buckets and more: one thread per
        // bucket keeps more of the multiply-add pipe busy (2^16 points
        // 0.104 -> 0.136 ms with groups)
        if (G <= kCoopFixupMaxBuckets)
            msm_fixup_coop_kernel<<<(G + kCoopGroups - 1) / kCoopGroups, 128, 0, s>>>(starts, G, L, head, tail,
                                                                                     buckets, longs, nlong);
        else
            msm_fixup_kernel<<<blocks_for(G, 128), 128, 0, s>>>(starts, G, L, head, tail, buckets, longs, nlong);
        GB_CHECK_LAUNCH();
        int sms = 0;
        GB_CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, current_device()));
        msm_fixup_long_kernel<<<(unsigned)sms * 2, 256, 0, s>>>(starts, L, head, tail, longs, nlong, buckets);
        GB_CHECK_LAUNCH();
    }
    timed_end(tok_fix, s, GB_SLOT_MSM_FIXUP);
    int tok_red = timed_begin(s);
    if (coop_reduce) {
        // latency-bound: one 8-lane group per sub-segment, 16 groups a block
        msm_reduce_coop_kernel<<<nseg * S_coop / kCoopGroups, 128, 0, s>>>(buckets, K, S_coop, partial);
        GB_CHECK_LAUNCH();
        const xyzz_t *src = partial;
        uint32_t len = S_coop / kCoopGroups;
        dev_buf<xyzz_t> tmp_a, tmp_b;
        bool use_a = true;
        while (len > 1) {
            const uint32_t blocks = (len + 2 * kCoopGroups - 1) / (2 * kCoopGroups);
            dev_buf<xyzz_t> &dst = use_a ? tmp_a : tmp_b;
            dst = dev_buf<xyzz_t>((size_t)nseg * blocks, s);
            xyzz_tree_sum_coop_kernel<<<dim3(blocks, nseg), 128, 0, s>>>(src, len, dst);
            GB_CHECK_LAUNCH();
            src = dst;
            len = blocks;
            use_a = !use_a;
        }
        GB_CUDA_OK(cudaMemcpyAsync(segsum, src, (size_t)nseg * sizeof(xyzz_t), cudaMemcpyDeviceToDevice, s));
    } else {
    msm_reduce_partial_kernel<<<blocks_for((size_t)nseg * S, 128), 128, 0, s>>>(buckets, K, S, nseg, partial);
    GB_CHECK_LAUNCH();
    {
        // tree-sum each segment's S / group partials down to one point
        const xyzz_t *src = partial;
        uint32_t len = S / std::min<uint32_t>(S, 128);
        dev_buf<xyzz_t> tmp_a, tmp_b;
        bool use_a = true;
        while (len > 1) {
            uint32_t blocks = (len + 511) / 512;
            dev_buf<xyzz_t> &dst = use_a ? tmp_a : tmp_b;
            dst = dev_buf<xyzz_t>((size_t)nseg * blocks, s);
            xyzz_tree_sum_kernel<<<dim3(blocks, nseg), 256, 0, s>>>(src, len, dst);
            GB_CHECK_LAUNCH();
            src = dst;
            len = blocks;
            use_a = !use_a;
        }
        GB_CUDA_OK(cudaMemcpyAsync(segsum, src, (size_t)nseg * sizeof(xyzz_t), cudaMemcpyDeviceToDevice, s));
    }
    }
    if (segs_per_item > 1) {
        // plain MSMs: a Horner chain per MSM, cooperative groups
        msm_combine_coop_kernel<<<(nitems + kCoopGroups - 1) / kCoopGroups, 128, 0, s>>>(segsum, nitems,
                                                                                          segs_per_item, c, d_out);
    } else {
        msm_combine_kernel<<<blocks_for(nitems, 32), 32, 0, s>>>(segsum, nitems, segs_per_item, c, d_out);
    }
    GB_CHECK_LAUNCH();
    timed_end(tok_red, s, GB_SLOT_MSM_REDUCE);
    timed_end(tok_all, s, GB_SLOT_MSM_TOTAL);
}

// CUDA-graph replay of a batch's launch sequence.  A batch whose shape
// (window, sizes, chunking, launch geometry) and bases pointer come a
// second time on the same stream is captured as a graph, replayed from then
// on: the graph reads its descriptors from device buffers of its own, refreshed by
// one copy each before the launch, and writes its results to a buffer of
// its own, copied to the caller's after it.  Its scratch is allocated and
// freed by the graph's memory nodes.  A proof or a server sends the same
// batch shapes round after round, so the host enqueues 4 operations instead
// of about 25, and the device runs the sequence without per-launch gaps.
struct graph_key {
    int device = 0;
    cudaStream_t stream = nullptr;
    const affine_t *points = nullptr;
    int c = 0, variant = 0;
    bool precomputed = false, coop_reduce = false;
    size_t stride = 0;
    uint32_t nitems = 0, K = 0, segs_per_item = 0, nseg = 0, G = 0, nblocks = 0, L = 0, S = 0, S_coop = 0;
    uint64_t points_total = 0, digits_total = 0, nchunks = 0;
    auto tie() const
    {
        return std::tie(device, stream, points, c, variant, precomputed, coop_reduce, stride, nitems, K,
                        segs_per_item, nseg, G, nblocks, L, S, S_coop, points_total, digits_total, nchunks);
    }
    bool operator<(const graph_key &o) const { return tie() < o.tie(); }
};

// A captured graph and its buffers, freed on its stream when the last user
// lets go of it (an executable graph still running is freed when it
// completes; the buffers go back in stream order behind it).
struct graph_entry {
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    item_desc *d_items = nullptr;
    seg_desc *d_segs = nullptr;
    blk_desc *d_blks = nullptr;
    jacobian_t *d_out = nullptr;
    uint64_t last_use = 0;
    std::mutex mu;  // descriptor upload, launch and result copy stay together
    ~graph_entry()
    {
        if (exec) cudaGraphExecDestroy(exec);
        dev_free(d_items, stream);
        dev_free(d_segs, stream);
        dev_free(d_blks, stream);
        dev_free(d_out, stream);
    }
};

// The cache lives until the process exits (never destroyed: its entries
// would otherwise call into a CUDA runtime that is already shutting down).
static std::mutex g_graph_mu;
static auto &g_graphs = *new std::map<graph_key, std::shared_ptr<graph_entry>>();
static auto &g_graph_failed = *new std::set<graph_key>();
// shapes seen once: a shape is captured the second time it comes, so that
// one-off shapes (a server's changing group sizes) cost no capture
static auto &g_graph_seen = *new std::set<graph_key>();
static uint64_t g_graph_clock = 0;
static std::atomic<unsigned long long> g_graph_launches{0}, g_graph_captures{0};
static constexpr size_t kMaxGraphs = 256;
// on unless GB_MSM_GRAPHS=0 or gb_msm_graphs_enable(0)
static std::atomic<int> g_graphs_on{-1};

static bool graphs_enabled()
{
    int on = g_graphs_on.load(std::memory_order_relaxed);
    if (on < 0) {
        const char *e = getenv("GB_MSM_GRAPHS");
        on = (e && e[0] == '0') ? 0 : 1;
        g_graphs_on.store(on, std::memory_order_relaxed);
    }
    return on && !profiling_enabled();
}

// Runs the planned batch through a cached graph; false when this shape
// cannot be captured (the caller then launches it directly).
static bool run_planned_graph(const batch_plan &P, const affine_t *points, jacobian_t *d_out, cudaStream_t s)
{
    graph_key key;
    key.device = current_device();
    key.stream = s;
    key.points = points;
    key.c = P.c, key.variant = P.variant, key.precomputed = P.precomputed, key.coop_reduce = P.coop_reduce;
    key.stride = P.stride, key.nitems = P.nitems, key.K = P.K, key.segs_per_item = P.segs_per_item;
    key.nseg = P.nseg, key.G = P.G, key.nblocks = P.nblocks, key.L = P.L, key.S = P.S, key.S_coop = P.S_coop;
    key.points_total = P.points_total, key.digits_total = P.digits_total, key.nchunks = P.nchunks;

    // a stream the caller is capturing gets the launches themselves
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    GB_CUDA_OK(cudaStreamIsCapturing(s, &capturing));
    if (capturing != cudaStreamCaptureStatusNone) return false;
    std::shared_ptr<graph_entry> e;
    {
        std::lock_guard<std::mutex> lk(g_graph_mu);
        if (g_graph_failed.count(key)) return false;
        auto it = g_graphs.find(key);
        if (it != g_graphs.end()) e = it->second;
        else if (g_graph_seen.insert(key).second) {
            if (g_graph_seen.size() > 4 * kMaxGraphs) g_graph_seen.clear();
            return false;
        } else {
            // captured under the cache lock: one capture at a time, and no
            // other thread uses this key until it is in the cache
            e = std::make_shared<graph_entry>();
            e->stream = s;
            e->d_items = (item_desc *)dev_alloc(P.nitems * sizeof(item_desc), s);
            e->d_segs = (seg_desc *)dev_alloc(P.nseg * sizeof(seg_desc), s);
            e->d_blks = (blk_desc *)dev_alloc(P.nblocks * sizeof(blk_desc), s);
            e->d_out = (jacobian_t *)dev_alloc(P.nitems * sizeof(jacobian_t), s);
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                (void)cudaGetLastError();
                g_graph_failed.insert(key);
                return false;
            }
            bool launched = true;
            try {
                run_planned(P, e->d_items, e->d_segs, e->d_blks, points, e->d_out, s);
            } catch (...) {
                launched = false;
            }
            const cudaError_t ec = cudaStreamEndCapture(s, &g);
            cudaError_t ei = cudaErrorUnknown;
            if (launched && ec == cudaSuccess && g) ei = cudaGraphInstantiate(&e->exec, g, 0);
            if (g) cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                (void)cudaGetLastError();
                e->exec = nullptr;
                g_graph_failed.insert(key);
                return false;
            }
            g_graph_captures++;
            if (g_graphs.size() >= kMaxGraphs) {
                auto lru = g_graphs.begin();
                for (auto j = g_graphs.begin(); j != g_graphs.end(); ++j)
                    if (j->second->last_use < lru->second->last_use) lru = j;
                g_graphs.erase(lru);
            }
            g_graphs.emplace(key, e);
        }
        e->last_use = ++g_graph_clock;
    }
    // the previous launch of this graph is on the same stream: the copies
    // into its descriptor buffers are ordered after it
    std::lock_guard<std::mutex> lk(e->mu);
    h2d(e->d_items, P.idesc.data(), P.nitems * sizeof(item_desc), s);
    h2d(e->d_segs, P.sdesc.data(), P.nseg * sizeof(seg_desc), s);
    h2d(e->d_blks, P.bdesc.data(), P.nblocks * sizeof(blk_desc), s);
    GB_CUDA_OK(cudaGraphLaunch(e->exec, s));
    GB_CUDA_OK(cudaMemcpyAsync(d_out, e->d_out, P.nitems * sizeof(jacobian_t), cudaMemcpyDeviceToDevice, s));
    g_graph_launches++;
    return true;
}

// Run a batch of MSMs.  precomputed: `points` is a table of nwin rows of
// `stride` bases (row j = 2^(c*j) P); plain: `points` holds the bases.
// Results (one Jacobian point per item) are written to d_out (device).
// use_graph: the bases pointer is stable across calls (a context's), so
// the batch may replay a captured graph.
static void msm_run_batch(const std::vector<msm_item> &items, int c, bool precomputed, const affine_t *points,
                          size_t stride, jacobian_t *d_out, cudaStream_t s, bool use_graph = false)
{
    set_smem_attrs();
    if (items.empty()) return;
    const batch_plan P = plan_batch(items, c, precomputed, stride);
    if (use_graph && graphs_enabled() && run_planned_graph(P, points, d_out, s)) return;
    dev_buf<item_desc> d_items(P.nitems, s);
    dev_buf<seg_desc> d_segs(P.nseg, s);
    dev_buf<blk_desc> d_blks(P.nblocks, s);
    h2d(d_items, P.idesc.data(), P.nitems * sizeof(item_desc), s);
    h2d(d_segs, P.sdesc.data(), P.nseg * sizeof(seg_desc), s);
    h2d(d_blks, P.bdesc.data(), P.nblocks * sizeof(blk_desc), s);
    run_planned(P, d_items, d_segs, d_blks, points, d_out, s);
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
    // read-only once created: calls from different lanes run concurrently,
    // each with its own stream-ordered scratch
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

// Plain MSMs of host bases + host scalars [nmsms][n] (nothing resident):
// one batch through the engine.
// Autotuner for the plain path: the key is the size class of the largest
// item, the batch-size class and the sparsity of a sample of the scalars
// (zero scalars, scalars below 2^64: both empty the high windows); a new key
// times every window size with a populated top window on this batch.
__global__ void scalar_sample_kernel(const fr_t *__restrict__ scalars, size_t n, unsigned *counts)
{
    unsigned zero = 0, small = 0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
        fr_t c = scalars[i].from_mont();
        bool hi_zero = true;
#pragma unroll
        for (int k = 2; k < 8; k++) hi_zero &= c.v[k] == 0;
        if (hi_zero) {
            if (c.v[0] == 0 && c.v[1] == 0) zero++;
            else small++;
        }
    }
    atomicAdd(&counts[0], zero);
    atomicAdd(&counts[1], small);
}

static int tuned_window(const std::vector<msm_item> &items, const affine_t *points, size_t stride, cudaStream_t s)
{
    size_t n_max = 0, total = 0;
    for (const msm_item &it : items) {
        n_max = std::max(n_max, it.n);
        total += it.n;
    }
    int c = choose_window(n_max, false);
    if (!autotune_enabled() || n_max < 256) return c;
    const msm_item &first = *std::max_element(items.begin(), items.end(),
                                              [](const msm_item &a, const msm_item &b) { return a.n < b.n; });
    const size_t sample = std::min<size_t>(first.n, 4096);
    dev_buf<unsigned> counts(2, s);
    GB_CUDA_OK(cudaMemsetAsync(counts.get(), 0, 2 * sizeof(unsigned), s));
    scalar_sample_kernel<<<1, 256, 0, s>>>(first.scalars, sample, counts);
    GB_CHECK_LAUNCH();
    unsigned h[2] = {0, 0};
    d2h(h, counts, sizeof(h), s);
    lane_sync(s);
    auto cls = [&](unsigned v) { return v * 20 < sample ? 0 : (v * 10 < sample * 3 ? 1 : 2); };
    int lg = 0;
    while (((size_t)1 << (lg + 1)) <= n_max) lg++;
    const size_t nitems = items.size();
    const int bclass = nitems == 1 ? 0 : nitems <= 8 ? 1 : nitems <= 64 ? 2 : 3;
    const std::string key = "msm:2^" + std::to_string(lg) + ":b" + std::to_string(bclass) + ":z" +
                            std::to_string(cls(h[0])) + ":s" + std::to_string(cls(h[1]));
    if (autotune_lookup(key, &c)) return c;
    dev_buf<jacobian_t> scratch(nitems, s);
    float best = 1e30f;
    for (int cand : {8, 10, 13, 16}) {
        if (cand > kMaxWindowBits || ((size_t)1 << (cand - 1)) > 8 * total) continue;
        float ms = time_on_stream(s, [&] { msm_run_batch(items, cand, false, points, stride, scratch, s); });
        if (ms < best) {
            best = ms;
            c = cand;
        }
    }
    autotune_store(key, c);
    return c;
}

static void msm_host_plain(jacobian_t *out, const affine_t *points, const fr_t *scalars, size_t n, size_t nmsms)
{
    cudaStream_t s = lane_stream();
    dev_buf<affine_t> d_points(n, s);
    dev_buf<fr_t> d_scalars(n * nmsms, s);
    dev_buf<jacobian_t> d_out(std::max<size_t>(nmsms, 1), s);
    h2d(d_points, points, n * sizeof(affine_t), s);
    h2d(d_scalars, scalars, n * nmsms * sizeof(fr_t), s);
    std::vector<msm_item> items;
    for (size_t m = 0; m < nmsms; m++) items.push_back(msm_item{d_scalars.get() + m * n, n, 0});
    msm_run_batch(items, tuned_window(items, d_points, 0, s), false, d_points, 0, d_out, s);
    d2h(out, d_out, nmsms * sizeof(jacobian_t), s);
    lane_sync(s);
    timed_collect();
}

// An MSM far smaller than the context's bucket count (2^(c-1)) skips the
// precomputed windows: a precomputed MSM always pays for all the buckets,
// while a small plain MSM with its own small window pays far less.  Below
// this ratio of points to buckets the plain path is taken.
static constexpr size_t kPrecomputedMinRatio = 8;

// A batch against the context, queued on stream s.  Large items use the
// precomputed table; small ones run as one plain batch over table row 0 (the
// bases themselves) with a window sized for them.  The results (one Jacobian
// point per item) are copied to `staging` on s, large items first; the
// returned vector gives the item index of each staging slot.  `staging` must
// be page-locked when the caller does not synchronise s before reading it.
static std::vector<size_t> context_enqueue_items(msm_context_t *ctx, jacobian_t *staging,
                                                 const std::vector<msm_item> &items, cudaStream_t s)
{
    std::vector<msm_item> big, small;
    std::vector<size_t> big_idx, small_idx;
    for (size_t i = 0; i < items.size(); i++) {
        if (items[i].n * kPrecomputedMinRatio >= ((size_t)1 << (ctx->c - 1)) || items.size() == 1) {
            big.push_back(items[i]);
            big_idx.push_back(i);
        } else {
            small.push_back(items[i]);
            small_idx.push_back(i);
        }
    }
    dev_buf<jacobian_t> d_big(std::max<size_t>(big.size(), 1), s), d_small(std::max<size_t>(small.size(), 1), s);
    if (!big.empty()) msm_run_batch(big, ctx->c, true, ctx->table, ctx->npoints, d_big, s, true);
    if (!small.empty())
        msm_run_batch(small, tuned_window(small, ctx->table, 0, s), false, ctx->table, 0, d_small, s, true);
    d2h(staging, d_big, big.size() * sizeof(jacobian_t), s);
    d2h(staging + big.size(), d_small, small.size() * sizeof(jacobian_t), s);
    big_idx.insert(big_idx.end(), small_idx.begin(), small_idx.end());
    return big_idx;
}

// The same, results to the host when it returns.
static void context_run_items(msm_context_t *ctx, jacobian_t *out_host, const std::vector<msm_item> &items,
                              cudaStream_t s)
{
    std::vector<jacobian_t> staging(items.size());
    const std::vector<size_t> order = context_enqueue_items(ctx, staging.data(), items, s);
    lane_sync(s);
    for (size_t i = 0; i < order.size(); i++) out_host[order[i]] = staging[i];
    timed_collect();
}

// Page-locked staging buffers of the asynchronous MSM calls, reused: a
// cudaFreeHost would synchronise the device, so buffers are kept until exit.
static std::mutex g_pinned_mu;
static std::multimap<size_t, jacobian_t *> g_pinned_free;

static jacobian_t *pinned_take(size_t n, size_t *cap)
{
    n = std::max<size_t>(n, 64);
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        auto it = g_pinned_free.lower_bound(n);
        if (it != g_pinned_free.end()) {
            *cap = it->first;
            jacobian_t *p = it->second;
            g_pinned_free.erase(it);
            return p;
        }
    }
    jacobian_t *p = nullptr;
    GB_CUDA_OK(cudaHostAlloc((void **)&p, n * sizeof(jacobian_t), cudaHostAllocPortable));
    *cap = n;
    return p;
}

static void pinned_give(jacobian_t *p, size_t cap)
{
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    g_pinned_free.emplace(cap, p);
}

// An MSM batch in flight: its completion event, the page-locked buffer its
// results land in and the item order of that buffer.
struct msm_ticket_t {
    int device = 0;
    uint32_t lane = 0;
    cudaEvent_t done = nullptr;
    jacobian_t *staging = nullptr;
    size_t cap = 0;
    std::vector<size_t> order;
};

static void ticket_release(msm_ticket_t *t)
{
    if (!t) return;
    if (t->done) cudaEventDestroy(t->done);
    pinned_give(t->staging, t->cap);
    delete t;
}

// The device address of page-locked host memory (mapped into the unified
// address space, so kernels read it over the host link), or null for
// pageable or device memory.
static const fr_t *pinned_device_view(const fr_t *p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return reinterpret_cast<const fr_t *>(a.devicePointer);
}

static void context_run_device(msm_context_t *ctx, jacobian_t *out_host, const fr_t *d_scalars, size_t npoints,
                               size_t nmsms, cudaStream_t s)
{
    std::vector<msm_item> items;
    for (size_t m = 0; m < nmsms; m++) items.push_back(msm_item{d_scalars + m * npoints, npoints, 0});
    context_run_items(ctx, out_host, items, s);
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

// One MSM over bases and scalars already in device memory (the caller's
// pointers, e.g. a resident SRS and a polynomial): the plain engine with
// windows combined by Horner's rule, no precomputed table, so it needs n x
// 96 bytes of bases instead of a context's nwin x n x 96.  No reference
// counterpart: the reference's resident MSMs all go through a context.
RustError gb_g1_msm_device(RawG1Projective *out_raw, const RawG1Affine *d_points_raw, const RawFr *d_scalars_raw,
                           size_t n)
{
    jacobian_t *out = reinterpret_cast<jacobian_t *>(out_raw);
    const affine_t *d_points = reinterpret_cast<const affine_t *>(d_points_raw);
    const fr_t *d_scalars = reinterpret_cast<const fr_t *>(d_scalars_raw);
    GB_ENTRY_BEGIN
    if (!out || (n && (!d_points || !d_scalars)))
        return make_error((int)cudaErrorInvalidValue, "invalid device MSM arguments");
    cudaStream_t s = lane_stream();
    dev_buf<jacobian_t> d_out(1, s);
    std::vector<msm_item> items{msm_item{d_scalars, n, 0}};
    msm_run_batch(items, tuned_window(items, d_points, 0, s), false, d_points, 0, d_out, s);
    d2h(out, d_out, sizeof(jacobian_t), s);
    lane_sync(s);
    timed_collect();
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
        lane_sync(s);
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

// Device bytes a context holds: its table of nwin x npoints affine points
// (the bases shifted by each window).  No reference counterpart.
size_t gb_g1_msm_context_device_bytes(const void *context)
{
    auto *ctx = reinterpret_cast<const msm_context_t *>(context);
    return ctx ? ctx->npoints * (size_t)ctx->nwin * sizeof(affine_t) : 0;
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
    cudaStream_t s = lane_stream();
    // page-locked host scalars are read in place by the recode kernel over
    // the host link, with no staging copy; pageable ones are staged
    if (const fr_t *view = pinned_device_view(scalars)) {
        count_transfer(true, npoints * nmsms * sizeof(fr_t));
        context_run_device(ctx, out, view, npoints, nmsms, s);
        return ok();
    }
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
    cudaStream_t s = lane_stream();
    device_vec_wait(dv, s);
    context_run_device(ctx, out, dv->values + scalar_offset, npoints, nmsms, s);
    return ok();
    GB_ENTRY_END
}

// The resident batch of midnight_sppark_bls12_381_g1_msm_context_device_batch,
// queued on the calling lane and returned at once: *ticket is completed by
// gb_msm_ticket_wait, which waits for the batch and writes its points.  The
// host can queue further work on the lane meanwhile (work that does not
// need the points), so the device is not left idle while the host waits for
// them.  No reference counterpart (the reference's calls return the points).
RustError gb_g1_msm_context_device_batch_async(void **ticket, void *context, const void *device_vec,
                                               size_t scalar_offset, size_t npoints, size_t nmsms)
{
    if (!ticket) return make_error((int)cudaErrorInvalidValue, "null MSM ticket output");
    *ticket = nullptr;
    if (!context || !device_vec) return make_error(-1, "invalid resident BLS12-381 G1 MSM arguments");
    GB_ENTRY_BEGIN
    auto *ctx = reinterpret_cast<msm_context_t *>(context);
    auto *dv = reinterpret_cast<const fr_device_vec *>(device_vec);
    if (npoints != 0 && nmsms > (SIZE_MAX - scalar_offset) / npoints)
        return make_error((int)cudaErrorInvalidValue, "resident MSM range overflow");
    if (scalar_offset + npoints * nmsms > dv->len)
        return make_error((int)cudaErrorInvalidValue, "resident MSM range exceeds device vector");
    if (npoints > ctx->npoints) return make_error((int)cudaErrorInvalidValue, "more scalars than context bases");
    cudaStream_t s = lane_stream();
    auto *t = new msm_ticket_t();
    try {
        t->device = current_device();
        t->lane = current_lane();
        t->staging = pinned_take(nmsms, &t->cap);
        GB_CUDA_OK(cudaEventCreateWithFlags(&t->done, cudaEventDisableTiming));
        if (nmsms) {
            device_vec_wait(dv, s);
            std::vector<msm_item> items;
            for (size_t m = 0; m < nmsms; m++)
                items.push_back(msm_item{dv->values + scalar_offset + m * npoints, npoints, 0});
            t->order = context_enqueue_items(ctx, t->staging, items, s);
        }
        GB_CUDA_OK(cudaEventRecord(t->done, s));
    } catch (...) {
        ticket_release(t);
        throw;
    }
    *ticket = t;
    return ok();
    GB_ENTRY_END
}

// Graph replay of context batches on (1) or off (0); the counters give the
// graphs captured and the batches replayed since the process started.
RustError gb_msm_graphs_enable(int on)
{
    gb::g_graphs_on.store(on ? 1 : 0, std::memory_order_relaxed);
    return ok();
}

RustError gb_msm_graph_stats(unsigned long long *captures, unsigned long long *launches)
{
    if (!captures || !launches) return make_error((int)cudaErrorInvalidValue, "null graph counter output");
    *captures = gb::g_graph_captures.load();
    *launches = gb::g_graph_launches.load();
    return ok();
}

// Waits for the batch of `ticket`, writes its points to out (nmsms of them,
// in batch order; out may be null to discard them) and releases the ticket,
// which must not be used again.  A wait that ran out in the lane's NTT work
// since its previous synchronisation is reported here, as by the lane's
// synchronising calls.
RustError gb_msm_ticket_wait(void *ticket, RawG1Projective *out_raw)
{
    auto *t = reinterpret_cast<msm_ticket_t *>(ticket);
    if (!t) return make_error((int)cudaErrorInvalidValue, "null MSM ticket");
    jacobian_t *out = reinterpret_cast<jacobian_t *>(out_raw);
    GB_ENTRY_BEGIN
    const cudaError_t e = cudaEventSynchronize(t->done);
    if (e != cudaSuccess) {
        ticket_release(t);
        return make_error((int)e, cudaGetErrorString(e));
    }
    int prev_dev = 0;
    GB_CUDA_OK(cudaGetDevice(&prev_dev));
    const uint32_t prev_lane = current_lane();
    try {
        if (prev_dev != t->device) GB_CUDA_OK(cudaSetDevice(t->device));
        set_lane(t->lane);
        lane_check();
    } catch (...) {
        set_lane(prev_lane);
        cudaSetDevice(prev_dev);
        ticket_release(t);
        throw;
    }
    set_lane(prev_lane);
    if (prev_dev != t->device) GB_CUDA_OK(cudaSetDevice(prev_dev));
    if (out)
        for (size_t i = 0; i < t->order.size(); i++) out[t->order[i]] = t->staging[i];
    ticket_release(t);
    timed_collect();
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
    cudaStream_t s = lane_stream();
    device_vec_wait(dv, s);
    std::vector<msm_item> items;
    for (size_t i = 0; i < count; i++)
        items.push_back(msm_item{dv->values + slices[i].scalar_offset, slices[i].len, slices[i].point_offset});
    context_run_items(ctx, out, items, s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:6379-6404 (test hooks): a delay for the next
// scrambled batches' mask producer on this thread; the masked scalars are
// zeroed and the stream held back before the mask is added, so that an MSM
// that did not wait for them would read zeros
static thread_local uint32_t t_mask_delay_ms = 0;

void midnight_sppark_test_mask_delay(uint32_t delay_ms)
{
    t_mask_delay_ms = delay_ms;
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
    cudaStream_t s = lane_stream();
    device_vec_wait(dv, s);
    device_vec_wait(mv, s);
    dev_buf<fr_t> masked(count, s);
    if (t_mask_delay_ms) {
        GB_CUDA_OK(cudaMemsetAsync(masked.get(), 0, count * sizeof(fr_t), s));
        lane_sync(s);
        stream_host_delay(s, t_mask_delay_ms);
    }
    add_mask_kernel<<<blocks_for(count, 256), 256, 0, s>>>(masked, dv->values + scalar_offset, mv->values, npoints,
                                                           count);
    GB_CHECK_LAUNCH();
    context_run_device(ctx, out, masked, npoints, nmsms, s);
    return ok();
    GB_ENTRY_END
}

}  // extern "C"
