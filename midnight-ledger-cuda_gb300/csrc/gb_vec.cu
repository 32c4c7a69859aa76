// Fr vector kernels: multiplicative prefix scan, Montgomery-trick batch
// inversion, permutation / lookup grand products, quotient limb split, linear
// combinations, canonical sort and the resident device-vector entry points of
// the C ABI (midnight-sppark-msm/src/bls12_381_g1_msm.cu:1188-1700 kernels,
// 2741-3442 device vectors, 3558-4634 vector ops and products).
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <vector>

#include "gb_ntt.cuh"
#include "gb_vec.cuh"

namespace gb {

static constexpr int kScanThreads = 256;
static constexpr int kScanPer = 8;  // elements per thread
static constexpr size_t kScanTile = (size_t)kScanThreads * kScanPer;

// ------------------------------------------------------------ block scans

// Inclusive multiplicative scan of one value per thread across the block
// (Hillis-Steele over shared memory).  Returns the inclusive prefix.
__device__ fr_t block_scan_mul(fr_t v, fr_t *sh)
{
    sh[threadIdx.x] = v;
    __syncthreads();
    for (unsigned off = 1; off < blockDim.x; off <<= 1) {
        fr_t other = threadIdx.x >= off ? sh[threadIdx.x - off] : fr_t::one();
        __syncthreads();
        if (threadIdx.x >= off) sh[threadIdx.x] = sh[threadIdx.x] * other;
        __syncthreads();
    }
    return sh[threadIdx.x];
}

// Inclusive multiplicative suffix scan (thread t gets prod_{t' >= t}).
__device__ fr_t block_suffix_scan_mul(fr_t v, fr_t *sh)
{
    sh[threadIdx.x] = v;
    __syncthreads();
    for (unsigned off = 1; off < blockDim.x; off <<= 1) {
        fr_t other = threadIdx.x + off < blockDim.x ? sh[threadIdx.x + off] : fr_t::one();
        __syncthreads();
        if (threadIdx.x + off < blockDim.x) sh[threadIdx.x] = sh[threadIdx.x] * other;
        __syncthreads();
    }
    return sh[threadIdx.x];
}

// ------------------------------------------------------------ prefix product

// phase 1: per tile product -> aux[tile]
__global__ void __launch_bounds__(kScanThreads) scan_tile_product_kernel(const fr_t *__restrict__ in, size_t n,
                                                                         fr_t *__restrict__ aux)
{
    __shared__ fr_t sh[kScanThreads];
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPer;
    fr_t p = fr_t::one();
#pragma unroll
    for (int e = 0; e < kScanPer; e++)
        if (base + e < n) p = p * in[base + e];
    fr_t incl = block_scan_mul(p, sh);
    if (threadIdx.x == blockDim.x - 1) aux[blockIdx.x] = incl;
}

// phase 3: out[i] = carry_in(tile) * prefix within tile (inclusive)
__global__ void __launch_bounds__(kScanThreads) scan_tile_apply_kernel(const fr_t *__restrict__ in, size_t n,
                                                                       const fr_t *__restrict__ aux_incl,
                                                                       fr_t *out)
{
    __shared__ fr_t sh[kScanThreads];
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPer;
    fr_t vals[kScanPer];
    fr_t p = fr_t::one();
#pragma unroll
    for (int e = 0; e < kScanPer; e++) {
        vals[e] = base + e < n ? in[base + e] : fr_t::one();
        p = p * vals[e];
    }
    fr_t incl = block_scan_mul(p, sh);
    __syncthreads();
    fr_t excl = threadIdx.x ? sh[threadIdx.x - 1] : fr_t::one();
    fr_t run = blockIdx.x ? aux_incl[blockIdx.x - 1] * excl : excl;
    (void)incl;
#pragma unroll
    for (int e = 0; e < kScanPer; e++) {
        run = run * vals[e];
        if (base + e < n) out[base + e] = run;
    }
}

// inclusive prefix product, out may alias in
void prefix_product(fr_t *out, const fr_t *in, size_t n, cudaStream_t s)
{
    if (!n) return;
    size_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles > 0x7fffffff) throw cuda_error(-1, "scan too large");
    dev_buf<fr_t> aux(tiles, s);
    scan_tile_product_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, aux);
    GB_CHECK_LAUNCH();
    if (tiles > 1) prefix_product(aux, aux, tiles, s);
    scan_tile_apply_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, aux, out);
    GB_CHECK_LAUNCH();
}

// ------------------------------------------------------------ additive suffix scan

// out[i] = sum_{j >= i} in[j], by tiles of 2048 counted from the top end
__global__ void __launch_bounds__(kScanThreads) sfx_tile_sum_kernel(const fr_t *__restrict__ in, size_t n,
                                                                    fr_t *__restrict__ aux)
{
    __shared__ fr_t sh[kScanThreads];
    // tile t covers reversed positions [t*2048, (t+1)*2048), element n-1-r
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPer;
    fr_t acc = fr_t::zero();
#pragma unroll
    for (int e = 0; e < kScanPer; e++)
        if (base + e < n) acc = acc + in[n - 1 - (base + e)];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (unsigned off = blockDim.x / 2; off; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) aux[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kScanThreads) sfx_tile_apply_kernel(const fr_t *in, size_t n,
                                                                      const fr_t *__restrict__ aux_incl, fr_t *out)
{
    __shared__ fr_t sh[kScanThreads];
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPer;
    fr_t v[kScanPer];
    fr_t acc = fr_t::zero();
#pragma unroll
    for (int e = 0; e < kScanPer; e++) {
        v[e] = base + e < n ? in[n - 1 - (base + e)] : fr_t::zero();
        acc = acc + v[e];
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (unsigned off = 1; off < blockDim.x; off <<= 1) {
        fr_t other = threadIdx.x >= off ? sh[threadIdx.x - off] : fr_t::zero();
        __syncthreads();
        if (threadIdx.x >= off) sh[threadIdx.x] = sh[threadIdx.x] + other;
        __syncthreads();
    }
    fr_t run = threadIdx.x ? sh[threadIdx.x - 1] : fr_t::zero();
    if (blockIdx.x) run = run + aux_incl[blockIdx.x - 1];
#pragma unroll
    for (int e = 0; e < kScanPer; e++) {
        run = run + v[e];
        if (base + e < n) out[n - 1 - (base + e)] = run;
    }
}

// inclusive prefix sum of tile totals, in place (reuses the suffix machinery
// on the reversed view of a reversed array: a plain forward scan)
__global__ void __launch_bounds__(kScanThreads) fwd_sum_scan_small_kernel(fr_t *a, size_t n)
{
    // single block, n <= kScanTile * kScanTile handled by recursion on the host
    __shared__ fr_t sh[kScanThreads];
    const size_t per = (n + blockDim.x - 1) / blockDim.x;
    const size_t lo = threadIdx.x * per, hi = min(lo + per, n);
    fr_t acc = fr_t::zero();
    for (size_t i = lo; i < hi; i++) acc = acc + a[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (unsigned off = 1; off < blockDim.x; off <<= 1) {
        fr_t other = threadIdx.x >= off ? sh[threadIdx.x - off] : fr_t::zero();
        __syncthreads();
        if (threadIdx.x >= off) sh[threadIdx.x] = sh[threadIdx.x] + other;
        __syncthreads();
    }
    fr_t run = threadIdx.x ? sh[threadIdx.x - 1] : fr_t::zero();
    for (size_t i = lo; i < hi; i++) {
        run = run + a[i];
        a[i] = run;
    }
}

void suffix_sum(fr_t *out, const fr_t *in, size_t n, cudaStream_t s)
{
    if (!n) return;
    size_t tiles = (n + kScanTile - 1) / kScanTile;
    dev_buf<fr_t> aux(tiles, s);
    sfx_tile_sum_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, aux);
    GB_CHECK_LAUNCH();
    fwd_sum_scan_small_kernel<<<1, kScanThreads, 0, s>>>(aux, tiles);
    GB_CHECK_LAUNCH();
    sfx_tile_apply_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, aux, out);
    GB_CHECK_LAUNCH();
}

// ------------------------------------------------------------ batch inversion

// Montgomery's trick per tile: one binary-GCD inversion per tile of 2048
// elements; zeros stay zero (the field inverse the reference applies maps
// 0 to 0).  out may alias in.  If `mul` is given, out[i] = mul[i] / in[i].
__global__ void __launch_bounds__(kScanThreads) batch_invert_kernel(const fr_t *in, size_t n,
                                                                    const fr_t *mul,
                                                                    fr_t *out)
{
    __shared__ fr_t sh[kScanThreads];
    __shared__ fr_t total_inv;
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPer;
    fr_t x[kScanPer], q[kScanPer];
    fr_t p = fr_t::one();
#pragma unroll
    for (int e = 0; e < kScanPer; e++) {
        fr_t v = base + e < n ? in[base + e] : fr_t::zero();
        x[e] = v;
        q[e] = p;  // product of this thread's earlier nonzero elements
        if (!v.is_zero()) p = p * v;
    }
    fr_t incl = block_scan_mul(p, sh);
    __syncthreads();
    fr_t excl = threadIdx.x ? sh[threadIdx.x - 1] : fr_t::one();
    if (threadIdx.x == blockDim.x - 1) total_inv = incl.inverse_binary();
    __syncthreads();
    fr_t suffix_incl = block_suffix_scan_mul(p, sh);
    __syncthreads();
    fr_t suffix_excl = threadIdx.x + 1 < blockDim.x ? sh[threadIdx.x + 1] : fr_t::one();
    (void)suffix_incl;
    // 1/p = total^-1 * (product of every other thread's p)
    fr_t J = total_inv * excl * suffix_excl;
#pragma unroll
    for (int e = kScanPer - 1; e >= 0; e--) {
        if (base + e >= n) continue;
        if (x[e].is_zero()) {
            out[base + e] = fr_t::zero();
            continue;
        }
        fr_t inv = J * q[e];
        J = J * x[e];
        out[base + e] = mul ? mul[base + e] * inv : inv;
    }
}

void batch_invert(fr_t *out, const fr_t *in, size_t n, const fr_t *mul, cudaStream_t s)
{
    if (!n) return;
    size_t tiles = (n + kScanTile - 1) / kScanTile;
    batch_invert_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, mul, out);
    GB_CHECK_LAUNCH();
}

__global__ void power_factors_kernel(fr_t *d, fr_t w, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = i ? w : fr_t::one();
}

// Power tables up to 2^24 entries: w^i = T0[i & 255] * T1[(i >> 8) & 255] *
// T2[i >> 16], where T0[j] = w^j, T1[j] = w^(256 j), T2[j] = w^(65536 j).
// One block builds the three 256-entry tables with block scans (exclusive:
// T[j] = base^j); the apply kernel spends two products per element.
__global__ void __launch_bounds__(256) power_tables_kernel(fr_t w, fr_t *__restrict__ tables)
{
    __shared__ fr_t sh[256];
    fr_t base = w;
    for (int level = 0; level < 3; level++) {
        fr_t incl = block_scan_mul(base, sh);  // base^(t+1)
        __syncthreads();
        tables[level * 256 + threadIdx.x] = threadIdx.x ? sh[threadIdx.x - 1] : fr_t::one();
        base = sh[255];  // base^256, the next level's base
        __syncthreads();
        (void)incl;
    }
}

__global__ void power_apply_kernel(const fr_t *__restrict__ tables, size_t n, fr_t *__restrict__ d)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fr_t v = tables[i & 255];
    if (i >> 8) v = v * tables[256 + ((i >> 8) & 255)];
    if (i >> 16) v = v * tables[512 + (i >> 16)];
    d[i] = v;
}

// the tables of power_tables_kernel for several points: block q reads
// points[q] and writes tables[q * 768 ..]
__global__ void __launch_bounds__(256) power_tables_many_kernel(const fr_t *__restrict__ points,
                                                                fr_t *__restrict__ tables)
{
    __shared__ fr_t sh[256];
    fr_t base = points[blockIdx.x];
    fr_t *t = tables + (size_t)blockIdx.x * 768;
    for (int level = 0; level < 3; level++) {
        block_scan_mul(base, sh);  // sh[t] = base^(t+1)
        __syncthreads();
        t[level * 256 + threadIdx.x] = threadIdx.x ? sh[threadIdx.x - 1] : fr_t::one();
        base = sh[255];
        __syncthreads();
    }
}

// d[q * n + i] = tables_q-powers, i < n <= 2^24, one grid row per point
__global__ void power_apply_many_kernel(const fr_t *__restrict__ tables, size_t n, fr_t *__restrict__ d)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const fr_t *t = tables + (size_t)blockIdx.y * 768;
    fr_t v = t[i & 255];
    if (i >> 8) v = v * t[256 + ((i >> 8) & 255)];
    if (i >> 16) v = v * t[512 + (i >> 16)];
    d[(size_t)blockIdx.y * n + i] = v;
}

void omega_powers_many(fr_t *d, const fr_t *d_points, size_t npoints, size_t n, cudaStream_t s)
{
    if (!n || !npoints) return;
    if (n > ((size_t)1 << 24) || npoints > 65535) throw cuda_error((int)cudaErrorInvalidValue, "power table too large");
    dev_buf<fr_t> tables(768 * npoints, s);
    power_tables_many_kernel<<<(unsigned)npoints, 256, 0, s>>>(d_points, tables);
    GB_CHECK_LAUNCH();
    power_apply_many_kernel<<<dim3(blocks_for(n, 256), (unsigned)npoints), 256, 0, s>>>(tables, n, d);
    GB_CHECK_LAUNCH();
}

void omega_powers(fr_t *d, const fr_t &w, size_t n, cudaStream_t s)
{
    if (!n) return;
    if (n > ((size_t)1 << 24)) {
        power_factors_kernel<<<blocks_for(n, 256), 256, 0, s>>>(d, w, n);
        GB_CHECK_LAUNCH();
        prefix_product(d, d, n, s);
        return;
    }
    dev_buf<fr_t> tables(3 * 256, s);
    power_tables_kernel<<<1, 256, 0, s>>>(w, tables);
    GB_CHECK_LAUNCH();
    power_apply_kernel<<<blocks_for(n, 256), 256, 0, s>>>(tables, n, d);
    GB_CHECK_LAUNCH();
}

// ------------------------------------------------------------ products

// z[0] = init, z[i] = init * prefix[i-1]; init read from device memory
__global__ void shifted_apply_kernel(fr_t *__restrict__ out, const fr_t *__restrict__ prefix,
                                     const fr_t *__restrict__ init, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fr_t a = *init;
    out[i] = i ? a * prefix[i - 1] : a;
}

__global__ void blind_tail_kernel(fr_t *__restrict__ values, const fr_t *__restrict__ blinds, size_t len, size_t bf)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < bf) values[len - bf + i] = blinds[i];
}

__global__ void copy_one_kernel(fr_t *dst, const fr_t *src) { *dst = *src; }

__global__ void set_scalar_kernel(fr_t *dst, fr_t v) { *dst = v; }

// Permutation fraction numerator / denominator per row (prover.rs:392-460):
// num = prod_j (v_j + delta^j w^i beta + gamma), den = prod_j (v_j + beta s_j + gamma).
// Column c is columns[c * len ..] or, with a pointer table, col_ptrs[c][..].
__global__ void perm_num_den_kernel(const fr_t *__restrict__ columns, const fr_t *const *__restrict__ col_ptrs,
                                    const fr_t *__restrict__ perms, const fr_t *__restrict__ delta_powers,
                                    fr_t omega, fr_t beta, fr_t gamma, size_t len, size_t c0, size_t ncols,
                                    fr_t *__restrict__ num, fr_t *__restrict__ den)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    fr_t wi = omega.pow_u64(i);
    fr_t bw = beta * wi;
    fr_t nn = fr_t::one(), dd = fr_t::one();
    for (size_t j = 0; j < ncols; j++) {
        size_t c = c0 + j;
        fr_t v = col_ptrs ? col_ptrs[c][i] : columns[c * len + i];
        nn = nn * (v + delta_powers[c] * bw + gamma);
        dd = dd * (v + beta * perms[c * len + i] + gamma);
    }
    num[i] = nn;
    den[i] = dd;
}

// Lookup fraction numerator / denominator (lookup/prover.rs:1075-1240):
// num = (A + beta)(S + gamma), den = (A' + beta)(S' + gamma)
__global__ void lookup_num_den_kernel(const fr_t *__restrict__ ci, const fr_t *__restrict__ ct,
                                      const fr_t *__restrict__ pi, const fr_t *__restrict__ pt, fr_t beta,
                                      fr_t gamma, size_t total, fr_t *__restrict__ num, fr_t *__restrict__ den)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    num[i] = (ci[i] + beta) * (ct[i] + gamma);
    den[i] = (pi[i] + beta) * (pt[i] + gamma);
}

// grand product of fractions with chained initial value; `out` gets z
static void grand_product(fr_t *out, fr_t *num, fr_t *den, size_t len, const fr_t *d_init, fr_t *scratch,
                          cudaStream_t s)
{
    // fraction = num / den (batch inversion), prefix product, shift by init
    batch_invert(num, den, len, num, s);
    prefix_product(scratch, num, len, s);
    shifted_apply_kernel<<<blocks_for(len, 256), 256, 0, s>>>(out, scratch, d_init, len);
    GB_CHECK_LAUNCH();
}

void permutation_products(fr_t *out, const fr_t *d_columns, const fr_t *const *d_col_ptrs, const fr_t *d_perms,
                          size_t len, size_t column_count, size_t chunk_len, const fr_t &beta, const fr_t &gamma,
                          const fr_t &omega, const fr_t *d_delta, const fr_t *d_blinds, size_t bf, cudaStream_t s)
{
    const size_t sets = (column_count + chunk_len - 1) / chunk_len;
    dev_buf<fr_t> num(len, s), den(len, s), scratch(len, s), init(1, s);
    set_scalar_kernel<<<1, 1, 0, s>>>(init, fr_t::one());
    GB_CHECK_LAUNCH();
    for (size_t set = 0; set < sets; set++) {
        size_t c0 = set * chunk_len;
        size_t nc = std::min(chunk_len, column_count - c0);
        fr_t *z = out + set * len;
        perm_num_den_kernel<<<blocks_for(len, 256), 256, 0, s>>>(d_columns, d_col_ptrs, d_perms, d_delta, omega, beta,
                                                                 gamma, len, c0, nc, num, den);
        GB_CHECK_LAUNCH();
        grand_product(z, num, den, len, init, scratch, s);
        // next set starts from this set's last unblinded value
        copy_one_kernel<<<1, 1, 0, s>>>(init, z + (len - (bf + 1)));
        GB_CHECK_LAUNCH();
        if (bf) {
            blind_tail_kernel<<<blocks_for(bf, 256), 256, 0, s>>>(z, d_blinds + set * bf, len, bf);
            GB_CHECK_LAUNCH();
        }
    }
}

void lookup_products(fr_t *out, const fr_t *ci, const fr_t *ct, const fr_t *pi, const fr_t *pt, size_t len,
                     size_t lookup_count, const fr_t &beta, const fr_t &gamma, const fr_t *d_blinds, size_t bf,
                     cudaStream_t s)
{
    size_t total = len * lookup_count;
    dev_buf<fr_t> num(total, s), den(total, s), scratch(len, s), init(1, s);
    set_scalar_kernel<<<1, 1, 0, s>>>(init, fr_t::one());
    GB_CHECK_LAUNCH();
    lookup_num_den_kernel<<<blocks_for(total, 256), 256, 0, s>>>(ci, ct, pi, pt, beta, gamma, total, num, den);
    GB_CHECK_LAUNCH();
    for (size_t l = 0; l < lookup_count; l++) {
        fr_t *z = out + l * len;
        grand_product(z, num.get() + l * len, den.get() + l * len, len, init, scratch, s);
        if (bf) {
            blind_tail_kernel<<<blocks_for(bf, 256), 256, 0, s>>>(z, d_blinds + l * bf, len, bf);
            GB_CHECK_LAUNCH();
        }
    }
}

// ------------------------------------------------------------ misc kernels

__global__ void lincomb_kernel(fr_t *__restrict__ out, const fr_t *__restrict__ polys, const fr_t *__restrict__ k,
                               size_t len, size_t count)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    fr_t acc = fr_t::zero();
    for (size_t p = 0; p < count; p++) acc = acc + polys[p * len + i] * k[p];
    out[i] = acc;
}

__global__ void quotient_pieces_kernel(fr_t *__restrict__ out, const fr_t *__restrict__ q, size_t poly_len,
                                       size_t pieces)
{
    size_t f = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= poly_len * pieces) return;
    size_t piece = f / poly_len, i = f % poly_len;
    out[f] = i == poly_len - 1 ? fr_t::zero() : q[piece * (poly_len - 1) + i];
}

__global__ void blind_quotient_pieces_kernel(fr_t *pieces, const fr_t *__restrict__ blinds, size_t poly_len,
                                             size_t count)
{
    // sequential over pieces: piece p's last slot and piece p+1's first slot
    if (threadIdx.x || blockIdx.x) return;
    for (size_t p = 0; p + 1 < count; p++) {
        fr_t b = blinds[p];
        pieces[p * poly_len + poly_len - 1] = b;
        pieces[(p + 1) * poly_len] = pieces[(p + 1) * poly_len] - b;
    }
}

// canonical big-endian key (fq.rs:152-164) as 4 x u64 for the radix sort
struct canon_key {
    uint64_t l[4];
};
struct canon_decomposer {
    __host__ __device__ ::cuda::std::tuple<uint64_t &, uint64_t &, uint64_t &, uint64_t &> operator()(
        canon_key &k) const
    {
        return {k.l[3], k.l[2], k.l[1], k.l[0]};
    }
};

__global__ void to_canon_kernel(const fr_t *__restrict__ in, canon_key *__restrict__ out, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fr_t c = in[i].from_mont();
    canon_key k;
#pragma unroll
    for (int j = 0; j < 4; j++) k.l[j] = (uint64_t)c.v[2 * j] | ((uint64_t)c.v[2 * j + 1] << 32);
    out[i] = k;
}

__global__ void from_canon_kernel(const canon_key *__restrict__ in, fr_t *__restrict__ out, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fr_t c;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        c.v[2 * j] = (uint32_t)in[i].l[j];
        c.v[2 * j + 1] = (uint32_t)(in[i].l[j] >> 32);
    }
    out[i] = c.to_mont();
}

void sort_canonical(fr_t *d, size_t n, cudaStream_t s)
{
    if (n < 2) return;
    dev_buf<canon_key> a(n, s), b(n, s);
    to_canon_kernel<<<blocks_for(n, 256), 256, 0, s>>>(d, a, n);
    GB_CHECK_LAUNCH();
    size_t temp = 0;
    GB_CUDA_OK(cub::DeviceRadixSort::SortKeys(nullptr, temp, a.get(), b.get(), (int64_t)n, canon_decomposer{}, 0, 256, s));
    dev_buf<uint8_t> t(temp, s);
    GB_CUDA_OK(cub::DeviceRadixSort::SortKeys(t.get(), temp, a.get(), b.get(), (int64_t)n, canon_decomposer{}, 0, 256, s));
    from_canon_kernel<<<blocks_for(n, 256), 256, 0, s>>>(b, d, n);
    GB_CHECK_LAUNCH();
}

// upload helper
static dev_buf<fr_t> upload(const fr_t *host, size_t n, cudaStream_t s)
{
    dev_buf<fr_t> d(n, s);
    h2d(d, host, n * sizeof(fr_t), s);
    return d;
}

}  // namespace gb

namespace gb {

static constexpr size_t kSuffixSlice = 8192;

__global__ void nonzero_init_kernel(unsigned long long *stats, size_t count, size_t len)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) {
        stats[i] = len;        // first nonzero (len: none)
        stats[count + i] = 0;  // nonzero count
    }
}

// block (slice, poly): the slice's first nonzero index and nonzero count,
// merged into the polynomial's by atomics
__global__ void nonzero_stats_kernel(unsigned long long *first, unsigned long long *live,
                                     const fr_t *__restrict__ values, size_t len)
{
    __shared__ unsigned long long f_sh[256], c_sh[256];
    const size_t p = blockIdx.y;
    const fr_t *poly = values + p * len;
    const size_t lo = (size_t)blockIdx.x * kSuffixSlice, hi = min(lo + kSuffixSlice, len);
    unsigned long long f = len, c = 0;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        if (!poly[i].is_zero()) {
            f = min(f, (unsigned long long)i);
            c++;
        }
    }
    f_sh[threadIdx.x] = f;
    c_sh[threadIdx.x] = c;
    __syncthreads();
    for (unsigned off = blockDim.x / 2; off; off >>= 1) {
        if (threadIdx.x < off) {
            f_sh[threadIdx.x] = min(f_sh[threadIdx.x], f_sh[threadIdx.x + off]);
            c_sh[threadIdx.x] += c_sh[threadIdx.x + off];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (f_sh[0] < len) atomicMin(first + p, f_sh[0]);
        if (c_sh[0]) atomicAdd(live + p, c_sh[0]);
    }
}

}  // namespace gb

using namespace gb;

extern "C" {

// ---------------------------------------------------------------- vector ops
// bls12_381_g1_msm.cu:3558-3600 (host vector in, result back in place)
RustError midnight_sppark_bls12_381_fr_mul_assign(RawFr *values_raw, RawFr scalar_raw, size_t len)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    const fr_t scalar = gb::from_raw(scalar_raw);
    if (len == 0) return ok();
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto d = upload(values, len, s);
    launch_mul_assign(d, scalar, len, s);
    d2h(values, d, len * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

RustError midnight_sppark_bls12_381_fr_mul_assign_zeta(RawFr *values_raw, RawFr first_raw, RawFr second_raw, size_t len)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    const fr_t first = gb::from_raw(first_raw);
    const fr_t second = gb::from_raw(second_raw);
    if (len == 0) return ok();
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto d = upload(values, len, s);
    launch_mul_assign_zeta(d, first, second, len, len, s);
    d2h(values, d, len * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

RustError midnight_sppark_bls12_381_fr_mul_assign_repeating(RawFr *values_raw, const RawFr *factors_raw, size_t factor_len, size_t len)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    const fr_t *factors = reinterpret_cast<const fr_t *>(factors_raw);
    if (len == 0) return ok();
    if (factor_len == 0 || !factors) return make_error((int)cudaErrorInvalidValue, "empty repeating factors");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto d = upload(values, len, s);
    auto f = upload(factors, factor_len, s);
    launch_mul_assign_repeating(d, f, factor_len, len, s);
    d2h(values, d, len * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:1225-1231 semantics (every element inverted, 0 -> 0),
// computed with Montgomery's trick instead of one exponentiation per element
RustError midnight_sppark_bls12_381_fr_invert_assign(RawFr *values_raw, size_t len)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    if (len == 0) return ok();
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto d = upload(values, len, s);
    batch_invert(d, d, len, nullptr, s);
    d2h(values, d, len * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

RustError midnight_sppark_bls12_381_fr_sort_canonical(RawFr *values_raw, size_t len)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    if (len < 2) return ok();
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto d = upload(values, len, s);
    sort_canonical(d, len, s);
    d2h(values, d, len * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3558 region: out[i] = sum_k scalars[k] * polys[k][i]
RustError midnight_sppark_bls12_381_fr_poly_lincomb(RawFr *out_raw, const RawFr *polys_raw, size_t poly_len, size_t poly_count, const RawFr *scalars_raw)
{
    fr_t *out = reinterpret_cast<fr_t *>(out_raw);
    const fr_t *polys = reinterpret_cast<const fr_t *>(polys_raw);
    const fr_t *scalars = reinterpret_cast<const fr_t *>(scalars_raw);
    if (poly_len == 0) return ok();
    if (!out || (poly_count && (!polys || !scalars)))
        return make_error((int)cudaErrorInvalidValue, "invalid lincomb arguments");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto d = upload(polys, poly_len * poly_count, s);
    auto k = upload(scalars, poly_count, s);
    dev_buf<fr_t> o(poly_len, s);
    lincomb_kernel<<<blocks_for(poly_len, 256), 256, 0, s>>>(o, d, k, poly_len, poly_count);
    GB_CHECK_LAUNCH();
    d2h(out, o, poly_len * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:4303-4340 (permutation/prover.rs:36-43 semantics)
RustError midnight_sppark_bls12_381_fr_shifted_prefix_product(RawFr *values_raw, RawFr initial_raw, size_t len)
{
    fr_t *values = reinterpret_cast<fr_t *>(values_raw);
    const fr_t initial = gb::from_raw(initial_raw);
    if (len == 0) return ok();
    if (!values) return make_error((int)cudaErrorInvalidValue, "null values");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto d = upload(values, len, s);
    dev_buf<fr_t> prefix(len, s), init(1, s);
    h2d(init, &initial, sizeof(fr_t), s);
    prefix_product(prefix, d, len, s);
    shifted_apply_kernel<<<blocks_for(len, 256), 256, 0, s>>>(d, prefix, init, len);
    GB_CHECK_LAUNCH();
    d2h(values, d, len * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:4342-4449: z of every permutation set, resident
RustError midnight_sppark_bls12_381_fr_permutation_products(void **out, const RawFr *columns_raw, const RawFr *permutations_raw, size_t len, size_t column_count, size_t chunk_len, RawFr beta_raw, RawFr gamma_raw, RawFr omega_raw, const RawFr *delta_powers_raw, const RawFr *blind_values_raw, size_t blinding_factors)
{
    const fr_t *columns = reinterpret_cast<const fr_t *>(columns_raw);
    const fr_t *permutations = reinterpret_cast<const fr_t *>(permutations_raw);
    const fr_t beta = gb::from_raw(beta_raw);
    const fr_t gamma = gb::from_raw(gamma_raw);
    const fr_t omega = gb::from_raw(omega_raw);
    const fr_t *delta_powers = reinterpret_cast<const fr_t *>(delta_powers_raw);
    const fr_t *blind_values = reinterpret_cast<const fr_t *>(blind_values_raw);
    if (!out || len == 0 || column_count == 0 || chunk_len == 0 || !columns || !permutations || !delta_powers ||
        blinding_factors >= len || (blinding_factors != 0 && !blind_values))
        return make_error((int)cudaErrorInvalidValue, "invalid permutation product arguments");
    *out = nullptr;
    const size_t sets = (column_count + chunk_len - 1) / chunk_len;
    if (column_count > SIZE_MAX / len || sets > SIZE_MAX / len)
        return make_error((int)cudaErrorInvalidValue, "permutation product size overflow");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto dc = upload(columns, column_count * len, s);
    auto dp = upload(permutations, column_count * len, s);
    auto dd = upload(delta_powers, column_count, s);
    auto db = upload(blind_values, sets * blinding_factors, s);
    fr_device_vec *v = device_vec_new(sets * len, s);
    try {
        permutation_products(v->values, dc, nullptr, dp, len, column_count, chunk_len, beta, gamma, omega, dd, db,
                             blinding_factors, s);
        device_vec_mark_ready(v, s);
        lane_sync(s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// The permutation products over resident columns and permutation values
// (column_count x len each); delta powers and blinds are host arrays.
RustError gb_fr_permutation_products_device(void **out, const void *columns_vec, const void *permutations_vec,
                                            size_t len, size_t column_count, size_t chunk_len, RawFr beta_raw,
                                            RawFr gamma_raw, RawFr omega_raw, const RawFr *delta_powers_raw,
                                            const RawFr *blind_values_raw, size_t blinding_factors)
{
    const fr_t *delta_powers = reinterpret_cast<const fr_t *>(delta_powers_raw);
    const fr_t *blind_values = reinterpret_cast<const fr_t *>(blind_values_raw);
    if (!out || len == 0 || column_count == 0 || chunk_len == 0 || !columns_vec || !permutations_vec ||
        !delta_powers || blinding_factors >= len || (blinding_factors != 0 && !blind_values))
        return make_error((int)cudaErrorInvalidValue, "invalid resident permutation product arguments");
    *out = nullptr;
    const size_t sets = (column_count + chunk_len - 1) / chunk_len;
    if (column_count > SIZE_MAX / len || sets > SIZE_MAX / len)
        return make_error((int)cudaErrorInvalidValue, "permutation product size overflow");
    GB_ENTRY_BEGIN
    auto *cv = reinterpret_cast<const fr_device_vec *>(columns_vec);
    auto *pv = reinterpret_cast<const fr_device_vec *>(permutations_vec);
    if (cv->len < column_count * len || pv->len < column_count * len)
        return make_error((int)cudaErrorInvalidValue, "resident permutation columns too short");
    cudaStream_t s = lane_stream();
    device_vec_wait(cv, s);
    device_vec_wait(pv, s);
    auto dd = upload(delta_powers, column_count, s);
    auto db = upload(blind_values, sets * blinding_factors, s);
    fr_device_vec *v = device_vec_new(sets * len, s);
    try {
        permutation_products(v->values, cv->values, nullptr, pv->values, len, column_count, chunk_len,
                             gb::from_raw(beta_raw), gb::from_raw(gamma_raw), gb::from_raw(omega_raw), dd, db,
                             blinding_factors, s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:4451-4548
RustError midnight_sppark_bls12_381_fr_lookup_products(void **out, const RawFr *compressed_inputs_raw, const RawFr *compressed_tables_raw, const RawFr *permuted_inputs_raw, const RawFr *permuted_tables_raw, size_t len, size_t lookup_count, RawFr beta_raw, RawFr gamma_raw, const RawFr *blind_values_raw, size_t blinding_factors)
{
    const fr_t *compressed_inputs = reinterpret_cast<const fr_t *>(compressed_inputs_raw);
    const fr_t *compressed_tables = reinterpret_cast<const fr_t *>(compressed_tables_raw);
    const fr_t *permuted_inputs = reinterpret_cast<const fr_t *>(permuted_inputs_raw);
    const fr_t *permuted_tables = reinterpret_cast<const fr_t *>(permuted_tables_raw);
    const fr_t beta = gb::from_raw(beta_raw);
    const fr_t gamma = gb::from_raw(gamma_raw);
    const fr_t *blind_values = reinterpret_cast<const fr_t *>(blind_values_raw);
    if (!out || len == 0 || lookup_count == 0 || !compressed_inputs || !compressed_tables || !permuted_inputs ||
        !permuted_tables || blinding_factors >= len || (blinding_factors != 0 && !blind_values))
        return make_error((int)cudaErrorInvalidValue, "invalid lookup product arguments");
    *out = nullptr;
    if (lookup_count > SIZE_MAX / len) return make_error((int)cudaErrorInvalidValue, "lookup product size overflow");
    GB_ENTRY_BEGIN
    const size_t total = lookup_count * len;
    cudaStream_t s = lane_stream();
    auto a = upload(compressed_inputs, total, s);
    auto b = upload(compressed_tables, total, s);
    auto c = upload(permuted_inputs, total, s);
    auto d = upload(permuted_tables, total, s);
    auto bl = upload(blind_values, lookup_count * blinding_factors, s);
    fr_device_vec *v = device_vec_new(total, s);
    try {
        lookup_products(v->values, a, b, c, d, len, lookup_count, beta, gamma, bl, blinding_factors, s);
        device_vec_mark_ready(v, s);
        lane_sync(s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:4550-4634: the four lookup columns already resident,
// laid out [compressed inputs | compressed tables | permuted inputs | permuted tables]
RustError midnight_sppark_bls12_381_fr_lookup_products_device(void **out, const void *trace_lagrange, size_t len, size_t lookup_count, RawFr beta_raw, RawFr gamma_raw, const RawFr *blind_values_raw, size_t blinding_factors)
{
    const fr_t beta = gb::from_raw(beta_raw);
    const fr_t gamma = gb::from_raw(gamma_raw);
    const fr_t *blind_values = reinterpret_cast<const fr_t *>(blind_values_raw);
    if (!out || len == 0 || lookup_count == 0 || !trace_lagrange || blinding_factors >= len ||
        (blinding_factors != 0 && !blind_values))
        return make_error((int)cudaErrorInvalidValue, "invalid resident lookup product arguments");
    *out = nullptr;
    if (lookup_count > SIZE_MAX / len)
        return make_error((int)cudaErrorInvalidValue, "resident lookup product size overflow");
    GB_ENTRY_BEGIN
    const size_t total = lookup_count * len;
    auto *tr = reinterpret_cast<const fr_device_vec *>(trace_lagrange);
    if (tr->len != total * 4) return make_error((int)cudaErrorInvalidValue, "resident lookup trace length mismatch");
    cudaStream_t s = lane_stream();
    device_vec_wait(tr, s);
    auto bl = upload(blind_values, lookup_count * blinding_factors, s);
    fr_device_vec *v = device_vec_new(total, s);
    try {
        const fr_t *base = tr->values;
        lookup_products(v->values, base, base + total, base + 2 * total, base + 3 * total, len, lookup_count, beta,
                        gamma, bl, blinding_factors, s);
        device_vec_mark_ready(v, s);
        lane_sync(s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3181-3240 (vanishing/prover.rs:141-220,304-318)
RustError midnight_sppark_bls12_381_fr_device_quotient_pieces(void **out, const void *quotient_vec, size_t poly_len, size_t piece_count, const RawFr *blinds_raw, size_t blind_count)
{
    const fr_t *blinds = reinterpret_cast<const fr_t *>(blinds_raw);
    if (!out || !quotient_vec || poly_len < 2 || piece_count < 2 || blind_count != piece_count - 1 || !blinds ||
        piece_count > SIZE_MAX / poly_len)
        return make_error((int)cudaErrorInvalidValue, "invalid resident quotient piece arguments");
    *out = nullptr;
    GB_ENTRY_BEGIN
    auto *q = reinterpret_cast<const fr_device_vec *>(quotient_vec);
    if (q->len < (poly_len - 1) * piece_count)
        return make_error((int)cudaErrorInvalidValue, "resident quotient is too short");
    cudaStream_t s = lane_stream();
    device_vec_wait(q, s);
    auto b = upload(blinds, blind_count, s);
    fr_device_vec *v = device_vec_new(poly_len * piece_count, s);
    try {
        quotient_pieces_kernel<<<blocks_for(poly_len * piece_count, 256), 256, 0, s>>>(v->values, q->values, poly_len,
                                                                                     piece_count);
        GB_CHECK_LAUNCH();
        blind_quotient_pieces_kernel<<<1, 32, 0, s>>>(v->values, b, poly_len, piece_count);
        GB_CHECK_LAUNCH();
        device_vec_mark_ready(v, s);
        lane_sync(s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3242-3278
RustError midnight_sppark_bls12_381_fr_device_poly_lincomb(void **out, const void *polys_vec, size_t poly_len, size_t poly_count, const RawFr *scalars_raw, size_t scalar_count)
{
    const fr_t *scalars = reinterpret_cast<const fr_t *>(scalars_raw);
    if (!out || !polys_vec || poly_len == 0 || poly_count == 0 || !scalars || scalar_count != poly_count)
        return make_error((int)cudaErrorInvalidValue, "invalid resident lincomb arguments");
    *out = nullptr;
    GB_ENTRY_BEGIN
    auto *pv = reinterpret_cast<const fr_device_vec *>(polys_vec);
    if (poly_count > SIZE_MAX / poly_len || pv->len < poly_len * poly_count)
        return make_error((int)cudaErrorInvalidValue, "resident lincomb source too short");
    cudaStream_t s = lane_stream();
    device_vec_wait(pv, s);
    auto k = upload(scalars, scalar_count, s);
    fr_device_vec *v = device_vec_new(poly_len, s);
    try {
        lincomb_kernel<<<blocks_for(poly_len, 256), 256, 0, s>>>(v->values, pv->values, k, poly_len, poly_count);
        GB_CHECK_LAUNCH();
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// ---------------------------------------------------------------- device vectors
// bls12_381_g1_msm.cu:2741-2780
RustError midnight_sppark_bls12_381_fr_device_vec_upload(void **out, const RawFr *values_raw, size_t len)
{
    const fr_t *values = reinterpret_cast<const fr_t *>(values_raw);
    if (!out || (len && !values)) return make_error((int)cudaErrorInvalidValue, "invalid device vector upload");
    *out = nullptr;
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    fr_device_vec *v = device_vec_new(len, s);
    try {
        h2d(v->values, values, len * sizeof(fr_t), s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:2782-2830: several host slices concatenated
RustError midnight_sppark_bls12_381_fr_device_vec_upload_many(void **out, const RawFr *const *values_raw, const size_t *lengths, size_t count)
{
    const fr_t *const *values = reinterpret_cast<const fr_t *const *>(values_raw);
    if (!out || (count && (!values || !lengths)))
        return make_error((int)cudaErrorInvalidValue, "invalid device vector upload");
    *out = nullptr;
    GB_ENTRY_BEGIN
    size_t total = 0;
    for (size_t i = 0; i < count; i++) {
        if (lengths[i] && !values[i]) return make_error((int)cudaErrorInvalidValue, "null upload slice");
        total += lengths[i];
    }
    cudaStream_t s = lane_stream();
    fr_device_vec *v = device_vec_new(total, s);
    try {
        size_t off = 0;
        for (size_t i = 0; i < count; i++) {
            h2d(v->values + off, values[i], lengths[i] * sizeof(fr_t), s);
            off += lengths[i];
        }
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3000-3060
RustError midnight_sppark_bls12_381_fr_device_vec_download(RawFr *out_raw, const void *device_vec, size_t len)
{
    fr_t *out = reinterpret_cast<fr_t *>(out_raw);
    if (!device_vec || (len && !out)) return make_error((int)cudaErrorInvalidValue, "invalid device vector download");
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<const fr_device_vec *>(device_vec);
    if (len > v->len) return make_error((int)cudaErrorInvalidValue, "download longer than device vector");
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    d2h(out, v->values, len * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

__global__ void scatter_kernel(fr_t *dst, const uint32_t *__restrict__ idx, const fr_t *__restrict__ vals,
                               size_t count)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) dst[idx[i]] = vals[i];
}

// bls12_381_g1_msm.cu:2860-2905
RustError midnight_sppark_bls12_381_fr_device_vec_scatter_host(void *device_vec, const uint32_t *indices, const RawFr *values_raw, size_t count)
{
    const fr_t *values = reinterpret_cast<const fr_t *>(values_raw);
    if (!device_vec || (count && (!indices || !values)))
        return make_error((int)cudaErrorInvalidValue, "invalid device vector scatter");
    if (count == 0) return ok();
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<fr_device_vec *>(device_vec);
    for (size_t i = 0; i < count; i++)
        if (indices[i] >= v->len) return make_error((int)cudaErrorInvalidValue, "scatter index out of range");
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    dev_buf<uint32_t> di(count, s);
    h2d(di, indices, count * sizeof(uint32_t), s);
    auto dv = upload(values, count, s);
    scatter_kernel<<<blocks_for(count, 256), 256, 0, s>>>(v->values, di, dv, count);
    GB_CHECK_LAUNCH();
    device_vec_mark_ready(v, s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:2907-2950: [prefix device vector | host suffix]
RustError midnight_sppark_bls12_381_fr_device_vec_concat_host(void **out, const void *prefix_device_vec, const RawFr *suffix_raw, size_t suffix_len)
{
    const fr_t *suffix = reinterpret_cast<const fr_t *>(suffix_raw);
    if (!out || !prefix_device_vec || (suffix_len && !suffix))
        return make_error((int)cudaErrorInvalidValue, "invalid device vector concat");
    *out = nullptr;
    GB_ENTRY_BEGIN
    auto *p = reinterpret_cast<const fr_device_vec *>(prefix_device_vec);
    cudaStream_t s = lane_stream();
    device_vec_wait(p, s);
    fr_device_vec *v = device_vec_new(p->len + suffix_len, s);
    try {
        if (p->len)
            GB_CUDA_OK(cudaMemcpyAsync(v->values, p->values, p->len * sizeof(fr_t), cudaMemcpyDeviceToDevice, s));
        h2d(v->values + p->len, suffix, suffix_len * sizeof(fr_t), s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:2952-2998
RustError midnight_sppark_bls12_381_fr_device_vec_concat_many_host(void **out, const void *const *sources, size_t source_count, const RawFr *suffix_raw, size_t suffix_len)
{
    const fr_t *suffix = reinterpret_cast<const fr_t *>(suffix_raw);
    if (!out || (source_count && !sources) || (suffix_len && !suffix))
        return make_error((int)cudaErrorInvalidValue, "invalid device vector concat");
    *out = nullptr;
    GB_ENTRY_BEGIN
    size_t total = suffix_len;
    for (size_t i = 0; i < source_count; i++) {
        if (!sources[i]) return make_error((int)cudaErrorInvalidValue, "null concat source");
        total += reinterpret_cast<const fr_device_vec *>(sources[i])->len;
    }
    cudaStream_t s = lane_stream();
    fr_device_vec *v = device_vec_new(total, s);
    try {
        size_t off = 0;
        for (size_t i = 0; i < source_count; i++) {
            auto *src = reinterpret_cast<const fr_device_vec *>(sources[i]);
            device_vec_wait(src, s);
            if (src->len)
                GB_CUDA_OK(cudaMemcpyAsync(v->values + off, src->values, src->len * sizeof(fr_t),
                                           cudaMemcpyDeviceToDevice, s));
            off += src->len;
        }
        h2d(v->values + off, suffix, suffix_len * sizeof(fr_t), s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3062-3120: selected polynomials of a resident batch
RustError midnight_sppark_bls12_381_fr_device_vec_gather_polys(void **out, const void *source_device_vec,
                                                               size_t poly_len, const uint32_t *indices,
                                                               size_t index_count)
{
    if (!out || !source_device_vec || (index_count && !indices))
        return make_error((int)cudaErrorInvalidValue, "invalid device vector gather");
    *out = nullptr;
    GB_ENTRY_BEGIN
    auto *src = reinterpret_cast<const fr_device_vec *>(source_device_vec);
    for (size_t i = 0; i < index_count; i++)
        if (poly_len && ((size_t)indices[i] + 1) * poly_len > src->len)
            return make_error((int)cudaErrorInvalidValue, "gather index out of range");
    cudaStream_t s = lane_stream();
    device_vec_wait(src, s);
    fr_device_vec *v = device_vec_new(poly_len * index_count, s);
    try {
        for (size_t i = 0; i < index_count; i++)
            if (poly_len)
                GB_CUDA_OK(cudaMemcpyAsync(v->values + i * poly_len, src->values + (size_t)indices[i] * poly_len,
                                           poly_len * sizeof(fr_t), cudaMemcpyDeviceToDevice, s));
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3101-3179: per polynomial the first nonzero
// coefficient (starts) and the nonzero count, then the suffixes from the
// first nonzero coefficient on, packed polynomial after polynomial.  With
// out == NULL and out_capacity == 0 only *out_len (the packed length) is
// returned.
RustError midnight_sppark_bls12_381_fr_device_vec_download_nonzero_suffixes(RawFr *out, size_t out_capacity,
                                                                           size_t *out_len, size_t *starts,
                                                                           size_t *nonzero_counts,
                                                                           const void *device_vec,
                                                                           size_t scalar_offset, size_t poly_len,
                                                                           size_t count)
{
    if (!out_len || !starts || !device_vec || poly_len == 0 || count == 0 || count > SIZE_MAX / poly_len ||
        (out_capacity != 0 && !out))
        return make_error((int)cudaErrorInvalidValue, "invalid nonzero suffix download arguments");
    *out_len = 0;
    auto *v = reinterpret_cast<const fr_device_vec *>(device_vec);
    const size_t required = poly_len * count;
    if (scalar_offset > v->len || required > v->len - scalar_offset)
        return make_error((int)cudaErrorInvalidValue, "nonzero suffix range exceeds device vector");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    const fr_t *base = v->values + scalar_offset;
    dev_buf<unsigned long long> d_stats(2 * count, s);
    const uint32_t slices = (uint32_t)((poly_len + kSuffixSlice - 1) / kSuffixSlice);
    nonzero_init_kernel<<<blocks_for(count, 256), 256, 0, s>>>(d_stats, count, poly_len);
    GB_CHECK_LAUNCH();
    for (size_t c0 = 0; c0 < count; c0 += 65535) {
        const unsigned m = (unsigned)std::min<size_t>(65535, count - c0);
        nonzero_stats_kernel<<<dim3(slices, m), 256, 0, s>>>(d_stats.get() + c0, d_stats.get() + count + c0,
                                                             base + c0 * poly_len, poly_len);
        GB_CHECK_LAUNCH();
    }
    std::vector<unsigned long long> h(2 * count);
    d2h(h.data(), d_stats, 2 * count * sizeof(unsigned long long), s);
    lane_sync(s);
    size_t total = 0;
    for (size_t p = 0; p < count; p++) {
        starts[p] = (size_t)h[p];
        if (nonzero_counts) nonzero_counts[p] = (size_t)h[count + p];
        total += poly_len - starts[p];
    }
    if (!out && out_capacity == 0) {
        *out_len = total;
        return ok();
    }
    if (total > out_capacity) return make_error((int)cudaErrorInvalidValue, "nonzero suffix output is too small");
    size_t cursor = 0;
    for (size_t p = 0; p < count; p++) {
        const size_t n = poly_len - starts[p];
        if (n) d2h(out + cursor, base + p * poly_len + starts[p], n * sizeof(fr_t), s);
        cursor += n;
    }
    lane_sync(s);
    *out_len = total;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:6406-6423 (test hooks): scales a resident vector in
// place on this lane after holding the lane's stream back for delay_ms; the
// vector's ready event moves past the scaling, so a reader on another lane
// waits for it
RustError midnight_sppark_test_delayed_scale(void *device_vec, RawFr scale, uint32_t delay_ms)
{
    if (!device_vec) return make_error((int)cudaErrorInvalidValue, "null device vector");
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<fr_device_vec *>(device_vec);
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    lane_sync(s);
    stream_host_delay(s, delay_ms);
    if (v->len) launch_mul_assign(v->values, gb::from_raw(scale), v->len, s);
    device_vec_mark_ready(v, s);
    return ok();
    GB_ENTRY_END
}

void midnight_sppark_bls12_381_fr_device_vec_free(void *device_vec)
{
    device_vec_delete(reinterpret_cast<fr_device_vec *>(device_vec));
}

// Length of a resident vector (library extension used by the host mirror).
size_t gb_fr_device_vec_len(const void *device_vec)
{
    return device_vec ? reinterpret_cast<const fr_device_vec *>(device_vec)->len : 0;
}

}  // extern "C"
