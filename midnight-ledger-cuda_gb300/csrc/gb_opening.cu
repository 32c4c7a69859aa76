// KZG opening helpers on the device: batched polynomial evaluation at a
// point (midnight-sppark-msm/src/bls12_381_g1_msm.cu:3985-4031,
// midnight_sppark_bls12_381_fr_device_eval_polys) and the Kate quotient
// (f(X) - f(z)) / (X - z) of every polynomial of a batch (the division the
// reference's multi-open computes with its kate scan, .cu:1923-1959).
//
// Evaluation: z^i is tabulated by a multiplicative scan, each block sums a
// slice of c_i z^i, a second pass adds the slices.  Kate quotient: with
// S_k = sum_{j >= k} f_j z^j (an additive suffix scan), q_i = S_{i+1} z^-(i+1)
// for i < n-1 and q_{n-1} = 0; z = 0 is the shift q_i = f_{i+1}.
#include <algorithm>
#include <vector>

#include "gb_vec.cuh"

namespace gb {

static constexpr int kEvalThreads = 256;
static constexpr size_t kEvalSlice = 8192;

__global__ void __launch_bounds__(kEvalThreads) eval_slices_kernel(const fr_t *__restrict__ polys, size_t len,
                                                                   const fr_t *__restrict__ pw, uint32_t slices,
                                                                   fr_t *__restrict__ partial)
{
    __shared__ fr_t sh[kEvalThreads];
    const size_t p = blockIdx.y, sl = blockIdx.x;
    const fr_t *c = polys + p * len;
    size_t lo = sl * kEvalSlice, hi = min(lo + kEvalSlice, len);
    fr_t acc = fr_t::zero();
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) acc = acc + c[i] * pw[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (unsigned off = blockDim.x / 2; off; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[p * slices + sl] = sh[0];
}

__global__ void sum_slices_kernel(const fr_t *__restrict__ partial, uint32_t slices, size_t count,
                                  fr_t *__restrict__ out)
{
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    fr_t acc = fr_t::zero();
    for (uint32_t s = 0; s < slices; s++) acc = acc + partial[p * slices + s];
    out[p] = acc;
}

void eval_polys(fr_t *d_out, const fr_t *polys, size_t len, size_t count, const fr_t &z, cudaStream_t s)
{
    dev_buf<fr_t> pw(len, s);
    omega_powers(pw, z, len, s);
    uint32_t slices = (uint32_t)((len + kEvalSlice - 1) / kEvalSlice);
    dev_buf<fr_t> partial(count * slices, s);
    eval_slices_kernel<<<dim3(slices, (unsigned)count), kEvalThreads, 0, s>>>(polys, len, pw, slices, partial);
    GB_CHECK_LAUNCH();
    sum_slices_kernel<<<blocks_for(count, 128), 128, 0, s>>>(partial, slices, count, d_out);
    GB_CHECK_LAUNCH();
}

// evaluations of a batch of (polynomial, point) pairs: pair p reads the
// coefficients at polys[p] and the power row pw + row[p] * len
struct eval_pair {
    const fr_t *polys;
    uint32_t row;
};

__global__ void __launch_bounds__(kEvalThreads) eval_slices_many_kernel(const eval_pair *__restrict__ pairs, size_t len,
                                                                        const fr_t *__restrict__ pw, uint32_t slices,
                                                                        fr_t *__restrict__ partial)
{
    __shared__ fr_t sh[kEvalThreads];
    const size_t p = blockIdx.y, sl = blockIdx.x;
    const eval_pair e = pairs[p];
    const fr_t *c = e.polys;
    const fr_t *z = pw + (size_t)e.row * len;
    size_t lo = sl * kEvalSlice, hi = min(lo + kEvalSlice, len);
    fr_t acc = fr_t::zero();
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) acc = acc + c[i] * z[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (unsigned off = blockDim.x / 2; off; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[p * slices + sl] = sh[0];
}

// evaluations of pairs (pair p: coefficients at pairs[p].polys of len
// values, at the host point points[pairs[p].row]) into d_out; the powers of
// every point tabulated once
static void eval_pairs(fr_t *d_out, const std::vector<eval_pair> &pairs, const RawFr *points, size_t npoints,
                       size_t len, cudaStream_t s)
{
    const size_t total = pairs.size();
    if (!total) return;
    dev_buf<fr_t> d_points(npoints, s), pw(npoints * len, s);
    dev_buf<eval_pair> d_pairs(total, s);
    h2d(d_points, points, npoints * sizeof(fr_t), s);
    h2d(d_pairs, pairs.data(), total * sizeof(eval_pair), s);
    if (len <= ((size_t)1 << 24)) {
        omega_powers_many(pw, d_points, npoints, len, s);
    } else {
        for (size_t q = 0; q < npoints; q++) omega_powers(pw.get() + q * len, from_raw(points[q]), len, s);
    }
    const uint32_t slices = (uint32_t)((len + kEvalSlice - 1) / kEvalSlice);
    const size_t chunk = 65535;  // grid.y limit
    dev_buf<fr_t> partial(std::min(total, chunk) * slices, s);
    for (size_t b = 0; b < total; b += chunk) {
        const size_t m = std::min(chunk, total - b);
        eval_slices_many_kernel<<<dim3(slices, (unsigned)m), kEvalThreads, 0, s>>>(d_pairs.get() + b, len, pw, slices,
                                                                                   partial);
        GB_CHECK_LAUNCH();
        sum_slices_kernel<<<blocks_for(m, 128), 128, 0, s>>>(partial, slices, m, d_out + b);
        GB_CHECK_LAUNCH();
    }
}

// g[p][j] = f[p][j] * z^j
__global__ void scale_by_powers_kernel(const fr_t *__restrict__ f, const fr_t *__restrict__ pw, size_t len,
                                       size_t total, fr_t *__restrict__ g)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < total) g[t] = f[t] * pw[t % len];
}

// q[p][i] = S[p][i+1] * zinv^(i+1), q[p][len-1] = 0, where S is the suffix sum
__global__ void kate_finish_kernel(const fr_t *__restrict__ S, const fr_t *__restrict__ zinv_pw, size_t len,
                                   size_t total, fr_t *__restrict__ q)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    size_t i = t % len;
    q[t] = i + 1 < len ? S[t + 1] * zinv_pw[i + 1] : fr_t::zero();
}

__global__ void shift_down_kernel(const fr_t *__restrict__ f, size_t len, size_t total, fr_t *__restrict__ q)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    size_t i = t % len;
    q[t] = i + 1 < len ? f[t + 1] : fr_t::zero();
}

void kate_divide(fr_t *d_out, const fr_t *f, size_t len, size_t count, const fr_t &z, cudaStream_t s)
{
    const size_t total = len * count;
    if (!total) return;
    if (z.is_zero()) {
        shift_down_kernel<<<blocks_for(total, 256), 256, 0, s>>>(f, len, total, d_out);
        GB_CHECK_LAUNCH();
        return;
    }
    // powers of z and of 1/z (rows 0 and 1 of pws), in one launch pair up
    // to 2^24 coefficients
    dev_buf<fr_t> zs(2, s), pws(2 * len, s), g(total, s);
    const fr_t hz[2] = {z, z.inverse()};
    if (len <= ((size_t)1 << 24)) {
        h2d(zs, hz, sizeof(hz), s);
        omega_powers_many(pws, zs, 2, len, s);
    } else {
        omega_powers(pws, hz[0], len, s);
        omega_powers(pws.get() + len, hz[1], len, s);
    }
    const fr_t *pw = pws.get(), *ipw = pws.get() + len;
    scale_by_powers_kernel<<<blocks_for(total, 256), 256, 0, s>>>(f, pw, len, total, g);
    GB_CHECK_LAUNCH();
    for (size_t p = 0; p < count; p++) suffix_sum(g.get() + p * len, g.get() + p * len, len, s);
    kate_finish_kernel<<<blocks_for(total, 256), 256, 0, s>>>(g, ipw, len, total, d_out);
    GB_CHECK_LAUNCH();
}

// q[k][i] = sum over the items t of q k (q_offsets[k] <= t < q_offsets[k+1])
// of coeffs[t] * poly(item_polys[t])[i]; polynomials through a pointer table
__global__ void multiopen_q_kernel(fr_t *__restrict__ out, const fr_t *const *__restrict__ polys,
                                   const uint32_t *__restrict__ q_offsets, const uint32_t *__restrict__ item_polys,
                                   const fr_t *__restrict__ coeffs, size_t len, size_t q_count)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= len * q_count) return;
    const size_t k = t / len, i = t - k * len;
    fr_t acc = fr_t::zero();
    for (uint32_t it = q_offsets[k]; it < q_offsets[k + 1]; it++) acc = acc + polys[item_polys[it]][i] * coeffs[it];
    out[t] = acc;
}

// out[i] = sum_p k[p] * polys[p][i], polynomials through a pointer table
__global__ void lincomb_table_kernel(fr_t *__restrict__ out, const fr_t *const *__restrict__ polys,
                                     const fr_t *__restrict__ k, size_t len, size_t count)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    fr_t acc = fr_t::zero();
    for (size_t p = 0; p < count; p++) acc = acc + polys[p][i] * k[p];
    out[i] = acc;
}

// checks of the q description shared by both preparation entry points
static const char *check_q_layout(const uint32_t *q_offsets, size_t q_offsets_len, const uint32_t *q_poly_indices,
                                  size_t q_items_len, size_t poly_count, const uint32_t *query_poly_indices,
                                  const uint32_t *query_point_indices, size_t query_count, size_t point_count)
{
    const size_t q_count = q_offsets_len - 1;
    if (q_offsets[0] != 0 || q_offsets[q_count] != q_items_len) return "invalid multi-open q offsets";
    for (size_t k = 0; k < q_count; k++)
        if (q_offsets[k] > q_offsets[k + 1]) return "non-monotonic multi-open q offsets";
    for (size_t t = 0; t < q_items_len; t++)
        if (q_poly_indices[t] >= poly_count) return "multi-open q polynomial index out of range";
    for (size_t r = 0; r < query_count; r++)
        if (query_poly_indices[r] >= poly_count || query_point_indices[r] >= point_count)
            return "multi-open query index out of range";
    return nullptr;
}

// the q polynomials into d_q and the query evaluations into d_eval, the
// polynomials named by a host table of device pointers
static void multiopen_prepare_core(fr_t *d_q, fr_t *d_eval, const std::vector<const fr_t *> &polys, size_t len,
                                   const uint32_t *q_offsets, size_t q_offsets_len, const uint32_t *q_poly_indices,
                                   const RawFr *q_coefficients, size_t q_items_len, const RawFr *points,
                                   size_t point_count, const uint32_t *query_poly_indices,
                                   const uint32_t *query_point_indices, size_t query_count, cudaStream_t s)
{
    const size_t q_count = q_offsets_len - 1;
    dev_buf<const fr_t *> d_polys(polys.size(), s);
    dev_buf<uint32_t> d_offsets(q_offsets_len, s), d_items(q_items_len, s);
    dev_buf<fr_t> d_coeffs(q_items_len, s);
    h2d(d_polys, polys.data(), polys.size() * sizeof(const fr_t *), s);
    h2d(d_offsets, q_offsets, q_offsets_len * sizeof(uint32_t), s);
    h2d(d_items, q_poly_indices, q_items_len * sizeof(uint32_t), s);
    h2d(d_coeffs, q_coefficients, q_items_len * sizeof(fr_t), s);
    if (q_count) {
        multiopen_q_kernel<<<blocks_for(len * q_count, 256), 256, 0, s>>>(d_q, d_polys, d_offsets, d_items, d_coeffs,
                                                                           len, q_count);
        GB_CHECK_LAUNCH();
    }
    std::vector<eval_pair> pairs(query_count);
    for (size_t r = 0; r < query_count; r++) pairs[r] = eval_pair{polys[query_poly_indices[r]], query_point_indices[r]};
    eval_pairs(d_eval, pairs, points, point_count, len, s);
}

}  // namespace gb

using namespace gb;

extern "C" {

// bls12_381_g1_msm.cu:3985-4031: out[p] = sum_i polys[p][i] * point^i
RustError midnight_sppark_bls12_381_fr_device_eval_polys(RawFr *out_raw, const void *device_vec, size_t poly_len,
                                                         size_t poly_count, RawFr point_raw)
{
    if (!out_raw || !device_vec || poly_len == 0 || poly_count == 0 || poly_count > SIZE_MAX / poly_len)
        return make_error((int)cudaErrorInvalidValue, "invalid resident polynomial evaluation arguments");
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<const fr_device_vec *>(device_vec);
    if (v->len != poly_len * poly_count)
        return make_error((int)cudaErrorInvalidValue, "resident polynomial evaluation shape mismatch");
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    dev_buf<fr_t> d(poly_count, s);
    eval_polys(d, v->values, poly_len, poly_count, from_raw(point_raw), s);
    d2h(out_raw, d, poly_count * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// Several evaluations in one call (no reference counterpart: the reference
// makes one midnight_sppark_bls12_381_fr_device_eval_polys call per point).
// Request r evaluates the counts[r] polynomials of poly_len coefficients held
// by vecs[r] at points[r]; out receives the values request by request.
RustError gb_fr_device_eval_many(RawFr *out_raw, const void *const *vecs, const size_t *counts,
                                 const RawFr *points_raw, size_t requests, size_t poly_len)
{
    if (!out_raw || !vecs || !counts || !points_raw || requests == 0 || poly_len == 0 || requests > 65535)
        return make_error((int)cudaErrorInvalidValue, "invalid batched evaluation arguments");
    GB_ENTRY_BEGIN
    std::vector<eval_pair> pairs;
    for (size_t r = 0; r < requests; r++) {
        auto *v = reinterpret_cast<const fr_device_vec *>(vecs[r]);
        if (!v || counts[r] == 0 || counts[r] > SIZE_MAX / poly_len || v->len != counts[r] * poly_len)
            return make_error((int)cudaErrorInvalidValue, "batched evaluation shape mismatch");
        for (size_t p = 0; p < counts[r]; p++) pairs.push_back(eval_pair{v->values + p * poly_len, (uint32_t)r});
    }
    cudaStream_t s = lane_stream();
    for (size_t r = 0; r < requests; r++) device_vec_wait(reinterpret_cast<const fr_device_vec *>(vecs[r]), s);
    const size_t total = pairs.size();
    dev_buf<fr_t> d_out(total, s);
    eval_pairs(d_out, pairs, points_raw, requests, poly_len, s);
    d2h(out_raw, d_out, total * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// Kate quotients (f - f(z)) / (X - z) of poly_count resident polynomials of
// poly_len coefficients, into a new device vector of the same shape.
RustError gb_fr_device_kate_divide(void **out, const void *device_vec, size_t poly_len, size_t poly_count,
                                   RawFr point_raw)
{
    if (!out || !device_vec || poly_len == 0 || poly_count == 0 || poly_count > SIZE_MAX / poly_len)
        return make_error((int)cudaErrorInvalidValue, "invalid Kate division arguments");
    *out = nullptr;
    GB_ENTRY_BEGIN
    auto *v = reinterpret_cast<const fr_device_vec *>(device_vec);
    if (v->len != poly_len * poly_count)
        return make_error((int)cudaErrorInvalidValue, "Kate division shape mismatch");
    cudaStream_t s = lane_stream();
    device_vec_wait(v, s);
    fr_device_vec *r = device_vec_new(poly_len * poly_count, s);
    try {
        kate_divide(r->values, v->values, poly_len, poly_count, from_raw(point_raw), s);
        device_vec_mark_ready(r, s);
    } catch (...) {
        device_vec_delete(r);
        throw;
    }
    *out = r;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3600-3721: host polynomials [poly_count][poly_len];
// q_out [q_count][poly_len] (q k = the sum of its items' coefficient times
// polynomial), eval_out[r] = polynomial query_poly_indices[r] at
// points[query_point_indices[r]]
RustError midnight_sppark_bls12_381_fr_multiopen_prepare(
    RawFr *q_out, RawFr *eval_out, const RawFr *polys, size_t poly_len, size_t poly_count, const uint32_t *q_offsets,
    size_t q_offsets_len, const uint32_t *q_poly_indices, const RawFr *q_coefficients, size_t q_items_len,
    const RawFr *points, size_t point_count, const uint32_t *query_poly_indices, const uint32_t *query_point_indices,
    size_t query_count)
{
    if (poly_len == 0 || poly_count == 0 || q_offsets_len < 2 || !q_out || !eval_out || !polys || !q_offsets ||
        !q_poly_indices || !q_coefficients || !points || point_count == 0 || !query_poly_indices ||
        !query_point_indices)
        return make_error((int)cudaErrorInvalidValue, "invalid multi-open preparation arguments");
    if (const char *bad = check_q_layout(q_offsets, q_offsets_len, q_poly_indices, q_items_len, poly_count,
                                         query_poly_indices, query_point_indices, query_count, point_count))
        return make_error((int)cudaErrorInvalidValue, bad);
    const size_t q_count = q_offsets_len - 1;
    if (poly_count > SIZE_MAX / poly_len || q_count > SIZE_MAX / poly_len || point_count > SIZE_MAX / poly_len)
        return make_error((int)cudaErrorInvalidValue, "multi-open preparation size overflow");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    dev_buf<fr_t> d_polys(poly_len * poly_count, s), d_q(poly_len * q_count, s), d_eval(query_count, s);
    h2d(d_polys, polys, poly_len * poly_count * sizeof(fr_t), s);
    std::vector<const fr_t *> table(poly_count);
    for (size_t p = 0; p < poly_count; p++) table[p] = d_polys.get() + p * poly_len;
    multiopen_prepare_core(d_q, d_eval, table, poly_len, q_offsets, q_offsets_len, q_poly_indices, q_coefficients,
                           q_items_len, points, point_count, query_poly_indices, query_point_indices, query_count, s);
    d2h(q_out, d_q, poly_len * q_count * sizeof(fr_t), s);
    d2h(eval_out, d_eval, query_count * sizeof(fr_t), s);
    lane_sync(s);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3723-3871: the same over resident polynomials; poly
// reference p names polynomial index of source 0 (dynamic), 1 (fixed) or 2
// (extra), each a device vector of whole polynomials.  q_out (host) and
// q_device_out (a new device vector) are each optional, not both absent.
RustError midnight_sppark_bls12_381_fr_multiopen_prepare_device(
    RawFr *q_out, void **q_device_out, RawFr *eval_out, const void *dynamic_source, const void *fixed_source,
    const void *extra_source, size_t poly_len, const RawDevicePolyRef *poly_refs, size_t poly_count,
    const uint32_t *q_offsets, size_t q_offsets_len, const uint32_t *q_poly_indices, const RawFr *q_coefficients,
    size_t q_items_len, const RawFr *points, size_t point_count, const uint32_t *query_poly_indices,
    const uint32_t *query_point_indices, size_t query_count)
{
    if (poly_len == 0 || poly_count == 0 || q_offsets_len < 2 || (!q_out && !q_device_out) || !eval_out ||
        !dynamic_source || !fixed_source || !extra_source || !poly_refs || !q_offsets || !q_poly_indices ||
        !q_coefficients || !points || point_count == 0 || !query_poly_indices || !query_point_indices)
        return make_error((int)cudaErrorInvalidValue, "invalid resident multi-open arguments");
    if (q_device_out) *q_device_out = nullptr;
    const fr_device_vec *src[3] = {reinterpret_cast<const fr_device_vec *>(dynamic_source),
                                   reinterpret_cast<const fr_device_vec *>(fixed_source),
                                   reinterpret_cast<const fr_device_vec *>(extra_source)};
    std::vector<const fr_t *> table(poly_count);
    for (size_t p = 0; p < poly_count; p++) {
        const RawDevicePolyRef r = poly_refs[p];
        if (r.source > 2 || (size_t)r.index >= src[r.source]->len / poly_len)
            return make_error((int)cudaErrorInvalidValue, "resident polynomial reference out of range");
        table[p] = src[r.source]->values + (size_t)r.index * poly_len;
    }
    if (const char *bad = check_q_layout(q_offsets, q_offsets_len, q_poly_indices, q_items_len, poly_count,
                                         query_poly_indices, query_point_indices, query_count, point_count))
        return make_error((int)cudaErrorInvalidValue, bad);
    const size_t q_count = q_offsets_len - 1;
    if (q_count > SIZE_MAX / poly_len || point_count > SIZE_MAX / poly_len)
        return make_error((int)cudaErrorInvalidValue, "multi-open preparation size overflow");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    for (const fr_device_vec *v : src) device_vec_wait(v, s);
    fr_device_vec *q = device_vec_new(poly_len * q_count, s);
    try {
        dev_buf<fr_t> d_eval(query_count, s);
        multiopen_prepare_core(q->values, d_eval, table, poly_len, q_offsets, q_offsets_len, q_poly_indices,
                               q_coefficients, q_items_len, points, point_count, query_poly_indices,
                               query_point_indices, query_count, s);
        device_vec_mark_ready(q, s);
        if (q_out) d2h(q_out, q->values, poly_len * q_count * sizeof(fr_t), s);
        d2h(eval_out, d_eval, query_count * sizeof(fr_t), s);
        lane_sync(s);
    } catch (...) {
        device_vec_delete(q);
        throw;
    }
    if (q_device_out) *q_device_out = q;
    else device_vec_delete(q);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:3873-3983: f = sum_k scalars[k] * floor(q_k / prod_j
// (X - points[j])) over q k's points (point_offsets[k] <= j <
// point_offsets[k+1]), one Kate division per point; a new device vector of
// poly_len coefficients
RustError midnight_sppark_bls12_381_fr_multiopen_f_poly_device(void **out, const void *q_device_vec, size_t poly_len,
                                                               const uint32_t *point_offsets,
                                                               size_t point_offsets_len, const RawFr *points,
                                                               size_t point_count, const RawFr *combination_scalars,
                                                               size_t scalar_count)
{
    if (!out || !q_device_vec || poly_len < 2 || !point_offsets || point_offsets_len < 2 || !points ||
        !combination_scalars)
        return make_error((int)cudaErrorInvalidValue, "invalid resident f-polynomial arguments");
    *out = nullptr;
    const size_t q_count = point_offsets_len - 1;
    auto *qv = reinterpret_cast<const fr_device_vec *>(q_device_vec);
    if (q_count != scalar_count || q_count > SIZE_MAX / poly_len || qv->len != q_count * poly_len ||
        point_offsets[0] != 0 || point_offsets[q_count] != point_count)
        return make_error((int)cudaErrorInvalidValue, "resident f-polynomial shape mismatch");
    for (size_t k = 0; k < q_count; k++)
        if (point_offsets[k] > point_offsets[k + 1])
            return make_error((int)cudaErrorInvalidValue, "non-monotonic f-polynomial point offsets");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    device_vec_wait(qv, s);
    dev_buf<fr_t> divided(q_count * poly_len, s), work(2 * poly_len, s);
    std::vector<const fr_t *> table(q_count);
    for (size_t k = 0; k < q_count; k++) {
        const fr_t *cur = qv->values + k * poly_len;
        const uint32_t p0 = point_offsets[k], p1 = point_offsets[k + 1];
        for (uint32_t j = p0; j < p1; j++) {
            fr_t *dst = j + 1 == p1 ? divided.get() + k * poly_len : work.get() + ((j - p0) & 1) * poly_len;
            kate_divide(dst, cur, poly_len, 1, from_raw(points[j]), s);
            cur = dst;
        }
        table[k] = cur;
    }
    dev_buf<const fr_t *> d_table(q_count, s);
    h2d(d_table, table.data(), q_count * sizeof(const fr_t *), s);
    dev_buf<fr_t> d_scalars(scalar_count, s);
    h2d(d_scalars, combination_scalars, scalar_count * sizeof(fr_t), s);
    fr_device_vec *v = device_vec_new(poly_len, s);
    try {
        lincomb_table_kernel<<<blocks_for(poly_len, 256), 256, 0, s>>>(v->values, d_table, d_scalars, poly_len,
                                                                       q_count);
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

// bls12_381_g1_msm.cu:4025-4118: pi = floor((sum_k scalars[k] q_k +
// scalars[q_count] f) / (X - point)), a new device vector of poly_len - 1
// coefficients (q_count = scalar_count - 1)
RustError midnight_sppark_bls12_381_fr_multiopen_pi_device(void **out, const void *q_device_vec,
                                                           const void *f_device_vec, size_t poly_len,
                                                           const RawFr *combination_scalars, size_t scalar_count,
                                                           RawFr point)
{
    if (!out || !q_device_vec || !f_device_vec || poly_len < 2 || !combination_scalars || scalar_count < 2)
        return make_error((int)cudaErrorInvalidValue, "invalid resident pi-polynomial arguments");
    *out = nullptr;
    const size_t q_count = scalar_count - 1;
    auto *qv = reinterpret_cast<const fr_device_vec *>(q_device_vec);
    auto *fv = reinterpret_cast<const fr_device_vec *>(f_device_vec);
    if (q_count > SIZE_MAX / poly_len || qv->len != q_count * poly_len || fv->len != poly_len)
        return make_error((int)cudaErrorInvalidValue, "resident pi-polynomial shape mismatch");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    device_vec_wait(qv, s);
    device_vec_wait(fv, s);
    std::vector<const fr_t *> table(scalar_count);
    for (size_t k = 0; k < q_count; k++) table[k] = qv->values + k * poly_len;
    table[q_count] = fv->values;
    dev_buf<const fr_t *> d_table(scalar_count, s);
    h2d(d_table, table.data(), scalar_count * sizeof(const fr_t *), s);
    dev_buf<fr_t> d_scalars(scalar_count, s), combined(poly_len, s), quotient(poly_len, s);
    h2d(d_scalars, combination_scalars, scalar_count * sizeof(fr_t), s);
    lincomb_table_kernel<<<blocks_for(poly_len, 256), 256, 0, s>>>(combined, d_table, d_scalars, poly_len,
                                                                   scalar_count);
    GB_CHECK_LAUNCH();
    // the quotient ignores the constant term, so subtracting the value at
    // the point (as the reference does first) changes nothing
    kate_divide(quotient, combined, poly_len, 1, from_raw(point), s);
    fr_device_vec *v = device_vec_new(poly_len - 1, s);
    try {
        GB_CUDA_OK(cudaMemcpyAsync(v->values, quotient.get(), (poly_len - 1) * sizeof(fr_t), cudaMemcpyDeviceToDevice,
                                   s));
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

}  // extern "C"
