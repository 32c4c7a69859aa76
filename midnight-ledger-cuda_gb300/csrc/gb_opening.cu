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
    GB_CUDA_OK(cudaStreamSynchronize(s));
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
    if (pairs.size() > 65535) return make_error((int)cudaErrorInvalidValue, "too many batched evaluations");
    cudaStream_t s = lane_stream();
    for (size_t r = 0; r < requests; r++) device_vec_wait(reinterpret_cast<const fr_device_vec *>(vecs[r]), s);
    const size_t total = pairs.size();
    dev_buf<fr_t> d_points(requests, s), pw(requests * poly_len, s), d_out(total, s);
    dev_buf<eval_pair> d_pairs(total, s);
    h2d(d_points, points_raw, requests * sizeof(fr_t), s);
    h2d(d_pairs, pairs.data(), total * sizeof(eval_pair), s);
    omega_powers_many(pw, d_points, requests, poly_len, s);
    const uint32_t slices = (uint32_t)((poly_len + kEvalSlice - 1) / kEvalSlice);
    dev_buf<fr_t> partial(total * slices, s);
    eval_slices_many_kernel<<<dim3(slices, (unsigned)total), kEvalThreads, 0, s>>>(d_pairs, poly_len, pw, slices,
                                                                                 partial);
    GB_CHECK_LAUNCH();
    sum_slices_kernel<<<blocks_for(total, 128), 128, 0, s>>>(partial, slices, total, d_out);
    GB_CHECK_LAUNCH();
    d2h(out_raw, d_out, total * sizeof(fr_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
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

}  // extern "C"
