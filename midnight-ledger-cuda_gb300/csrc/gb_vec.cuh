// Fr vector building blocks shared across translation units.
#pragma once

#include "gb_runtime.cuh"

namespace gb {

// inclusive multiplicative prefix scan; out may alias in
void prefix_product(fr_t *out, const fr_t *in, size_t n, cudaStream_t s);
// out[i] = (mul ? mul[i] : 1) / in[i], zeros stay zero; out may alias in or mul
void batch_invert(fr_t *out, const fr_t *in, size_t n, const fr_t *mul, cudaStream_t s);
// out[i] = sum_{j >= i} in[j]; out may alias in
void suffix_sum(fr_t *out, const fr_t *in, size_t n, cudaStream_t s);
// d[i] = w^i for i < n
void omega_powers(fr_t *d, const fr_t &w, size_t n, cudaStream_t s);
// d[q * n + i] = points[q]^i for q < npoints, i < n <= 2^24 (points on the
// device)
void omega_powers_many(fr_t *d, const fr_t *d_points, size_t npoints, size_t n, cudaStream_t s);

}  // namespace gb
