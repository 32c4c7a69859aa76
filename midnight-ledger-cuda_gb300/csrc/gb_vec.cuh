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
// z of every permutation set into out [sets][len] (bls12_381_g1_msm.cu:4342-4449):
// column c is d_columns[c * len ..], or d_col_ptrs[c][..] when the device
// pointer table is given; delta powers and blinds on the device
void permutation_products(fr_t *out, const fr_t *d_columns, const fr_t *const *d_col_ptrs, const fr_t *d_perms,
                          size_t len, size_t column_count, size_t chunk_len, const fr_t &beta, const fr_t &gamma,
                          const fr_t &omega, const fr_t *d_delta, const fr_t *d_blinds, size_t bf, cudaStream_t s);
// permute_expression_pair for lookup_count lookups (lookup/prover.rs:1573-1690):
// lookup l's compressed input / table at inputs + l * in_stride / tables +
// l * in_stride, its A' / S' into a_out + l * out_stride / s_out + l *
// out_stride, rows usable_rows.. of A' / S' from the host blinds
// ([lookup_count][len - usable_rows] each).  Returns nullptr, or the message
// of a failed permutation (an input missing from the table).
const char *lookup_permute_core(const fr_t *inputs, const fr_t *tables, size_t in_stride, fr_t *a_out, fr_t *s_out,
                                size_t out_stride, size_t len, size_t usable_rows, size_t lookup_count,
                                const RawFr *input_blinds, const RawFr *table_blinds, cudaStream_t s);

}  // namespace gb
