// Fr number-theoretic transforms on the device (shared by the NTT entry
// points, the coset LDE and the quotient path).
#pragma once

#include "gb_runtime.cuh"

namespace gb {

// Root of unity of order 2^log_n (forward) or its inverse: the reference's
// domain construction squares ROOT_OF_UNITY (S - k) times
// (vendor/midnight-proofs-0.8.1/src/poly/domain.rs:72-88; fq.rs:70,481).
fr_t host_omega(uint32_t log_n, bool inverse);
fr_t host_fr_from_u64(uint64_t v);
fr_t host_fr_inverse(const fr_t &a);

// In-place NTT of `count` contiguous polynomials of length 2^log_n on stream s,
// natural order in and out (the reference's NN order).  forward: a_k =
// sum_j a_j w^(jk); inverse uses w^-1 and multiplies by `scale`
// (pass n^-1 for the reference's inverse, which includes 1/n).  Bounded
// waits that run out are counted in status[0..1] (device memory the caller
// owns and zeroes; may be null to not count them).
void ntt_inplace(fr_t *d, uint32_t log_n, size_t count, bool inverse, const fr_t *scale, uint32_t *status,
                 cudaStream_t s);

// elementwise helpers (launch on stream s)
void launch_mul_assign(fr_t *d, const fr_t &k, size_t len, cudaStream_t s);
void launch_mul_assign_zeta(fr_t *d, const fr_t &first, const fr_t &second, size_t len, size_t period_len,
                            cudaStream_t s);
void launch_mul_assign_repeating(fr_t *d, const fr_t *factors, size_t factor_len, size_t len, cudaStream_t s);
void launch_scale_zeta(fr_t *d, const fr_t &scale, const fr_t &first, const fr_t &second, size_t len,
                       size_t period_len, cudaStream_t s);
void launch_coeff_to_extended_prepare(fr_t *out, const fr_t *in, const fr_t &first, const fr_t &second,
                                      size_t input_len, size_t output_len, size_t count, cudaStream_t s);

}  // namespace gb
