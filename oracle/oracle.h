/*
 * CPU oracle for the BLS12-381 prover hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C, the CPU
 * semantics of the reference prover (midnight-curves / midnight-proofs, which
 * sit on blst and rayon) so that the CUDA library can be checked against it.
 * Only tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py
 * may load it; the product path never links or calls it.
 *
 * Representation (identical to blst and to the reference FFI structs in
 * midnight-sppark-msm/src/lib.rs:17-36):
 *   Fr  : 4 x u64 little-endian limbs, Montgomery form, R = 2^256.
 *   Fp  : 6 x u64 little-endian limbs, Montgomery form, R = 2^384.
 *   G1 affine   : {x[6], y[6]}; the point at infinity is all-zero.
 *   G1 Jacobian : {x[6], y[6], z[6]}; the point at infinity has z = 0.
 */
#ifndef GB_ORACLE_H
#define GB_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint64_t l[4]; } orc_fr;
typedef struct { uint64_t l[6]; } orc_fp;
typedef struct { orc_fp x, y; } orc_g1_affine;
typedef struct { orc_fp x, y, z; } orc_g1_jac;

/* ---- scalar field Fr ---------------------------------------------------- */
void orc_fr_mul(orc_fr *out, const orc_fr *a, const orc_fr *b);
void orc_fr_add(orc_fr *out, const orc_fr *a, const orc_fr *b);
void orc_fr_sub(orc_fr *out, const orc_fr *a, const orc_fr *b);
void orc_fr_inv(orc_fr *out, const orc_fr *a);               /* 0 -> 0 */
void orc_fr_to_mont(orc_fr *out, const orc_fr *canonical);
void orc_fr_from_mont(orc_fr *out, const orc_fr *mont);
void orc_fr_from_u64(orc_fr *out, uint64_t v);
void orc_fr_pow(orc_fr *out, const orc_fr *a, const uint64_t *exp, size_t exp_limbs);
/* Named constants (Montgomery form): 0 one, 1 generator(7), 2 root_of_unity,
 * 3 root_of_unity_inv, 4 delta, 5 zeta, 6 two_inv. */
int orc_fr_constant(orc_fr *out, int which);
/* from_uniform_bytes (fq.rs:704-725): a0 * R^2 + a1 * R^3 over raw limbs. */
void orc_fr_from_uniform_bytes(orc_fr *out, const uint8_t bytes[64]);
/* canonical big-endian order (fq.rs:152-164): -1, 0, 1 */
int orc_fr_cmp_canonical(const orc_fr *a, const orc_fr *b);

/* ---- base field Fp ------------------------------------------------------ */
void orc_fp_mul(orc_fp *out, const orc_fp *a, const orc_fp *b);
void orc_fp_to_mont(orc_fp *out, const orc_fp *canonical);
void orc_fp_from_mont(orc_fp *out, const orc_fp *mont);
int orc_fp_sqrt(orc_fp *out, const orc_fp *a); /* 1 if a square */

/* ---- G1 ----------------------------------------------------------------- */
void orc_g1_generator(orc_g1_affine *out);
int orc_g1_is_on_curve(const orc_g1_affine *p);
void orc_g1_to_affine(orc_g1_affine *out, const orc_g1_jac *p);
void orc_g1_jac_to_affine_batch(orc_g1_affine *out, const orc_g1_jac *p, size_t n);
void orc_g1_from_affine(orc_g1_jac *out, const orc_g1_affine *p);
void orc_g1_add(orc_g1_jac *out, const orc_g1_jac *a, const orc_g1_jac *b);
void orc_g1_add_affine(orc_g1_jac *out, const orc_g1_jac *a, const orc_g1_affine *b);
void orc_g1_double(orc_g1_jac *out, const orc_g1_jac *a);
void orc_g1_neg(orc_g1_jac *out, const orc_g1_jac *a);
/* out = [scalar] p, scalar in Montgomery form */
void orc_g1_mul(orc_g1_jac *out, const orc_g1_affine *p, const orc_fr *scalar);
/* out[i] = affine([s_i] G) for scalars in Montgomery form */
void orc_g1_generator_mul_batch(orc_g1_affine *out, const orc_fr *scalars, size_t n, int threads);
int orc_g1_affine_eq(const orc_g1_affine *a, const orc_g1_affine *b);
int orc_g1_jac_eq(const orc_g1_jac *a, const orc_g1_jac *b);

/* zcash encodings (g1.rs:1179-1211): 48-byte compressed, 96-byte uncompressed.
 * Decoders return 0 on success, nonzero on an invalid encoding. */
int orc_g1_decompress(orc_g1_affine *out, const uint8_t in[48]);
void orc_g1_compress(uint8_t out[48], const orc_g1_affine *p);
int orc_g1_from_uncompressed(orc_g1_affine *out, const uint8_t in[96]);
void orc_g1_to_uncompressed(uint8_t out[96], const orc_g1_affine *p);

/* ---- multiexp ----------------------------------------------------------- */
/* Booth window index (msm.rs:13-56) of a canonical little-endian 32-byte scalar */
int32_t orc_booth_index(size_t window_index, size_t window_size, const uint8_t el[32]);
/* sum_i [s_i] P_i by per-point double-and-add (small n only) */
void orc_g1_msm_naive(orc_g1_jac *out, const orc_g1_affine *bases, const orc_fr *scalars, size_t n);
/* Pippenger with Booth windows (msm.rs:477-550 semantics); window_bits 0 = ceil(ln n) */
void orc_g1_msm(orc_g1_jac *out, const orc_g1_affine *bases, const orc_fr *scalars, size_t n,
                int threads, int window_bits);

/* ---- NTT / domain ------------------------------------------------------- */
/* best_fft (fft.rs:35-113): in place, natural order in and out, no scaling */
void orc_fr_fft(orc_fr *a, uint32_t log_n, const orc_fr *omega, int threads);
/* 2^k-th root of unity: ROOT_OF_UNITY squared (S - k) times (domain.rs:72-88) */
void orc_fr_omega(orc_fr *out, uint32_t k);
/* Reference FFI semantics of midnight_sppark_bls12_381_fr_ntt: forward = FFT(omega),
 * inverse = FFT(omega^-1) * n^-1. */
void orc_fr_ntt(orc_fr *a, uint32_t log_n, int inverse, int threads);
/* values[i] *= {1, first, second}[i mod 3] */
void orc_fr_mul_assign_zeta(orc_fr *a, const orc_fr *first, const orc_fr *second, size_t len);
void orc_fr_mul_assign(orc_fr *a, const orc_fr *s, size_t len);
void orc_fr_mul_assign_repeating(orc_fr *a, const orc_fr *f, size_t flen, size_t len);
/* ntt_zeta: NTT(inverse?) then * scale then zeta distribution */
void orc_fr_ntt_zeta(orc_fr *a, uint32_t log_n, int inverse, const orc_fr *scale,
                     const orc_fr *first, const orc_fr *second, int threads);
/* divide_ntt_zeta: *= factors[i mod m]; inverse NTT; * scale; zeta distribution */
void orc_fr_divide_ntt_zeta(orc_fr *a, uint32_t log_n, const orc_fr *factors, size_t m,
                            const orc_fr *scale, const orc_fr *first, const orc_fr *second,
                            int threads);
/* coeff_to_extended for `count` polynomials of input_len coefficients each */
int orc_fr_coeff_to_extended_batch(orc_fr *out, const orc_fr *in, size_t input_len, size_t count,
                                   uint32_t ext_log_n, const orc_fr *first, const orc_fr *second,
                                   int threads);
/* a[i] *= shift^i for i < len (sppark LDE_distribute_powers, natural index) */
void orc_fr_distribute_powers(orc_fr *a, size_t len, const orc_fr *shift);
/* coset NTT by powers of `shift`, natural order in and out (sppark NTT::Base with
 * Type::coset): forward = NTT(a_i shift^i); inverse = iNTT(a)_i shift^-i */
void orc_fr_ntt_coset(orc_fr *a, uint32_t log_n, int inverse, const orc_fr *shift, int threads);
/* coefficients -> evaluations on the coset shift * <w_ext>: a_i shift^i, zero-pad to
 * 2^ext_log_n, forward NTT, for `count` polynomials of input_len coefficients */
int orc_fr_coeff_to_extended_coset_batch(orc_fr *out, const orc_fr *in, size_t input_len, size_t count,
                                         uint32_t ext_log_n, const orc_fr *shift, int threads);
/* sppark NTT::LDE: 2^lg_dsz evaluations -> 2^(lg_dsz+lg_blowup) evaluations on the coset
 * by the multiplicative generator (iNTT, distribute powers, zero-pad, NTT) */
void orc_fr_lde_coset(orc_fr *out, const orc_fr *in, uint32_t lg_dsz, uint32_t lg_blowup, int threads);
/* EvaluationDomain::new(j, k) constants: extended_k and t_evaluations (inverted) */
uint32_t orc_domain_extended_k(uint32_t j, uint32_t k);
void orc_domain_t_evaluations(orc_fr *out, uint32_t j, uint32_t k); /* 2^(ext_k-k) entries */

/* ---- grand products & vector ops ---------------------------------------- */
void orc_fr_batch_invert(orc_fr *a, size_t len);
void orc_fr_shifted_prefix_product(orc_fr *values, const orc_fr *initial, size_t len);
int orc_fr_permutation_products(orc_fr *out, const orc_fr *columns, const orc_fr *permutations,
                                size_t len, size_t column_count, size_t chunk_len,
                                const orc_fr *beta, const orc_fr *gamma, const orc_fr *omega,
                                const orc_fr *delta_powers, const orc_fr *blinds,
                                size_t blinding_factors);
int orc_fr_lookup_products(orc_fr *out, const orc_fr *compressed_inputs,
                           const orc_fr *compressed_tables, const orc_fr *permuted_inputs,
                           const orc_fr *permuted_tables, size_t len, size_t lookup_count,
                           const orc_fr *beta, const orc_fr *gamma, const orc_fr *blinds,
                           size_t blinding_factors);
void orc_fr_poly_lincomb(orc_fr *out, const orc_fr *polys, size_t poly_len, size_t poly_count,
                         const orc_fr *scalars);
int orc_fr_quotient_pieces(orc_fr *out, const orc_fr *quotient, size_t quotient_len,
                           size_t poly_len, size_t piece_count, const orc_fr *blinds,
                           size_t blind_count);
void orc_fr_sort_canonical(orc_fr *a, size_t len);
/* eval_polynomial (arithmetic.rs:53-77): sum_i poly[i] * point^i */
void orc_fr_eval_poly(orc_fr *out, const orc_fr *poly, size_t len, const orc_fr *point);
/* kate_division (arithmetic.rs:97-116): len - 1 quotient coefficients */
void orc_fr_kate_division(orc_fr *q, const orc_fr *a, size_t len, const orc_fr *b);

/* ---- quotient numerator ------------------------------------------------- */
/* Same memory layout as the C ABI's RawValueSource / RawCalculation /
 * RawGraph / RawColumnRef (midnight-sppark-msm/src/lib.rs:38-86). */
typedef struct { uint32_t kind, a, b; } orc_value_source;
typedef struct {
    uint32_t op, target, parts_offset, parts_len;
    orc_value_source lhs, rhs;
} orc_calculation;
typedef struct {
    const orc_fr *constants;
    size_t constants_len;
    const int32_t *rotations;
    size_t rotations_len;
    const orc_calculation *calculations;
    size_t calculations_len;
    const orc_value_source *horner_parts;
    size_t horner_parts_len;
    uint32_t num_intermediates;
} orc_graph;
typedef struct { uint32_t kind, index; } orc_column_ref;

/* Evaluator::evaluate_numerator (evaluation.rs:3114-3528) with the argument
 * shapes of midnight_sppark_bls12_381_eval_numerator (.cu:5196). */
int orc_eval_numerator(orc_fr *out, size_t len, const orc_fr *initial_out, uint32_t run_custom,
                       const orc_fr *fixed, size_t fixed_cols, const orc_fr *advice, size_t advice_cols,
                       const orc_fr *instance, size_t instance_cols, const orc_fr *challenges,
                       size_t challenge_len, const orc_fr *beta, const orc_fr *gamma, const orc_fr *theta,
                       const orc_fr *trash_challenge, const orc_fr *y, const orc_fr *omega,
                       const orc_fr *delta_start, const orc_fr *delta_const, int32_t rot_scale,
                       int32_t last_rotation, uint32_t chunk_len, const orc_fr *l0, const orc_fr *l_last,
                       const orc_fr *l_active, const orc_fr *permutation_products, size_t permutation_sets,
                       const orc_column_ref *permutation_columns, size_t permutation_columns_len,
                       const orc_fr *permutation_pk_cosets, const orc_fr *lookup_product_cosets,
                       const orc_fr *lookup_input_cosets, const orc_fr *lookup_table_cosets,
                       size_t lookup_count, const orc_fr *trash_cosets,
                       const uint32_t *trash_selector_fixed_indices, size_t trash_count,
                       const orc_graph *custom_graph, const orc_graph *lookup_graphs,
                       const orc_graph *trash_graphs, int threads);

/* ---- transcript ---------------------------------------------------------- */
void orc_blake2b(uint8_t *out, size_t outlen, const uint8_t *key, size_t keylen, const uint8_t *in, size_t len);
void orc_transcript_replay(const uint8_t *ops, size_t nops, const uint8_t *const *msgs, const size_t *lens,
                           orc_fr *challenges);

#ifdef __cplusplus
}
#endif
#endif
