/*
 * gb_prover.h -- C ABI of the GB300 (sm_103a) BLS12-381 prover library,
 * libgbprover.so.
 *
 * Drop-in boundary: every `midnight_sppark_*` entry point below has the
 * symbol name, argument list, argument meaning and error behaviour of the
 * function of the same name that the reference's Rust crate binds in
 * midnight-sppark-msm/src/lib.rs:763-1362 (implemented there in
 * midnight-sppark-msm/src/bls12_381_g1_msm.cu).  Linking this library in
 * place of the reference's sppark-built archive needs no change on the Rust
 * side.  Entries prefixed `gb_` are additions of this library.
 *
 * Data layout (all little-endian, Montgomery form, blst-compatible):
 *   RawFr           = Bls12_381Fr           (lib.rs:17-21)  4 x u64, R = 2^256
 *   RawG1Affine     = Bls12_381G1Affine     (lib.rs:23-28)  x[6], y[6]; infinity = all zero
 *   RawG1Projective = Bls12_381G1Projective (lib.rs:30-36)  Jacobian x[6], y[6], z[6]; infinity z = 0
 *
 * Errors: RustError is returned by value; code 0 = success, otherwise a
 * cudaError_t value or -1; `message` is NULL or a strdup()'d string the
 * caller releases with free() (vendor/sppark-0.1.15/src/lib.rs:8-23).
 * Invalid arguments give cudaErrorInvalidValue (1) with a message, as in
 * bls12_381_g1_msm.cu:6318-6331.  There is no CPU fallback: without a CUDA
 * device every compute entry point returns an error.
 *
 * Threading and ordering: work runs on the calling thread's execution lane
 * (one CUDA stream per lane, midnight_sppark_execution_lane_set).  Calls that
 * take or return host buffers are synchronous.  Calls that produce a device
 * vector return once the work is queued; a consumer on any lane waits for it
 * (each device vector carries a completion event).
 */
#ifndef GB_PROVER_H
#define GB_PROVER_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GB_API __attribute__((visibility("default")))
#else
#define GB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint64_t limbs[4]; } RawFr;
typedef struct { uint64_t x[6]; uint64_t y[6]; } RawG1Affine;
typedef struct { uint64_t x[6]; uint64_t y[6]; uint64_t z[6]; } RawG1Projective;
typedef struct { int code; char *message; } RustError;

/* bls12_381_g1_msm.cu:50-61; Rust mirror Bls12_381MsmConfig lib.rs:126-160.
 * window_bits 0 = chosen by the library; this library accepts 0 or 8..16. */
typedef struct {
    uint32_t domain_k;
    uint32_t min_msm_scalars;
    uint32_t unfiltered_min_scalars;
    uint32_t window_bits;
    uint32_t sort_grid_divisor;
    uint32_t sort_window_lanes;
    uint32_t integration_blocks;
    uint32_t batch_lanes;
    uint32_t reuse_event;
    uint32_t device_reduce;
} RawMsmConfig;

/* bls12_381_g1_msm.cu:63-68 */
typedef struct {
    size_t scalar_offset;
    size_t point_offset;
    size_t len;
    size_t nonzero_len;
} RawMsmSlice;

/* Compiled gate graph (lib.rs:38-79; bls12_381_g1_msm.cu:351-381), the
 * flattened form of midnight-proofs' GraphEvaluator (evaluation.rs:47-241).
 * ValueSource kinds: 0 constant[a], 1 intermediate[a], 2 fixed[a] at
 * rotation rotations[b], 3 advice[a]@b, 4 instance[a]@b, 5 challenge[a],
 * 6 beta, 7 gamma, 8 theta, 9 trash challenge, 10 y, 11 previous value.
 * Calculation ops: 0 add, 1 sub, 2 mul, 3 square, 4 double, 5 negate,
 * 6 Horner (v = lhs; v = v * rhs + part for each of the parts_len parts
 * starting at horner_parts[parts_offset]), 7 store.  Each result goes to
 * intermediates[target]; the graph's value is the last calculation's. */
typedef struct { uint32_t kind; uint32_t a; uint32_t b; } RawValueSource;
typedef struct {
    uint32_t op;
    uint32_t target;
    uint32_t parts_offset;
    uint32_t parts_len;
    RawValueSource lhs;
    RawValueSource rhs;
} RawCalculation;
typedef struct {
    const RawFr *constants;
    size_t constants_len;
    const int32_t *rotations;
    size_t rotations_len;
    const RawCalculation *calculations;
    size_t calculations_len;
    const RawValueSource *horner_parts;
    size_t horner_parts_len;
    uint32_t num_intermediates;
} RawGraph;
/* permutation column: kind 0 fixed, 1 advice, 2 instance (lib.rs:81-86) */
typedef struct { uint32_t kind; uint32_t index; } RawColumnRef;
/* resident polynomial: source 0 dynamic, 1 fixed, 2 extra device vector,
 * index-th polynomial in it (bls12_381_g1_msm.cu:383-386) */
typedef struct { uint32_t source; uint32_t index; } RawDevicePolyRef;

/* ---- lanes ---------------------------------------------------------------- */
/* bls12_381_g1_msm.cu:134-146: 0 = shared lane, 1..8 private lanes */
GB_API RustError midnight_sppark_execution_lane_set(uint32_t lane);

/* ---- G1 multiexp ------------------------------------------------------------ */
/* bls12_381_g1_msm.cu:6164-6200: out = sum_i scalars[i] * points[i] */
GB_API RustError midnight_sppark_bls12_381_g1_msm(RawG1Projective *out, const RawG1Affine *points,
                                                  const RawFr *scalars, size_t len);
/* bls12_381_g1_msm.cu:6202-6245: scalars laid out [nmsms][npoints] */
GB_API RustError midnight_sppark_bls12_381_g1_msm_batch(RawG1Projective *out, const RawG1Affine *points,
                                                        const RawFr *scalars, size_t npoints, size_t nmsms);
/* bls12_381_g1_msm.cu:6247-6281: resident bases (and their per-window
 * shifted copies, computed here once) */
GB_API RustError midnight_sppark_bls12_381_g1_msm_context_create(void **out, const RawG1Affine *points,
                                                                 size_t npoints);
GB_API RustError midnight_sppark_bls12_381_g1_msm_context_create_with_config(void **out,
                                                                             const RawG1Affine *points,
                                                                             size_t npoints,
                                                                             RawMsmConfig config);
/* bls12_381_g1_msm.cu:6283-6286 */
GB_API void midnight_sppark_bls12_381_g1_msm_context_free(void *context);
/* device bytes held by a context (its nwin x npoints table of affine
 * points); no reference counterpart, for HBM budgeting */
GB_API size_t gb_g1_msm_context_device_bytes(const void *context);
/* bls12_381_g1_msm.cu:6288-6308: host scalars [nmsms][npoints] */
GB_API RustError midnight_sppark_bls12_381_g1_msm_context_batch(RawG1Projective *out, void *context,
                                                                const RawFr *scalars, size_t npoints,
                                                                size_t nmsms);
/* bls12_381_g1_msm.cu:6310-6344: scalars from a device vector */
GB_API RustError midnight_sppark_bls12_381_g1_msm_context_device_batch(RawG1Projective *out, void *context,
                                                                       const void *device_vec,
                                                                       size_t scalar_offset, size_t npoints,
                                                                       size_t nmsms);
/* bls12_381_g1_msm.cu:6346-6377 */
GB_API RustError midnight_sppark_bls12_381_g1_msm_context_device_ragged(RawG1Projective *out, void *context,
                                                                        const void *device_vec,
                                                                        const RawMsmSlice *slices, size_t count);
/* bls12_381_g1_msm.cu:6426-6486: per batch entry, MSM(scalars + mask)
 * (mask_device_vec holds npoints values); as in the reference, the caller
 * subtracts its precomputed MSM(mask, bases) (lib.rs:3302-3354) */
GB_API RustError midnight_sppark_bls12_381_g1_msm_context_device_scrambled_batch(
    RawG1Projective *out, void *context, const void *device_vec, size_t scalar_offset, size_t npoints,
    size_t nmsms, const void *mask_device_vec);

/* ---- NTT / coset LDE -------------------------------------------------------- */
/* bls12_381_g1_msm.cu:6488-6502: in place, natural order; inverse includes 1/n */
GB_API RustError midnight_sppark_bls12_381_fr_ntt(RawFr *values, uint32_t log_n, bool inverse);
/* bls12_381_g1_msm.cu:3447-3495: NTT, then *scale, then *{1,first,second}[i mod 3] */
GB_API RustError midnight_sppark_bls12_381_fr_ntt_zeta(RawFr *values, uint32_t log_n, bool inverse, RawFr scale,
                                                       RawFr first, RawFr second);
/* bls12_381_g1_msm.cu:3497-3556: *factors[i mod m], inverse NTT, *scale, zeta */
GB_API RustError midnight_sppark_bls12_381_fr_divide_ntt_zeta(RawFr *values, uint32_t log_n,
                                                              const RawFr *factors, size_t factor_len,
                                                              RawFr scale, RawFr first, RawFr second);
/* bls12_381_g1_msm.cu:2542-2602: zeta-distribute, zero-pad, forward NTT */
GB_API RustError midnight_sppark_bls12_381_fr_coeff_to_extended_batch(RawFr *out, const RawFr *inputs,
                                                                      size_t input_len, size_t count,
                                                                      uint32_t extended_log_n, RawFr first,
                                                                      RawFr second);
/* bls12_381_g1_msm.cu:2604-2740: same, result resident */
GB_API RustError midnight_sppark_bls12_381_fr_device_coeff_to_extended_batch(void **out, const RawFr *inputs,
                                                                             size_t input_len, size_t count,
                                                                             uint32_t extended_log_n,
                                                                             RawFr first, RawFr second);
GB_API RustError midnight_sppark_bls12_381_fr_device_coeff_to_extended_from_device_batch(
    void **out, const void *source, size_t input_len, size_t count, uint32_t extended_log_n, RawFr first,
    RawFr second);
/* bls12_381_g1_msm.cu:3280-3440 */
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_ntt_zeta(void *device_vec, uint32_t log_n, bool inverse,
                                                                  RawFr scale, RawFr first, RawFr second);
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_ntt_zeta_batch(void *device_vec, uint32_t log_n,
                                                                        size_t count, bool inverse, RawFr scale,
                                                                        RawFr first, RawFr second);
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_divide_ntt_zeta(void *device_vec, uint32_t log_n,
                                                                         const RawFr *factors, size_t factor_len,
                                                                         RawFr scale, RawFr first,
                                                                         RawFr second);

/* ---- vector ops ------------------------------------------------------------- */
/* bls12_381_g1_msm.cu:1188-1231 kernels behind lib.rs:1000-1140 */
GB_API RustError midnight_sppark_bls12_381_fr_mul_assign(RawFr *values, RawFr scalar, size_t len);
GB_API RustError midnight_sppark_bls12_381_fr_mul_assign_zeta(RawFr *values, RawFr first, RawFr second,
                                                              size_t len);
GB_API RustError midnight_sppark_bls12_381_fr_mul_assign_repeating(RawFr *values, const RawFr *factors,
                                                                   size_t factor_len, size_t len);
GB_API RustError midnight_sppark_bls12_381_fr_invert_assign(RawFr *values, size_t len);
GB_API RustError midnight_sppark_bls12_381_fr_sort_canonical(RawFr *values, size_t len);
GB_API RustError midnight_sppark_bls12_381_fr_poly_lincomb(RawFr *out, const RawFr *polys, size_t poly_len,
                                                           size_t poly_count, const RawFr *scalars);
/* bls12_381_g1_msm.cu:4303-4340 (permutation/prover.rs:36-43) */
GB_API RustError midnight_sppark_bls12_381_fr_shifted_prefix_product(RawFr *values, RawFr initial, size_t len);

/* ---- grand products --------------------------------------------------------- */
/* bls12_381_g1_msm.cu:4342-4449: out = device vector [sets][len] */
GB_API RustError midnight_sppark_bls12_381_fr_permutation_products(
    void **out, const RawFr *columns, const RawFr *permutations, size_t len, size_t column_count,
    size_t chunk_len, RawFr beta, RawFr gamma, RawFr omega, const RawFr *delta_powers,
    const RawFr *blind_values, size_t blinding_factors);
/* bls12_381_g1_msm.cu:4451-4548: out = device vector [lookup_count][len] */
GB_API RustError midnight_sppark_bls12_381_fr_lookup_products(
    void **out, const RawFr *compressed_inputs, const RawFr *compressed_tables, const RawFr *permuted_inputs,
    const RawFr *permuted_tables, size_t len, size_t lookup_count, RawFr beta, RawFr gamma,
    const RawFr *blind_values, size_t blinding_factors);
/* bls12_381_g1_msm.cu:4550-4634 */
GB_API RustError midnight_sppark_bls12_381_fr_lookup_products_device(void **out, const void *trace_lagrange,
                                                                     size_t len, size_t lookup_count, RawFr beta,
                                                                     RawFr gamma, const RawFr *blind_values,
                                                                     size_t blinding_factors);

/* ---- quotient --------------------------------------------------------------- */
/* bls12_381_g1_msm.cu:3181-3240 (vanishing/prover.rs:141-220,304-318) */
GB_API RustError midnight_sppark_bls12_381_fr_device_quotient_pieces(void **out, const void *quotient_vec,
                                                                     size_t poly_len, size_t piece_count,
                                                                     const RawFr *blinds, size_t blind_count);
/* bls12_381_g1_msm.cu:3242-3278 */
GB_API RustError midnight_sppark_bls12_381_fr_device_poly_lincomb(void **out, const void *polys_vec,
                                                                  size_t poly_len, size_t poly_count,
                                                                  const RawFr *scalars, size_t scalar_count);

/* bls12_381_g1_msm.cu:5196-5432 (evaluation.rs:3114-3528): the quotient
 * numerator nu on the extended coset, len rows.  If run_custom, out starts
 * from the custom-gate graph, else from initial_out; then, folded with
 * v = v*y + term: the permutation terms (permutation_sets products of len
 * values, columns chunked by chunk_len, cosets of the sigma polynomials),
 * lookup_count lookups (product / permuted input / permuted table cosets and
 * each lookup's table graph) and trash_count trash arguments.  Columns are
 * laid out [column][len]. */
GB_API RustError midnight_sppark_bls12_381_eval_numerator(
    RawFr *out, size_t len, const RawFr *initial_out, uint32_t run_custom, const RawFr *fixed, size_t fixed_cols,
    const RawFr *advice, size_t advice_cols, const RawFr *instance, size_t instance_cols, const RawFr *challenges,
    size_t challenge_len, RawFr beta, RawFr gamma, RawFr theta, RawFr trash_challenge, RawFr y, RawFr omega,
    RawFr delta_start, RawFr delta_const, int32_t rot_scale, int32_t last_rotation, uint32_t chunk_len,
    const RawFr *l0, const RawFr *l_last, const RawFr *l_active, const RawFr *permutation_products,
    size_t permutation_sets, const RawColumnRef *permutation_columns, size_t permutation_columns_len,
    const RawFr *permutation_pk_cosets, size_t permutation_pk_cosets_len, const RawFr *lookup_product_cosets,
    const RawFr *lookup_input_cosets, const RawFr *lookup_table_cosets, size_t lookup_count,
    const RawFr *trash_cosets, const uint32_t *trash_selector_fixed_indices, size_t trash_count,
    RawGraph custom_graph, const RawGraph *lookup_graphs, const RawGraph *trash_graphs);
/* bls12_381_g1_msm.cu:5434-5515: graph_count graphs evaluated over len rows,
 * out laid out [graph][len] */
GB_API RustError midnight_sppark_bls12_381_eval_graph_batch(
    RawFr *out, size_t len, const RawFr *fixed, size_t fixed_cols, const RawFr *advice, size_t advice_cols,
    const RawFr *instance, size_t instance_cols, const RawFr *challenges, size_t challenge_len, RawFr beta,
    RawFr gamma, RawFr theta, RawFr trash_challenge, RawFr y, int32_t rot_scale, const RawGraph *graphs,
    size_t graph_count);

/* ---- resident forms of the argument and quotient entry points ---------------- */
/* midnight_sppark_bls12_381_fr_permutation_products over device vectors
 * (the resident trace path of .cu:4342-4449, prover.rs:216-262) */
GB_API RustError gb_fr_permutation_products_device(void **out, const void *columns_vec,
                                                   const void *permutations_vec, size_t len, size_t column_count,
                                                   size_t chunk_len, RawFr beta, RawFr gamma, RawFr omega,
                                                   const RawFr *delta_powers, const RawFr *blind_values,
                                                   size_t blinding_factors);
/* midnight_sppark_bls12_381_eval_graph_batch over device vectors, into a new
 * device vector [graph_count][len] (the resident lookup compression of
 * lookup/prover.rs:556-590) */
GB_API RustError gb_eval_graph_batch_device(void **out, size_t len, const void *fixed_vec, size_t fixed_cols,
                                            const void *advice_vec, size_t advice_cols, const void *instance_vec,
                                            size_t instance_cols, const RawFr *challenges, size_t challenge_len,
                                            RawFr beta, RawFr gamma, RawFr theta, RawFr trash_challenge, RawFr y,
                                            int32_t rot_scale, const RawGraph *graphs, size_t graph_count);
/* midnight_sppark_bls12_381_eval_numerator over device vectors (the numerator
 * context of .cu:5968-6162): lagrange_vec = l0 | l_last | l_active (3 x len),
 * lookup_permuted_vec = per lookup its permuted input then permuted table
 * coset; out = a new device vector of len rows */
GB_API RustError gb_eval_numerator_device(
    void **out, size_t len, const void *initial_vec, uint32_t run_custom, const void *fixed_vec, size_t fixed_cols,
    const void *advice_vec, size_t advice_cols, const void *instance_vec, size_t instance_cols,
    const RawFr *challenges, size_t challenge_len, RawFr beta, RawFr gamma, RawFr theta, RawFr trash_challenge,
    RawFr y, RawFr omega, RawFr delta_start, RawFr delta_const, int32_t rot_scale, int32_t last_rotation,
    uint32_t chunk_len, const void *lagrange_vec, const void *permutation_products_vec, size_t permutation_sets,
    const RawColumnRef *permutation_columns, size_t permutation_columns_len, const void *permutation_pk_vec,
    size_t permutation_pk_cosets_len, const void *lookup_products_vec, const void *lookup_permuted_vec,
    size_t lookup_count, const void *trash_vec, const uint32_t *trash_selector_fixed_indices, size_t trash_count,
    RawGraph custom_graph, const RawGraph *lookup_graphs, const RawGraph *trash_graphs);

/* ---- numerator context (stateful resident quotient) -------------------------- */
/* bls12_381_g1_msm.cu:5517-5660: the circuit's fixed data resident once.
 * fixed [fixed_cols][len] extended cosets, fixed_lagrange [fixed_cols][input_len],
 * l0 / l_last / l_active [len], permutation sigma cosets [pk_len][len] and
 * Lagrange values [pk_len][input_len], trash selectors (fixed column indices),
 * the graphs (copied into device memory), omega (extended domain), trace_omega
 * (input domain), g_coset (the coset shift: delta_start = beta * g_coset). */
GB_API RustError midnight_sppark_bls12_381_numerator_context_create(
    void **out, size_t len, size_t input_len, const RawFr *fixed, const RawFr *fixed_lagrange, size_t fixed_cols,
    const RawFr *l0, const RawFr *l_last, const RawFr *l_active, const RawColumnRef *permutation_columns,
    size_t permutation_columns_len, const RawFr *permutation_pk_cosets, const RawFr *permutation_pk_lagrange,
    size_t permutation_pk_cosets_len, const uint32_t *trash_selector_fixed_indices, size_t trash_count,
    RawGraph custom_graph, const RawGraph *lookup_graphs, const RawGraph *lookup_input_graphs,
    const RawGraph *lookup_table_graphs, size_t lookup_count, const RawGraph *trash_graphs, RawFr omega,
    RawFr trace_omega, RawFr g_coset, RawFr delta_const, int32_t rot_scale, int32_t last_rotation,
    uint32_t chunk_len);
/* bls12_381_g1_msm.cu:5662-5665 (drains the device first) */
GB_API void midnight_sppark_bls12_381_numerator_context_free(void *context);
/* bls12_381_g1_msm.cu:5968-6162: the numerator over one resident column vector
 * of total_columns x len values; each group (advice, instance, permutation
 * products, lookup products / permuted inputs / permuted tables, trash) is a
 * run of columns at its offset; out = a new device vector of len rows */
GB_API RustError midnight_sppark_bls12_381_numerator_context_eval(
    void **out, const void *context, const void *columns, size_t total_columns, size_t advice_offset,
    size_t advice_cols, size_t instance_offset, size_t instance_cols, const RawFr *challenges, size_t challenge_len,
    RawFr beta, RawFr gamma, RawFr theta, RawFr trash_challenge, RawFr y, size_t permutation_offset,
    size_t permutation_sets, size_t lookup_product_offset, size_t lookup_input_offset, size_t lookup_table_offset,
    size_t lookup_count, size_t trash_offset, size_t trash_count);
/* bls12_381_g1_msm.cu:5667-5736: trash compressed expressions over the trace
 * (input_len rows; advice / instance device vectors [cols][input_len]),
 * out [trash_count][input_len] */
GB_API RustError midnight_sppark_bls12_381_trace_context_trash(void **out, const void *context, const void *advice,
                                                               size_t advice_cols, const void *instance,
                                                               size_t instance_cols, const RawFr *challenges,
                                                               size_t challenge_len, RawFr trash_challenge);
/* bls12_381_g1_msm.cu:5738-5847: permutation products over the trace,
 * out [sets][input_len], sets = ceil(permutation columns / chunk_len);
 * delta_powers one per column, blind_values [sets][blinding_factors] */
GB_API RustError midnight_sppark_bls12_381_trace_context_permutation(
    void **out, const void *context, const void *advice, size_t advice_cols, const void *instance,
    size_t instance_cols, RawFr beta, RawFr gamma, const RawFr *delta_powers, size_t delta_powers_len,
    const RawFr *blind_values, size_t blind_values_len, size_t blinding_factors);
/* bls12_381_g1_msm.cu:5849-5966: compressed lookup inputs and tables over the
 * trace and their permutations, out [inputs | tables | permuted inputs |
 * permuted tables], each [lookup_count][input_len] (the layout
 * midnight_sppark_bls12_381_fr_lookup_products_device reads); blinds
 * [lookup_count][blind_count], blind_count = input_len - usable_rows */
GB_API RustError midnight_sppark_bls12_381_trace_context_lookup_permute(
    void **out, const void *context, const void *advice, size_t advice_cols, const void *instance,
    size_t instance_cols, const RawFr *challenges, size_t challenge_len, RawFr theta, size_t usable_rows,
    const RawFr *input_blinds, const RawFr *table_blinds, size_t blind_count);

/* bls12_381_g1_msm.cu:5139-5194: lookup permutation from host compressed
 * inputs / tables ([lookup_count][len] each); out = a new device vector
 * [inputs | tables | permuted inputs | permuted tables], blinds
 * [lookup_count][blind_count], blind_count = len - usable_rows */
GB_API RustError midnight_sppark_bls12_381_fr_lookup_permute_batch(void **out, const RawFr *compressed_inputs,
                                                                   const RawFr *compressed_tables, size_t len,
                                                                   size_t lookup_count, size_t usable_rows,
                                                                   const RawFr *input_blinds,
                                                                   const RawFr *table_blinds, size_t blind_count);
/* permute_expression_pair (lookup/prover.rs:1573-1690) for lookup_count
 * lookups on the device: compressed_vec = per lookup its compressed input
 * then compressed table column (len rows each); out = a new device vector,
 * per lookup A' then S' (len rows each), rows usable_rows.. taken from
 * input_blinds / table_blinds ([lookup_count][len - usable_rows] each).
 * An input value missing from the table is an error. */
GB_API RustError gb_fr_lookup_permute_device(void **out, const void *compressed_vec, size_t len, size_t usable_rows,
                                             size_t lookup_count, const RawFr *input_blinds,
                                             const RawFr *table_blinds);

/* ---- blinding draws ---------------------------------------------------------- */
/* nblocks ChaCha20 keystream blocks (RFC 8439 block function, 64-bit block
 * counter in words 12-13 and stream id in words 14-15, as rand_chacha's
 * ChaCha20Rng) from block `counter`, 16 words each, computed on the host: the
 * prover's host-side draws.  No reference counterpart (rand_chacha 0.3.1 on
 * the Rust side). */
GB_API RustError gb_chacha20_blocks(const uint32_t *key, uint64_t counter, uint64_t stream, size_t nblocks,
                                    uint32_t *out);
/* n values by Fq::random's rejection rule (fq.rs:373-387) from the
 * ChaCha20Rng stream with this 32-byte seed, starting at keystream word
 * word_offset, into a new device vector in Montgomery form;
 * *words_consumed = the keystream words the n draws used (the large draw of
 * vanishing/prover.rs:41-75 made on the device) */
GB_API RustError gb_fr_random_chacha20(void **out, const uint8_t *key32, uint64_t word_offset, size_t n,
                                       uint64_t *words_consumed);

/* ---- KZG opening helpers ---------------------------------------------------- */
/* bls12_381_g1_msm.cu:3985-4031: out[p] = sum_i polys[p][i] * point^i for the
 * poly_count resident polynomials of poly_len coefficients */
GB_API RustError midnight_sppark_bls12_381_fr_device_eval_polys(RawFr *out, const void *device_vec, size_t poly_len,
                                                                size_t poly_count, RawFr point);

/* bls12_381_g1_msm.cu:3600-3721: multi-open preparation over host
 * polynomials [poly_count][poly_len]: q_out [q_count][poly_len], q k = sum of
 * q_coefficients[t] * polys[q_poly_indices[t]] for q_offsets[k] <= t <
 * q_offsets[k+1] (q_count = q_offsets_len - 1); eval_out[r] = polynomial
 * query_poly_indices[r] at points[query_point_indices[r]] */
GB_API RustError midnight_sppark_bls12_381_fr_multiopen_prepare(
    RawFr *q_out, RawFr *eval_out, const RawFr *polys, size_t poly_len, size_t poly_count, const uint32_t *q_offsets,
    size_t q_offsets_len, const uint32_t *q_poly_indices, const RawFr *q_coefficients, size_t q_items_len,
    const RawFr *points, size_t point_count, const uint32_t *query_poly_indices, const uint32_t *query_point_indices,
    size_t query_count);
/* bls12_381_g1_msm.cu:3723-3871: the same over resident polynomials named by
 * poly_refs; q_out (host) and *q_device_out (new device vector) optional,
 * not both absent */
GB_API RustError midnight_sppark_bls12_381_fr_multiopen_prepare_device(
    RawFr *q_out, void **q_device_out, RawFr *eval_out, const void *dynamic_source, const void *fixed_source,
    const void *extra_source, size_t poly_len, const RawDevicePolyRef *poly_refs, size_t poly_count,
    const uint32_t *q_offsets, size_t q_offsets_len, const uint32_t *q_poly_indices, const RawFr *q_coefficients,
    size_t q_items_len, const RawFr *points, size_t point_count, const uint32_t *query_poly_indices,
    const uint32_t *query_point_indices, size_t query_count);
/* bls12_381_g1_msm.cu:3873-3983: f = sum_k combination_scalars[k] * q_k /
 * prod (X - points[j]) over q k's points (point_offsets, remainders
 * dropped); a new device vector of poly_len coefficients */
GB_API RustError midnight_sppark_bls12_381_fr_multiopen_f_poly_device(void **out, const void *q_device_vec,
                                                                      size_t poly_len, const uint32_t *point_offsets,
                                                                      size_t point_offsets_len, const RawFr *points,
                                                                      size_t point_count,
                                                                      const RawFr *combination_scalars,
                                                                      size_t scalar_count);
/* bls12_381_g1_msm.cu:4025-4118: pi = (sum_k scalars[k] q_k + scalars[last] f)
 * / (X - point), remainder dropped; a new device vector of poly_len - 1
 * coefficients */
GB_API RustError midnight_sppark_bls12_381_fr_multiopen_pi_device(void **out, const void *q_device_vec,
                                                                  const void *f_device_vec, size_t poly_len,
                                                                  const RawFr *combination_scalars,
                                                                  size_t scalar_count, RawFr point);

/* ---- Poseidon hash chains (default-off in the reference's Rust callers) --- */
/* bls12_381_g1_msm.cu:4121-4190 (lib.rs:1029-1040,4185-4236): out[i] = the
 * i-th hash of a chain of len 3-element Poseidon hashes (width 3, x^5,
 * 4 + 60 + 4 rounds): prev = initial; per hash, permute (prev, tail0,
 * input_len), add tail1 to the first element, permute again, prev = its
 * first element.  mds: 9 values (row-major), round_constants: 68 x 3. */
GB_API RustError midnight_sppark_bls12_381_fr_poseidon_hash_chain(RawFr *out, size_t len, RawFr initial,
                                                                  RawFr tail0, RawFr tail1, RawFr input_len,
                                                                  const RawFr *mds, size_t mds_len,
                                                                  const RawFr *round_constants,
                                                                  size_t round_constants_len);
/* bls12_381_g1_msm.cu:4192-4268 (lib.rs:1042-1053,4238-4290): the chain's
 * circuit witness, 256 values per hash (128 per permutation: per full
 * round the three cubes then the three new state values; per run of six
 * partial rounds five new third elements, then the three new values) */
GB_API RustError midnight_sppark_bls12_381_fr_poseidon_hash_chain_witness(RawFr *out, size_t len, RawFr initial,
                                                                          RawFr tail0, RawFr tail1,
                                                                          RawFr input_len, const RawFr *mds,
                                                                          size_t mds_len,
                                                                          const RawFr *round_constants,
                                                                          size_t round_constants_len);
/* bls12_381_g1_msm.cu:2820-2876 (lib.rs:854-863,1687-1730): a new device
 * vector of 8 advice columns x domain_len rows holding the chip's cells for
 * hash_count hashes: witness (256 per hash) placed by layout (128 entries,
 * column << 8 | row within a permutation's 21-row region; hash h's regions
 * start at rows 2 + 41 h and 2 + 41 h + 21), each permutation's input rows
 * and the chain's first cells from metadata (11 values).  Every layout
 * entry must name a column below 8 and a row inside the domain. */
GB_API RustError midnight_sppark_bls12_381_fr_poseidon_advice_from_witness(void **out, const RawFr *witness,
                                                                           size_t hash_count, size_t domain_len,
                                                                           const RawFr *metadata,
                                                                           size_t metadata_len,
                                                                           const uint16_t *layout,
                                                                           size_t layout_len);

/* ---- device vectors --------------------------------------------------------- */
/* bls12_381_g1_msm.cu:2741-3442 */
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_upload(void **out, const RawFr *values, size_t len);
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_upload_many(void **out, const RawFr *const *values,
                                                                     const size_t *lengths, size_t count);
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_download(RawFr *out, const void *device_vec, size_t len);
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_scatter_host(void *device_vec, const uint32_t *indices,
                                                                      const RawFr *values, size_t count);
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_concat_host(void **out, const void *prefix_device_vec,
                                                                     const RawFr *suffix, size_t suffix_len);
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_concat_many_host(void **out,
                                                                          const void *const *source_device_vecs,
                                                                          size_t source_count,
                                                                          const RawFr *suffix, size_t suffix_len);
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_gather_polys(void **out, const void *source_device_vec,
                                                                      size_t poly_len, const uint32_t *indices,
                                                                      size_t index_count);
GB_API void midnight_sppark_bls12_381_fr_device_vec_free(void *device_vec);
/* bls12_381_g1_msm.cu:3101-3179: for count polynomials of poly_len values at
 * scalar_offset: starts[p] = first nonzero coefficient (poly_len if none),
 * nonzero_counts[p] (optional) = nonzero coefficients, out = the suffixes
 * from starts[p] on, packed; *out_len = packed length.  out == NULL with
 * out_capacity == 0 asks for *out_len only. */
GB_API RustError midnight_sppark_bls12_381_fr_device_vec_download_nonzero_suffixes(
    RawFr *out, size_t out_capacity, size_t *out_len, size_t *starts, size_t *nonzero_counts, const void *device_vec,
    size_t scalar_offset, size_t poly_len, size_t count);

/* ---- test hooks (bls12_381_g1_msm.cu:6379-6423) ---------------------------- */
/* the next scrambled batches on this thread zero their masked scalars and
 * hold the stream back delay_ms before the mask is added */
GB_API void midnight_sppark_test_mask_delay(uint32_t delay_ms);
/* device_vec *= scale on this lane after holding the lane back delay_ms; the
 * vector is ready for other lanes only after the scaling */
GB_API RustError midnight_sppark_test_delayed_scale(void *device_vec, RawFr scale, uint32_t delay_ms);

/* ---- library additions (no reference counterpart) ---------------------------- */
/* number of Fr elements held by a device vector */
GB_API size_t gb_fr_device_vec_len(const void *device_vec);
/* out[i] = affine([scalars[i]] G), host buffers (SRS bases [tau^i] G) */
GB_API RustError gb_g1_generator_mul(RawG1Affine *out, const RawFr *scalars, size_t n);
/* same with device pointers; queued on the calling lane's stream */
GB_API RustError gb_g1_generator_mul_device(RawG1Affine *d_out, const RawFr *d_scalars, size_t n);
/* one MSM over n bases and n scalars already in device memory (caller's
 * pointers), result to the host: the plain engine (Horner over windows),
 * no precomputed table (a context keeps nwin x n x 96 bytes) */
GB_API RustError gb_g1_msm_device(RawG1Projective *out, const RawG1Affine *d_points, const RawFr *d_scalars,
                                  size_t n);
/* midnight_sppark_bls12_381_g1_msm_context_device_batch
 * (bls12_381_g1_msm.cu:6310-6344) queued on the calling lane without
 * waiting: *ticket receives a handle that gb_msm_ticket_wait completes.
 * Work queued on the lane meanwhile runs after the batch; the host is free
 * until it needs the points (a prover queues the transforms that do not
 * depend on the next challenge before waiting for the commitments).  Every
 * ticket must be waited for exactly once. */
GB_API RustError gb_g1_msm_context_device_batch_async(void **ticket, void *context, const void *device_vec,
                                                      size_t scalar_offset, size_t npoints, size_t nmsms);
/* waits for a ticket's batch, writes its nmsms points to out in batch order
 * (out may be NULL) and releases the ticket; a lane wait status set since
 * the lane's previous synchronisation is returned as cudaErrorLaunchTimeout */
GB_API RustError gb_msm_ticket_wait(void *ticket, RawG1Projective *out);
/* CUDA-graph replay of context batches (no FFI counterpart: the reference
 * launches each stage of bls12_381_g1_msm.cu:172-215 one by one).  A batch
 * shape (and bases) that comes a second time on the same lane is captured
 * as a graph and replayed from then on, with its descriptors refreshed; on by default
 * (GB_MSM_GRAPHS=0 turns it off at start-up).  The counters are the graphs
 * captured and the batches replayed since the process started. */
GB_API RustError gb_msm_graphs_enable(int on);
GB_API RustError gb_msm_graph_stats(unsigned long long *captures, unsigned long long *launches);
/* KZG SRS (no FFI counterpart; the reference does these in Rust on the CPU):
 * g_lagrange = iFFT(g) * n^-1 over G1 for 2^k points (arithmetic.rs:34-50,
 * params.rs:60-77 downsize), and the seeded-tau setup of params.rs:79-129
 * (g[i] = [tau^i]G, g_lagrange[i] = [(tau^n-1)/n * w^i/(tau - w^i)]G; either
 * output may be NULL).  Host buffers of 2^k affine points. */
GB_API RustError gb_g1_to_lagrange(RawG1Affine *out, const RawG1Affine *g, uint32_t k);
GB_API RustError gb_kzg_setup(RawG1Affine *g_out, RawG1Affine *g_lagrange_out, RawFr tau, uint32_t k);
/* Jacobian MSM results (Montgomery limbs) to affine Montgomery coordinates
 * on the host, with one field inversion for the batch; the point at
 * infinity becomes all zeros.  The reference's Rust callers do this with
 * blst's p1_to_affine on every commitment before it is written to the
 * transcript (vendor/midnight-curves-0.3.1/src/bls12_381/g1.rs:109-123
 * From<G1Projective>, :1127 batch_normalize).  No device work. */
GB_API RustError gb_g1_jacobian_to_affine_batch(RawG1Affine *out, const RawG1Projective *in, size_t n);
/* Kate quotients (f(X) - f(point)) / (X - point) of poly_count resident
 * polynomials (the division of the reference's multi-open kate scan,
 * bls12_381_g1_msm.cu:1923-1959), into a new device vector */
/* several evaluations in one call: request r evaluates the counts[r]
 * polynomials of poly_len coefficients in the device vector vecs[r] at
 * points[r]; out gets sum(counts) values, request by request.  The batched
 * form of bls12_381_g1_msm.cu:3985-4031 (one point per call there), for the
 * evaluations a proof makes at x and its rotations. */
GB_API RustError gb_fr_device_eval_many(RawFr *out, const void *const *vecs, const size_t *counts,
                                        const RawFr *points, size_t requests, size_t poly_len);
GB_API RustError gb_fr_device_kate_divide(void **out, const void *device_vec, size_t poly_len, size_t poly_count,
                                          RawFr point);
/* Autotuner: when enabled, the plain MSM path times the window sizes
 * {8, 10, 13, 16} and the NTT its pass variants the first time it meets a
 * (size, batch, scalar-sparsity) key, and keeps the fastest; off by default */
GB_API void gb_autotune_set(int enabled);
/* Forces the NTT pass variant, process-wide: 1 = one radix-2 butterfly per
 * thread, 2 / 3 = 4 / 8 elements per thread with twiddles from the global
 * table, 4 / 5 = 4 / 8 elements per thread with each pass's twiddles staged
 * in shared memory by a bulk copy; 0 restores the default (4) or the
 * autotuned choice */
GB_API void gb_ntt_variant_set(int variant);
/* bounded waits of NTT work (staged-pass twiddle copies, work-queue waits)
 * that ran out since the last read, process-wide, after synchronising the
 * calling lane; resets the count.  A wait that runs out is recorded in its
 * lane's status word, and the lane's next synchronising call (every call
 * that returns data to the host, e.g. a download or an MSM) returns
 * cudaErrorLaunchTimeout: results that depend on it are never returned as
 * success, as CUDA reports errors of asynchronous work at a later call. */
GB_API RustError gb_ntt_wait_timeouts(uint32_t *out);
/* test hook: poll limit of the first twiddle-copy wait of staged NTT passes
 * launched from now on, process-wide (negative = default; 0 = the wait gives
 * up at once and the error is reported as above, while the copy still lands
 * in a second, longer wait before the CTA moves on) */
GB_API void gb_ntt_wait_limit_set(int64_t spins);
/* ---- coset by the powers of a shift: sppark's coset NTT and LDE form
 * (vendor/sppark-0.1.15/sppark/ntt/ntt.cuh:78-97,196-209,283-342; kernels.cu
 * LDE_distribute_powers / LDE_spread_distribute_powers), which the
 * reference's vendored sppark uses with the multiplicative generator 7
 * (parameters/bls12_381.h:11, fq.rs:31-33 GENERATOR).  The reference's
 * midnight_sppark_* FFI exports only the ZETA coset; these are the
 * generator-coset counterparts. */
/* coefficients -> evaluations on shift * <w_ext>: out[p][j] = sum_i
 * inputs[p][i] (shift w_ext^j)^i for count polynomials of input_len values,
 * out count x 2^extended_log_n; host buffers */
GB_API RustError gb_fr_coeff_to_extended_coset_batch(RawFr *out, const RawFr *inputs, size_t input_len,
                                                     size_t count, uint32_t extended_log_n, RawFr shift);
/* the same from resident coefficients into a new device vector */
GB_API RustError gb_fr_device_coeff_to_extended_coset_batch(void **out, const void *source, size_t input_len,
                                                            size_t count, uint32_t extended_log_n, RawFr shift);
/* coset NTT in place on count resident polynomials of 2^log_n values
 * (NTT::Base with Type::coset, natural order): forward NTT(a_i shift^i),
 * inverse iNTT(a)_i shift^-i with the iNTT's 1/n */
GB_API RustError gb_fr_device_vec_ntt_coset_batch(void *device_vec, uint32_t log_n, size_t count, bool inverse,
                                                  RawFr shift);
/* the same on one host polynomial */
GB_API RustError gb_fr_ntt_coset(RawFr *values, uint32_t log_n, bool inverse, RawFr shift);
/* NTT::LDE: 2^lg_domain_size evaluations -> 2^(lg_domain_size + lg_blowup)
 * evaluations of the same polynomial on the coset of the generator 7 */
GB_API RustError gb_fr_lde_coset(RawFr *out, const RawFr *in, uint32_t lg_domain_size, uint32_t lg_blowup);
/* NTTs of `count` polynomials of different sizes held in one device vector,
 * in one persistent launch fed by a device work queue: polynomial j is the
 * 2^log_ns[j] values at element offset offsets[j] (ranges inside the vector,
 * not overlapping, log_ns[j] <= 30) and gets the semantics of
 * midnight_sppark_bls12_381_fr_device_vec_ntt_zeta (inverse includes 1/n,
 * then out[i] *= scale * [1, first, second][i mod 3]; a single value is
 * left unchanged).  Sizes of 2 and 4 values take the plain path.  The batched form of the reference's
 * one-transform-per-call device NTT (bls12_381_g1_msm.cu:3280-3380). */
GB_API RustError gb_fr_device_vec_ntt_ragged(void *device_vec, const size_t *offsets, const uint32_t *log_ns,
                                             size_t count, bool inverse, RawFr scale, RawFr first, RawFr second);
GB_API void gb_autotune_reset(void);
/* "key=value;" per tuned key into buf (NUL-terminated, truncated); returns
 * the full length */
GB_API size_t gb_autotune_report(char *buf, size_t len);
/* measured device throughput of 32x32->64 multiply-adds (64-bit products)
 * per second: the fastest probe form */
GB_API RustError gb_imad_peak(double *out_per_sec);
/* one probe form: 0 = mad.wide chains, 1..3 = carry-chained 12-limb rows
 * with 1, 2 or 4 independent accumulator sets per thread */
GB_API RustError gb_imad_probe(int form, double *out_per_sec);
/* cumulative host<->device bytes moved by this library */
GB_API void gb_transfer_counters(uint64_t *h2d_bytes, uint64_t *d2h_bytes);
GB_API void gb_transfer_counters_reset(void);
/* kernel launches issued by the library since it was loaded */
GB_API uint64_t gb_launch_counter(void);
/* the calling thread's lane stream (a cudaStream_t) */
GB_API void *gb_lane_stream(void);
/* CUDA-event timing of individual kernels on their launching stream;
 * slot 0 = MSM bucket accumulation, 1 = whole MSM, 2 = NTT passes, 3 = MSM
 * recode and sort, 4 = MSM bucket fix-up, 5 = MSM bucket reduction and window
 * combination */
GB_API void gb_profile_enable(int on);
GB_API void gb_profile_read(int slot, double *total_ms, uint64_t *launches);
GB_API void gb_profile_reset(void);
/* Allocation-free shifted prefix product; no counterpart in the reference.
 * For callers that cannot allocate device memory when they need it (a
 * server that reserved its HBM budget up front, or a prover lane that must
 * not trigger the device-wide synchronisation of cudaMalloc/cudaFree): in
 * place on caller-owned device memory, z[0] = initial,
 * z[i] = initial * prod_{j<i} values[j], same result as
 * midnight_sppark_bls12_381_fr_shifted_prefix_product.  Scratch is a fixed
 * 64 KiB device array per GPU (held until exit), so len <= 4194304 (2^22);
 * longer inputs get cudaErrorInvalidValue.  Queued on `stream` (NULL = the
 * calling thread's lane) and returns without waiting.  All calls share the
 * scratch: calls that overlap on the GPU (unordered streams) race.  The first
 * call on a device looks up the scratch address; make it before any stream
 * capture on that device. */
GB_API RustError gb_fr_shifted_prefix_product_noalloc(RawFr *d_values, RawFr initial, size_t len, void *stream);
/* releases a RustError message for callers without access to free() */
GB_API void gb_error_free(char *message);

#ifdef __cplusplus
}
#endif

#endif /* GB_PROVER_H */
