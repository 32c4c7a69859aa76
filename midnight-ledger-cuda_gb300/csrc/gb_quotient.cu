// Quotient numerator on the extended coset for sm_103a, and its C ABI
// (midnight-sppark-msm/src/bls12_381_g1_msm.cu:5196-5515, semantics of
// vendor/midnight-proofs-0.8.1/src/plonk/evaluation.rs:3114-3528).
//
// One fused kernel per call: each thread owns one extended-domain row and
// evaluates the custom-gate graph, then folds in the permutation, lookup and
// trash constraints (v = v*y + term), writing the row once.  The compiled
// graph is interpreted: every thread of a warp walks the same calculation
// list (uniform control flow, broadcast loads), with its intermediates in a
// per-thread local array sized to the graph.
#include <algorithm>
#include <vector>

#include "gb_vec.cuh"

namespace gb {

struct dgraph {
    const fr_t *constants;
    uint32_t nconst;
    const int32_t *rotations;
    uint32_t nrot;
    const RawCalculation *calcs;
    uint32_t ncalc;
    const RawValueSource *parts;
    uint32_t nparts;
    uint32_t ninter;
};

struct num_params {
    fr_t *out;
    size_t len;
    int32_t rot_scale;
    const fr_t *fixed;
    size_t fixed_cols;
    const fr_t *advice;
    size_t advice_cols;
    const fr_t *instance;
    size_t instance_cols;
    const fr_t *challenges;
    size_t challenge_len;
    fr_t beta, gamma, theta, trash, y;
    int run_custom;
    const fr_t *initial;
    dgraph custom;
    size_t perm_sets;
    const fr_t *perm_products;
    const RawColumnRef *perm_columns;
    size_t perm_columns_len;
    const fr_t *perm_pk_cosets;
    const fr_t *omega_powers;
    fr_t delta_start, delta_const;
    int32_t last_rotation;
    uint32_t chunk_len;
    const fr_t *l0, *l_last, *l_active;
    size_t lookup_count;
    const fr_t *lk_product, *lk_input, *lk_table;
    size_t lk_stride;  // distance between consecutive lookups' input (and table) columns
    const dgraph *lookup_graphs;
    size_t trash_count;
    const fr_t *trash_cosets;
    const uint32_t *trash_sel;
    const dgraph *trash_graphs;
};

// (idx + rot * rot_scale) mod len, Euclidean (evaluation.rs:40-45)
__device__ __forceinline__ size_t rot_index(size_t idx, int32_t rot, int32_t rot_scale, size_t len)
{
    int64_t v = (int64_t)idx + (int64_t)rot * rot_scale;
    int64_t m = (int64_t)len;
    v %= m;
    if (v < 0) v += m;
    return (size_t)v;
}

__device__ __forceinline__ const fr_t *column_base(const num_params &p, uint32_t kind, uint32_t index)
{
    if (kind == 0 && index < p.fixed_cols) return p.fixed + (size_t)index * p.len;
    if (kind == 1 && index < p.advice_cols) return p.advice + (size_t)index * p.len;
    if (kind == 2 && index < p.instance_cols) return p.instance + (size_t)index * p.len;
    return nullptr;
}

// ValueSource::get (evaluation.rs:83-129); out-of-range references read zero
template <int MAX>
__device__ fr_t source_value(const RawValueSource &src, const dgraph &g, const num_params &p, size_t idx,
                             const fr_t *inter, const fr_t &prev)
{
    switch (src.kind) {
    case 0:
        return src.a < g.nconst ? g.constants[src.a] : fr_t::zero();
    case 1:
        return src.a < MAX ? inter[src.a] : fr_t::zero();
    case 2:
    case 3:
    case 4: {
        const fr_t *base = column_base(p, src.kind - 2, src.a);
        if (!base || src.b >= g.nrot) return fr_t::zero();
        return base[rot_index(idx, g.rotations[src.b], p.rot_scale, p.len)];
    }
    case 5:
        return src.a < p.challenge_len ? p.challenges[src.a] : fr_t::zero();
    case 6:
        return p.beta;
    case 7:
        return p.gamma;
    case 8:
        return p.theta;
    case 9:
        return p.trash;
    case 10:
        return p.y;
    case 11:
        return prev;
    default:
        return fr_t::zero();
    }
}

// GraphEvaluator::evaluate (evaluation.rs:3797-3846): every calculation in
// order, results cached as intermediates; the value of the last one
template <int MAX>
__device__ fr_t evaluate_graph(const dgraph &g, const num_params &p, size_t idx, const fr_t &prev)
{
    fr_t inter[MAX];
    const uint32_t nint = g.ninter < MAX ? g.ninter : MAX;
    for (uint32_t i = 0; i < nint; i++) inter[i] = fr_t::zero();
    fr_t last = fr_t::zero();
    for (uint32_t c = 0; c < g.ncalc; c++) {
        const RawCalculation calc = g.calcs[c];
        fr_t v;
        switch (calc.op) {
        case 0:
            v = source_value<MAX>(calc.lhs, g, p, idx, inter, prev) + source_value<MAX>(calc.rhs, g, p, idx, inter, prev);
            break;
        case 1:
            v = source_value<MAX>(calc.lhs, g, p, idx, inter, prev) - source_value<MAX>(calc.rhs, g, p, idx, inter, prev);
            break;
        case 2:
            v = source_value<MAX>(calc.lhs, g, p, idx, inter, prev) * source_value<MAX>(calc.rhs, g, p, idx, inter, prev);
            break;
        case 3:
            v = source_value<MAX>(calc.lhs, g, p, idx, inter, prev).sqr();
            break;
        case 4:
            v = source_value<MAX>(calc.lhs, g, p, idx, inter, prev).dbl();
            break;
        case 5:
            v = -source_value<MAX>(calc.lhs, g, p, idx, inter, prev);
            break;
        case 6: {
            fr_t factor = source_value<MAX>(calc.rhs, g, p, idx, inter, prev);
            v = source_value<MAX>(calc.lhs, g, p, idx, inter, prev);
            for (uint32_t k = 0; k < calc.parts_len; k++) {
                uint32_t pi = calc.parts_offset + k;
                fr_t part = pi < g.nparts ? source_value<MAX>(g.parts[pi], g, p, idx, inter, prev) : fr_t::zero();
                v = v * factor + part;
            }
            break;
        }
        case 7:
            v = source_value<MAX>(calc.lhs, g, p, idx, inter, prev);
            break;
        default:
            v = fr_t::zero();
            break;
        }
        if (calc.target < MAX) inter[calc.target] = v;
        last = v;
    }
    return last;
}

template <int MAX>
__global__ void numerator_kernel(num_params p)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= p.len) return;
    const fr_t one = fr_t::one();
    const fr_t zero = fr_t::zero();
    fr_t value = p.run_custom ? evaluate_graph<MAX>(p.custom, p, idx, zero) : p.initial[idx];

    if (p.perm_sets && p.chunk_len) {
        // permutation argument (evaluation.rs:3282-3352)
        const size_t len = p.len;
        const size_t r_next = rot_index(idx, 1, p.rot_scale, len);
        const size_t r_last = rot_index(idx, p.last_rotation, p.rot_scale, len);
        const fr_t *first = p.perm_products;
        const fr_t *lastp = p.perm_products + (p.perm_sets - 1) * len;
        const fr_t l0 = p.l0[idx];
        value = value * p.y + (one - first[idx]) * l0;
        value = value * p.y + (lastp[idx].sqr() - lastp[idx]) * p.l_last[idx];
        for (size_t s = 1; s < p.perm_sets; s++)
            value = value * p.y + (p.perm_products[s * len + idx] - p.perm_products[(s - 1) * len + r_last]) * l0;
        fr_t delta = p.delta_start * p.omega_powers[idx];
        const fr_t l_active = p.l_active[idx];
        for (size_t s = 0; s < p.perm_sets; s++) {
            const fr_t *prod = p.perm_products + s * len;
            fr_t left = prod[r_next];
            fr_t right = prod[idx];
            const size_t base = s * p.chunk_len;
            for (uint32_t j = 0; j < p.chunk_len && base + j < p.perm_columns_len; j++) {
                const RawColumnRef ref = p.perm_columns[base + j];
                const fr_t *col = column_base(p, ref.kind, ref.index);
                if (!col) continue;
                const fr_t v = col[idx];
                left = left * (v + p.beta * p.perm_pk_cosets[(base + j) * len + idx] + p.gamma);
                right = right * (v + delta + p.gamma);
                delta = delta * p.delta_const;
            }
            value = value * p.y + (left - right) * l_active;
        }
    }

    for (size_t n = 0; n < p.lookup_count; n++) {
        // lookup argument (evaluation.rs:3408-3472)
        const size_t len = p.len;
        const size_t r_next = rot_index(idx, 1, p.rot_scale, len);
        const size_t r_prev = rot_index(idx, -1, p.rot_scale, len);
        const fr_t *prod = p.lk_product + n * len;
        const fr_t *pin = p.lk_input + n * p.lk_stride;
        const fr_t *ptab = p.lk_table + n * p.lk_stride;
        const fr_t table_value = evaluate_graph<MAX>(p.lookup_graphs[n], p, idx, zero);
        const fr_t a_minus_s = pin[idx] - ptab[idx];
        const fr_t l0 = p.l0[idx], l_active = p.l_active[idx];
        value = value * p.y + (one - prod[idx]) * l0;
        value = value * p.y + (prod[idx].sqr() - prod[idx]) * p.l_last[idx];
        value = value * p.y +
                (prod[r_next] * (pin[idx] + p.beta) * (ptab[idx] + p.gamma) - prod[idx] * table_value) * l_active;
        value = value * p.y + a_minus_s * l0;
        value = value * p.y + a_minus_s * (pin[idx] - pin[r_prev]) * l_active;
    }

    for (size_t n = 0; n < p.trash_count; n++) {
        // trash argument (evaluation.rs:3489-3521)
        const uint32_t sel = p.trash_sel[n];
        if (sel >= p.fixed_cols) continue;
        const fr_t compressed = evaluate_graph<MAX>(p.trash_graphs[n], p, idx, zero);
        const fr_t q = p.fixed[(size_t)sel * p.len + idx];
        value = value * p.y + (compressed - (one - q) * p.trash_cosets[n * p.len + idx]);
    }
    p.out[idx] = value;
}

template <int MAX>
__global__ void graph_batch_kernel(num_params p, fr_t *out)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= p.len) return;
    out[idx] = evaluate_graph<MAX>(p.custom, p, idx, fr_t::zero());
}

// ---------------------------------------------------------------- host

struct graph_upload {
    dev_buf<fr_t> constants;
    dev_buf<int32_t> rotations;
    dev_buf<RawCalculation> calcs;
    dev_buf<RawValueSource> parts;
    dgraph g{};
};

static void upload_graph(graph_upload &u, const RawGraph &raw, cudaStream_t s)
{
    if ((raw.constants_len && !raw.constants) || (raw.rotations_len && !raw.rotations) ||
        (raw.calculations_len && !raw.calculations) || (raw.horner_parts_len && !raw.horner_parts))
        throw cuda_error((int)cudaErrorInvalidValue, "graph arrays missing");
    u.constants = dev_buf<fr_t>(raw.constants_len, s);
    u.rotations = dev_buf<int32_t>(raw.rotations_len, s);
    u.calcs = dev_buf<RawCalculation>(raw.calculations_len, s);
    u.parts = dev_buf<RawValueSource>(raw.horner_parts_len, s);
    h2d(u.constants, raw.constants, raw.constants_len * sizeof(fr_t), s);
    h2d(u.rotations, raw.rotations, raw.rotations_len * sizeof(int32_t), s);
    h2d(u.calcs, raw.calculations, raw.calculations_len * sizeof(RawCalculation), s);
    h2d(u.parts, raw.horner_parts, raw.horner_parts_len * sizeof(RawValueSource), s);
    u.g.constants = u.constants;
    u.g.nconst = (uint32_t)raw.constants_len;
    u.g.rotations = u.rotations;
    u.g.nrot = (uint32_t)raw.rotations_len;
    u.g.calcs = u.calcs;
    u.g.ncalc = (uint32_t)raw.calculations_len;
    u.g.parts = u.parts;
    u.g.nparts = (uint32_t)raw.horner_parts_len;
    u.g.ninter = raw.num_intermediates;
}

static int capacity_for(uint32_t n)
{
    if (n <= 16) return 16;
    if (n <= 64) return 64;
    if (n <= 256) return 256;
    return 0;
}

template <class F16, class F64, class F256>
static void launch_by_capacity(int cap, F16 f16, F64 f64, F256 f256)
{
    if (cap == 16) f16();
    else if (cap == 64) f64();
    else if (cap == 256) f256();
    else throw cuda_error((int)cudaErrorInvalidValue, "graph needs more than 256 intermediates");
}

static dev_buf<fr_t> upload_fr(const RawFr *h, size_t n, cudaStream_t s)
{
    dev_buf<fr_t> d(n, s);
    h2d(d, h, n * sizeof(fr_t), s);
    return d;
}


// graph_count graphs over device columns into d_out [graph_count][len];
// challenges are a host array
static void graph_batch_core(fr_t *d_out, size_t len, const fr_t *fixed, size_t fixed_cols, const fr_t *advice,
                             size_t advice_cols, const fr_t *instance, size_t instance_cols, const RawFr *challenges,
                             size_t challenge_len, RawFr beta, RawFr gamma, RawFr theta, RawFr trash_challenge,
                             RawFr y, int32_t rot_scale, const RawGraph *graphs, size_t graph_count, cudaStream_t s)
{
    num_params p{};
    p.len = len;
    p.rot_scale = rot_scale;
    auto d_chal = upload_fr(challenges, challenge_len, s);
    p.fixed = fixed;
    p.fixed_cols = fixed_cols;
    p.advice = advice;
    p.advice_cols = advice_cols;
    p.instance = instance;
    p.instance_cols = instance_cols;
    p.challenges = d_chal;
    p.challenge_len = challenge_len;
    p.beta = from_raw(beta);
    p.gamma = from_raw(gamma);
    p.theta = from_raw(theta);
    p.trash = from_raw(trash_challenge);
    p.y = from_raw(y);
    std::vector<graph_upload> up(graph_count);
    const unsigned grid = blocks_for(len, 128);
    for (size_t gi = 0; gi < graph_count; gi++) {
        upload_graph(up[gi], graphs[gi], s);
        p.custom = up[gi].g;
        fr_t *o = d_out + gi * len;
        launch_by_capacity(
            capacity_for(graphs[gi].num_intermediates), [&] { graph_batch_kernel<16><<<grid, 128, 0, s>>>(p, o); },
            [&] { graph_batch_kernel<64><<<grid, 128, 0, s>>>(p, o); },
            [&] { graph_batch_kernel<256><<<grid, 128, 0, s>>>(p, o); });
        GB_CHECK_LAUNCH();
    }
}

// Device pointers of one numerator evaluation; graphs still in host memory.
struct numerator_inputs {
    size_t len;
    const fr_t *fixed, *advice, *instance, *challenges, *initial;
    size_t fixed_cols, advice_cols, instance_cols, challenge_len;
    const fr_t *l0, *l_last, *l_active;
    const fr_t *perm_products, *perm_pk;
    size_t perm_sets;
    const RawColumnRef *perm_columns;  // host
    size_t perm_columns_len, perm_pk_len;
    const fr_t *lk_product, *lk_input, *lk_table;
    size_t lk_stride, lookup_count;
    const fr_t *trash_cosets;
    const uint32_t *trash_sel;  // host
    size_t trash_count;
    uint32_t run_custom;
    const RawGraph *custom_graph, *lookup_graphs, *trash_graphs;  // host
};

static void numerator_core(fr_t *d_out, const numerator_inputs &in, RawFr beta, RawFr gamma, RawFr theta,
                           RawFr trash_challenge, RawFr y, RawFr omega, RawFr delta_start, RawFr delta_const,
                           int32_t rot_scale, int32_t last_rotation, uint32_t chunk_len, cudaStream_t s)
{
    const size_t len = in.len;
    num_params p{};
    p.out = d_out;
    p.len = len;
    p.rot_scale = rot_scale;
    p.fixed = in.fixed;
    p.fixed_cols = in.fixed_cols;
    p.advice = in.advice;
    p.advice_cols = in.advice_cols;
    p.instance = in.instance;
    p.instance_cols = in.instance_cols;
    p.challenges = in.challenges;
    p.challenge_len = in.challenge_len;
    p.beta = from_raw(beta);
    p.gamma = from_raw(gamma);
    p.theta = from_raw(theta);
    p.trash = from_raw(trash_challenge);
    p.y = from_raw(y);
    p.run_custom = in.run_custom ? 1 : 0;
    p.initial = in.initial;
    uint32_t max_inter = in.run_custom ? in.custom_graph->num_intermediates : 0;
    graph_upload custom;
    if (in.run_custom) upload_graph(custom, *in.custom_graph, s);
    p.custom = custom.g;
    p.l0 = in.l0;
    p.l_last = in.l_last;
    p.l_active = in.l_active;
    dev_buf<RawColumnRef> d_pcols(in.perm_columns_len, s);
    h2d(d_pcols, in.perm_columns, in.perm_columns_len * sizeof(RawColumnRef), s);
    dev_buf<fr_t> d_omega(in.perm_sets ? len : 0, s);
    if (in.perm_sets) omega_powers(d_omega, from_raw(omega), len, s);
    p.perm_sets = in.perm_sets;
    p.perm_products = in.perm_products;
    p.perm_columns = d_pcols;
    p.perm_columns_len = in.perm_columns_len;
    p.perm_pk_cosets = in.perm_pk;
    p.omega_powers = d_omega;
    p.delta_start = from_raw(delta_start);
    p.delta_const = from_raw(delta_const);
    p.last_rotation = last_rotation;
    p.chunk_len = chunk_len;
    std::vector<graph_upload> lk(in.lookup_count), tr(in.trash_count);
    std::vector<dgraph> lkg(in.lookup_count), trg(in.trash_count);
    for (size_t i = 0; i < in.lookup_count; i++) {
        upload_graph(lk[i], in.lookup_graphs[i], s);
        lkg[i] = lk[i].g;
        max_inter = std::max(max_inter, in.lookup_graphs[i].num_intermediates);
    }
    for (size_t i = 0; i < in.trash_count; i++) {
        upload_graph(tr[i], in.trash_graphs[i], s);
        trg[i] = tr[i].g;
        max_inter = std::max(max_inter, in.trash_graphs[i].num_intermediates);
    }
    dev_buf<dgraph> d_lkg(in.lookup_count, s), d_trg(in.trash_count, s);
    h2d(d_lkg, lkg.data(), in.lookup_count * sizeof(dgraph), s);
    h2d(d_trg, trg.data(), in.trash_count * sizeof(dgraph), s);
    p.lookup_count = in.lookup_count;
    p.lk_product = in.lk_product;
    p.lk_input = in.lk_input;
    p.lk_table = in.lk_table;
    p.lk_stride = in.lk_stride;
    p.lookup_graphs = d_lkg;
    dev_buf<uint32_t> d_tsel(in.trash_count, s);
    h2d(d_tsel, in.trash_sel, in.trash_count * sizeof(uint32_t), s);
    p.trash_count = in.trash_count;
    p.trash_cosets = in.trash_cosets;
    p.trash_sel = d_tsel;
    p.trash_graphs = d_trg;
    const unsigned grid = blocks_for(len, 128);
    launch_by_capacity(
        capacity_for(max_inter), [&] { numerator_kernel<16><<<grid, 128, 0, s>>>(p); },
        [&] { numerator_kernel<64><<<grid, 128, 0, s>>>(p); }, [&] { numerator_kernel<256><<<grid, 128, 0, s>>>(p); });
    GB_CHECK_LAUNCH();
    // the graph and column-reference buffers are released in stream order
    // after the launch; the caller's stream keeps the kernel ahead of them
}

static const fr_t *vec_values(const void *v, size_t need, const char *what)
{
    if (!need) return nullptr;
    if (!v) throw cuda_error((int)cudaErrorInvalidValue, what);
    auto *dv = reinterpret_cast<const fr_device_vec *>(v);
    if (dv->len < need) throw cuda_error((int)cudaErrorInvalidValue, what);
    return dv->values;
}

}  // namespace gb

using namespace gb;

extern "C" {

RustError midnight_sppark_bls12_381_eval_numerator(
    RawFr *out_raw, size_t len, const RawFr *initial_out, uint32_t run_custom, const RawFr *fixed, size_t fixed_cols,
    const RawFr *advice, size_t advice_cols, const RawFr *instance, size_t instance_cols, const RawFr *challenges,
    size_t challenge_len, RawFr beta, RawFr gamma, RawFr theta, RawFr trash_challenge, RawFr y, RawFr omega,
    RawFr delta_start, RawFr delta_const, int32_t rot_scale, int32_t last_rotation, uint32_t chunk_len,
    const RawFr *l0, const RawFr *l_last, const RawFr *l_active, const RawFr *permutation_products,
    size_t permutation_sets, const RawColumnRef *permutation_columns, size_t permutation_columns_len,
    const RawFr *permutation_pk_cosets, size_t permutation_pk_cosets_len, const RawFr *lookup_product_cosets,
    const RawFr *lookup_input_cosets, const RawFr *lookup_table_cosets, size_t lookup_count,
    const RawFr *trash_cosets, const uint32_t *trash_selector_fixed_indices, size_t trash_count,
    RawGraph custom_graph, const RawGraph *lookup_graphs, const RawGraph *trash_graphs)
{
    if (len == 0) return ok();
    if (!out_raw) return make_error((int)cudaErrorInvalidValue, "null numerator output");
    if (!run_custom && !initial_out)
        return make_error((int)cudaErrorInvalidValue, "initial_out is required when custom evaluation is skipped");
    if ((lookup_count && (!lookup_graphs || !lookup_product_cosets || !lookup_input_cosets || !lookup_table_cosets)) ||
        (trash_count && (!trash_graphs || !trash_cosets || !trash_selector_fixed_indices)) ||
        (permutation_sets && (!permutation_products || !l0 || !l_last || !l_active)) ||
        (lookup_count && (!l0 || !l_last || !l_active)))
        return make_error((int)cudaErrorInvalidValue, "invalid numerator arguments");
    if (permutation_sets && permutation_pk_cosets_len < permutation_columns_len)
        return make_error((int)cudaErrorInvalidValue, "fewer permutation cosets than permutation columns");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    dev_buf<fr_t> d_out(len, s);
    auto d_fixed = upload_fr(fixed, fixed_cols * len, s);
    auto d_advice = upload_fr(advice, advice_cols * len, s);
    auto d_instance = upload_fr(instance, instance_cols * len, s);
    auto d_chal = upload_fr(challenges, challenge_len, s);
    dev_buf<fr_t> d_init;
    if (!run_custom) d_init = upload_fr(initial_out, len, s);
    const bool lagrange = permutation_sets || lookup_count;
    auto d_l0 = upload_fr(l0, lagrange ? len : 0, s);
    auto d_llast = upload_fr(l_last, lagrange ? len : 0, s);
    auto d_lact = upload_fr(l_active, lagrange ? len : 0, s);
    auto d_pprod = upload_fr(permutation_products, permutation_sets * len, s);
    auto d_pk = upload_fr(permutation_pk_cosets, permutation_pk_cosets_len * len, s);
    auto d_lprod = upload_fr(lookup_product_cosets, lookup_count * len, s);
    auto d_lin = upload_fr(lookup_input_cosets, lookup_count * len, s);
    auto d_ltab = upload_fr(lookup_table_cosets, lookup_count * len, s);
    auto d_trash = upload_fr(trash_cosets, trash_count * len, s);
    numerator_inputs in{};
    in.len = len;
    in.fixed = d_fixed;
    in.fixed_cols = fixed_cols;
    in.advice = d_advice;
    in.advice_cols = advice_cols;
    in.instance = d_instance;
    in.instance_cols = instance_cols;
    in.challenges = d_chal;
    in.challenge_len = challenge_len;
    in.initial = d_init;
    in.run_custom = run_custom;
    in.l0 = d_l0;
    in.l_last = d_llast;
    in.l_active = d_lact;
    in.perm_products = d_pprod;
    in.perm_sets = permutation_sets;
    in.perm_columns = permutation_columns;
    in.perm_columns_len = permutation_columns_len;
    in.perm_pk = d_pk;
    in.perm_pk_len = permutation_pk_cosets_len;
    in.lk_product = d_lprod;
    in.lk_input = d_lin;
    in.lk_table = d_ltab;
    in.lk_stride = len;
    in.lookup_count = lookup_count;
    in.trash_cosets = d_trash;
    in.trash_sel = trash_selector_fixed_indices;
    in.trash_count = trash_count;
    in.custom_graph = &custom_graph;
    in.lookup_graphs = lookup_graphs;
    in.trash_graphs = trash_graphs;
    numerator_core(d_out, in, beta, gamma, theta, trash_challenge, y, omega, delta_start, delta_const, rot_scale,
                   last_rotation, chunk_len, s);
    d2h(out_raw, d_out, len * sizeof(fr_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
    return ok();
    GB_ENTRY_END
}

// The numerator over resident columns, into a new device vector of len rows.
RustError gb_eval_numerator_device(
    void **out, size_t len, const void *initial_vec, uint32_t run_custom, const void *fixed_vec, size_t fixed_cols,
    const void *advice_vec, size_t advice_cols, const void *instance_vec, size_t instance_cols,
    const RawFr *challenges, size_t challenge_len, RawFr beta, RawFr gamma, RawFr theta, RawFr trash_challenge,
    RawFr y, RawFr omega, RawFr delta_start, RawFr delta_const, int32_t rot_scale, int32_t last_rotation,
    uint32_t chunk_len, const void *lagrange_vec, const void *permutation_products_vec, size_t permutation_sets,
    const RawColumnRef *permutation_columns, size_t permutation_columns_len, const void *permutation_pk_vec,
    size_t permutation_pk_cosets_len, const void *lookup_products_vec, const void *lookup_permuted_vec,
    size_t lookup_count, const void *trash_vec, const uint32_t *trash_selector_fixed_indices, size_t trash_count,
    RawGraph custom_graph, const RawGraph *lookup_graphs, const RawGraph *trash_graphs)
{
    if (!out) return make_error((int)cudaErrorInvalidValue, "null numerator output");
    *out = nullptr;
    if (len == 0) return make_error((int)cudaErrorInvalidValue, "empty numerator domain");
    if ((lookup_count && !lookup_graphs) || (trash_count && (!trash_graphs || !trash_selector_fixed_indices)) ||
        (permutation_columns_len && !permutation_columns) || (challenge_len && !challenges))
        return make_error((int)cudaErrorInvalidValue, "invalid resident numerator arguments");
    if (permutation_sets && permutation_pk_cosets_len < permutation_columns_len)
        return make_error((int)cudaErrorInvalidValue, "fewer permutation cosets than permutation columns");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    for (const void *v : {initial_vec, fixed_vec, advice_vec, instance_vec, lagrange_vec, permutation_products_vec,
                          permutation_pk_vec, lookup_products_vec, lookup_permuted_vec, trash_vec})
        if (v) device_vec_wait(reinterpret_cast<const fr_device_vec *>(v), s);
    const bool lagrange = permutation_sets || lookup_count;
    numerator_inputs in{};
    in.len = len;
    in.run_custom = run_custom;
    in.initial = run_custom ? nullptr : vec_values(initial_vec, len, "initial values missing");
    in.fixed = vec_values(fixed_vec, fixed_cols * len, "fixed cosets too short");
    in.fixed_cols = fixed_cols;
    in.advice = vec_values(advice_vec, advice_cols * len, "advice cosets too short");
    in.advice_cols = advice_cols;
    in.instance = vec_values(instance_vec, instance_cols * len, "instance cosets too short");
    in.instance_cols = instance_cols;
    auto d_chal = upload_fr(challenges, challenge_len, s);
    in.challenges = d_chal;
    in.challenge_len = challenge_len;
    const fr_t *lag = vec_values(lagrange_vec, lagrange ? 3 * len : 0, "l0 | l_last | l_active cosets too short");
    in.l0 = lag;
    in.l_last = lag ? lag + len : nullptr;
    in.l_active = lag ? lag + 2 * len : nullptr;
    in.perm_products = vec_values(permutation_products_vec, permutation_sets * len, "permutation products too short");
    in.perm_sets = permutation_sets;
    in.perm_columns = permutation_columns;
    in.perm_columns_len = permutation_columns_len;
    in.perm_pk = vec_values(permutation_pk_vec, permutation_pk_cosets_len * len, "permutation cosets too short");
    in.perm_pk_len = permutation_pk_cosets_len;
    in.lk_product = vec_values(lookup_products_vec, lookup_count * len, "lookup products too short");
    const fr_t *perm = vec_values(lookup_permuted_vec, 2 * lookup_count * len, "permuted lookup columns too short");
    in.lk_input = perm;
    in.lk_table = perm ? perm + len : nullptr;
    in.lk_stride = 2 * len;
    in.lookup_count = lookup_count;
    in.trash_cosets = vec_values(trash_vec, trash_count * len, "trash cosets too short");
    in.trash_sel = trash_selector_fixed_indices;
    in.trash_count = trash_count;
    in.custom_graph = &custom_graph;
    in.lookup_graphs = lookup_graphs;
    in.trash_graphs = trash_graphs;
    fr_device_vec *v = device_vec_new(len, s);
    try {
        numerator_core(v->values, in, beta, gamma, theta, trash_challenge, y, omega, delta_start, delta_const,
                       rot_scale, last_rotation, chunk_len, s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

RustError midnight_sppark_bls12_381_eval_graph_batch(RawFr *out_raw, size_t len, const RawFr *fixed, size_t fixed_cols,
                                                      const RawFr *advice, size_t advice_cols, const RawFr *instance,
                                                      size_t instance_cols, const RawFr *challenges,
                                                      size_t challenge_len, RawFr beta, RawFr gamma, RawFr theta,
                                                      RawFr trash_challenge, RawFr y, int32_t rot_scale,
                                                      const RawGraph *graphs, size_t graph_count)
{
    if (len == 0 || graph_count == 0) return ok();
    if (!out_raw || !graphs || (fixed_cols && !fixed) || (advice_cols && !advice) || (instance_cols && !instance) ||
        (challenge_len && !challenges))
        return make_error((int)cudaErrorInvalidValue, "invalid graph batch arguments");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto d_fixed = upload_fr(fixed, fixed_cols * len, s);
    auto d_advice = upload_fr(advice, advice_cols * len, s);
    auto d_instance = upload_fr(instance, instance_cols * len, s);
    dev_buf<fr_t> d_out(len * graph_count, s);
    graph_batch_core(d_out, len, d_fixed, fixed_cols, d_advice, advice_cols, d_instance, instance_cols, challenges,
                     challenge_len, beta, gamma, theta, trash_challenge, y, rot_scale, graphs, graph_count, s);
    d2h(out_raw, d_out, len * graph_count * sizeof(fr_t), s);
    GB_CUDA_OK(cudaStreamSynchronize(s));
    return ok();
    GB_ENTRY_END
}

// graph_count graphs over resident columns (len rows each), into a new
// device vector [graph_count][len]
RustError gb_eval_graph_batch_device(void **out, size_t len, const void *fixed_vec, size_t fixed_cols,
                                     const void *advice_vec, size_t advice_cols, const void *instance_vec,
                                     size_t instance_cols, const RawFr *challenges, size_t challenge_len, RawFr beta,
                                     RawFr gamma, RawFr theta, RawFr trash_challenge, RawFr y, int32_t rot_scale,
                                     const RawGraph *graphs, size_t graph_count)
{
    if (!out) return make_error((int)cudaErrorInvalidValue, "null graph batch output");
    *out = nullptr;
    if (len == 0 || graph_count == 0 || !graphs || (challenge_len && !challenges))
        return make_error((int)cudaErrorInvalidValue, "invalid resident graph batch arguments");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    for (const void *v : {fixed_vec, advice_vec, instance_vec})
        if (v) device_vec_wait(reinterpret_cast<const fr_device_vec *>(v), s);
    const fr_t *fx = vec_values(fixed_vec, fixed_cols * len, "fixed columns too short");
    const fr_t *ad = vec_values(advice_vec, advice_cols * len, "advice columns too short");
    const fr_t *in = vec_values(instance_vec, instance_cols * len, "instance columns too short");
    fr_device_vec *v = device_vec_new(len * graph_count, s);
    try {
        graph_batch_core(v->values, len, fx, fixed_cols, ad, advice_cols, in, instance_cols, challenges,
                         challenge_len, beta, gamma, theta, trash_challenge, y, rot_scale, graphs, graph_count, s);
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
