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
#include <functional>
#include <mutex>
#include <memory>
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
    // the same program with its intermediates given slots by liveness
    // (compile_graph): kind-1 sources name a slot, a target of kNoSlot is
    // not stored; nslots = kNoSlot when the graph needs more slots than a
    // block's shared memory holds (the kernels then interpret `calcs`)
    const RawCalculation *ccalcs;
    const RawValueSource *cparts;
    uint32_t nslots;
};

static constexpr uint32_t kNoSlot = 0xffffffffu;
// slots of one row in shared memory: 128 rows a block x 48 slots x 32 B
// = 192 KB at most
static constexpr uint32_t kMaxSlots = 48;
static constexpr unsigned kNumThreads = 128;

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
        return src.a < MAX && src.a < g.ninter ? inter[src.a] : fr_t::zero();
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
        if (calc.target < nint) inter[calc.target] = v;
        last = v;
    }
    return last;
}

// Products of the interpreted graphs go through the out-of-line Fr product:
// one copy of its code instead of one per call site keeps the interpreter's
// loop and the argument terms small enough for the instruction cache.
__device__ __forceinline__ fr_t qmul(const fr_t &a, const fr_t &b)
{
#if defined(__CUDA_ARCH__) && !defined(GB_FP_MUL_INLINE)
    return fr_t::mul_by_value(a, b);
#else
    return a * b;
#endif
}

// A row's slots: slot k of the calling thread at sh[k * blockDim.x].
__device__ __forceinline__ fr_t slot_ld(const fr_t *sh, uint32_t k) { return sh[(size_t)k * blockDim.x]; }
__device__ __forceinline__ void slot_st(fr_t *sh, uint32_t k, const fr_t &v) { sh[(size_t)k * blockDim.x] = v; }

__device__ fr_t source_value_slots(const RawValueSource &src, const dgraph &g, const num_params &p, size_t idx,
                                   const fr_t *sh, const fr_t &prev)
{
    switch (src.kind) {
    case 0:
        return src.a < g.nconst ? g.constants[src.a] : fr_t::zero();
    case 1:
        return slot_ld(sh, src.a);
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

// evaluate_graph over the compiled program: intermediates live in the row's
// shared-memory slots, so nothing goes to local memory
__device__ fr_t evaluate_graph_slots(const dgraph &g, const num_params &p, size_t idx, const fr_t &prev, fr_t *sh)
{
    fr_t last = fr_t::zero();
    for (uint32_t c = 0; c < g.ncalc; c++) {
        const RawCalculation calc = g.ccalcs[c];
        const fr_t a = source_value_slots(calc.lhs, g, p, idx, sh, prev);
        fr_t v;
        switch (calc.op) {
        case 0:
            v = a + source_value_slots(calc.rhs, g, p, idx, sh, prev);
            break;
        case 1:
            v = a - source_value_slots(calc.rhs, g, p, idx, sh, prev);
            break;
        case 2:
            v = qmul(a, source_value_slots(calc.rhs, g, p, idx, sh, prev));
            break;
        case 3:
            v = qmul(a, a);
            break;
        case 4:
            v = a.dbl();
            break;
        case 5:
            v = -a;
            break;
        case 6: {
            const fr_t factor = source_value_slots(calc.rhs, g, p, idx, sh, prev);
            v = a;
            for (uint32_t k = 0; k < calc.parts_len; k++) {
                const uint32_t pi = calc.parts_offset + k;
                const fr_t part = pi < g.nparts ? source_value_slots(g.cparts[pi], g, p, idx, sh, prev) : fr_t::zero();
                v = qmul(v, factor) + part;
            }
            break;
        }
        case 7:
            v = a;
            break;
        default:
            v = fr_t::zero();
            break;
        }
        if (calc.target != kNoSlot) slot_st(sh, calc.target, v);
        last = v;
    }
    return last;
}

// The graph of a row: the compiled program when SLOTS, else the interpreter
// with a local array of MAX intermediates.
template <int MAX, bool SLOTS>
__device__ __forceinline__ fr_t eval_row_graph(const dgraph &g, const num_params &p, size_t idx, const fr_t &prev,
                                               fr_t *sh)
{
    if (SLOTS) return evaluate_graph_slots(g, p, idx, prev, sh);
    return evaluate_graph<MAX>(g, p, idx, prev);
}

template <int MAX, bool SLOTS = false>
__global__ void numerator_kernel(num_params p)
{
    extern __shared__ fr_t num_slots[];
    fr_t *sh = num_slots + threadIdx.x;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= p.len) return;
    const fr_t one = fr_t::one();
    const fr_t zero = fr_t::zero();
    fr_t value = p.run_custom ? eval_row_graph<MAX, SLOTS>(p.custom, p, idx, zero, sh) : p.initial[idx];

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
        const fr_t table_value = eval_row_graph<MAX, SLOTS>(p.lookup_graphs[n], p, idx, zero, sh);
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
        const fr_t compressed = eval_row_graph<MAX, SLOTS>(p.trash_graphs[n], p, idx, zero, sh);
        const fr_t q = p.fixed[(size_t)sel * p.len + idx];
        value = value * p.y + (compressed - (one - q) * p.trash_cosets[n * p.len + idx]);
    }
    p.out[idx] = value;
}

template <int MAX, bool SLOTS = false>
__global__ void graph_batch_kernel(num_params p, fr_t *out)
{
    extern __shared__ fr_t num_slots[];
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= p.len) return;
    out[idx] = eval_row_graph<MAX, SLOTS>(p.custom, p, idx, fr_t::zero(), num_slots + threadIdx.x);
}

// ---------------------------------------------------------------- host

struct graph_upload {
    dev_buf<fr_t> constants;
    dev_buf<int32_t> rotations;
    dev_buf<RawCalculation> calcs, ccalcs;
    dev_buf<RawValueSource> parts, cparts;
    dgraph g{};
};

static int capacity_for(uint32_t n);

// Gives the graph's intermediates slots by liveness, for the slot
// interpreter: every write of an intermediate starts a new value, which
// takes the lowest free slot and holds it until its last read (a value never
// read takes none).  Reads follow the interpreter exactly: an intermediate
// not yet written, or with an index at or above num_intermediates, reads
// zero; a target at or above num_intermediates is not stored.  Operands are
// read before the target is written, so a target may take a slot that one of
// its own operands frees.  Returns the slots used, or kNoSlot if more than
// kMaxSlots would be live at once.
static uint32_t compile_graph(const RawGraph &raw, std::vector<RawCalculation> &out_calcs,
                              std::vector<RawValueSource> &out_parts)
{
    const uint32_t cap = raw.num_intermediates;
    const size_t nc = raw.calculations_len;
    // the sources each calculation reads, as the interpreter reads them
    auto reads = [&](const RawCalculation &c, std::vector<const RawValueSource *> &r) {
        r.clear();
        switch (c.op) {
        case 0: case 1: case 2: r.push_back(&c.lhs); r.push_back(&c.rhs); break;
        case 3: case 4: case 5: case 7: r.push_back(&c.lhs); break;
        case 6:
            r.push_back(&c.rhs);
            r.push_back(&c.lhs);
            for (uint32_t k = 0; k < c.parts_len; k++) {
                const uint64_t pi = (uint64_t)c.parts_offset + k;
                if (pi < raw.horner_parts_len) r.push_back(&raw.horner_parts[pi]);
            }
            break;
        default: break;
        }
    };
    // pass 1: versions and their last reads
    std::vector<int64_t> cur(cap, -1), last_read;
    std::vector<int64_t> ver_of(nc, -1);
    std::vector<const RawValueSource *> r;
    for (size_t c = 0; c < nc; c++) {
        const RawCalculation &calc = raw.calculations[c];
        reads(calc, r);
        for (const RawValueSource *v : r)
            if (v->kind == 1 && v->a < cap && cur[v->a] >= 0) last_read[cur[v->a]] = (int64_t)c;
        if (calc.target < cap) {
            ver_of[c] = (int64_t)last_read.size();
            cur[calc.target] = ver_of[c];
            last_read.push_back(-1);
        }
    }
    // pass 2: slots
    std::fill(cur.begin(), cur.end(), -1);
    std::vector<uint32_t> slot_of(last_read.size(), kNoSlot);
    std::vector<uint32_t> free_slots;  // a min-heap by slot number
    uint32_t nslots = 0;
    auto take = [&]() {
        if (free_slots.empty()) return nslots++;
        std::pop_heap(free_slots.begin(), free_slots.end(), std::greater<uint32_t>());
        const uint32_t k = free_slots.back();
        free_slots.pop_back();
        return k;
    };
    auto give = [&](uint32_t k) {
        free_slots.push_back(k);
        std::push_heap(free_slots.begin(), free_slots.end(), std::greater<uint32_t>());
    };
    auto map_src = [&](const RawValueSource &v) {
        RawValueSource o = v;
        if (v.kind == 1) {
            if (v.a < cap && cur[v.a] >= 0) {
                o.a = slot_of[cur[v.a]];
            } else {
                o.kind = 0;  // reads zero: an out-of-range constant index
                o.a = kNoSlot;
            }
        }
        return o;
    };
    out_calcs.resize(nc);
    out_parts.clear();
    for (size_t c = 0; c < nc; c++) {
        const RawCalculation &calc = raw.calculations[c];
        RawCalculation o = calc;
        o.lhs = map_src(calc.lhs);
        o.rhs = map_src(calc.rhs);
        if (calc.op == 6) {
            o.parts_offset = (uint32_t)out_parts.size();
            for (uint32_t k = 0; k < calc.parts_len; k++) {
                const uint64_t pi = (uint64_t)calc.parts_offset + k;
                if (pi < raw.horner_parts_len) {
                    out_parts.push_back(map_src(raw.horner_parts[pi]));
                } else {
                    RawValueSource z{0, kNoSlot, 0};
                    out_parts.push_back(z);
                }
            }
        }
        // values whose last read is this calculation free their slots
        reads(calc, r);
        std::vector<int64_t> done;
        for (const RawValueSource *v : r)
            if (v->kind == 1 && v->a < cap && cur[v->a] >= 0 && last_read[cur[v->a]] == (int64_t)c)
                done.push_back(cur[v->a]);
        std::sort(done.begin(), done.end());
        done.erase(std::unique(done.begin(), done.end()), done.end());
        for (int64_t v : done) give(slot_of[v]);
        o.target = kNoSlot;
        if (ver_of[c] >= 0) {
            const int64_t v = ver_of[c];
            if (last_read[v] >= 0) {
                slot_of[v] = take();
                o.target = slot_of[v];
            }
            cur[calc.target] = v;
        }
        out_calcs[c] = o;
    }
    return nslots > kMaxSlots ? kNoSlot : nslots;
}

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
    u.g.nslots = kNoSlot;
    if (capacity_for(raw.num_intermediates)) {
        std::vector<RawCalculation> cc;
        std::vector<RawValueSource> cp;
        const uint32_t ns = compile_graph(raw, cc, cp);
        if (ns != kNoSlot) {
            u.ccalcs = dev_buf<RawCalculation>(cc.size(), s);
            u.cparts = dev_buf<RawValueSource>(cp.size(), s);
            h2d(u.ccalcs, cc.data(), cc.size() * sizeof(RawCalculation), s);
            h2d(u.cparts, cp.data(), cp.size() * sizeof(RawValueSource), s);
            u.g.ccalcs = u.ccalcs;
            u.g.cparts = u.cparts;
            u.g.nslots = ns;
        }
    }
}

// the slot count a launch over these graphs needs: kNoSlot when one of them
// could not be compiled
static uint32_t slots_for(uint32_t acc, const dgraph &g)
{
    return acc == kNoSlot || g.nslots == kNoSlot ? kNoSlot : std::max(acc, g.nslots);
}

static void set_slot_smem()
{
    static std::once_flag once;
    std::call_once(once, [] {
        const int bytes = (int)(kNumThreads * kMaxSlots * sizeof(fr_t));
        cudaFuncSetAttribute(numerator_kernel<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cudaFuncSetAttribute(graph_batch_kernel<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    });
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


// one launch per graph, graph gi (device-resident, its descriptor on the
// host) into d_out + gi * p.len; p carries the columns and challenges
static void graph_batch_launch(fr_t *d_out, num_params p, const dgraph *graphs, size_t graph_count, cudaStream_t s)
{
    set_slot_smem();
    const unsigned grid = blocks_for(p.len, kNumThreads);
    for (size_t gi = 0; gi < graph_count; gi++) {
        p.custom = graphs[gi];
        fr_t *o = d_out + gi * p.len;
        if (graphs[gi].nslots != kNoSlot) {
            const size_t smem = (size_t)kNumThreads * graphs[gi].nslots * sizeof(fr_t);
            graph_batch_kernel<16, true><<<grid, kNumThreads, smem, s>>>(p, o);
        } else {
            launch_by_capacity(
                capacity_for(graphs[gi].ninter), [&] { graph_batch_kernel<16><<<grid, kNumThreads, 0, s>>>(p, o); },
                [&] { graph_batch_kernel<64><<<grid, kNumThreads, 0, s>>>(p, o); },
                [&] { graph_batch_kernel<256><<<grid, kNumThreads, 0, s>>>(p, o); });
        }
        GB_CHECK_LAUNCH();
    }
}

// the numerator kernel: the slot interpreter when every graph compiled
// (max_slots != kNoSlot), else the local-array interpreter sized for
// max_inter intermediates per row
static void numerator_launch(const num_params &p, uint32_t max_inter, uint32_t max_slots, cudaStream_t s)
{
    set_slot_smem();
    const unsigned grid = blocks_for(p.len, kNumThreads);
    if (max_slots != kNoSlot) {
        numerator_kernel<16, true><<<grid, kNumThreads, (size_t)kNumThreads * max_slots * sizeof(fr_t), s>>>(p);
    } else {
        launch_by_capacity(
            capacity_for(max_inter), [&] { numerator_kernel<16><<<grid, kNumThreads, 0, s>>>(p); },
            [&] { numerator_kernel<64><<<grid, kNumThreads, 0, s>>>(p); },
            [&] { numerator_kernel<256><<<grid, kNumThreads, 0, s>>>(p); });
    }
    GB_CHECK_LAUNCH();
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
    std::vector<dgraph> dg(graph_count);
    for (size_t gi = 0; gi < graph_count; gi++) {
        upload_graph(up[gi], graphs[gi], s);
        dg[gi] = up[gi].g;
    }
    graph_batch_launch(d_out, p, dg.data(), graph_count, s);
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
    uint32_t max_slots = 0;
    graph_upload custom;
    if (in.run_custom) {
        upload_graph(custom, *in.custom_graph, s);
        max_slots = slots_for(max_slots, custom.g);
    }
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
        max_slots = slots_for(max_slots, lkg[i]);
    }
    for (size_t i = 0; i < in.trash_count; i++) {
        upload_graph(tr[i], in.trash_graphs[i], s);
        trg[i] = tr[i].g;
        max_inter = std::max(max_inter, in.trash_graphs[i].num_intermediates);
        max_slots = slots_for(max_slots, trg[i]);
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
    numerator_launch(p, max_inter, max_slots, s);
    // the graph and column-reference buffers are released in stream order
    // after the launch; the caller's stream keeps the kernel ahead of them
}

// Resident numerator state of one circuit (numerator_context_t,
// bls12_381_g1_msm.cu:1116 and :5517-5660): the fixed columns as extended
// cosets and as Lagrange values, l0 / l_last / l_active, the permutation
// columns with their sigma cosets and Lagrange values, omega^i over the
// extended domain and every graph uploaded once.  Read-only once created, so
// calls from several lanes may share it.
struct numerator_context {
    cudaStream_t owner = nullptr;
    size_t len = 0, input_len = 0, fixed_cols = 0, perm_columns_len = 0, perm_pk_len = 0;
    size_t lookup_count = 0, trash_count = 0;
    int32_t rot_scale = 1, last_rotation = 0;
    uint32_t chunk_len = 0, max_inter = 0, max_slots = 0;
    fr_t g_coset, delta_const, trace_omega;
    dev_buf<fr_t> fixed, fixed_lagrange, l0, l_last, l_active, pk_cosets, pk_lagrange, omega_pows;
    std::vector<RawColumnRef> perm_columns;
    dev_buf<RawColumnRef> d_perm_columns;
    dev_buf<uint32_t> d_trash_sel;
    graph_upload custom;
    std::vector<graph_upload> lookup, lookup_input, lookup_table, trash;
    std::vector<dgraph> lookup_input_g, lookup_table_g, trash_g;  // descriptors, host copies
    dev_buf<dgraph> d_lookup, d_trash;
};

static void upload_graphs(std::vector<graph_upload> &up, std::vector<dgraph> &desc, const RawGraph *graphs, size_t n,
                          cudaStream_t s)
{
    up = std::vector<graph_upload>(n);
    desc.resize(n);
    for (size_t i = 0; i < n; i++) {
        upload_graph(up[i], graphs[i], s);
        desc[i] = up[i].g;
    }
}

// the Lagrange-basis column a permutation column reference names, over the
// context's input domain; nullptr when out of range
static const fr_t *lagrange_column(const numerator_context &c, const RawColumnRef &ref, const fr_t *advice,
                                   size_t advice_cols, const fr_t *instance, size_t instance_cols)
{
    const size_t n = c.input_len;
    if (ref.kind == 0) return ref.index < c.fixed_cols ? c.fixed_lagrange.get() + (size_t)ref.index * n : nullptr;
    if (ref.kind == 1) return ref.index < advice_cols ? advice + (size_t)ref.index * n : nullptr;
    if (ref.kind == 2) return ref.index < instance_cols ? instance + (size_t)ref.index * n : nullptr;
    return nullptr;
}

// advice / instance device vectors of at least cols * n values
static const fr_t *trace_values(const void *v, size_t cols, size_t n, cudaStream_t s, const char *what)
{
    if (!cols) return nullptr;
    auto *dv = reinterpret_cast<const fr_device_vec *>(v);
    if (!dv || dv->len < cols * n) throw cuda_error((int)cudaErrorInvalidValue, what);
    device_vec_wait(dv, s);
    return dv->values;
}

// num_params over the context's Lagrange-basis fixed columns and the trace's
// advice / instance values (input_len rows, rotations unscaled), with every
// challenge but the named ones zero
static num_params trace_params(const numerator_context &c, const fr_t *advice, size_t advice_cols,
                               const fr_t *instance, size_t instance_cols, const fr_t *d_chal, size_t challenge_len)
{
    num_params p{};
    p.len = c.input_len;
    p.rot_scale = 1;
    p.fixed = c.fixed_lagrange;
    p.fixed_cols = c.fixed_cols;
    p.advice = advice;
    p.advice_cols = advice_cols;
    p.instance = instance;
    p.instance_cols = instance_cols;
    p.challenges = d_chal;
    p.challenge_len = challenge_len;
    p.beta = p.gamma = p.theta = p.trash = p.y = fr_t::zero();
    return p;
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
    lane_sync(s);
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

// bls12_381_g1_msm.cu:5517-5660: the circuit's fixed data resident once,
// for numerator evaluations and the trace-context calls below.
RustError midnight_sppark_bls12_381_numerator_context_create(
    void **out, size_t len, size_t input_len, const RawFr *fixed, const RawFr *fixed_lagrange, size_t fixed_cols,
    const RawFr *l0, const RawFr *l_last, const RawFr *l_active, const RawColumnRef *permutation_columns,
    size_t permutation_columns_len, const RawFr *permutation_pk_cosets, const RawFr *permutation_pk_lagrange,
    size_t permutation_pk_cosets_len, const uint32_t *trash_selector_fixed_indices, size_t trash_count,
    RawGraph custom_graph, const RawGraph *lookup_graphs, const RawGraph *lookup_input_graphs,
    const RawGraph *lookup_table_graphs, size_t lookup_count, const RawGraph *trash_graphs, RawFr omega,
    RawFr trace_omega, RawFr g_coset, RawFr delta_const, int32_t rot_scale, int32_t last_rotation,
    uint32_t chunk_len)
{
    if (!out || len == 0 || input_len == 0 || !l0 || !l_last || !l_active)
        return make_error((int)cudaErrorInvalidValue, "invalid numerator context arguments");
    if ((fixed_cols && (!fixed || !fixed_lagrange)) || (permutation_columns_len && !permutation_columns) ||
        (permutation_pk_cosets_len && (!permutation_pk_cosets || !permutation_pk_lagrange)) ||
        (lookup_count && (!lookup_graphs || !lookup_input_graphs || !lookup_table_graphs)) ||
        (trash_count && (!trash_graphs || !trash_selector_fixed_indices)))
        return make_error((int)cudaErrorInvalidValue, "missing numerator context data");
    *out = nullptr;
    if (permutation_pk_cosets_len < permutation_columns_len)
        return make_error((int)cudaErrorInvalidValue, "fewer permutation cosets than permutation columns");
    for (size_t i = 0; i < trash_count; i++)
        if (trash_selector_fixed_indices[i] >= fixed_cols)
            return make_error((int)cudaErrorInvalidValue, "trash selector is not a fixed column");
    if (fixed_cols > SIZE_MAX / len || permutation_pk_cosets_len > SIZE_MAX / len)
        return make_error((int)cudaErrorInvalidValue, "numerator context size overflow");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    auto c = std::make_unique<numerator_context>();
    c->owner = s;
    c->len = len;
    c->input_len = input_len;
    c->fixed_cols = fixed_cols;
    c->perm_columns_len = permutation_columns_len;
    c->perm_pk_len = permutation_pk_cosets_len;
    c->lookup_count = lookup_count;
    c->trash_count = trash_count;
    c->rot_scale = rot_scale;
    c->last_rotation = last_rotation;
    c->chunk_len = chunk_len;
    c->g_coset = from_raw(g_coset);
    c->delta_const = from_raw(delta_const);
    c->trace_omega = from_raw(trace_omega);
    c->fixed = upload_fr(fixed, fixed_cols * len, s);
    c->fixed_lagrange = upload_fr(fixed_lagrange, fixed_cols * input_len, s);
    c->l0 = upload_fr(l0, len, s);
    c->l_last = upload_fr(l_last, len, s);
    c->l_active = upload_fr(l_active, len, s);
    c->pk_cosets = upload_fr(permutation_pk_cosets, permutation_pk_cosets_len * len, s);
    c->pk_lagrange = upload_fr(permutation_pk_lagrange, permutation_pk_cosets_len * input_len, s);
    c->perm_columns.assign(permutation_columns, permutation_columns + permutation_columns_len);
    c->d_perm_columns = dev_buf<RawColumnRef>(permutation_columns_len, s);
    h2d(c->d_perm_columns, permutation_columns, permutation_columns_len * sizeof(RawColumnRef), s);
    c->d_trash_sel = dev_buf<uint32_t>(trash_count, s);
    h2d(c->d_trash_sel, trash_selector_fixed_indices, trash_count * sizeof(uint32_t), s);
    c->omega_pows = dev_buf<fr_t>(len, s);
    omega_powers(c->omega_pows, from_raw(omega), len, s);
    upload_graph(c->custom, custom_graph, s);
    c->max_inter = custom_graph.num_intermediates;
    std::vector<dgraph> lookup_g;
    upload_graphs(c->lookup, lookup_g, lookup_graphs, lookup_count, s);
    upload_graphs(c->lookup_input, c->lookup_input_g, lookup_input_graphs, lookup_count, s);
    upload_graphs(c->lookup_table, c->lookup_table_g, lookup_table_graphs, lookup_count, s);
    upload_graphs(c->trash, c->trash_g, trash_graphs, trash_count, s);
    for (const dgraph &g : lookup_g) c->max_inter = std::max(c->max_inter, g.ninter);
    for (const dgraph &g : c->trash_g) c->max_inter = std::max(c->max_inter, g.ninter);
    c->max_slots = slots_for(0, c->custom.g);
    for (const dgraph &g : lookup_g) c->max_slots = slots_for(c->max_slots, g);
    for (const dgraph &g : c->trash_g) c->max_slots = slots_for(c->max_slots, g);
    if (!capacity_for(c->max_inter))
        return make_error((int)cudaErrorInvalidValue, "graph needs more than 256 intermediates");
    c->d_lookup = dev_buf<dgraph>(lookup_count, s);
    h2d(c->d_lookup, lookup_g.data(), lookup_count * sizeof(dgraph), s);
    c->d_trash = dev_buf<dgraph>(trash_count, s);
    h2d(c->d_trash, c->trash_g.data(), trash_count * sizeof(dgraph), s);
    lane_sync(s);
    *out = c.release();
    return ok();
    GB_ENTRY_END
}

// Evaluations issued on any lane may still read the context: the whole
// device is drained before its buffers go.
void midnight_sppark_bls12_381_numerator_context_free(void *context)
{
    auto *c = reinterpret_cast<numerator_context *>(context);
    if (!c) return;
    cudaDeviceSynchronize();
    delete c;
}

// bls12_381_g1_msm.cu:5968-6162: the numerator over one resident column
// vector (each group of columns a run of len-row columns at its offset),
// into a new device vector of len rows.
RustError midnight_sppark_bls12_381_numerator_context_eval(
    void **out, const void *raw_context, const void *raw_columns, size_t total_columns, size_t advice_offset,
    size_t advice_cols, size_t instance_offset, size_t instance_cols, const RawFr *challenges, size_t challenge_len,
    RawFr beta, RawFr gamma, RawFr theta, RawFr trash_challenge, RawFr y, size_t permutation_offset,
    size_t permutation_sets, size_t lookup_product_offset, size_t lookup_input_offset, size_t lookup_table_offset,
    size_t lookup_count, size_t trash_offset, size_t trash_count)
{
    if (!out || !raw_context || (challenge_len && !challenges))
        return make_error((int)cudaErrorInvalidValue, "invalid numerator evaluation arguments");
    *out = nullptr;
    const auto *c = reinterpret_cast<const numerator_context *>(raw_context);
    const auto *cols = reinterpret_cast<const fr_device_vec *>(raw_columns);
    const size_t len = c->len;
    auto in_bounds = [total_columns](size_t offset, size_t count) {
        return offset <= total_columns && count <= total_columns - offset;
    };
    if (lookup_count != c->lookup_count || trash_count != c->trash_count || total_columns > SIZE_MAX / len ||
        !cols || cols->len < total_columns * len || !in_bounds(advice_offset, advice_cols) ||
        !in_bounds(instance_offset, instance_cols) || !in_bounds(permutation_offset, permutation_sets) ||
        !in_bounds(lookup_product_offset, lookup_count) || !in_bounds(lookup_input_offset, lookup_count) ||
        !in_bounds(lookup_table_offset, lookup_count) || !in_bounds(trash_offset, trash_count))
        return make_error((int)cudaErrorInvalidValue, "resident numerator vector length mismatch");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    device_vec_wait(cols, s);
    auto view = [cols, len](size_t offset, size_t count) -> const fr_t * {
        return count ? cols->values + offset * len : nullptr;
    };
    auto d_chal = upload_fr(challenges, challenge_len, s);
    num_params p{};
    p.len = len;
    p.rot_scale = c->rot_scale;
    p.fixed = c->fixed;
    p.fixed_cols = c->fixed_cols;
    p.advice = view(advice_offset, advice_cols);
    p.advice_cols = advice_cols;
    p.instance = view(instance_offset, instance_cols);
    p.instance_cols = instance_cols;
    p.challenges = d_chal;
    p.challenge_len = challenge_len;
    p.beta = from_raw(beta);
    p.gamma = from_raw(gamma);
    p.theta = from_raw(theta);
    p.trash = from_raw(trash_challenge);
    p.y = from_raw(y);
    p.run_custom = 1;
    p.custom = c->custom.g;
    p.l0 = c->l0;
    p.l_last = c->l_last;
    p.l_active = c->l_active;
    p.perm_sets = permutation_sets;
    p.perm_products = view(permutation_offset, permutation_sets);
    p.perm_columns = c->d_perm_columns;
    p.perm_columns_len = c->perm_columns_len;
    p.perm_pk_cosets = c->pk_cosets;
    p.omega_powers = c->omega_pows;
    p.delta_start = p.beta * c->g_coset;
    p.delta_const = c->delta_const;
    p.last_rotation = c->last_rotation;
    p.chunk_len = c->chunk_len;
    p.lookup_count = lookup_count;
    p.lk_product = view(lookup_product_offset, lookup_count);
    p.lk_input = view(lookup_input_offset, lookup_count);
    p.lk_table = view(lookup_table_offset, lookup_count);
    p.lk_stride = len;
    p.lookup_graphs = c->d_lookup;
    p.trash_count = trash_count;
    p.trash_cosets = view(trash_offset, trash_count);
    p.trash_sel = c->d_trash_sel;
    p.trash_graphs = c->d_trash;
    fr_device_vec *v = device_vec_new(len, s);
    try {
        p.out = v->values;
        numerator_launch(p, c->max_inter, c->max_slots, s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:5667-5736: every trash argument's compressed
// expression over the trace (input_len rows), out [trash_count][input_len]
RustError midnight_sppark_bls12_381_trace_context_trash(void **out, const void *raw_context, const void *raw_advice,
                                                        size_t advice_cols, const void *raw_instance,
                                                        size_t instance_cols, const RawFr *challenges,
                                                        size_t challenge_len, RawFr trash_challenge)
{
    if (!out || !raw_context || (challenge_len && !challenges))
        return make_error((int)cudaErrorInvalidValue, "invalid resident trash arguments");
    *out = nullptr;
    const auto *c = reinterpret_cast<const numerator_context *>(raw_context);
    const size_t n = c->input_len;
    if (c->trash_count == 0) return make_error((int)cudaErrorInvalidValue, "resident trash vector length mismatch");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    const fr_t *advice = trace_values(raw_advice, advice_cols, n, s, "resident trash vector length mismatch");
    const fr_t *instance = trace_values(raw_instance, instance_cols, n, s, "resident trash vector length mismatch");
    auto d_chal = upload_fr(challenges, challenge_len, s);
    num_params p = trace_params(*c, advice, advice_cols, instance, instance_cols, d_chal, challenge_len);
    p.trash = from_raw(trash_challenge);
    fr_device_vec *v = device_vec_new(c->trash_count * n, s);
    try {
        graph_batch_launch(v->values, p, c->trash_g.data(), c->trash_count, s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:5738-5847: z of every permutation set over the trace,
// out [sets][input_len]; the columns are the context's permutation column
// references into its fixed Lagrange values and the given advice / instance
RustError midnight_sppark_bls12_381_trace_context_permutation(
    void **out, const void *raw_context, const void *raw_advice, size_t advice_cols, const void *raw_instance,
    size_t instance_cols, RawFr beta, RawFr gamma, const RawFr *delta_powers, size_t delta_powers_len,
    const RawFr *blind_values, size_t blind_values_len, size_t blinding_factors)
{
    if (!out || !raw_context || !delta_powers)
        return make_error((int)cudaErrorInvalidValue, "invalid resident permutation arguments");
    *out = nullptr;
    const auto *c = reinterpret_cast<const numerator_context *>(raw_context);
    const size_t n = c->input_len, cc = c->perm_columns_len, chunk = c->chunk_len;
    if (cc == 0 || chunk == 0 || delta_powers_len != cc)
        return make_error((int)cudaErrorInvalidValue, "resident permutation vector length mismatch");
    const size_t sets = (cc + chunk - 1) / chunk;
    if (blinding_factors >= n || blind_values_len != sets * blinding_factors || (blind_values_len && !blind_values))
        return make_error((int)cudaErrorInvalidValue, "resident permutation blind mismatch");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    const char *what = "resident permutation vector length mismatch";
    const fr_t *advice = trace_values(raw_advice, advice_cols, n, s, what);
    const fr_t *instance = trace_values(raw_instance, instance_cols, n, s, what);
    std::vector<const fr_t *> ptrs(cc);
    for (size_t i = 0; i < cc; i++) {
        ptrs[i] = lagrange_column(*c, c->perm_columns[i], advice, advice_cols, instance, instance_cols);
        if (!ptrs[i]) return make_error((int)cudaErrorInvalidValue, "permutation column out of range");
    }
    dev_buf<const fr_t *> d_ptrs(cc, s);
    h2d(d_ptrs, ptrs.data(), cc * sizeof(const fr_t *), s);
    auto dd = upload_fr(delta_powers, cc, s);
    auto db = upload_fr(blind_values, blind_values_len, s);
    fr_device_vec *v = device_vec_new(sets * n, s);
    try {
        permutation_products(v->values, nullptr, d_ptrs, c->pk_lagrange, n, cc, chunk, from_raw(beta),
                             from_raw(gamma), c->trace_omega, dd, db, blinding_factors, s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:5849-5966: every lookup's compressed input and table
// expressions over the trace and their permutations, one device vector
// [inputs | tables | permuted inputs | permuted tables], each
// [lookup_count][input_len]; rows usable_rows.. of the permuted columns from
// the blinds ([lookup_count][blind_count] each)
RustError midnight_sppark_bls12_381_trace_context_lookup_permute(
    void **out, const void *raw_context, const void *raw_advice, size_t advice_cols, const void *raw_instance,
    size_t instance_cols, const RawFr *challenges, size_t challenge_len, RawFr theta, size_t usable_rows,
    const RawFr *input_blinds, const RawFr *table_blinds, size_t blind_count)
{
    if (!out || !raw_context || (challenge_len && !challenges))
        return make_error((int)cudaErrorInvalidValue, "invalid resident lookup permutation arguments");
    *out = nullptr;
    const auto *c = reinterpret_cast<const numerator_context *>(raw_context);
    const size_t n = c->input_len, lc = c->lookup_count;
    if (lc == 0 || usable_rows == 0 || usable_rows > n || blind_count != n - usable_rows ||
        (blind_count && (!input_blinds || !table_blinds)))
        return make_error((int)cudaErrorInvalidValue, "resident lookup permutation shape mismatch");
    if (n > ((size_t)1 << 31) || lc > SIZE_MAX / n || lc * n > SIZE_MAX / 4)
        return make_error((int)cudaErrorInvalidValue, "resident lookup permutation size overflow");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    const char *what = "resident lookup permutation shape mismatch";
    const fr_t *advice = trace_values(raw_advice, advice_cols, n, s, what);
    const fr_t *instance = trace_values(raw_instance, instance_cols, n, s, what);
    auto d_chal = upload_fr(challenges, challenge_len, s);
    num_params p = trace_params(*c, advice, advice_cols, instance, instance_cols, d_chal, challenge_len);
    p.theta = from_raw(theta);
    const size_t group = lc * n;
    fr_device_vec *v = device_vec_new(4 * group, s);
    const char *failed = nullptr;
    try {
        fr_t *t = v->values;
        graph_batch_launch(t, p, c->lookup_input_g.data(), lc, s);
        graph_batch_launch(t + group, p, c->lookup_table_g.data(), lc, s);
        failed = lookup_permute_core(t, t + group, n, t + 2 * group, t + 3 * group, n, n, usable_rows, lc,
                                     input_blinds, table_blinds, s);
        device_vec_mark_ready(v, s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    if (failed) {
        device_vec_delete(v);
        return make_error((int)cudaErrorInvalidValue, failed);
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
    lane_sync(s);
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
