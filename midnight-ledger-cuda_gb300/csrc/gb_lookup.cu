// Lookup permutation on the device: permute_expression_pair
// (vendor/midnight-proofs-0.8.1/src/plonk/lookup/prover.rs:1573-1690) for
// every lookup of a proof, over the resident compressed input and table
// columns.
//
// Per lookup, with u usable rows:
//   A' = the compressed inputs sorted in canonical order;
//   S'[i] = A'[i] where row i starts a run of equal inputs; the table
//   values left after removing one copy of every distinct input, in sorted
//   order, fill the remaining rows from the bottom up;
//   rows u.. of A' and S' are the caller's blinds.
// Sorting is a radix sort of canonical keys (by their top 64-bit limb; by
// the whole key only when two distinct values share a top limb, which a
// check after the sort detects); every run start looks up the
// first equal table entry by binary search (marking it used); two exclusive
// scans give each leftover table value its rank and each repeated row its
// rank from the bottom.  An input value missing from the table is the
// reference's ConstraintSystemFailure.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "gb_vec.cuh"

namespace gb {

struct ckey {
    uint64_t l[4];  // canonical value, little-endian limbs
};

struct ckey_decomposer {
    __host__ __device__ ::cuda::std::tuple<uint64_t &, uint64_t &, uint64_t &, uint64_t &> operator()(ckey &k) const
    {
        return {k.l[3], k.l[2], k.l[1], k.l[0]};
    }
};

// the top limb alone: canonical order whenever no two distinct values
// share it (equal values may sit in any order)
struct ckey_top_decomposer {
    __host__ __device__ ::cuda::std::tuple<uint64_t &> operator()(ckey &k) const { return {k.l[3]}; }
};

__device__ __forceinline__ int ckey_cmp(const ckey &a, const ckey &b)
{
#pragma unroll
    for (int i = 3; i >= 0; i--)
        if (a.l[i] != b.l[i]) return a.l[i] < b.l[i] ? -1 : 1;
    return 0;
}

__device__ __forceinline__ ckey to_ckey(const fr_t &m)
{
    fr_t c = m.from_mont();
    ckey k;
#pragma unroll
    for (int j = 0; j < 4; j++) k.l[j] = (uint64_t)c.v[2 * j] | ((uint64_t)c.v[2 * j + 1] << 32);
    return k;
}

__device__ __forceinline__ fr_t from_ckey(const ckey &k)
{
    fr_t c;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        c.v[2 * j] = (uint32_t)k.l[j];
        c.v[2 * j + 1] = (uint32_t)(k.l[j] >> 32);
    }
    return c.to_mont();
}

__global__ void lk_keys_kernel(const fr_t *__restrict__ a, const fr_t *__restrict__ t, size_t u, ckey *ka, ckey *kt)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= u) return;
    ka[i] = to_ckey(a[i]);
    kt[i] = to_ckey(t[i]);
}

// run starts of the sorted inputs; each takes the first equal table entry
__global__ void lk_match_kernel(const ckey *__restrict__ as, const ckey *__restrict__ ts, size_t u,
                                uint32_t *__restrict__ repeated, uint32_t *__restrict__ keep, int *missing)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= u) return;
    const bool first = i == 0 || ckey_cmp(as[i], as[i - 1]) != 0;
    repeated[i] = first ? 0u : 1u;
    if (!first) return;
    size_t lo = 0, hi = u;  // lower bound of as[i] in ts
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (ckey_cmp(ts[mid], as[i]) < 0) lo = mid + 1;
        else hi = mid;
    }
    if (lo < u && ckey_cmp(ts[lo], as[i]) == 0) keep[lo] = 0u;
    else atomicExch(missing, 1);
}

// after a sort by the top limb: flag two neighbours with the same top limb
// but different values (the order among them is then not canonical)
__global__ void lk_tie_kernel(const ckey *__restrict__ as, const ckey *__restrict__ ts, size_t u, int *tie)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 || i >= u) return;
    if ((as[i].l[3] == as[i - 1].l[3] && ckey_cmp(as[i], as[i - 1]) != 0) ||
        (ts[i].l[3] == ts[i - 1].l[3] && ckey_cmp(ts[i], ts[i - 1]) != 0))
        atomicExch(tie, 1);
}

__global__ void lk_fill_kernel(uint32_t *keep, size_t u)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < u) keep[i] = 1u;
}

__global__ void lk_leftovers_kernel(const ckey *__restrict__ ts, const uint32_t *__restrict__ keep,
                                    const uint32_t *__restrict__ keep_pos, size_t u, ckey *__restrict__ leftovers)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < u && keep[i]) leftovers[keep_pos[i]] = ts[i];
}

__global__ void lk_write_kernel(const ckey *__restrict__ as, const ckey *__restrict__ leftovers,
                                const uint32_t *__restrict__ repeated, const uint32_t *__restrict__ rep_pos,
                                const uint32_t *__restrict__ keep, const uint32_t *__restrict__ keep_pos, size_t u,
                                fr_t *__restrict__ a_out, fr_t *__restrict__ s_out, int *mismatch)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= u) return;
    const uint32_t rep_total = rep_pos[u - 1] + repeated[u - 1];
    const uint32_t left_total = keep_pos[u - 1] + keep[u - 1];
    const fr_t a = from_ckey(as[i]);
    a_out[i] = a;
    if (!repeated[i]) {
        s_out[i] = a;
    } else {
        // repeated rows from the bottom up take the leftovers in order
        const uint32_t rank = rep_total - 1 - rep_pos[i];
        if (rank < left_total) s_out[i] = from_ckey(leftovers[rank]);
        else atomicExch(mismatch, 1);
    }
    if (i == 0 && rep_total != left_total) atomicExch(mismatch, 1);
}

static void exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, cudaStream_t s)
{
    size_t temp = 0;
    GB_CUDA_OK(cub::DeviceScan::ExclusiveSum(nullptr, temp, in, out, (int)n, s));
    dev_buf<uint8_t> t(temp, s);
    GB_CUDA_OK(cub::DeviceScan::ExclusiveSum(t.get(), temp, in, out, (int)n, s));
}

template <class D>
static void sort_ckeys(ckey *in_a, ckey *out_a, ckey *in_t, ckey *out_t, size_t u, int end_bit, cudaStream_t s)
{
    size_t temp = 0;
    GB_CUDA_OK(cub::DeviceRadixSort::SortKeys(nullptr, temp, in_a, out_a, (int64_t)u, D{}, 0, end_bit, s));
    dev_buf<uint8_t> tmp(temp, s);
    GB_CUDA_OK(cub::DeviceRadixSort::SortKeys(tmp.get(), temp, in_a, out_a, (int64_t)u, D{}, 0, end_bit, s));
    GB_CUDA_OK(cub::DeviceRadixSort::SortKeys(tmp.get(), temp, in_t, out_t, (int64_t)u, D{}, 0, end_bit, s));
}

// one lookup: a, t = compressed input / table (u rows read); outputs u rows.
// full = false sorts by the top limb and raises d_flags[2] when that order
// is not canonical (the caller then repeats with full = true).
static void permute_pair(const fr_t *a, const fr_t *t, size_t u, fr_t *a_out, fr_t *s_out, int *d_flags, bool full,
                         cudaStream_t s)
{
    dev_buf<ckey> ka(u, s), kt(u, s), sa(u, s), st(u, s), left(u, s);
    dev_buf<uint32_t> repeated(u, s), rep_pos(u, s), keep(u, s), keep_pos(u, s);
    const unsigned grid = blocks_for(u, 256);
    lk_keys_kernel<<<grid, 256, 0, s>>>(a, t, u, ka, kt);
    GB_CHECK_LAUNCH();
    if (full) {
        sort_ckeys<ckey_decomposer>(ka, sa, kt, st, u, 256, s);
    } else {
        sort_ckeys<ckey_top_decomposer>(ka, sa, kt, st, u, 64, s);
        lk_tie_kernel<<<grid, 256, 0, s>>>(sa, st, u, d_flags + 2);
        GB_CHECK_LAUNCH();
    }
    lk_fill_kernel<<<grid, 256, 0, s>>>(keep, u);
    GB_CHECK_LAUNCH();
    lk_match_kernel<<<grid, 256, 0, s>>>(sa, st, u, repeated, keep, d_flags);
    GB_CHECK_LAUNCH();
    exclusive_scan_u32(keep, keep_pos, u, s);
    exclusive_scan_u32(repeated, rep_pos, u, s);
    lk_leftovers_kernel<<<grid, 256, 0, s>>>(st, keep, keep_pos, u, left);
    GB_CHECK_LAUNCH();
    lk_write_kernel<<<grid, 256, 0, s>>>(sa, left, repeated, rep_pos, keep, keep_pos, u, a_out, s_out, d_flags + 1);
    GB_CHECK_LAUNCH();
}

const char *lookup_permute_core(const fr_t *inputs, const fr_t *tables, size_t in_stride, fr_t *a_out, fr_t *s_out,
                                size_t out_stride, size_t len, size_t usable_rows, size_t lookup_count,
                                const RawFr *input_blinds, const RawFr *table_blinds, cudaStream_t s)
{
    const size_t nb = len - usable_rows;
    int flags[3] = {0, 0, 0};
    dev_buf<int> d_flags(3, s);
    // sorted by the top limb first; on a tie of distinct values, again with
    // the whole canonical key
    for (int full = 0; full < 2; full++) {
        GB_CUDA_OK(cudaMemsetAsync(d_flags.get(), 0, 3 * sizeof(int), s));
        for (size_t l = 0; l < lookup_count; l++) {
            fr_t *ao = a_out + l * out_stride, *so = s_out + l * out_stride;
            permute_pair(inputs + l * in_stride, tables + l * in_stride, usable_rows, ao, so, d_flags, full != 0, s);
            if (full == 0 && nb) {
                h2d(ao + usable_rows, input_blinds + l * nb, nb * sizeof(fr_t), s);
                h2d(so + usable_rows, table_blinds + l * nb, nb * sizeof(fr_t), s);
            }
        }
        d2h(flags, d_flags, 3 * sizeof(int), s);
        lane_sync(s);
        if (!flags[2]) break;
    }
    if (flags[0]) return "lookup input value missing from the table";
    if (flags[1]) return "lookup table/input multiset mismatch";
    return nullptr;
}

}  // namespace gb

using namespace gb;

extern "C" {

// compressed_vec = per lookup its compressed input column then its
// compressed table column (len rows each); out = per lookup A' then S' (len
// rows each), rows usable_rows.. taken from the blinds
// ([lookup_count][len - usable_rows] each).
RustError gb_fr_lookup_permute_device(void **out, const void *compressed_vec, size_t len, size_t usable_rows,
                                      size_t lookup_count, const RawFr *input_blinds, const RawFr *table_blinds)
{
    if (!out || !compressed_vec || lookup_count == 0 || usable_rows == 0 || usable_rows > len ||
        len > ((size_t)1 << 31) || (usable_rows < len && (!input_blinds || !table_blinds)))
        return make_error((int)cudaErrorInvalidValue, "invalid lookup permutation arguments");
    *out = nullptr;
    GB_ENTRY_BEGIN
    auto *cv = reinterpret_cast<const fr_device_vec *>(compressed_vec);
    if (cv->len < 2 * lookup_count * len)
        return make_error((int)cudaErrorInvalidValue, "compressed lookup columns too short");
    cudaStream_t s = lane_stream();
    device_vec_wait(cv, s);
    fr_device_vec *v = device_vec_new(2 * lookup_count * len, s);
    const char *failed = nullptr;
    try {
        failed = lookup_permute_core(cv->values, cv->values + len, 2 * len, v->values, v->values + len, 2 * len, len,
                                     usable_rows, lookup_count, input_blinds, table_blinds, s);
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

// bls12_381_g1_msm.cu:5139-5194: host compressed inputs and tables
// ([lookup_count][len] each) in, one device vector [inputs | tables |
// permuted inputs | permuted tables] out (the layout
// midnight_sppark_bls12_381_fr_lookup_products_device reads); blinds
// [lookup_count][blind_count], blind_count = len - usable_rows
RustError midnight_sppark_bls12_381_fr_lookup_permute_batch(void **out, const RawFr *compressed_inputs,
                                                            const RawFr *compressed_tables, size_t len,
                                                            size_t lookup_count, size_t usable_rows,
                                                            const RawFr *input_blinds, const RawFr *table_blinds,
                                                            size_t blind_count)
{
    if (!out || !compressed_inputs || !compressed_tables || !input_blinds || !table_blinds || len == 0 ||
        lookup_count == 0 || usable_rows == 0 || usable_rows > len || blind_count != len - usable_rows ||
        usable_rows > UINT32_MAX || lookup_count > SIZE_MAX / len)
        return make_error((int)cudaErrorInvalidValue, "invalid resident lookup permutation arguments");
    *out = nullptr;
    const size_t group = lookup_count * len;
    if (group > SIZE_MAX / 4 || len > ((size_t)1 << 31))
        return make_error((int)cudaErrorInvalidValue, "resident lookup permutation size overflow");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    fr_device_vec *v = device_vec_new(4 * group, s);
    const char *failed = nullptr;
    try {
        fr_t *t = v->values;
        h2d(t, compressed_inputs, group * sizeof(fr_t), s);
        h2d(t + group, compressed_tables, group * sizeof(fr_t), s);
        failed = lookup_permute_core(t, t + group, len, t + 2 * group, t + 3 * group, len, len, usable_rows,
                                     lookup_count, input_blinds, table_blinds, s);
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

}  // extern "C"
