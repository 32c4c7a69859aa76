// Poseidon hash chains and their circuit witness over BLS12-381 Fr, and the
// scatter of that witness into the Poseidon chip's advice columns: the three
// Poseidon entry points of the reference FFI
// (midnight-sppark-msm/src/lib.rs:854-863,1029-1051,4185-4290;
// bls12_381_g1_msm.cu:2018-2216,2820-2876,4121-4268), which the reference's
// ZKIR preprocessing calls for chains of 3-element hashes
// (zkir/src/ir_vm.rs:300-340,540-560).
//
// The permutation (width 3, x^5 S-box, 4 full rounds, 60 partial rounds, 4
// full rounds; midnight-circuits hash/poseidon/constants, poseidon_cpu.rs):
//   state += rc[0];
//   for r in 0..68:
//       s_i = state_i^5 for every i in a full round (r < 4 or r >= 64),
//             only for i = 2 in a partial round (state_i unchanged otherwise)
//       state_i = sum_j mds[i][j] s_j + (rc[r + 1][i] if r + 1 < 68 else 0)
// A chain of len hashes: prev = initial; for each hash, state = (prev, tail0,
// input_len), permute, state_0 += tail1, permute, prev = state_0.
//
// The witness of one permutation (128 values, the reference's order,
// midnight-circuits poseidon_chip.rs:55-60,108-128): per full round the three
// cubes state_i^3 (taken after the round constant) then the three new state
// values; per run of 6 partial rounds the new state_2 of its first 5 rounds,
// then the three new state values after the 6th.  A hash's witness is its two
// permutations' (256 values).
//
// A chain is sequential, so one warp computes it: lanes 0-2 hold the three
// state elements and exchange the S-box outputs by shuffles.
#include <vector>

#include "gb_runtime.cuh"

namespace gb {

static constexpr int kPosWidth = 3;
static constexpr int kPosRounds = 68;
static constexpr int kPosFullHalf = 4;
static constexpr size_t kPosPermWitness = 128;
static constexpr size_t kPosHashWitness = 256;
static constexpr size_t kPosAdviceColumns = 8;
static constexpr size_t kPosRowsPerHash = 41;
static constexpr size_t kPosRowsPerPerm = 21;

__device__ __forceinline__ fr_t shfl_fr(const fr_t &v, int src)
{
    fr_t r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = __shfl_sync(0xffffffffu, v.v[i], src);
    return r;
}

// One permutation of the lane's state element x (lanes 0..2); the whole warp
// calls it.  wit: the permutation's 128 witness values, or null.
__device__ fr_t poseidon_permute_lane(fr_t x, const fr_t *mds, const fr_t *rc, fr_t *wit)
{
    const int lane = threadIdx.x;
    const bool on = lane < kPosWidth;
    const int i = on ? lane : 0;
    fr_t m[kPosWidth];
#pragma unroll
    for (int j = 0; j < kPosWidth; j++) m[j] = mds[i * kPosWidth + j];
    x = x + rc[i];
    size_t at = 0;
    for (int r = 0; r < kPosRounds; r++) {
        const bool full = r < kPosFullHalf || r >= kPosRounds - kPosFullHalf;
        fr_t s = x;
        if (full || i == 2) {
            const fr_t sq = x.sqr();
            const fr_t cube = sq * x;
            if (full && wit && on) wit[at + i] = cube;
            s = sq * cube;
        }
        fr_t acc = r + 1 < kPosRounds ? rc[(r + 1) * kPosWidth + i] : fr_t::zero();
#pragma unroll
        for (int j = 0; j < kPosWidth; j++) acc = acc + m[j] * shfl_fr(s, j);
        x = acc;
        if (wit && on) {
            if (full) {
                wit[at + kPosWidth + i] = x;
            } else {
                const int p = (r - kPosFullHalf) % 6;
                if (p < 5) {
                    if (i == 2) wit[at + p] = x;
                } else {
                    wit[at + 5 + i] = x;
                }
            }
        }
        if (full) at += 2 * kPosWidth;
        else if ((r - kPosFullHalf) % 6 == 5) at += 5 + kPosWidth;
    }
    return x;
}

// one warp: the chain's outputs (out, may be null) and witness (wit, may be null)
__global__ void __launch_bounds__(32) poseidon_chain_kernel(fr_t *out, fr_t *wit, fr_t initial, fr_t tail0,
                                                            fr_t tail1, fr_t input_len, const fr_t *mds,
                                                            const fr_t *rc, size_t len)
{
    const int lane = threadIdx.x;
    fr_t prev = initial;
    for (size_t h = 0; h < len; h++) {
        fr_t x = lane == 0 ? prev : lane == 1 ? tail0 : input_len;
        fr_t *w = wit ? wit + h * kPosHashWitness : nullptr;
        x = poseidon_permute_lane(x, mds, rc, w);
        if (lane == 0) x = x + tail1;
        x = poseidon_permute_lane(x, mds, rc, w ? w + kPosPermWitness : nullptr);
        prev = shfl_fr(x, 0);
        if (out && lane == 0) out[h] = prev;
    }
}

// advice[column * domain_len + row] = witness value, for every witness value
// of every hash: layout[k] = column << 8 | row places value k of a
// permutation at that row of the permutation's 21-row region
__global__ void poseidon_advice_scatter_kernel(fr_t *advice, size_t domain_len, const fr_t *witness,
                                               size_t hash_count, const uint16_t *layout)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= hash_count * kPosHashWitness) return;
    const size_t h = idx / kPosHashWitness, k = idx % kPosHashWitness;
    const uint16_t packed = layout[k % kPosPermWitness];
    const size_t row0 = 2 + kPosRowsPerHash * h + kPosRowsPerPerm * (k / kPosPermWitness);
    advice[(size_t)(packed >> 8) * domain_len + row0 + (packed & 0xffu)] = witness[idx];
}

// The cells of each hash that are not in the witness (bls12_381_g1_msm.cu:
// 2035-2068): each permutation's input row and its input plus the first
// round constants (metadata[8..10]), the second input's absorption of
// metadata[6] at row 20, and the chain's first cells at rows 0 and 1.
// Written after the scatter, so they take precedence over a layout that
// names the same cells.
__global__ void poseidon_advice_fixed_kernel(fr_t *advice, size_t domain_len, const fr_t *witness,
                                             size_t hash_count, const fr_t *meta)
{
    const size_t h = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= hash_count) return;
    const size_t row0 = 2 + kPosRowsPerHash * h;
    fr_t *col[3] = {advice, advice + domain_len, advice + 2 * domain_len};
    const fr_t *w = witness + h * kPosHashWitness;
    const fr_t first[3] = {h == 0 ? meta[4] : w[-(ptrdiff_t)kPosHashWitness + 253], meta[5], meta[7]};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        col[c][row0] = first[c];
        col[c][row0 + 1] = first[c] + meta[8 + c];
    }
    const fr_t absorbed = w[125] + meta[6];
    col[0][row0 + 20] = absorbed;
    col[1][row0 + 20] = w[125];
    col[2][row0 + 20] = meta[6];
    const fr_t second[3] = {absorbed, w[126], w[127]};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        col[c][row0 + 21] = second[c];
        col[c][row0 + 22] = second[c] + meta[8 + c];
    }
    if (h == 0) {
        col[0][0] = meta[0];
        col[1][0] = meta[1];
        col[2][0] = meta[2];
        col[0][1] = meta[3];
    }
}

// shared by the two chain entry points: out_len values of the chain's
// outputs or witness to host `out`
static void poseidon_chain_run(fr_t *out, bool witness, size_t len, const RawFr &initial, const RawFr &tail0,
                               const RawFr &tail1, const RawFr &input_len, const RawFr *mds,
                               const RawFr *round_constants)
{
    cudaStream_t s = lane_stream();
    const size_t out_len = witness ? len * kPosHashWitness : len;
    dev_buf<fr_t> d_out(out_len, s), d_mds(kPosWidth * kPosWidth, s), d_rc(kPosRounds * kPosWidth, s);
    h2d(d_mds, mds, kPosWidth * kPosWidth * sizeof(fr_t), s);
    h2d(d_rc, round_constants, kPosRounds * kPosWidth * sizeof(fr_t), s);
    poseidon_chain_kernel<<<1, 32, 0, s>>>(witness ? nullptr : d_out.get(), witness ? d_out.get() : nullptr,
                                           from_raw(initial), from_raw(tail0), from_raw(tail1),
                                           from_raw(input_len), d_mds, d_rc, len);
    GB_CHECK_LAUNCH();
    d2h(out, d_out, out_len * sizeof(fr_t), s);
    lane_sync(s);
}

}  // namespace gb

using namespace gb;

extern "C" {

// bls12_381_g1_msm.cu:4121-4190 (lib.rs:4185-4236): the chain's len outputs
RustError midnight_sppark_bls12_381_fr_poseidon_hash_chain(RawFr *out, size_t len, RawFr initial, RawFr tail0,
                                                           RawFr tail1, RawFr input_len, const RawFr *mds,
                                                           size_t mds_len, const RawFr *round_constants,
                                                           size_t round_constants_len)
{
    if (len == 0) return ok();
    if (!out || !mds || mds_len != kPosWidth * kPosWidth || !round_constants ||
        round_constants_len != (size_t)kPosRounds * kPosWidth)
        return make_error((int)cudaErrorInvalidValue, "invalid Poseidon hash-chain arguments");
    GB_ENTRY_BEGIN
    poseidon_chain_run(reinterpret_cast<fr_t *>(out), false, len, initial, tail0, tail1, input_len, mds,
                       round_constants);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:4192-4268 (lib.rs:4238-4290): 256 witness values per hash
RustError midnight_sppark_bls12_381_fr_poseidon_hash_chain_witness(RawFr *out, size_t len, RawFr initial,
                                                                   RawFr tail0, RawFr tail1, RawFr input_len,
                                                                   const RawFr *mds, size_t mds_len,
                                                                   const RawFr *round_constants,
                                                                   size_t round_constants_len)
{
    if (len == 0) return ok();
    if (!out || !mds || mds_len != kPosWidth * kPosWidth || !round_constants ||
        round_constants_len != (size_t)kPosRounds * kPosWidth || len > SIZE_MAX / kPosHashWitness / sizeof(fr_t))
        return make_error((int)cudaErrorInvalidValue, "invalid Poseidon witness arguments");
    GB_ENTRY_BEGIN
    poseidon_chain_run(reinterpret_cast<fr_t *>(out), true, len, initial, tail0, tail1, input_len, mds,
                       round_constants);
    return ok();
    GB_ENTRY_END
}

// bls12_381_g1_msm.cu:2820-2876 (lib.rs:1687-1730): a new device vector of
// 8 advice columns x domain_len rows, zero except the cells of hash_count
// hashes (41 rows each from row 2).  Unlike the reference, every layout
// entry is checked to name a column below 8 and a row inside the domain.
RustError midnight_sppark_bls12_381_fr_poseidon_advice_from_witness(void **out, const RawFr *witness,
                                                                    size_t hash_count, size_t domain_len,
                                                                    const RawFr *metadata, size_t metadata_len,
                                                                    const uint16_t *layout, size_t layout_len)
{
    if (!out || hash_count == 0 || domain_len == 0 || !witness || !metadata || metadata_len != 11 || !layout ||
        layout_len != kPosPermWitness || hash_count > SIZE_MAX / kPosHashWitness ||
        domain_len > SIZE_MAX / kPosAdviceColumns || hash_count > (SIZE_MAX - 2) / kPosRowsPerHash ||
        2 + kPosRowsPerHash * hash_count >= domain_len)
        return make_error((int)cudaErrorInvalidValue, "invalid Poseidon advice arguments");
    *out = nullptr;
    const size_t last_region = 2 + kPosRowsPerHash * (hash_count - 1) + kPosRowsPerPerm;
    for (size_t k = 0; k < layout_len; k++)
        if ((layout[k] >> 8) >= kPosAdviceColumns || last_region + (layout[k] & 0xffu) >= domain_len)
            return make_error((int)cudaErrorInvalidValue, "Poseidon advice layout entry outside the columns");
    GB_ENTRY_BEGIN
    cudaStream_t s = lane_stream();
    const size_t wlen = hash_count * kPosHashWitness;
    fr_device_vec *v = device_vec_new(kPosAdviceColumns * domain_len, s);
    try {
        dev_buf<fr_t> d_wit(wlen, s), d_meta(metadata_len, s);
        dev_buf<uint16_t> d_layout(layout_len, s);
        h2d(d_wit, witness, wlen * sizeof(fr_t), s);
        h2d(d_meta, metadata, metadata_len * sizeof(fr_t), s);
        h2d(d_layout, layout, layout_len * sizeof(uint16_t), s);
        GB_CUDA_OK(cudaMemsetAsync(v->values, 0, v->len * sizeof(fr_t), s));
        poseidon_advice_scatter_kernel<<<blocks_for(wlen, 256), 256, 0, s>>>(v->values, domain_len, d_wit,
                                                                            hash_count, d_layout);
        GB_CHECK_LAUNCH();
        poseidon_advice_fixed_kernel<<<blocks_for(hash_count, 128), 128, 0, s>>>(v->values, domain_len, d_wit,
                                                                                hash_count, d_meta);
        GB_CHECK_LAUNCH();
        device_vec_mark_ready(v, s);
        lane_sync(s);
    } catch (...) {
        device_vec_delete(v);
        throw;
    }
    *out = v;
    return ok();
    GB_ENTRY_END
}

}  // extern "C"
