// Field elements sampled on the device from a ChaCha20 stream.
//
// The prover draws its blinding values with Fq::random
// (vendor/midnight-curves-0.3.1/src/bls12_381/fq.rs:373-387): four u64 words
// of the rng, the top bit masked, rejected when >= r, stored in Montgomery
// form.  The rng is rand_chacha's ChaCha20Rng: the 20-round block function
// of RFC 8439 with a 64-bit block counter (words 12-13) and stream id 0
// (words 14-15), consumed word by word.  For a large draw (the vanishing
// argument's random polynomial, vanishing/prover.rs:41-75) the host rng
// hands its key and its word position to this entry point, which produces
// the same n values the host would, and reports how many words they used
// so the host rng can skip past them.
//
// Candidate j of a draw is keystream words [w0 + 8j, w0 + 8j + 8); one
// thread per candidate computes the (one or two) blocks that hold them and
// tests the candidate against r; an exclusive scan of the accept flags gives
// each accepted candidate its output index.
#include <cub/device/device_scan.cuh>

#include "gb_vec.cuh"

namespace gb {

struct chacha_key {
    uint32_t k[8];
};

__device__ __forceinline__ uint32_t rotl32(uint32_t x, int n) { return __funnelshift_l(x, x, n); }

#define GB_QR(a, b, c, d)                                                                                            \
    x[a] += x[b];                                                                                                    \
    x[d] = rotl32(x[d] ^ x[a], 16);                                                                                  \
    x[c] += x[d];                                                                                                    \
    x[b] = rotl32(x[b] ^ x[c], 12);                                                                                  \
    x[a] += x[b];                                                                                                    \
    x[d] = rotl32(x[d] ^ x[a], 8);                                                                                   \
    x[c] += x[d];                                                                                                    \
    x[b] = rotl32(x[b] ^ x[c], 7)

__device__ void chacha20_block(const chacha_key &key, uint64_t counter, uint32_t *out)
{
    uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key.k[0], key.k[1], key.k[2], key.k[3],
                       key.k[4],    key.k[5],    key.k[6],    key.k[7],    (uint32_t)counter,
                       (uint32_t)(counter >> 32), 0u, 0u};
    uint32_t x[16];
#pragma unroll
    for (int i = 0; i < 16; i++) x[i] = st[i];
#pragma unroll 1
    for (int r = 0; r < 10; r++) {
        GB_QR(0, 4, 8, 12);
        GB_QR(1, 5, 9, 13);
        GB_QR(2, 6, 10, 14);
        GB_QR(3, 7, 11, 15);
        GB_QR(0, 5, 10, 15);
        GB_QR(1, 6, 11, 12);
        GB_QR(2, 7, 8, 13);
        GB_QR(3, 4, 9, 14);
    }
#pragma unroll
    for (int i = 0; i < 16; i++) out[i] = x[i] + st[i];
}
#undef GB_QR

__global__ void fr_candidates_kernel(chacha_key key, uint64_t word0, size_t count, fr_t *raw_out, uint32_t *flags)
{
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count) return;
    const uint64_t w = word0 + 8 * (uint64_t)j;
    const uint64_t b0 = w >> 4;
    const uint32_t o = (uint32_t)(w & 15);
    uint32_t blk[32];
    chacha20_block(key, b0, blk);
    if (o > 8) chacha20_block(key, b0 + 1, blk + 16);
    fr_t v;
#pragma unroll
    for (int i = 0; i < 8; i++) v.v[i] = blk[o + i];
    v.v[7] &= 0x7fffffffu;
    // v < r, comparing from the top limb
    const fr_t m = fr_t::modulus();
    int state = 0;  // 0 equal so far, 1 less, 2 greater
#pragma unroll
    for (int i = 7; i >= 0; i--)
        if (state == 0 && v.v[i] != m.v[i]) state = v.v[i] < m.v[i] ? 1 : 2;
    raw_out[j] = v;
    flags[j] = state == 1 ? 1u : 0u;
}

__global__ void fr_accept_kernel(const fr_t *__restrict__ raw, const uint32_t *__restrict__ flags,
                                 const uint32_t *__restrict__ pos, size_t count, size_t n, fr_t r2,
                                 fr_t *__restrict__ out, unsigned long long *consumed)
{
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count || !flags[j]) return;
    const uint32_t p = pos[j];
    if (p >= n) return;
    out[p] = raw[j] * r2;  // canonical * R^2 / R = Montgomery form
    if (p == n - 1) *consumed = 8ull * (j + 1);
}

static fr_t host_r2()
{
    fr_t x = fr_t::one();  // R mod r
    for (int i = 0; i < 256; i++) x = x + x;
    return x;  // R * 2^256 = R^2 mod r
}

}  // namespace gb

using namespace gb;

// The same block function on the host (the prover's own draws: blinding
// values, challenges' seeds); plain C, no device involved.
static inline uint32_t host_rotl32(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }

static void host_chacha20_block(const uint32_t *key, uint64_t counter, uint64_t stream, uint32_t *out)
{
    uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                       key[4], key[5], key[6], key[7], (uint32_t)counter, (uint32_t)(counter >> 32),
                       (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t x[16];
    for (int i = 0; i < 16; i++) x[i] = st[i];
    auto qr = [&x](int a, int b, int c, int d) {
        x[a] += x[b];
        x[d] = host_rotl32(x[d] ^ x[a], 16);
        x[c] += x[d];
        x[b] = host_rotl32(x[b] ^ x[c], 12);
        x[a] += x[b];
        x[d] = host_rotl32(x[d] ^ x[a], 8);
        x[c] += x[d];
        x[b] = host_rotl32(x[b] ^ x[c], 7);
    };
    for (int r = 0; r < 10; r++) {
        qr(0, 4, 8, 12);
        qr(1, 5, 9, 13);
        qr(2, 6, 10, 14);
        qr(3, 7, 11, 15);
        qr(0, 5, 10, 15);
        qr(1, 6, 11, 12);
        qr(2, 7, 8, 13);
        qr(3, 4, 9, 14);
    }
    for (int i = 0; i < 16; i++) out[i] = x[i] + st[i];
}

extern "C" {

// nblocks consecutive keystream blocks (16 words each) of the ChaCha20 stream
// with this key (8 little-endian words) and stream id, from block `counter`.
// Host only: no device memory or stream is touched.
RustError gb_chacha20_blocks(const uint32_t *key, uint64_t counter, uint64_t stream, size_t nblocks, uint32_t *out)
{
    if (nblocks && (!key || !out)) return make_error((int)cudaErrorInvalidValue, "invalid ChaCha20 arguments");
    for (size_t b = 0; b < nblocks; b++) host_chacha20_block(key, counter + b, stream, out + 16 * b);
    return ok();
}

// n values by Fq::random's rejection rule from the ChaCha20Rng stream with
// this 32-byte seed, starting at keystream word `word_offset`, into a new
// device vector (Montgomery form); *words_consumed = keystream words used.
RustError gb_fr_random_chacha20(void **out, const uint8_t *key32, uint64_t word_offset, size_t n,
                                uint64_t *words_consumed)
{
    if (!out || !key32 || !words_consumed || n == 0 || n > ((size_t)1 << 30))
        return make_error((int)cudaErrorInvalidValue, "invalid random draw arguments");
    *out = nullptr;
    GB_ENTRY_BEGIN
    chacha_key key;
    for (int i = 0; i < 8; i++)
        key.k[i] = (uint32_t)key32[4 * i] | (uint32_t)key32[4 * i + 1] << 8 | (uint32_t)key32[4 * i + 2] << 16 |
                   (uint32_t)key32[4 * i + 3] << 24;
    cudaStream_t s = lane_stream();
    const fr_t r2 = host_r2();
    // each candidate is accepted with probability r / 2^255 > 0.9; the
    // margin makes a second round vanishingly rare, and it is handled
    size_t count = n + n / 8 + 64;
    for (int round = 0; round < 8; round++, count *= 2) {
        dev_buf<fr_t> raw(count, s);
        dev_buf<uint32_t> flags(count, s), pos(count, s);
        fr_candidates_kernel<<<blocks_for(count, 128), 128, 0, s>>>(key, word_offset, count, raw, flags);
        GB_CHECK_LAUNCH();
        size_t temp = 0;
        GB_CUDA_OK(cub::DeviceScan::ExclusiveSum(nullptr, temp, flags.get(), pos.get(), (int)count, s));
        dev_buf<uint8_t> t(temp, s);
        GB_CUDA_OK(cub::DeviceScan::ExclusiveSum(t.get(), temp, flags.get(), pos.get(), (int)count, s));
        uint32_t last_pos = 0, last_flag = 0;
        d2h(&last_pos, pos.get() + count - 1, sizeof(uint32_t), s);
        d2h(&last_flag, flags.get() + count - 1, sizeof(uint32_t), s);
        lane_sync(s);
        if ((size_t)last_pos + last_flag < n) continue;
        fr_device_vec *v = device_vec_new(n, s);
        try {
            dev_buf<unsigned long long> d_used(1, s);
            fr_accept_kernel<<<blocks_for(count, 256), 256, 0, s>>>(raw, flags, pos, count, n, r2, v->values, d_used);
            GB_CHECK_LAUNCH();
            unsigned long long used = 0;
            d2h(&used, d_used, sizeof(used), s);
            device_vec_mark_ready(v, s);
            lane_sync(s);
            *words_consumed = used;
        } catch (...) {
            device_vec_delete(v);
            throw;
        }
        *out = v;
        return ok();
    }
    return make_error(-1, "random draw did not reach the requested count");
    GB_ENTRY_END
}

}  // extern "C"
