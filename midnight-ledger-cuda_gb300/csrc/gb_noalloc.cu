// Allocation-free variant of the shifted prefix product (the grand-product
// building block z[0] = initial, z[i] = initial * prod_{j<i} values[j]).
//
// Some callers of this library cannot allocate device memory at the moment
// they need the product: a proof server that reserved its whole HBM budget up
// front and hands out fixed buffers, or a latency-critical prover lane where a
// cudaMalloc / cudaFree (which can synchronise the whole device) would stall
// every other lane.  This entry point takes the caller's own device buffer,
// works in place, and keeps its only temporaries -- one partial product per
// 2048-element tile -- in a fixed, file-scope device array.  It calls no
// cudaMalloc, cudaFree or any allocating routine.
//
// Limits and sharing rules:
//   * at most GB_NOALLOC_PREFIX_MAX_LEN = 4,194,304 (2^22) elements; longer
//     inputs are rejected with cudaErrorInvalidValue;
//   * the scratch array (2048 Fr = 64 KiB) exists once per GPU that loads the
//     library and lives until process exit;
//   * every call shares that array and leaves its contents behind; each call
//     overwrites all the scratch it reads, so nothing needs clearing, but two
//     calls whose work overlaps on the GPU (different streams, not ordered by
//     an event) race on it and give wrong results.  Calls queued on one stream
//     are ordered and safe;
//   * the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture on the device.
#include <mutex>

#include "gb_runtime.cuh"

namespace gb {

static constexpr int kNaThreads = 256;
static constexpr int kNaPer = 8;
static constexpr size_t kNaTile = (size_t)kNaThreads * kNaPer;     // 2048
static constexpr size_t kNaMaxTiles = 2048;                         // one scan block of 256 x 8
static constexpr size_t kNaMaxLen = kNaTile * kNaMaxTiles;           // 2^22

// The scratch: one inclusive tile product per tile.  In host code this name
// is only a handle for cudaGetSymbolAddress, never a device address.
static __device__ __align__(256) fr_t g_noalloc_tile_products[kNaMaxTiles];

static_assert(kNaMaxLen == ((size_t)1 << 22), "allocation-free prefix product maximum");

__device__ fr_t na_block_scan(fr_t v, fr_t *sh)
{
    sh[threadIdx.x] = v;
    __syncthreads();
    for (unsigned off = 1; off < blockDim.x; off <<= 1) {
        fr_t other = threadIdx.x >= off ? sh[threadIdx.x - off] : fr_t::one();
        __syncthreads();
        if (threadIdx.x >= off) sh[threadIdx.x] = sh[threadIdx.x] * other;
        __syncthreads();
    }
    return sh[threadIdx.x];
}

// tiles[t] = product of tile t's values
__global__ void __launch_bounds__(kNaThreads) na_tile_product_kernel(const fr_t *values, size_t n, fr_t *tiles)
{
    __shared__ fr_t sh[kNaThreads];
    size_t base = (size_t)blockIdx.x * kNaTile + (size_t)threadIdx.x * kNaPer;
    fr_t p = fr_t::one();
#pragma unroll
    for (int e = 0; e < kNaPer; e++)
        if (base + e < n) p = p * values[base + e];
    fr_t incl = na_block_scan(p, sh);
    if (threadIdx.x == blockDim.x - 1) tiles[blockIdx.x] = incl;
}

// inclusive scan of the tile products, in place (one block, <= 2048 tiles)
__global__ void __launch_bounds__(kNaThreads) na_tile_scan_kernel(fr_t *tiles, size_t ntiles)
{
    __shared__ fr_t sh[kNaThreads];
    size_t base = (size_t)threadIdx.x * kNaPer;
    fr_t v[kNaPer];
    fr_t p = fr_t::one();
#pragma unroll
    for (int e = 0; e < kNaPer; e++) {
        v[e] = base + e < ntiles ? tiles[base + e] : fr_t::one();
        p = p * v[e];
    }
    na_block_scan(p, sh);
    __syncthreads();
    fr_t run = threadIdx.x ? sh[threadIdx.x - 1] : fr_t::one();
#pragma unroll
    for (int e = 0; e < kNaPer; e++) {
        run = run * v[e];
        if (base + e < ntiles) tiles[base + e] = run;
    }
}

// z[i] = initial * (scanned product of earlier tiles) * (product of earlier
// elements in this tile); each block reads only its own tile before writing
// it, so the update is in place.
__global__ void __launch_bounds__(kNaThreads) na_shifted_apply_kernel(fr_t *values, size_t n, const fr_t *tiles,
                                                                      fr_t initial)
{
    __shared__ fr_t sh[kNaThreads];
    size_t base = (size_t)blockIdx.x * kNaTile + (size_t)threadIdx.x * kNaPer;
    fr_t v[kNaPer];
    fr_t p = fr_t::one();
#pragma unroll
    for (int e = 0; e < kNaPer; e++) {
        v[e] = base + e < n ? values[base + e] : fr_t::one();
        p = p * v[e];
    }
    na_block_scan(p, sh);
    __syncthreads();
    fr_t run = threadIdx.x ? sh[threadIdx.x - 1] : fr_t::one();
    if (blockIdx.x) run = tiles[blockIdx.x - 1] * run;
    run = initial * run;
#pragma unroll
    for (int e = 0; e < kNaPer; e++) {
        if (base + e < n) values[base + e] = run;
        run = run * v[e];
    }
}

namespace {
constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
fr_t *g_na_scratch[kNaMaxDevices];

// Device address of the scratch array on the current device, looked up once
// per device with that device current.
fr_t *noalloc_scratch(int dev)
{
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_scratch[dev]) {
        void *ptr = nullptr;
        GB_CUDA_OK(cudaGetSymbolAddress(&ptr, g_noalloc_tile_products));
        g_na_scratch[dev] = (fr_t *)ptr;
    }
    return g_na_scratch[dev];
}
}  // namespace

}  // namespace gb

using namespace gb;

extern "C" {

// In-place shifted prefix product over caller-owned device memory, with no
// device allocation (see the file comment for who needs it and its limits).
RustError gb_fr_shifted_prefix_product_noalloc(RawFr *d_values_raw, RawFr initial_raw, size_t len, void *stream)
{
    if (len == 0) return ok();
    if (!d_values_raw) return make_error((int)cudaErrorInvalidValue, "null device buffer");
    if (len > kNaMaxLen)
        return make_error((int)cudaErrorInvalidValue,
                          "allocation-free prefix product: length exceeds the maximum of 4194304 (2^22) elements");
    GB_ENTRY_BEGIN
    int dev = current_device();
    if (dev < 0 || dev >= kNaMaxDevices) return make_error(-1, "device index out of range");
    cudaPointerAttributes attr;
    GB_CUDA_OK(cudaPointerGetAttributes(&attr, d_values_raw));
    if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
        return make_error((int)cudaErrorInvalidValue, "values must be device memory of the current device");
    if (attr.type == cudaMemoryTypeDevice && attr.device != dev)
        return make_error((int)cudaErrorInvalidValue, "values live on another device than the current one");
    fr_t *scratch = noalloc_scratch(dev);
    cudaStream_t s = stream ? (cudaStream_t)stream : lane_stream();
    fr_t *values = reinterpret_cast<fr_t *>(d_values_raw);
    const fr_t initial = from_raw(initial_raw);
    const size_t tiles = (len + kNaTile - 1) / kNaTile;
    na_tile_product_kernel<<<(unsigned)tiles, kNaThreads, 0, s>>>(values, len, scratch);
    GB_CHECK_LAUNCH();
    na_tile_scan_kernel<<<1, kNaThreads, 0, s>>>(scratch, tiles);
    GB_CHECK_LAUNCH();
    na_shifted_apply_kernel<<<(unsigned)tiles, kNaThreads, 0, s>>>(values, len, scratch, initial);
    GB_CHECK_LAUNCH();
    return ok();
    GB_ENTRY_END
}

}  // extern "C"
