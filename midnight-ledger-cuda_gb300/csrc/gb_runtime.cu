// Host runtime: lanes, stream-ordered memory, device vectors, transfer
// counters and the lane / device-vector entry points of the C ABI.
#include <atomic>
#include <chrono>
#include <cstdint>
#include <thread>
#include <algorithm>
#include <cstring>
#include <string>
#include <map>
#include <mutex>
#include <vector>

#include "gb_runtime.cuh"

namespace gb {

static thread_local uint32_t t_lane = 0;

uint32_t current_lane() { return t_lane; }
void set_lane(uint32_t lane) { t_lane = lane; }

int current_device()
{
    int d = 0;
    GB_CUDA_OK(cudaGetDevice(&d));
    return d;
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
cudaStream_t g_streams[kMaxDevices][GB_MAX_LANES + 1];
// lane status words: host view and device view of 2 words per lane
uint32_t *g_status_host[kMaxDevices][GB_MAX_LANES + 1];
uint32_t *g_status_dev[kMaxDevices][GB_MAX_LANES + 1];
std::atomic<unsigned long long> g_timeouts{0};
bool g_pool_ready[kMaxDevices];
std::atomic<unsigned long long> g_h2d{0}, g_d2h{0};

void ensure_pool(int dev)
{
    if (g_pool_ready[dev]) return;
    cudaMemPool_t pool;
    GB_CUDA_OK(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t threshold = UINT64_MAX;
    GB_CUDA_OK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
    g_pool_ready[dev] = true;
}
}  // namespace

cudaStream_t lane_stream()
{
    int dev = current_device();
    if (dev < 0 || dev >= kMaxDevices) throw cuda_error(-1, "device index out of range");
    uint32_t lane = t_lane;
    std::lock_guard<std::mutex> lk(g_mutex);
    ensure_pool(dev);
    cudaStream_t &s = g_streams[dev][lane];
    if (!s) GB_CUDA_OK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    return s;
}

// the calling thread's lane status words (created with the lane's stream)
static void lane_status_words(uint32_t **host, uint32_t **dev)
{
    const int d = current_device();
    if (d < 0 || d >= kMaxDevices) throw cuda_error(-1, "device index out of range");
    const uint32_t lane = t_lane;
    std::lock_guard<std::mutex> lk(g_mutex);
    if (!g_status_host[d][lane]) {
        uint32_t *h = nullptr, *dv = nullptr;
        GB_CUDA_OK(cudaHostAlloc((void **)&h, 2 * sizeof(uint32_t), cudaHostAllocMapped | cudaHostAllocPortable));
        h[0] = h[1] = 0;
        GB_CUDA_OK(cudaHostGetDevicePointer((void **)&dv, h, 0));
        g_status_host[d][lane] = h;
        g_status_dev[d][lane] = dv;
    }
    *host = g_status_host[d][lane];
    *dev = g_status_dev[d][lane];
}

uint32_t *lane_status_device()
{
    uint32_t *h, *d;
    lane_status_words(&h, &d);
    return d;
}

void lane_check()
{
    uint32_t *h, *d;
    lane_status_words(&h, &d);
    volatile uint32_t *w = h;
    const uint32_t a = w[0], b = w[1];
    if (a || b) {
        w[0] = 0;
        w[1] = 0;
        g_timeouts.fetch_add((unsigned long long)a + b);
        throw cuda_error((int)cudaErrorLaunchTimeout,
                         a ? "an NTT twiddle copy of this lane's work did not complete; results since the "
                             "previous synchronisation are invalid"
                           : "an NTT work-queue wait of this lane's work ran out; results since the previous "
                             "synchronisation are invalid");
    }
}

void lane_sync(cudaStream_t s)
{
    GB_CUDA_OK(cudaStreamSynchronize(s));
    lane_check();
}

unsigned long long lane_timeouts_take() { return g_timeouts.exchange(0); }

void *dev_alloc(size_t bytes, cudaStream_t s)
{
    void *p = nullptr;
    if (bytes == 0) return nullptr;
    GB_CUDA_OK(cudaMallocAsync(&p, bytes, s));
    return p;
}

void dev_free(void *p, cudaStream_t s)
{
    if (p) cudaFreeAsync(p, s);
}

fr_device_vec *device_vec_new(size_t len, cudaStream_t s)
{
    auto *v = new fr_device_vec();
    v->len = len;
    v->device = current_device();
    v->owner = s;
    try {
        if (len) v->values = (fr_t *)dev_alloc(len * sizeof(fr_t), s);
        GB_CUDA_OK(cudaEventCreateWithFlags(&v->ready, cudaEventDisableTiming));
    } catch (...) {
        if (v->values) dev_free(v->values, s);
        delete v;
        throw;
    }
    return v;
}

void device_vec_mark_ready(fr_device_vec *v, cudaStream_t s)
{
    GB_CUDA_OK(cudaEventRecord(v->ready, s));
    v->owner = s;
}

void device_vec_wait(const fr_device_vec *v, cudaStream_t s)
{
    if (v->ready && v->owner != s) GB_CUDA_OK(cudaStreamWaitEvent(s, v->ready, 0));
}

static void CUDART_CB host_sleep(void *ms)
{
    std::this_thread::sleep_for(std::chrono::milliseconds((uintptr_t)ms));
}

void stream_host_delay(cudaStream_t s, uint32_t ms)
{
    if (ms) GB_CUDA_OK(cudaLaunchHostFunc(s, host_sleep, (void *)(uintptr_t)ms));
}

void device_vec_delete(fr_device_vec *v)
{
    if (!v) return;
    cudaStream_t s = v->owner;
    if (v->values) {
        // free after every queued user of the vector on its owner stream
        dev_free(v->values, s);
    }
    if (v->ready) cudaEventDestroy(v->ready);
    delete v;
}

void h2d(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    if (!bytes) return;
    GB_CUDA_OK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    count_transfer(true, bytes);
}

void d2h(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    if (!bytes) return;
    GB_CUDA_OK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    count_transfer(false, bytes);
}

void count_transfer(bool to_device, size_t bytes)
{
    (to_device ? g_h2d : g_d2h).fetch_add(bytes, std::memory_order_relaxed);
}

static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ---- per-kernel event timing ----
namespace {
std::atomic<bool> g_prof{false};
struct pending_t {
    cudaEvent_t a, b;
    int slot;
};
std::mutex g_prof_mu;
std::vector<cudaEvent_t> g_event_pool;
std::vector<pending_t> g_pending;
std::vector<std::pair<cudaEvent_t, int>> g_open;  // token -> (start event, unused)
double g_slot_ms[GB_SLOTS];
unsigned long long g_slot_n[GB_SLOTS];

cudaEvent_t take_event()
{
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    GB_CUDA_OK(cudaEventCreate(&e));
    return e;
}
}  // namespace

bool profiling_enabled() { return g_prof.load(std::memory_order_relaxed); }

int timed_begin(cudaStream_t s)
{
    if (!profiling_enabled()) return -1;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEvent_t e = take_event();
    GB_CUDA_OK(cudaEventRecord(e, s));
    g_open.push_back({e, 0});
    return (int)g_open.size() - 1;
}

void timed_end(int token, cudaStream_t s, int slot)
{
    if (token < 0) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEvent_t e = take_event();
    GB_CUDA_OK(cudaEventRecord(e, s));
    g_pending.push_back({g_open[token].first, e, slot});
}

void timed_collect()
{
    if (!profiling_enabled()) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto &p : g_pending) {
        if (cudaEventSynchronize(p.b) == cudaSuccess) {
            float ms = 0;
            if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
                g_slot_ms[p.slot] += ms;
                g_slot_n[p.slot] += 1;
            }
        }
        g_event_pool.push_back(p.a);
        g_event_pool.push_back(p.b);
    }
    g_pending.clear();
    g_open.clear();
}

}  // namespace gb

using namespace gb;

// ---------------------------------------------------------------- autotuner
namespace gb {
namespace {
std::atomic<bool> g_autotune{false};
std::mutex g_tune_mu;
std::map<std::string, int> g_tune;
}  // namespace

bool autotune_enabled() { return g_autotune.load(std::memory_order_relaxed); }

bool autotune_lookup(const std::string &key, int *value)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it == g_tune.end()) return false;
    *value = it->second;
    return true;
}

void autotune_store(const std::string &key, int value)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = value;
}

}  // namespace gb

extern "C" {

void gb_autotune_set(int enabled) { g_autotune.store(enabled != 0); }

void gb_autotune_reset(void)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}

// "key=value;" for every tuned key, truncated to len - 1 characters;
// returns the full length
size_t gb_autotune_report(char *buf, size_t len)
{
    std::string out;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (auto &kv : g_tune) out += kv.first + "=" + std::to_string(kv.second) + ";";
    }
    if (buf && len) {
        size_t k = std::min(len - 1, out.size());
        memcpy(buf, out.data(), k);
        buf[k] = 0;
    }
    return out.size();
}



// midnight-sppark-msm/src/bls12_381_g1_msm.cu:134-146
RustError midnight_sppark_execution_lane_set(uint32_t lane)
{
    if (lane > GB_MAX_LANES) return make_error((int)cudaErrorInvalidValue, "execution lane out of range");
    set_lane(lane);
    return ok();
}

// Transfer counters (reference: midnight-sppark-msm/src/lib.rs:485-760 keeps
// them on the Rust side per op; here the library counts its own copies).
void gb_transfer_counters(uint64_t *h2d_bytes, uint64_t *d2h_bytes)
{
    if (h2d_bytes) *h2d_bytes = g_h2d.load();
    if (d2h_bytes) *d2h_bytes = g_d2h.load();
}

void gb_transfer_counters_reset(void)
{
    g_h2d.store(0);
    g_d2h.store(0);
}

// Kernel launches issued by the library since load.
uint64_t gb_launch_counter(void) { return g_launches.load(); }

// The calling thread's lane stream (cudaStream_t), for callers that want to
// order or time their own work against the library's.
void *gb_lane_stream(void)
{
    try {
        return (void *)lane_stream();
    } catch (...) {
        return nullptr;
    }
}

// Per-kernel CUDA-event timing (slot 0: MSM bucket accumulation kernel,
// slot 1: whole MSM, slot 2: NTT passes, slots 3-5: the MSM's recode and
// sort, bucket fix-up, and bucket reduction with window combination).
void gb_profile_enable(int on)
{
    g_prof.store(on != 0);
}

void gb_profile_read(int slot, double *total_ms, uint64_t *launches)
{
    timed_collect();
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (slot < 0 || slot >= GB_SLOTS) {
        if (total_ms) *total_ms = 0;
        if (launches) *launches = 0;
        return;
    }
    if (total_ms) *total_ms = g_slot_ms[slot];
    if (launches) *launches = g_slot_n[slot];
}

void gb_profile_reset(void)
{
    timed_collect();
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (int i = 0; i < GB_SLOTS; i++) {
        g_slot_ms[i] = 0;
        g_slot_n[i] = 0;
    }
}

// Frees a message string returned inside a RustError (for callers that do
// not share the C runtime's free()).
void gb_error_free(char *message) { free(message); }

}  // extern "C"
