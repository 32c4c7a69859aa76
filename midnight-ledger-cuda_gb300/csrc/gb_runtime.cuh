// Host runtime shared by every entry point of the library: the error ABI,
// execution lanes (one CUDA stream per lane), stream-ordered device memory
// and the resident device-vector handle.
//
// Error ABI: every fallible entry point returns `RustError` by value,
// {int code; char *message}, code 0 = success, otherwise a cudaError_t value
// or -1; `message` is strdup()'d here and released by the caller with free().
// This is the by-value struct of vendor/sppark-0.1.15/sppark/util/rusterror.h
// that the reference's Rust side declares as `sppark::Error`
// (vendor/sppark-0.1.15/src/lib.rs:8-23).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <stdexcept>
#include <string>

#include "gb_curve.cuh"
#include "gb_prover.h"

namespace gb {

struct cuda_error : std::runtime_error {
    int code_;
    cuda_error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }
};

inline RustError ok() { return RustError{0, nullptr}; }

// boundary conversions: the C ABI's plain structs and the device types share
// one memory image (checked by the static_asserts at the end of this file)
inline fr_t from_raw(const RawFr &r)
{
    fr_t f;
    memcpy(&f, &r, sizeof(f));
    return f;
}

inline RustError make_error(int code, const char *msg)
{
    return RustError{code, msg ? strdup(msg) : nullptr};
}

#define GB_CUDA_OK(expr)                                                               \
    do {                                                                               \
        cudaError_t gb_e_ = (expr);                                                    \
        if (gb_e_ != cudaSuccess) {                                                    \
            throw ::gb::cuda_error((int)gb_e_, std::string(#expr " failed: ") +        \
                                                   cudaGetErrorString(gb_e_));         \
        }                                                                              \
    } while (0)

// every kernel launch of the library is followed by GB_CHECK_LAUNCH(), which
// also counts it (gb_launch_counter)
void note_launch();
#define GB_CHECK_LAUNCH()                  \
    do {                                   \
        ::gb::note_launch();               \
        GB_CUDA_OK(cudaGetLastError());    \
    } while (0)

// Wrap an entry-point body: C++ exceptions never cross the C ABI.
#define GB_ENTRY_BEGIN try {
#define GB_ENTRY_END                                                                   \
    }                                                                                  \
    catch (const ::gb::cuda_error &e)                                                  \
    {                                                                                  \
        return ::gb::make_error(e.code(), e.what());                                   \
    }                                                                                  \
    catch (const std::bad_alloc &)                                                     \
    {                                                                                  \
        return ::gb::make_error((int)cudaErrorMemoryAllocation, "host allocation failed"); \
    }                                                                                  \
    catch (const std::exception &e)                                                    \
    {                                                                                  \
        return ::gb::make_error(-1, e.what());                                         \
    }

// ---------------------------------------------------------------------------
// Lanes.  Lane 0 is the default; lanes 1..8 are private streams for
// concurrent proofs (midnight-sppark-msm/src/bls12_381_g1_msm.cu:46-146).
// The lane is a per-thread setting.
// ---------------------------------------------------------------------------
static constexpr uint32_t GB_MAX_LANES = 8;

uint32_t current_lane();
void set_lane(uint32_t lane);
// The calling thread's lane stream on the current device (created lazily).
cudaStream_t lane_stream();
int current_device();

// Status words of the bounded device waits (NTT twiddle copies, work-queue
// dependencies), two per (device, lane), in mapped page-locked host memory:
// a kernel whose wait runs out adds to its lane's word instead of failing,
// and the host reads the word after the lane's next synchronisation, as
// CUDA reports errors of asynchronous work at a later call.  lane_sync()
// synchronises the calling thread's lane stream and then throws
// cudaErrorLaunchTimeout if a wait of the lane's work ran out since the last
// check (the words are cleared); lane_check() does the check alone, without
// waiting.  Entry points that return data to the host synchronise through
// lane_sync(), so results that depend on a failed wait are never returned
// as success.
uint32_t *lane_status_device();
void lane_check();
void lane_sync(cudaStream_t s);
// waits that ran out since the last call, process-wide (the count is reset)
unsigned long long lane_timeouts_take();

// Stream-ordered device memory from the device's default memory pool, whose
// release threshold is raised once so freed blocks are reused, not returned.
void *dev_alloc(size_t bytes, cudaStream_t s);
void dev_free(void *p, cudaStream_t s);

template <class T>
struct dev_buf {
    T *ptr = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    dev_buf() = default;
    dev_buf(size_t count, cudaStream_t stream) : n(count), s(stream)
    {
        if (count) ptr = (T *)dev_alloc(count * sizeof(T), stream);
    }
    dev_buf(const dev_buf &) = delete;
    dev_buf &operator=(const dev_buf &) = delete;
    dev_buf(dev_buf &&o) noexcept : ptr(o.ptr), n(o.n), s(o.s) { o.ptr = nullptr; o.n = 0; }
    dev_buf &operator=(dev_buf &&o) noexcept
    {
        if (this != &o) { reset(); ptr = o.ptr; n = o.n; s = o.s; o.ptr = nullptr; o.n = 0; }
        return *this;
    }
    ~dev_buf() { reset(); }
    void reset()
    {
        if (ptr) dev_free(ptr, s);
        ptr = nullptr;
        n = 0;
    }
    T *release() { T *p = ptr; ptr = nullptr; n = 0; return p; }
    T *get() const { return ptr; }
    operator T *() const { return ptr; }
};

// Resident device vector of Fr values: the opaque `device_vec` handle of the
// reference FFI (scalar_device_vec_t, bls12_381_g1_msm.cu:1116-1147 usage).
// `ready` is recorded on the producing lane's stream after the last write so
// that a consumer on another lane can wait for it.
struct fr_device_vec {
    fr_t *values = nullptr;
    size_t len = 0;
    int device = 0;
    cudaEvent_t ready = nullptr;
    cudaStream_t owner = nullptr;
};

fr_device_vec *device_vec_new(size_t len, cudaStream_t s);
void device_vec_mark_ready(fr_device_vec *v, cudaStream_t s);
void device_vec_wait(const fr_device_vec *v, cudaStream_t s);
void device_vec_delete(fr_device_vec *v);

// holds stream s back on the host for ms milliseconds (a host function on
// the stream; the test hooks' stand-in for a slow producer)
void stream_host_delay(cudaStream_t s, uint32_t ms);

// host<->device copies on the lane stream (pageable or pinned host memory)
void h2d(void *dst, const void *src, size_t bytes, cudaStream_t s);
void d2h(void *dst, const void *src, size_t bytes, cudaStream_t s);

// Transfer accounting (bytes per direction), the counterpart of the
// reference's per-op transfer counters (midnight-sppark-msm/src/lib.rs:485-760).
void count_transfer(bool to_device, size_t bytes);

// Optional per-kernel timing with CUDA events on the launching stream:
// when enabled, timed_begin/timed_end bracket a launch and the elapsed time
// is folded into the named slot at the next timed_collect (after a sync).
bool profiling_enabled();
int timed_begin(cudaStream_t s);
void timed_end(int token, cudaStream_t s, int slot);
void timed_collect();
enum { GB_SLOT_MSM_ACCUMULATE = 0, GB_SLOT_MSM_TOTAL = 1, GB_SLOT_NTT = 2, GB_SLOT_MSM_SORT = 3,
       GB_SLOT_MSM_FIXUP = 4, GB_SLOT_MSM_REDUCE = 5, GB_SLOTS = 8 };

// Autotuner: when enabled, an operation with several launch shapes (the MSM
// window, the NTT pass variant) times its candidates the first time it meets
// a key and remembers the fastest.  Off by default: the cost models decide.
bool autotune_enabled();
bool autotune_lookup(const std::string &key, int *value);
void autotune_store(const std::string &key, int value);

// elapsed milliseconds of fn() on stream s (CUDA events, synchronises)
template <class F>
float time_on_stream(cudaStream_t s, F fn)
{
    cudaEvent_t a, b;
    GB_CUDA_OK(cudaEventCreate(&a));
    GB_CUDA_OK(cudaEventCreate(&b));
    GB_CUDA_OK(cudaEventRecord(a, s));
    fn();
    GB_CUDA_OK(cudaEventRecord(b, s));
    GB_CUDA_OK(cudaEventSynchronize(b));
    float ms = 0;
    GB_CUDA_OK(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

inline unsigned blocks_for(size_t n, unsigned threads)
{
    return (unsigned)((n + threads - 1) / threads);
}

}  // namespace gb

// RawFr etc. as plain-memory views
static_assert(sizeof(gb::fr_t) == 32, "Fr must be 32 bytes");
static_assert(sizeof(gb::fp_t) == 48, "Fp must be 48 bytes");
static_assert(sizeof(gb::affine_t) == 96, "affine must be 96 bytes");
static_assert(sizeof(gb::jacobian_t) == 144, "jacobian must be 144 bytes");
static_assert(sizeof(RawFr) == sizeof(gb::fr_t), "RawFr layout");
static_assert(sizeof(RawG1Affine) == sizeof(gb::affine_t), "RawG1Affine layout");
static_assert(sizeof(RawG1Projective) == sizeof(gb::jacobian_t), "RawG1Projective layout");
