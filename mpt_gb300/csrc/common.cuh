// common.cuh - shared host/device plumbing for the mptg C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>
#include <string.h>
#include <math.h>
#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/mptg.h"
#include "../../include/mptg_detmath.h"

#define MPTG_BUCKET 32       // points per kd-tree leaf bucket (one per lane)
#define MPTG_MAX_DIM 16      // largest state dimension supported by the kernels
#define MPTG_MAX_DEPTH 60    // deepest kd-tree node (register stack holds 64)
#define MPTG_MAX_EDGE_SAMPLES (1 << 22)  // longer discretised edges are reported invalid

// device-side error bits (per tree / per scene status word)
#define MPTG_DEVERR_CAPACITY 1u
#define MPTG_DEVERR_DEPTH 2u
#define MPTG_DEVERR_BAD_STATE 4u
#define MPTG_DEVERR_STACK 8u

struct mptg_ctx {
    int device = 0;
    int sms = 152;  // multiprocessors of the device
    char err[512] = {0};
    std::atomic<uint64_t> launches{0};
    std::mutex mu;
};

// Records a message for mptg_last_error and returns the status.
mptg_status mptg_fail(mptg_ctx* ctx, mptg_status st, const char* fmt, ...);

#define MPTG_CUDA_TRY(ctx, call)                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return mptg_fail((ctx), e_ == cudaErrorMemoryAllocation ? MPTG_ERR_OOM      \
                                                                    : MPTG_ERR_CUDA,    \
                             "%s failed: %s", #call, cudaGetErrorString(e_));           \
    } while (0)

#define MPTG_LAUNCHED(ctx) ((ctx)->launches.fetch_add(1, std::memory_order_relaxed))

// true when p is device (or managed) memory usable by kernels directly
bool mptg_is_device_ptr(const void* p);

// A device view of a caller buffer: the caller's pointer when it is device
// memory, else a stream-ordered temporary (copied in for inputs).
struct DevBuf {
    void* dptr = nullptr;
    const void* user = nullptr;
    size_t bytes = 0;
    bool owned = false;
};
mptg_status mptg_stage_in(mptg_ctx* ctx, const void* user, size_t bytes, cudaStream_t s, DevBuf* out);
mptg_status mptg_stage_out_alloc(mptg_ctx* ctx, void* user, size_t bytes, cudaStream_t s, DevBuf* out);
// copies an output temporary back to the caller (async) and releases temporaries
mptg_status mptg_stage_finish(mptg_ctx* ctx, cudaStream_t s, DevBuf* outs, int nouts, DevBuf* ins, int nins);

// Runs fn() (returning cudaError_t) the first time for (key, the current
// device) and after any call that failed: for per-device one-time settings
// such as cudaFuncSetAttribute, which applies to the current device only.
// Thread-safe; the settings of different keys may run concurrently.
template <class Fn>
inline cudaError_t mptg_once_per_device(const void* key, Fn fn) {
    static std::mutex mu;
    static std::vector<std::pair<const void*, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto& d : done)
        if (d.first == key && d.second == dev) return cudaSuccess;
    e = fn();
    if (e == cudaSuccess) done.emplace_back(key, dev);
    return e;
}

static inline unsigned mptg_blocks(size_t n, unsigned threads) {
    return (unsigned)((n + threads - 1) / threads);
}

// ordered float <-> int mapping so atomicMin/atomicMax on int order floats
__device__ __forceinline__ int mptg_f2ord(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float mptg_ord2f(int i) {
    return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}
