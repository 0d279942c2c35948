// cpdlp_common.cuh -- shared infrastructure of libcoolpdlp_cuda (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>
#include <vector>

#include "../../include/coolpdlp_cuda.h"

namespace cpdlp {

// ---------------------------------------------------------------------------
// errors: every internal failure is a cpdlp::Error carrying a CPDLP_ERR_* code;
// the C-ABI layer turns it into a status and cpdlp_last_error().
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(int code, const std::string& msg) { throw Error(code, msg); }

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
    if (e != cudaSuccess) {
        char buf[512];
        snprintf(buf, sizeof(buf), "%s failed at %s:%d: %s", what, file, line,
                 cudaGetErrorString(e));
        if (e == cudaErrorMemoryAllocation) fail(CPDLP_ERR_OUT_OF_MEMORY, buf);
        fail(CPDLP_ERR_CUDA, buf);
    }
}
#define CK(x) ::cpdlp::cuda_check((x), #x, __FILE__, __LINE__)
#define CK_LAUNCH() ::cpdlp::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)

// ---------------------------------------------------------------------------
// device buffer (owning, move-only), stream-ordered: allocated with
// cudaMallocAsync on the calling thread's current allocation stream and freed
// with cudaFreeAsync on the same stream, so that creating or dropping buffers
// never waits for kernels running on other streams (a plain cudaFree would
// synchronise the device, stalling every batch in flight).  Buffers must be
// released before the stream they were allocated on is destroyed.
// ---------------------------------------------------------------------------
inline cudaStream_t& alloc_stream() {
    static thread_local cudaStream_t s = nullptr;
    return s;
}
struct AllocScope {
    cudaStream_t prev;
    explicit AllocScope(cudaStream_t s) : prev(alloc_stream()) { alloc_stream() = s; }
    ~AllocScope() { alloc_stream() = prev; }
    AllocScope(const AllocScope&) = delete;
    AllocScope& operator=(const AllocScope&) = delete;
};

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    DBuf() = default;
    explicit DBuf(size_t count) { alloc(count); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; s = o.s; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DBuf() { release(); }
    void alloc(size_t count) {
        release();
        n = count;
        s = alloc_stream();
        if (count) CK(cudaMallocAsync((void**)&p, sizeof(T) * count, s));
    }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return sizeof(T) * n; }
    T* get() const { return p; }
};

// ---------------------------------------------------------------------------
// scalar semantics shared by host and device (src/utils/linalg.jl:1-53)
// Base.max/min on floats: NaN propagates and -0.0 < +0.0.
// ---------------------------------------------------------------------------
template <class T>
__host__ __device__ __forceinline__ T jl_max(T x, T y) {
    bool sx = signbit(x), sy = signbit(y);
    if ((y > x) || (sy < sx)) return (x != x) ? x : y;
    return (y != y) ? y : x;
}
template <class T>
__host__ __device__ __forceinline__ T jl_min(T x, T y) {
    bool sx = signbit(x), sy = signbit(y);
    if ((y < x) || (sy > sx)) return (x != x) ? x : y;
    return (y != y) ? y : x;
}
template <class T>
__host__ __device__ __forceinline__ T proj_box(T x, T l, T u) { return jl_min(u, jl_max(l, x)); }
template <class T>
__host__ __device__ __forceinline__ T pos_part(T a) { return jl_max(a, T(0)); }
template <class T>
__host__ __device__ __forceinline__ T neg_part(T a) { return -jl_min(a, T(0)); }
template <class T>
__host__ __device__ __forceinline__ T safeprod_left(T l, T r) { return isinf(l) ? r : l * r; }
template <class T>
__host__ __device__ __forceinline__ T proj_multiplier(T lam, T l, T u) {
    bool lmin = (l == -INFINITY), umax = (u == INFINITY);
    if (lmin) return umax ? T(0) : -neg_part(lam);
    return umax ? pos_part(lam) : lam;
}
template <class T>
__host__ __device__ __forceinline__ T combine(T l, T u) {
    T ls = isfinite(l) ? fabs(l) : T(0);
    T us = isfinite(u) ? fabs(u) : T(0);
    return jl_max(jl_max(T(0), ls), us);
}

// Exact IEEE products/sums without contraction into FMA, so that sequential
// sums match the Float64 reference operation by operation.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// Scalar loads as volatile PTX: volatile asm statements keep their relative
// order, so loads meant to be in flight together (prefetches) are issued
// before the code that consumes them instead of being sunk to their use.
// ld_stream: read once per pass (evict-first); ld_keep: read-only data that
// other kernels of the same step re-read (normal L2 policy).
__device__ __forceinline__ float ld_stream(const float* p) {
    float v;
    asm volatile("ld.global.cs.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ double ld_stream(const double* p) {
    double v;
    asm volatile("ld.global.cs.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ float ld_keep(const float* p) {
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ double ld_keep(const double* p) {
    double v;
    asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ int ld_keep(const int* p) {
    int v;
    asm volatile("ld.global.nc.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------
struct Handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    int num_sms = 0;
    // error history of the last cpdlp_solve on this handle (every phase of a
    // mixed-precision solve, passes counted from the start of the solve)
    std::vector<int64_t> solve_hist_passes;
    std::vector<cpdlp_kkt_errors> solve_hist_err;
    // reusable small host-pinned area for reductions read back each check
    double* pinned = nullptr;
    size_t pinned_bytes = 0;
    double* pinned_area(size_t bytes) {
        if (bytes > pinned_bytes) {
            if (pinned) cudaFreeHost(pinned);
            pinned = nullptr;
            pinned_bytes = 0;
            CK(cudaMallocHost((void**)&pinned, bytes));
            pinned_bytes = bytes;
        }
        return pinned;
    }
    // Reusable blocks of mapped, page-locked host memory that kernels write
    // results into while they run.  Blocks are returned to the pool instead of
    // freed, because freeing page-locked memory waits for the whole device.
    struct HostBlock {
        void* p;
        size_t bytes;
        bool used;
    };
    std::vector<HostBlock> host_blocks;
    void* host_get(size_t bytes) {
        int best = -1;
        for (size_t i = 0; i < host_blocks.size(); i++) {
            const HostBlock& b = host_blocks[i];
            if (!b.used && b.bytes >= bytes && (best < 0 || b.bytes < host_blocks[best].bytes))
                best = (int)i;
        }
        if (best >= 0) {
            host_blocks[best].used = true;
            return host_blocks[best].p;
        }
        void* p = nullptr;
        const size_t sz = std::max<size_t>(bytes, 1 << 16);
        CK(cudaHostAlloc(&p, sz, cudaHostAllocMapped | cudaHostAllocPortable));
        host_blocks.push_back(HostBlock{p, sz, true});
        return p;
    }
    void host_put(void* p) {
        for (HostBlock& b : host_blocks)
            if (b.p == p) b.used = false;
    }
    void host_release_all() {
        for (HostBlock& b : host_blocks) cudaFreeHost(b.p);
        host_blocks.clear();
    }
};

inline unsigned grid_for(int64_t items, int threads, int64_t cap = 1 << 30) {
    int64_t g = (items + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// wall clock (seconds)
double now_seconds();

// f(k) for k in [0, count) on up to 16 host threads, each a contiguous block
// of k (f must not depend on which thread runs it)
template <class F>
void parallel_for(int64_t count, F&& f) {
    const int64_t hw = std::max<int64_t>(1, std::min<int64_t>(16, std::thread::hardware_concurrency()));
    const int64_t nt = std::min<int64_t>(hw, std::max<int64_t>(1, count / 64));
    if (nt <= 1) {
        for (int64_t k = 0; k < count; k++) f(k);
        return;
    }
    std::vector<std::thread> th;
    for (int64_t t = 0; t < nt; t++)
        th.emplace_back([&, t] {
            for (int64_t k = count * t / nt; k < count * (t + 1) / nt; k++) f(k);
        });
    for (auto& x : th) x.join();
}

}  // namespace cpdlp
