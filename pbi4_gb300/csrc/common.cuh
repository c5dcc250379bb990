// common.cuh -- shared definitions for the PBI4 GB300 estimator library.
//
// Grid conventions (identical to the reference's Fortran arrays):
//   a 3-D grid a(ix,iy,iz), 1-based, first index fastest, is stored as the
//   C array a[z][y][x] with x = ix-1 fastest.  A real-to-complex transform of
//   that array gives the kx >= 0 half spectrum h[z][y][x], x in [0, N/2],
//   i.e. exactly the part ix <= N/2+1 that the reference's routines read.
// Frequencies follow powerI4.f90:435: index i -> k = i for i <= N/2, else i-N
// (the Nyquist plane maps to +N/2).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <stddef.h>

#include <atomic>
#include <vector>

#include "../../include/pbi4gpu.h"

namespace pbi4g {

// float32 constant of the reference: `real, parameter :: twopi = 6.28319`.
constexpr float kTwoPiF = 6.28319f;

// Set the thread-local error message; returns `code`.
int set_error(int code, const char* fmt, ...);

#define PBI4G_CUDA(call)                                                                      \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return ::pbi4g::set_error(PBI4G_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, \
                                      cudaGetErrorString(e_));                                \
    } while (0)

#define PBI4G_CUFFT(call)                                                                     \
    do {                                                                                      \
        cufftResult r_ = (call);                                                              \
        if (r_ != CUFFT_SUCCESS)                                                              \
            return ::pbi4g::set_error(PBI4G_ERR_CUFFT, "%s:%d %s: cufft error %d", __FILE__,  \
                                      __LINE__, #call, (int)r_);                              \
    } while (0)

#define PBI4G_CHECK(call)          \
    do {                           \
        int s_ = (call);           \
        if (s_ != PBI4G_OK) return s_; \
    } while (0)

#define PBI4G_LAUNCH_CHECK() PBI4G_CUDA(cudaGetLastError())

// Fortran nint(): round half away from zero.
__host__ __device__ inline long long f_nint(double x) { return llround(x); }

// signed frequency of 0-based index i on an n grid, Nyquist -> +n/2
__host__ __device__ inline int kfreq0(int i, int n) { return i <= n / 2 ? i : i - n; }
// |k| along one axis as the shell binning sees it: min(i, n-i)
__host__ __device__ inline int kabs0(int i, int n) { return i < n - i ? i : n - i; }
// 0-based index of -k
__host__ __device__ inline int kneg0(int i, int n) { return i == 0 ? 0 : n - i; }

inline int grid_blocks(size_t n, int threads, int cap = 152 * 32) {
    size_t b = (n + threads - 1) / threads;
    if (b > (size_t)cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

inline size_t half_cells(int N) { return (size_t)N * N * (N / 2 + 1); }
inline size_t full_cells(int N) { return (size_t)N * N * N; }

// Per-box scalars the graph-captured pipeline reads from device memory (a
// captured launch cannot carry a per-box value): the particle count and the
// two factors derived from it, computed on the host by the same formulas the
// direct path passes by value.
struct BoxPar {
    long long npart;
    double fcomb_cf;    // interlacing / window normalisation over npart (fcomb_half)
    double pow_sn;      // 1 / npart / kf^3 (bk_finalize)
    const double *pos;  // the box's positions, rows of the capacity (read by the captured assignment)
};

// Device allocations this library has made through DevBuf since it was loaded
// (pbi4g_device_allocs), and the host-side failure hook of
// pbi4g_debug_fail_alloc: armed with k > 0, the k-th next DevBuf allocation
// reports PBI4G_ERR_NOMEM without calling cudaMalloc.
inline std::atomic<long long> g_dev_allocs{0};
inline std::atomic<int> g_fail_alloc_in{0};

// true when an armed failure hook has come to this allocation (and disarms it)
inline bool injected_alloc_failure() {
    int k = g_fail_alloc_in.load();
    while (k > 0 && !g_fail_alloc_in.compare_exchange_weak(k, k - 1)) {
    }
    return k == 1;
}

// RAII device buffer
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    int ensure(size_t n) {
        if (n <= bytes && p) return PBI4G_OK;
        release();
        if (n == 0) n = 16;
        if (injected_alloc_failure())
            return set_error(PBI4G_ERR_NOMEM, "cudaMalloc(%zu) failed: injected by pbi4g_debug_fail_alloc", n);
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return set_error(PBI4G_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", n, cudaGetErrorString(e));
        }
        g_dev_allocs.fetch_add(1);
        bytes = n;
        return PBI4G_OK;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Per-stage CUDA-event timing on a stream (see pbi4g_plan_enable_timing).
struct Prof {
    bool on = false;
    struct Rec { int stage; cudaEvent_t a, b; };
    std::vector<cudaEvent_t> pool;
    std::vector<Rec> recs;
    cudaEvent_t cur_a = nullptr;
    int cur_stage = -1;
    ~Prof();
    cudaEvent_t get();
    void begin(int stage, cudaStream_t st);
    void end(cudaStream_t st);
};

}  // namespace pbi4g
