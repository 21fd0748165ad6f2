// Shared helpers of the autojax_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "autojax_gb300.h"

namespace aj {

// last CUDA error seen by a launch check (exported through aj_last_cuda_error)
extern int g_last_cuda_error;
// kernel launches checked so far in this process (exported through aj_launch_count)
extern unsigned long long g_launches;

inline int check_launch() {
    __atomic_add_fetch(&g_launches, 1ull, __ATOMIC_RELAXED);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        g_last_cuda_error = static_cast<int>(e);
        return AJ_ERR_CUDA;
    }
    return AJ_OK;
}

#define AJ_TRY(...)                          \
    do {                                     \
        int _aj_rc = (__VA_ARGS__);          \
        if (_aj_rc != AJ_OK) return _aj_rc;  \
    } while (0)

#define AJ_LAUNCHED() AJ_TRY(::aj::check_launch())

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// streaming multiprocessors of the current device (cached per device)
int num_sms();

inline unsigned blocks_for(int64_t n, int threads, int64_t cap = (1ll << 31) - 1) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return static_cast<unsigned>(b);
}

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// true when every pointer is 16-byte aligned (for float4 loads)
template <typename... T>
inline bool aligned16(const T*... p) {
    return ((reinterpret_cast<uintptr_t>(p) % 16 == 0) && ...);
}

// Carves typed sub-buffers out of a caller workspace.
struct Carver {
    char* base;
    size_t used = 0;
    size_t cap;
    Carver(void* p, size_t bytes) : base(static_cast<char*>(p)), cap(bytes) {}
    template <typename T>
    T* take(size_t count) {
        size_t off = align_up(used);
        used = off + count * sizeof(T);
        return reinterpret_cast<T*>(base ? base + off : nullptr);
    }
    bool fits() const { return used <= cap; }
};

// Sizes a workspace with the same sequence of take() calls as the user.
struct Sizer {
    size_t used = 0;
    template <typename T>
    void take(size_t count) { used = align_up(used) + count * sizeof(T); }
    size_t total() const { return align_up(used); }
};

// ------------------------------------------------------------ device side

// Records a data-dependent failure: first writer wins the code, index is informative.
__device__ __forceinline__ void report(int* info, int code, int64_t where) {
    if (info) {
        if (atomicCAS(info, 0, code) == 0) info[1] = static_cast<int>(where < 0x7fffffff ? where : 0x7fffffff);
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum (blockDim.x a multiple of 32, <= 1024); result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* smem32) {
    v = warp_sum(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem32[wid] = v;
    __syncthreads();
    int nw = blockDim.x >> 5;
    v = (threadIdx.x < nw) ? smem32[threadIdx.x] : 0.0;
    if (wid == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}

// Kahan-compensated add of a float into a (hi, lo) pair.
__device__ __forceinline__ void kahan_add(float& hi, float& lo, float x) {
    float y = x - lo;
    float t = hi + y;
    lo = (t - hi) - y;
    hi = t;
}

}  // namespace aj
