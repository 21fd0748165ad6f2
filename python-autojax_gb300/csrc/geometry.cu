// Mask geometry and runtime helpers.
//
// mask_2d_circular_from (numba.py:50-86) is reproduced bit-exactly: the same
// float64 operations in the same order, with explicitly rounded intrinsics so
// the compiler cannot contract them into fused multiply-adds.

#include "aj_common.cuh"

namespace aj {

int g_last_cuda_error = 0;
unsigned long long g_launches = 0;

// Throughput probe: 8 independent fused multiply-add chains per thread.
template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

int num_sms() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    if (cached[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
        cached[dev] = n;
    }
    return cached[dev];
}

__global__ void mask_circular_kernel(int64_t ny, int64_t nx, double psy, double psx, double r2, double cy,
                                     double cx, uint8_t* mask) {
    int64_t n = ny * nx;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t y = t / nx, x = t - y * nx;
        double dy = __dmul_rn(__dsub_rn((double)y, cy), psy);
        double dx = __dmul_rn(__dsub_rn((double)x, cx), psx);
        double d2 = __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx));
        mask[t] = (r2 < d2) ? 1 : 0;
    }
}

// One block: row-major compaction of the unmasked pixels (argwhere(~mask)).
__global__ void slim_from_mask_kernel(const uint8_t* mask, int64_t ny, int64_t nx, const double* grid_2d,
                                      int64_t max_out, int64_t* native, double* grid_slim, int64_t* count) {
    __shared__ int64_t warp_tot[32];
    __shared__ int64_t base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const int64_t n = ny * nx;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t c0 = 0; c0 < n; c0 += blockDim.x) {
        int64_t t = c0 + threadIdx.x;
        int flag = (t < n && mask[t] == 0) ? 1 : 0;
        unsigned ball = __ballot_sync(0xffffffffu, flag);
        int in_warp = __popc(ball & ((1u << lane) - 1u));
        if (lane == 31) warp_tot[wid] = __popc(ball);
        __syncthreads();
        int64_t before = 0;
        for (int w = 0; w < wid; ++w) before += warp_tot[w];
        int64_t pos = base + before + in_warp;
        if (flag && pos < max_out) {
            int64_t y = t / nx, x = t - y * nx;
            if (native) {
                native[2 * pos] = y;
                native[2 * pos + 1] = x;
            }
            if (grid_slim && grid_2d) {
                grid_slim[2 * pos] = grid_2d[2 * t];
                grid_slim[2 * pos + 1] = grid_2d[2 * t + 1];
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int64_t tot = 0;
            for (int w = 0; w < nw; ++w) tot += warp_tot[w];
            base += tot;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = base;
}

}  // namespace aj

using namespace aj;

extern "C" {

const char* aj_version(void) { return "autojax_gb300 0.1.0 (sm_103a)"; }

int aj_last_cuda_error(void) { return g_last_cuda_error; }

unsigned long long aj_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

int aj_probe_fma(int precision, int64_t blocks, int iters, void* out, void* stream) {
    if (blocks <= 0 || iters <= 0 || !out) return AJ_ERR_ARG;
    if (precision == AJ_FP64)
        fma_probe_kernel<double><<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(static_cast<double*>(out), iters,
                                                                                  0.999, 0.001);
    else
        fma_probe_kernel<float><<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(static_cast<float*>(out), iters,
                                                                                 0.999f, 0.001f);
    return check_launch();
}

int aj_mask_2d_circular(int64_t ny, int64_t nx, double psy, double psx, double radius, double centre_y,
                        double centre_x, uint8_t* mask, void* stream) {
    if (ny < 0 || nx < 0 || (!mask && ny * nx > 0)) return AJ_ERR_ARG;
    if (ny * nx == 0) return AJ_OK;
    // numba.py:41-44: centres_scaled
    double cy = 0.5 * (double)(ny - 1) - (centre_y / psy);
    double cx = 0.5 * (double)(nx - 1) + (centre_x / psx);
    double r2 = radius * radius;
    mask_circular_kernel<<<blocks_for(ny * nx, 256, 4096), 256, 0, as_stream(stream)>>>(ny, nx, psy, psx, r2, cy, cx,
                                                                                      mask);
    return check_launch();
}

int aj_slim_from_mask(const uint8_t* mask, int64_t ny, int64_t nx, const double* grid_2d, int64_t max_out,
                      int64_t* native_index, double* grid_slim, int64_t* count, void* stream) {
    if (!mask || !count || ny < 0 || nx < 0 || max_out < 0) return AJ_ERR_ARG;
    slim_from_mask_kernel<<<1, 1024, 0, as_stream(stream)>>>(mask, ny, nx, grid_2d, max_out, native_index, grid_slim,
                                                             count);
    return check_launch();
}

}  // extern "C"
