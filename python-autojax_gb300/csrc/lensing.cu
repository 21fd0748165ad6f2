// The mapping-weight builder: SIS ray-tracing and barycentric / bilinear
// weights of the traced image pixels, with their adjoints.
//
// The reference's likelihood takes the mapping (pix_indexes, pix_weights) as
// an input (numba.py:294-376, 761-857); the weights come from PyAutoLens,
// which it does not vendor.  Building them on the device lets a sampler go
// from lens parameters (Einstein radius, source-pixel positions) to logE and
// back to their gradients without leaving the GPU:
//   theta_E, points --(trace, weights)--> pix_weights --(aj_log_evidence)--> logE
//   dlogE/dtheta_E, dlogE/dpoints <--(these adjoints)-- dlogE/dpix_weights
//
// Delaunay point location is exact and deterministic: a pixel maps to the
// first triangle (lowest index) whose three edge functions share the sign of
// its area, evaluated in float64 without contraction (__dmul_rn/__dsub_rn),
// so the choice on shared edges is the same as a float64 restatement's.  A
// float32 pre-test with a margin larger than its rounding error (so it never
// rejects a containing triangle) keeps most tests off the float64 pipe.

#include <math.h>

#include "aj_internal.cuh"

namespace aj {

namespace {

constexpr int LOC_THREADS = 256;
constexpr int LOC_TILE = 4096;  // triangles staged in shared memory per pass (6 floats each)

__device__ __forceinline__ double cross_rn(double ux, double uy, double vx, double vy) {
    return __dsub_rn(__dmul_rn(ux, vy), __dmul_rn(uy, vx));
}

// exact containment of (x, y) in triangle (a, b, c): every edge function shares D's sign (or is 0)
__device__ bool contains_exact(const double* __restrict__ P, const int64_t* __restrict__ tri, int64_t t, double x,
                               double y) {
    const int64_t ia = tri[3 * t], ib = tri[3 * t + 1], ic = tri[3 * t + 2];
    const double ax = P[2 * ia], ay = P[2 * ia + 1], bx = P[2 * ib], by = P[2 * ib + 1];
    const double cx = P[2 * ic], cy = P[2 * ic + 1];
    const double D = cross_rn(__dsub_rn(bx, ax), __dsub_rn(by, ay), __dsub_rn(cx, ax), __dsub_rn(cy, ay));
    if (D == 0.0) return false;
    const double na = cross_rn(__dsub_rn(bx, x), __dsub_rn(by, y), __dsub_rn(cx, x), __dsub_rn(cy, y));
    const double nb = cross_rn(__dsub_rn(cx, x), __dsub_rn(cy, y), __dsub_rn(ax, x), __dsub_rn(ay, y));
    const double nc = cross_rn(__dsub_rn(ax, x), __dsub_rn(ay, y), __dsub_rn(bx, x), __dsub_rn(by, y));
    const double s = D > 0.0 ? 1.0 : -1.0;
    return na * s >= 0.0 && nb * s >= 0.0 && nc * s >= 0.0;
}

// One warp per traced pixel: the lanes test the staged triangles, a warp-wide
// minimum picks the first exact hit.  Pixels still unplaced after every tile
// get their nearest vertex (first minimum of the squared distance).
__global__ void __launch_bounds__(LOC_THREADS)
    delaunay_weights_kernel(const double* __restrict__ beta, int64_t M, const double* __restrict__ P, int64_t S,
                            const int64_t* __restrict__ tri, int64_t T, int64_t* __restrict__ idx,
                            double* __restrict__ w, int* info) {
    extern __shared__ float tri_s[];  // LOC_TILE x 6: ax ay bx by cx cy
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t wpb = LOC_THREADS / 32;
    const int64_t stride = (int64_t)gridDim.x * wpb;
    for (int64_t t0 = 0; t0 < T; t0 += LOC_TILE) {
        const int64_t nt = (T - t0) < LOC_TILE ? (T - t0) : LOC_TILE;
        __syncthreads();
        for (int64_t e = threadIdx.x; e < nt; e += LOC_THREADS) {
            const int64_t t = t0 + e;
            bool ok = true;
            for (int v = 0; v < 3; ++v) {
                const int64_t k = tri[3 * t + v];
                if (k < 0 || k >= S) {
                    ok = false;
                    break;
                }
                tri_s[6 * e + 2 * v] = (float)P[2 * k];
                tri_s[6 * e + 2 * v + 1] = (float)P[2 * k + 1];
            }
            if (!ok) {
                report(info, AJ_INFO_INDEX_RANGE, 3 * t);
                for (int v = 0; v < 6; ++v) tri_s[6 * e + v] = 0.f;  // a degenerate triangle never matches
            }
        }
        __syncthreads();
        for (int64_t m = blockIdx.x * wpb + warp; m < M; m += stride) {
            if (t0 > 0 && idx[3 * m] != -2) continue;  // placed by an earlier tile
            const double xd = beta[2 * m], yd = beta[2 * m + 1];
            const float xf = (float)xd, yf = (float)yd;
            int best = 0x7fffffff;
            for (int64_t e = lane; e < nt; e += 32) {
                const float* q = tri_s + 6 * e;
                const float ux = q[0] - xf, uy = q[1] - yf, vx = q[2] - xf, vy = q[3] - yf;
                const float wx = q[4] - xf, wy = q[5] - yf;
                const float D = (q[2] - q[0]) * (q[5] - q[1]) - (q[3] - q[1]) * (q[4] - q[0]);
                const float na = vx * wy - vy * wx, nb = wx * uy - wy * ux, nc = ux * vy - uy * vx;
                float R = fmaxf(fmaxf(fabsf(xf), fabsf(yf)), fmaxf(fmaxf(fabsf(q[0]), fabsf(q[1])),
                                                                   fmaxf(fmaxf(fabsf(q[2]), fabsf(q[3])),
                                                                         fmaxf(fabsf(q[4]), fabsf(q[5])))));
                // rounding of these float32 edge functions stays below ~1.2e-6 R^2
                const float tol = 4e-6f * R * R;
                const float s = D > 0.f ? 1.f : -1.f;
                const bool maybe = fabsf(D) <= tol || (na * s >= -tol && nb * s >= -tol && nc * s >= -tol);
                if (maybe && contains_exact(P, tri, t0 + e, xd, yd)) {
                    best = (int)e;
                    break;  // the lane's triangles are in increasing order
                }
            }
            best = __reduce_min_sync(0xffffffffu, best);
            if (lane == 0) idx[3 * m] = best != 0x7fffffff ? t0 + best : -2;
        }
    }
    __syncwarp();
    for (int64_t m = blockIdx.x * wpb + warp; m < M; m += stride) {
        const int64_t t = T > 0 ? idx[3 * m] : -2;
        const double x = beta[2 * m], y = beta[2 * m + 1];
        if (t >= 0) {
            if (lane == 0) {
                const int64_t ia = tri[3 * t], ib = tri[3 * t + 1], ic = tri[3 * t + 2];
                const double ax = P[2 * ia], ay = P[2 * ia + 1], bx = P[2 * ib], by = P[2 * ib + 1];
                const double cx = P[2 * ic], cy = P[2 * ic + 1];
                const double D =
                    cross_rn(__dsub_rn(bx, ax), __dsub_rn(by, ay), __dsub_rn(cx, ax), __dsub_rn(cy, ay));
                const double na = cross_rn(__dsub_rn(bx, x), __dsub_rn(by, y), __dsub_rn(cx, x), __dsub_rn(cy, y));
                const double nb = cross_rn(__dsub_rn(cx, x), __dsub_rn(cy, y), __dsub_rn(ax, x), __dsub_rn(ay, y));
                const double nc = cross_rn(__dsub_rn(ax, x), __dsub_rn(ay, y), __dsub_rn(bx, x), __dsub_rn(by, y));
                idx[3 * m] = ia;
                idx[3 * m + 1] = ib;
                idx[3 * m + 2] = ic;
                w[3 * m] = __ddiv_rn(na, D);
                w[3 * m + 1] = __ddiv_rn(nb, D);
                w[3 * m + 2] = __ddiv_rn(nc, D);
            }
        } else {
            // outside the hull: nearest vertex, first minimum
            double bd = INFINITY;
            int64_t bk = S;
            for (int64_t k = lane; k < S; k += 32) {
                const double dx = __dsub_rn(x, P[2 * k]), dy = __dsub_rn(y, P[2 * k + 1]);
                const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
                if (d2 < bd) {
                    bd = d2;
                    bk = k;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double od = __shfl_xor_sync(0xffffffffu, bd, o);
                const int64_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
                if (od < bd || (od == bd && ok < bk)) {
                    bd = od;
                    bk = ok;
                }
            }
            if (lane == 0) {
                idx[3 * m] = bk < S ? bk : -1;
                idx[3 * m + 1] = -1;
                idx[3 * m + 2] = -1;
                w[3 * m] = bk < S ? 1.0 : 0.0;
                w[3 * m + 1] = 0.0;
                w[3 * m + 2] = 0.0;
            }
        }
    }
}

__global__ void init_minus2_kernel(int64_t* __restrict__ idx, int64_t M) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x)
        idx[3 * m] = -2;
}

__device__ __forceinline__ void dcross_du(double ux, double uy, double vx, double vy, double& gx, double& gy) {
    gx = vy;
    gy = -vx;
}

__device__ __forceinline__ void dcross_dv(double ux, double uy, double vx, double vy, double& gx, double& gy) {
    gx = -uy;
    gy = ux;
}

// l = sum_j g_j N_j / D = Q / D;  dl/dv = (dQ/dv - l dD/dv) / D for each vertex, dl/dx = -(sum of dQ/dv) / D
__global__ void delaunay_weights_vjp_kernel(const double* __restrict__ beta, int64_t M, const double* __restrict__ P,
                                            const int64_t* __restrict__ idx, const double* __restrict__ G,
                                            double* __restrict__ gP, double* __restrict__ gB) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ia = idx[3 * m], ib = idx[3 * m + 1], ic = idx[3 * m + 2];
        if (ib < 0 || ia < 0 || ic < 0) {
            gB[2 * m] = 0.0;
            gB[2 * m + 1] = 0.0;
            continue;
        }
        const double x = beta[2 * m], y = beta[2 * m + 1];
        const double ax = P[2 * ia], ay = P[2 * ia + 1], bx = P[2 * ib], by = P[2 * ib + 1];
        const double cx = P[2 * ic], cy = P[2 * ic + 1];
        const double g0 = G[3 * m], g1 = G[3 * m + 1], g2 = G[3 * m + 2];
        // u = b - x, v = c - x, q = a - x
        const double ux = bx - x, uy = by - y, vx = cx - x, vy = cy - y, qx = ax - x, qy = ay - y;
        const double D = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
        const double Q = g0 * (ux * vy - uy * vx) + g1 * (vx * qy - vy * qx) + g2 * (qx * uy - qy * ux);
        const double ell = Q / D;
        double t0x, t0y, t1x, t1y;
        // dQ/da = g1 d cross(c-x, a-x)/dv + g2 d cross(a-x, b-x)/du
        dcross_dv(vx, vy, qx, qy, t0x, t0y);
        dcross_du(qx, qy, ux, uy, t1x, t1y);
        const double dQax = g1 * t0x + g2 * t1x, dQay = g1 * t0y + g2 * t1y;
        // dQ/db = g0 d cross(b-x, c-x)/du + g2 d cross(a-x, b-x)/dv
        dcross_du(ux, uy, vx, vy, t0x, t0y);
        dcross_dv(qx, qy, ux, uy, t1x, t1y);
        const double dQbx = g0 * t0x + g2 * t1x, dQby = g0 * t0y + g2 * t1y;
        // dQ/dc = g0 d cross(b-x, c-x)/dv + g1 d cross(c-x, a-x)/du
        dcross_dv(ux, uy, vx, vy, t0x, t0y);
        dcross_du(vx, vy, qx, qy, t1x, t1y);
        const double dQcx = g0 * t0x + g1 * t1x, dQcy = g0 * t0y + g1 * t1y;
        // dD/db, dD/dc with D = cross(b - a, c - a); dD/da = -(dD/db + dD/dc)
        double dDbx, dDby, dDcx, dDcy;
        dcross_du(bx - ax, by - ay, cx - ax, cy - ay, dDbx, dDby);
        dcross_dv(bx - ax, by - ay, cx - ax, cy - ay, dDcx, dDcy);
        const double dDax = -(dDbx + dDcx), dDay = -(dDby + dDcy);
        const double r = 1.0 / D;
        atomicAdd(gP + 2 * ia, (dQax - ell * dDax) * r);
        atomicAdd(gP + 2 * ia + 1, (dQay - ell * dDay) * r);
        atomicAdd(gP + 2 * ib, (dQbx - ell * dDbx) * r);
        atomicAdd(gP + 2 * ib + 1, (dQby - ell * dDby) * r);
        atomicAdd(gP + 2 * ic, (dQcx - ell * dDcx) * r);
        atomicAdd(gP + 2 * ic + 1, (dQcy - ell * dDcy) * r);
        gB[2 * m] = -(dQax + dQbx + dQcx) * r;
        gB[2 * m + 1] = -(dQay + dQby + dQcy) * r;
    }
}

// beta = theta - theta_E theta / |theta|
__global__ void sis_trace_kernel(const double* __restrict__ theta, int64_t M, double theta_e,
                                 const double* __restrict__ theta_e_dev, double* __restrict__ beta) {
    const double te = theta_e_dev ? *theta_e_dev : theta_e;
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
        const double ty = theta[2 * m], tx = theta[2 * m + 1];
        const double r = hypot(ty, tx);
        beta[2 * m] = ty - te * ty / r;
        beta[2 * m + 1] = tx - te * tx / r;
    }
}

// dL/dtheta_E = -sum_m grad_beta_m . theta_m / |theta_m|  (one block)
__global__ void sis_trace_vjp_kernel(const double* __restrict__ theta, int64_t M, const double* __restrict__ gB,
                                     double* __restrict__ out) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int64_t m = threadIdx.x; m < M; m += blockDim.x) {
        const double ty = theta[2 * m], tx = theta[2 * m + 1];
        const double r = hypot(ty, tx);
        acc += (gB[2 * m] * ty + gB[2 * m + 1] * tx) / r;
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) *out = -acc;
}

// bilinear weights on the n x n mesh over [-hw, hw]^2 (rows grow downwards in y)
__global__ void bilinear_weights_kernel(const double* __restrict__ beta, int64_t M, int64_t n, double hw,
                                        int64_t* __restrict__ idx, double* __restrict__ w) {
    const double h = 2.0 * hw / (double)(n - 1);
    const double top = (double)(n - 1) - 1e-9;
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
        const double fy = fmin(fmax(__ddiv_rn(__dsub_rn(hw, beta[2 * m]), h), 0.0), top);
        const double fx = fmin(fmax(__ddiv_rn(__dadd_rn(beta[2 * m + 1], hw), h), 0.0), top);
        const double ry = floor(fy), rx = floor(fx);
        const int64_t r0 = (int64_t)ry, c0 = (int64_t)rx;
        const double ty = __dsub_rn(fy, ry), tx = __dsub_rn(fx, rx);
        idx[4 * m] = r0 * n + c0;
        idx[4 * m + 1] = r0 * n + c0 + 1;
        idx[4 * m + 2] = (r0 + 1) * n + c0;
        idx[4 * m + 3] = (r0 + 1) * n + c0 + 1;
        w[4 * m] = __dmul_rn(__dsub_rn(1.0, ty), __dsub_rn(1.0, tx));
        w[4 * m + 1] = __dmul_rn(__dsub_rn(1.0, ty), tx);
        w[4 * m + 2] = __dmul_rn(ty, __dsub_rn(1.0, tx));
        w[4 * m + 3] = __dmul_rn(ty, tx);
    }
}

__global__ void bilinear_weights_vjp_kernel(const double* __restrict__ beta, int64_t M, int64_t n, double hw,
                                            const double* __restrict__ G, double* __restrict__ gB) {
    const double h = 2.0 * hw / (double)(n - 1);
    const double top = (double)(n - 1) - 1e-9;
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
        const double fy_raw = (hw - beta[2 * m]) / h, fx_raw = (beta[2 * m + 1] + hw) / h;
        const double fy = fmin(fmax(fy_raw, 0.0), top), fx = fmin(fmax(fx_raw, 0.0), top);
        const double ty = fy - floor(fy), tx = fx - floor(fx);
        const double* g = G + 4 * m;
        const double dty = -g[0] * (1 - tx) - g[1] * tx + g[2] * (1 - tx) + g[3] * tx;
        const double dtx = -g[0] * (1 - ty) + g[1] * (1 - ty) - g[2] * ty + g[3] * ty;
        gB[2 * m] = (fy_raw > 0.0 && fy_raw < top) ? -dty / h : 0.0;
        gB[2 * m + 1] = (fx_raw > 0.0 && fx_raw < top) ? dtx / h : 0.0;
    }
}

}  // namespace

}  // namespace aj

using namespace aj;

extern "C" {

int aj_sis_trace(const double* theta, int64_t M, double einstein_radius, const double* einstein_radius_dev,
                 double* beta, void* stream) {
    if (M < 0) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    if (!theta || !beta) return AJ_ERR_ARG;
    sis_trace_kernel<<<blocks_for(M, 256, 4 * num_sms()), 256, 0, as_stream(stream)>>>(theta, M, einstein_radius,
                                                                                      einstein_radius_dev, beta);
    return check_launch();
}

int aj_sis_trace_vjp(const double* theta, int64_t M, const double* grad_beta, double* grad_einstein_radius,
                     void* stream) {
    if (M < 0 || !grad_einstein_radius || (M > 0 && (!theta || !grad_beta))) return AJ_ERR_ARG;
    sis_trace_vjp_kernel<<<1, 1024, 0, as_stream(stream)>>>(theta, M, grad_beta, grad_einstein_radius);
    return check_launch();
}

int aj_delaunay_weights(const double* beta, int64_t M, const double* points, int64_t S, const int64_t* simplices,
                        int64_t T, int64_t* pix_indexes, double* pix_weights, int* info, void* stream) {
    if (M < 0 || S < 0 || T < 0) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    if (!beta || !pix_indexes || !pix_weights || (S > 0 && !points) || (T > 0 && !simplices)) return AJ_ERR_ARG;
    if (T > 0 && S < 3) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    static bool attr_set[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    const size_t smem = sizeof(float) * 6 * LOC_TILE;
    if (dev < 64 && !attr_set[dev]) {
        if (cudaFuncSetAttribute(delaunay_weights_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return AJ_ERR_CUDA;
        attr_set[dev] = true;
    }
    init_minus2_kernel<<<blocks_for(M, 256, 4 * num_sms()), 256, 0, st>>>(pix_indexes, M);
    AJ_LAUNCHED();
    // each block stages the triangles once and serves a strided set of pixels (8 per pass)
    const int64_t want = (M + LOC_THREADS / 32 - 1) / (LOC_THREADS / 32);
    const int64_t cap = 2 * (int64_t)num_sms();
    const unsigned g = (unsigned)(want < cap ? want : cap);
    delaunay_weights_kernel<<<g, LOC_THREADS, smem, st>>>(beta, M, points, S, simplices, T, pix_indexes, pix_weights,
                                                          info);
    return check_launch();
}

int aj_delaunay_weights_vjp(const double* beta, int64_t M, const double* points, int64_t S,
                            const int64_t* pix_indexes, const double* grad_weights, double* grad_points,
                            double* grad_beta, void* stream) {
    if (M < 0 || S < 0) return AJ_ERR_ARG;
    if (!grad_points || (M > 0 && (!beta || !pix_indexes || !grad_weights || !grad_beta))) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (S > 0 && cudaMemsetAsync(grad_points, 0, sizeof(double) * 2 * S, st) != cudaSuccess) return AJ_ERR_CUDA;
    if (M == 0) return AJ_OK;
    delaunay_weights_vjp_kernel<<<blocks_for(M, 256, 4 * num_sms()), 256, 0, st>>>(beta, M, points, pix_indexes,
                                                                                grad_weights, grad_points, grad_beta);
    return check_launch();
}

int aj_bilinear_weights(const double* beta, int64_t M, int64_t n, double half_width, int64_t* pix_indexes,
                        double* pix_weights, void* stream) {
    if (M < 0 || n < 2 || !(half_width > 0.0)) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    if (!beta || !pix_indexes || !pix_weights) return AJ_ERR_ARG;
    bilinear_weights_kernel<<<blocks_for(M, 256, 4 * num_sms()), 256, 0, as_stream(stream)>>>(beta, M, n, half_width,
                                                                                            pix_indexes, pix_weights);
    return check_launch();
}

int aj_bilinear_weights_vjp(const double* beta, int64_t M, int64_t n, double half_width, const double* grad_weights,
                            double* grad_beta, void* stream) {
    if (M < 0 || n < 2 || !(half_width > 0.0)) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    if (!beta || !grad_weights || !grad_beta) return AJ_ERR_ARG;
    bilinear_weights_vjp_kernel<<<blocks_for(M, 256, 4 * num_sms()), 256, 0, as_stream(stream)>>>(
        beta, M, n, half_width, grad_weights, grad_beta);
    return check_launch();
}

}  // extern "C"
