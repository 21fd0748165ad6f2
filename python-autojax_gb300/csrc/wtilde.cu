// w_tilde and its compact / preload forms (numba.py:95-290, original.py:230-449).
//
// Direct w_tilde.  cos(a - b) = cos a cos b + sin a sin b turns
//     W_ij = sum_k w_k cos(2 pi (t_ik - t_jk)),  t_ik = x_i u_k + y_i v_k,
// into the K-deep symmetric product W = P^T P of the panel
//     P[k][i] = sqrt(w_k) cos(2 pi t_ik),  P[K + k][i] = sqrt(w_k) sin(2 pi t_ik).
// A panel kernel evaluates the phases once per (pixel, visibility) with the
// argument reduction t - rint(t) in float64; the product then costs 2 fused
// multiply-adds per (pixel pair, visibility) instead of one cos per pair.
//   AJ_FP64 : float64 panel and float64 tiles (parity path).
//   AJ_MIXED: float64 sincospi panel split into double-float (hi, lo) float32
//             planes; the product runs in double-float on the float32 pipe
//             (gemm_df, lower tiles, accumulated over K chunks) and yields
//             the double-float planes the mixed likelihood reads.  (A float32
//             panel, even with exactly summed products, moves logE by 1-5e-6
//             at the benchmark's conditioning, so no float32 rounding of the
//             panel values is allowed.)
// Only lower-triangular tiles are computed; each writes its mirror too.
//
// Compact table (numba.py:211-234).  With a = D n1 u, b = D n0 v the same
// identity gives w_c[n0][n1+N-1] = P1[|n1|][n0] + sgn(n1) P2[|n1|][n0] where
// P1 = Cu^T Cv and P2 = Su^T Sv are N x N products over K, run split-K.
//
// Preload (original.py:230-403) and w_tilde_data (numba.py:95-152) are sums
// sum_k a_k cos(2 pi (X_c u_k + Y_c v_k)) over a list of offsets c, run as a
// split-K cos-sum kernel with partial sums reduced in a fixed order.

#include <math.h>

#include "aj_internal.cuh"

namespace aj {

constexpr int PANEL_ROW_PAD = 128;  // panel columns (pixels) padded to the tile size
constexpr int FOLD = 256;           // k-rows summed in registers before a Kahan fold
constexpr size_t PANEL_BUDGET = size_t(1) << 30;  // bytes of panel per K chunk

inline int64_t pad_to(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// ------------------------------------------------------------------ panels

// P[kk][i] = sqrt(w) cos(2 pi t), P[kc + kk][i] = sqrt(w) sin(2 pi t) for
// k = k0 + kk < K and i < M; zeros elsewhere (padding).
template <typename T>
__global__ void wtilde_panel_kernel(const double* __restrict__ sigma, const double* __restrict__ uv,
                                    const double* __restrict__ grid, int64_t K, int64_t M, int64_t k0, int64_t kc,
                                    int64_t Mp, T* __restrict__ P) {
    const int64_t kk = blockIdx.x;
    const int64_t i = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
    if (i >= Mp) return;
    const int64_t k = k0 + kk;
    T c = T(0), s = T(0);
    if (k < K && i < M) {
        const double u = uv[2 * k], v = uv[2 * k + 1];
        const double t = fma(grid[2 * i + 1], u, grid[2 * i] * v);
        const double sw = 1.0 / fabs(sigma[k]);
        if constexpr (sizeof(T) == 8) {
            double sd, cd;
            sincospi(2.0 * t, &sd, &cd);
            c = T(cd * sw);
            s = T(sd * sw);
        } else {
            const float r = static_cast<float>(t - rint(t));
            float sf, cf;
            sincospif(2.0f * r, &sf, &cf);
            const float swf = static_cast<float>(sw);
            c = cf * swf;
            s = sf * swf;
        }
    }
    P[kk * Mp + i] = c;
    P[(kc + kk) * Mp + i] = s;
}

// lower-triangular tile index -> (row tile, col tile), row >= col
__device__ __forceinline__ void lower_tile(int64_t t, int64_t& bi, int64_t& bj) {
    int64_t r = static_cast<int64_t>((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    bi = r;
    bj = t - r * (r + 1) / 2;
}

// ---------------------------------------------------------- float64 SYRK

// C (+)= P^T P on lower 64x64 tiles, mirrored. P: kd x Mp float64.
__global__ void __launch_bounds__(256)
    syrk_f64_kernel(const double* __restrict__ P, int64_t Mp, int64_t kd, int64_t M, double* __restrict__ C,
                    int accumulate) {
    __shared__ double As[16][64];
    __shared__ double Bs[16][64];
    int64_t bi, bj;
    lower_tile(blockIdx.x, bi, bj);
    const int64_t a0 = bi * 64, b0 = bj * 64;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    double acc[4][4] = {};
    for (int64_t k0 = 0; k0 < kd; k0 += 16) {
        for (int e = tid; e < 16 * 64; e += 256) {
            const int r = e >> 6, c = e & 63;
            const int64_t kr = k0 + r;
            As[r][c] = (kr < kd && a0 + c < Mp) ? P[kr * Mp + a0 + c] : 0.0;
            Bs[r][c] = (kr < kd && b0 + c < Mp) ? P[kr * Mp + b0 + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t gi = a0 + ty * 4 + i;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t gj = b0 + tx * 4 + j;
            if (gi < M && gj < M) {
                double v = acc[i][j];
                if (accumulate) v += C[gi * M + gj];
                C[gi * M + gj] = v;
                if (bi != bj) C[gj * M + gi] = v;
            }
        }
    }
}

// --------------------------------------------------------------- compact

// Tab[q][kk][n] for q = 0..3: sqrt(w) {cos, sin}(2 pi ps n u_k), {cos, sin}(2 pi ps n v_k), n < N.
template <typename T>
__global__ void compact_panel_kernel(const double* __restrict__ sigma, const double* __restrict__ uv, int64_t K,
                                     int64_t N, int64_t Np, double ps_rad, int64_t k0, int64_t kc,
                                     T* __restrict__ tab) {
    const int64_t kk = blockIdx.x;
    const int64_t n = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
    if (n >= Np) return;
    const int64_t k = k0 + kk;
    T cu = 0, su = 0, cv = 0, sv = 0;
    if (k < K && n < N) {
        const double sw = 1.0 / fabs(sigma[k]);
        const double tu = (ps_rad * (double)n) * uv[2 * k];
        const double tv = (ps_rad * (double)n) * uv[2 * k + 1];
        if constexpr (sizeof(T) == 8) {
            double s1, c1, s2, c2;
            sincospi(2.0 * tu, &s1, &c1);
            sincospi(2.0 * tv, &s2, &c2);
            cu = c1 * sw;
            su = s1 * sw;
            cv = c2 * sw;
            sv = s2 * sw;
        } else {
            float s1, c1, s2, c2;
            sincospif(2.0f * static_cast<float>(tu - rint(tu)), &s1, &c1);
            sincospif(2.0f * static_cast<float>(tv - rint(tv)), &s2, &c2);
            const float swf = static_cast<float>(sw);
            cu = c1 * swf;
            su = s1 * swf;
            cv = c2 * swf;
            sv = s2 * swf;
        }
    }
    const int64_t plane = kc * Np;
    tab[0 * plane + kk * Np + n] = cu;
    tab[1 * plane + kk * Np + n] = su;
    tab[2 * plane + kk * Np + n] = cv;
    tab[3 * plane + kk * Np + n] = sv;
}

// partial[split][p][a][b] = sum over this split's k of tab[p][k][a] * tab[2 + p][k][b], p = 0, 1.
// 64x64 output tile per block (grid.x tiles, grid.y splits, grid.z = p).
template <typename T>
__global__ void __launch_bounds__(256)
    compact_gemm_kernel(const T* __restrict__ tab, int64_t kc, int64_t Np, int64_t k_per_split,
                        double* __restrict__ partial) {
    __shared__ T As[16][64];
    __shared__ T Bs[16][64];
    const int p = blockIdx.z;
    const int64_t ntile = Np / 64;
    const int64_t ta = blockIdx.x / ntile, tb = blockIdx.x % ntile;
    const int64_t kb = blockIdx.y * k_per_split;
    const int64_t ke = min(kc, kb + k_per_split);
    const T* A = tab + (int64_t)p * kc * Np;
    const T* B = tab + (int64_t)(2 + p) * kc * Np;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    T acc[4][4] = {};
    float hi[4][4] = {}, lo[4][4] = {};
    int since_fold = 0;
    for (int64_t k0 = kb; k0 < ke; k0 += 16) {
        for (int e = tid; e < 16 * 64; e += 256) {
            const int r = e >> 6, c = e & 63;
            const int64_t kr = k0 + r;
            As[r][c] = kr < ke ? A[kr * Np + ta * 64 + c] : T(0);
            Bs[r][c] = kr < ke ? B[kr * Np + tb * 64 + c] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] += As[kk][ty * 4 + i] * Bs[kk][tx * 4 + j];
        }
        __syncthreads();
        if constexpr (sizeof(T) == 4) {
            since_fold += 16;
            if (since_fold >= FOLD) {
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        kahan_add(hi[i][j], lo[i][j], acc[i][j]);
                        acc[i][j] = 0;
                    }
                since_fold = 0;
            }
        }
    }
    double* out = partial + ((int64_t)blockIdx.y * 2 + p) * Np * Np;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double v;
            if constexpr (sizeof(T) == 4) {
                kahan_add(hi[i][j], lo[i][j], acc[i][j]);
                v = (double)hi[i][j] - (double)lo[i][j];
            } else {
                v = acc[i][j];
            }
            out[(ta * 64 + ty * 4 + i) * Np + tb * 64 + tx * 4 + j] = v;
        }
}

// Sum the split partials (fixed order) into accum[2][Np][Np] (accumulate across K chunks).
__global__ void compact_reduce_kernel(const double* __restrict__ partial, int64_t nsplit, int64_t Np,
                                      double* __restrict__ accum, int first) {
    const int64_t n = 2 * Np * Np;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        double s = first ? 0.0 : accum[t];
        for (int64_t q = 0; q < nsplit; ++q) s += partial[q * n + t];
        accum[t] = s;
    }
}

// w_c[n0][c] with n1 = c - (N - 1): P1[|n1|][n0] + sgn(n1) P2[|n1|][n0].
__global__ void compact_assemble_kernel(const double* __restrict__ accum, int64_t N, int64_t Np,
                                        double* __restrict__ out) {
    const int64_t W = 2 * N - 1;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * W; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n0 = t / W, c = t - n0 * W;
        const int64_t n1 = c - (N - 1);
        const int64_t a = n1 < 0 ? -n1 : n1;
        const double p1 = accum[a * Np + n0];
        const double p2 = accum[Np * Np + a * Np + n0];
        out[t] = n1 > 0 ? p1 + p2 : (n1 < 0 ? p1 - p2 : p1);
    }
}

// --------------------------------------------------------------- cos sums

// partial[split][c] = sum over this split's k of a_k cos(2 pi (X_c u_k + Y_c v_k)).
// Weight modes: 0 -> a_k = sigma_k^-2 (w_tilde), 1 -> a_k = (sigma_k^2 / vis_k)^2 (w_tilde_data),
// 2 -> the dirty image (float64 only): a_k cos + b_k sin with a_k = sigma_k^-2 Re V_k,
// b_k = -sigma_k^-2 Im V_k, vis interleaved complex.
template <bool MIXED>
__global__ void __launch_bounds__(256)
    cos_sum_kernel(const double* __restrict__ X, const double* __restrict__ Y, int64_t stride, int64_t C,
                   const double* __restrict__ uv, const double* __restrict__ sigma, const double* __restrict__ vis,
                   int weight_mode, int64_t K, int64_t k_per_split, double* __restrict__ partial) {
    __shared__ double su[512], sv[512], sa[512], sb[512];
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double x = c < C ? X[c * stride] : 0.0;
    const double y = c < C ? Y[c * stride] : 0.0;
    const int64_t kb = blockIdx.y * k_per_split;
    const int64_t ke = min(K, kb + k_per_split);
    double acc = 0.0;
    float hi = 0.f, lo = 0.f, accf = 0.f;
    int cnt = 0;
    for (int64_t k0 = kb; k0 < ke; k0 += 512) {
        const int nk = (int)((ke - k0) < 512 ? (ke - k0) : 512);
        for (int e = threadIdx.x; e < nk; e += blockDim.x) {
            const int64_t k = k0 + e;
            su[e] = uv[2 * k];
            sv[e] = uv[2 * k + 1];
            const double s = sigma[k];
            if (weight_mode == 0) {
                sa[e] = 1.0 / (s * s);
            } else if (weight_mode == 2) {
                const double w = 1.0 / (s * s);
                sa[e] = w * vis[2 * k];
                sb[e] = -w * vis[2 * k + 1];
            } else {
                const double q = (s * s) / vis[k];
                sa[e] = q * q;
            }
        }
        __syncthreads();
        if (c < C) {
            for (int e = 0; e < nk; ++e) {
                const double t = fma(x, su[e], y * sv[e]);
                if constexpr (MIXED) {
                    const float r = static_cast<float>(t - rint(t));
                    accf = fmaf(static_cast<float>(sa[e]), cospif(2.0f * r), accf);
                    if (++cnt == 64) {
                        kahan_add(hi, lo, accf);
                        accf = 0.f;
                        cnt = 0;
                    }
                } else if (weight_mode == 2) {
                    double sn, cs;
                    sincospi(2.0 * t, &sn, &cs);
                    acc = fma(sa[e], cs, fma(sb[e], sn, acc));
                } else {
                    acc = fma(sa[e], cospi(2.0 * t), acc);
                }
            }
        }
        __syncthreads();
    }
    if (c < C) {
        if constexpr (MIXED) {
            kahan_add(hi, lo, accf);
            acc = (double)hi - (double)lo;
        }
        partial[blockIdx.y * C + c] = acc;
    }
}

// out[dst[c]] (or out[c]) = sum over splits of partial[split][c]
__global__ void cos_sum_reduce_kernel(const double* __restrict__ partial, int64_t nsplit, int64_t C,
                                      const int64_t* __restrict__ dst, double* __restrict__ out) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int64_t q = 0; q < nsplit; ++q) s += partial[q * C + c];
        out[dst ? dst[c] : c] = s;
    }
}

// Offsets of the four preload quadrants (original.py:352-401).
// cells: 0 .. Y*X-1 quadrant (0,0); then (0,-1) j>0; (-1,0) i>0; (-1,-1) i,j>0.
__global__ void preload_offsets_kernel(const double* __restrict__ g, int64_t gy, int64_t gx, int64_t Y, int64_t X,
                                       double* __restrict__ xo, double* __restrict__ yo, int64_t* __restrict__ dst) {
    const int64_t YX = Y * X;
    // The reference slices grid_2d[0:Y, 0:X] first (original.py:347), so "-1" is row Y-1 / column X-1.
    (void)gy;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 4 * YX; t += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(t / YX);
        const int64_t r = t - q * YX;
        const int64_t i = r / X, j = r - i * X;
        int64_t ci, cj, si, sj, di, dj;
        bool valid;
        if (q == 0) {
            ci = 0; cj = 0; si = i; sj = j; di = i; dj = j; valid = true;
        } else if (q == 1) {
            ci = 0; cj = X - 1; si = i; sj = X - j - 1; di = i; dj = 2 * X - j; valid = j > 0;
        } else if (q == 2) {
            ci = Y - 1; cj = 0; si = Y - i - 1; sj = j; di = 2 * Y - i; dj = j; valid = i > 0;
        } else {
            ci = Y - 1; cj = X - 1; si = Y - i - 1; sj = X - j - 1; di = 2 * Y - i; dj = 2 * X - j;
            valid = i > 0 && j > 0;
        }
        const double* gc = g + (ci * gx + cj) * 2;
        const double* gs = g + (si * gx + sj) * 2;
        yo[t] = gc[0] - gs[0];
        xo[t] = gc[1] - gs[1];
        dst[t] = valid ? di * (2 * X) + dj : -1;
    }
}

// The four quadrants overlap nowhere except through invalid cells, which
// the reduce writes to a scratch slot; zero the output first.
__global__ void scatter_valid_kernel(const double* __restrict__ vals, const int64_t* __restrict__ dst, int64_t C,
                                     double* __restrict__ out) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x)
        if (dst[c] >= 0) out[dst[c]] += vals[c];
}

// ------------------------------------------------------------ expansions

template <bool COMPACT>
__global__ void expand_kernel(const double* __restrict__ table, int64_t rows, int64_t cols,
                              const int64_t* __restrict__ nat, int64_t M, double* __restrict__ out64,
                              float* __restrict__ out32, int* info) {
    for (int64_t i = blockIdx.y; i < M; i += gridDim.y) {
    const int64_t yi = nat[2 * i], xi = nat[2 * i + 1];
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t yj = nat[2 * j], xj = nat[2 * j + 1];
        int64_t r, c;
        if constexpr (COMPACT) {
            // numba.py:251-254
            const int64_t m = yi - yj;
            c = (m >= 0 ? xi - xj : xj - xi) + (rows - 1);
            r = m < 0 ? -m : m;
        } else {
            // numba.py:287-289: preload[y_j - y_i][x_j - x_i], negative indices wrap once
            r = yj - yi;
            c = xj - xi;
            if (r < 0) r += rows;
            if (c < 0) c += cols;
        }
        double v = 0.0;
        if (r >= 0 && r < rows && c >= 0 && c < cols) {
            v = table[r * cols + c];
        } else {
            report(info, AJ_INFO_INDEX_RANGE, i * M + j);
        }
        if (out64) out64[i * M + j] = v;
        if (out32) out32[i * M + j] = static_cast<float>(v);
    }
    }
}

// ----------------------------------------------------------- host plans

struct WtildePlan {
    int64_t Mp, kc, nchunk;
    size_t elem;
};

// (both precisions store 8 bytes a panel element: a float64, or a hi + lo pair of float32)
WtildePlan wtilde_plan(int64_t K, int64_t M) {
    WtildePlan p;
    p.Mp = pad_to(M > 0 ? M : 1, PANEL_ROW_PAD);
    p.elem = 8;  // float64, or a hi + lo pair of float32
    int64_t kc = (int64_t)(PANEL_BUDGET / (2 * p.Mp * p.elem));
    kc = kc / 64 * 64;
    if (kc < 64) kc = 64;
    const int64_t Kp = pad_to(K > 0 ? K : 1, 64);
    if (kc > Kp) kc = Kp;
    p.kc = kc;
    p.nchunk = (K + kc - 1) / kc;
    return p;
}

struct CompactPlan {
    int64_t Np, kc, nchunk, nsplit, k_per_split;
    size_t elem;
};

CompactPlan compact_plan(int64_t N, int64_t K, int precision) {
    (void)precision;  // the compact table always runs the float64 kernels (~30 ms at K = 1e6)
    CompactPlan p;
    p.Np = pad_to(N > 0 ? N : 1, 64);
    p.elem = 8;
    int64_t kc = (int64_t)((size_t(256) << 20) / (4 * p.Np * p.elem));
    kc = kc / 64 * 64;
    if (kc < 64) kc = 64;
    const int64_t Kp = pad_to(K > 0 ? K : 1, 64);
    if (kc > Kp) kc = Kp;
    p.kc = kc;
    p.nchunk = (K + kc - 1) / kc;
    const int64_t tiles = (p.Np / 64) * (p.Np / 64) * 2;
    int64_t want = (4 * (int64_t)num_sms() + tiles - 1) / tiles;
    int64_t kps = (kc + want - 1) / want;
    kps = pad_to(kps < 16 ? 16 : kps, 16);
    p.k_per_split = kps;
    p.nsplit = (kc + kps - 1) / kps;
    return p;
}

struct CosSumPlan {
    int64_t nsplit, k_per_split;
};

CosSumPlan cos_sum_plan(int64_t C, int64_t K) {
    CosSumPlan p;
    const int64_t cblocks = (C + 255) / 256;
    int64_t want = (8 * (int64_t)num_sms() + cblocks - 1) / cblocks;
    if (want < 1) want = 1;
    int64_t kps = (K + want - 1) / want;
    if (kps < 512) kps = 512;
    p.k_per_split = kps;
    p.nsplit = (K + kps - 1) / kps;
    if (p.nsplit < 1) p.nsplit = 1;
    return p;
}

int launch_cos_sum(const double* X, const double* Y, int64_t stride, int64_t C, const double* uv,
                   const double* sigma, const double* vis, int weight_mode, int64_t K, const int64_t* dst,
                   double* out, double* partial, const CosSumPlan& pl, int precision, cudaStream_t st) {
    dim3 grid(blocks_for(C, 256), (unsigned)pl.nsplit);
    if (precision == AJ_MIXED)
        cos_sum_kernel<true><<<grid, 256, 0, st>>>(X, Y, stride, C, uv, sigma, vis, weight_mode, K, pl.k_per_split,
                                                   partial);
    else
        cos_sum_kernel<false><<<grid, 256, 0, st>>>(X, Y, stride, C, uv, sigma, vis, weight_mode, K, pl.k_per_split,
                                                    partial);
    AJ_LAUNCHED();
    cos_sum_reduce_kernel<<<blocks_for(C, 256, 4096), 256, 0, st>>>(partial, pl.nsplit, C, dst, out);
    return check_launch();
}

}  // namespace aj

using namespace aj;

extern "C" {

size_t aj_w_tilde_curvature_workspace_size(int64_t K, int64_t M, int precision) {
    if (precision == AJ_MIXED) {
        // the digit panel; the planes may also be joined through this buffer
        size_t b = wtilde_tc_workspace_bytes(K, M);
        if (b < sizeof(double) * M * M) b = sizeof(double) * M * M;
        return align_up(b);
    }
    WtildePlan p = wtilde_plan(K, M);
    Sizer s;
    s.take<char>(2 * p.kc * p.Mp * p.elem);
    return s.total();
}

int aj_w_tilde_curvature(const double* noise_map_real, const double* uv, const double* grid_slim, int64_t K,
                         int64_t M, double* out64, float* out_planes, void* workspace, size_t workspace_bytes,
                         int precision, void* stream) {
    if (K < 0 || M < 0 || (precision != AJ_FP64 && precision != AJ_MIXED)) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    if (!out64 || !grid_slim || (K > 0 && (!noise_map_real || !uv))) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    float* ph = out_planes;
    float* pl = out_planes ? out_planes + M * M : nullptr;
    if (K == 0) {
        if (cudaMemsetAsync(out64, 0, sizeof(double) * M * M, st) != cudaSuccess) return AJ_ERR_CUDA;
        if (out_planes && cudaMemsetAsync(out_planes, 0, sizeof(float) * 2 * M * M, st) != cudaSuccess)
            return AJ_ERR_CUDA;
        return AJ_OK;
    }
    WtildePlan p = wtilde_plan(K, M);
    if (workspace_bytes < aj_w_tilde_curvature_workspace_size(K, M, precision) || !workspace) return AJ_ERR_WORKSPACE;
    if (precision == AJ_MIXED) {
        // the double-float result accumulates in planes: the caller's, else the float64 output's bytes
        const bool own = out_planes == nullptr;
        if (own) {
            ph = reinterpret_cast<float*>(out64);
            pl = ph + M * M;  // out64 holds exactly 2 M^2 floats
        }
        // W's lower triangle from exact digit products on the tensor cores (wtilde_tc.cu)
        AJ_TRY(wtilde_tc(noise_map_real, uv, grid_slim, K, M, ph, pl, workspace, workspace_bytes, st));
        AJ_TRY(df_mirror_lower(ph, pl, M, st));
        if (own) {
            // planes live in out64's storage: join in place from the back is unsafe, so join via the panel buffer
            // the workspace holds at least M^2 doubles for this join (see the size function)
            double* tmp = reinterpret_cast<double*>(workspace);
            AJ_TRY(df_join(ph, pl, M * M, tmp, st));
            if (cudaMemcpyAsync(out64, tmp, sizeof(double) * M * M, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                return AJ_ERR_CUDA;
        } else {
            AJ_TRY(df_join(ph, pl, M * M, out64, st));
        }
        return AJ_OK;
    }
    const int64_t nt = p.Mp / 64;
    const int64_t ntiles = nt * (nt + 1) / 2;
    for (int64_t ch = 0; ch < p.nchunk; ++ch) {
        const int64_t k0 = ch * p.kc;
        dim3 pg((unsigned)p.kc, (unsigned)((p.Mp + 255) / 256));
        double* P = static_cast<double*>(workspace);
        wtilde_panel_kernel<double><<<pg, 256, 0, st>>>(noise_map_real, uv, grid_slim, K, M, k0, p.kc, p.Mp, P);
        AJ_LAUNCHED();
        syrk_f64_kernel<<<(unsigned)ntiles, 256, 0, st>>>(P, p.Mp, 2 * p.kc, M, out64, ch > 0);
        AJ_LAUNCHED();
    }
    if (out_planes) AJ_TRY(df_split(out64, M * M, ph, pl, st));
    return AJ_OK;
}

size_t aj_w_compact_curvature_workspace_size(int64_t N, int64_t K, int precision) {
    CompactPlan p = compact_plan(N, K, precision);
    Sizer s;
    s.take<char>(4 * p.kc * p.Np * p.elem);
    s.take<double>(p.nsplit * 2 * p.Np * p.Np);
    s.take<double>(2 * p.Np * p.Np);
    return s.total();
}

int aj_w_compact_curvature(int64_t N, const double* noise_map_real, const double* uv, int64_t K,
                           double pixel_scale, double* out, void* workspace, size_t workspace_bytes,
                           int precision, void* stream) {
    if (N < 0 || K < 0 || (precision != AJ_FP64 && precision != AJ_MIXED)) return AJ_ERR_ARG;
    if (N == 0) return AJ_OK;
    if (!out || (K > 0 && (!noise_map_real || !uv))) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (K == 0) return cudaMemsetAsync(out, 0, sizeof(double) * N * (2 * N - 1), st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    CompactPlan p = compact_plan(N, K, precision);
    if (!workspace || workspace_bytes < aj_w_compact_curvature_workspace_size(N, K, precision)) return AJ_ERR_WORKSPACE;
    Carver cv(workspace, workspace_bytes);
    char* tab = cv.take<char>(4 * p.kc * p.Np * p.elem);
    double* partial = cv.take<double>(p.nsplit * 2 * p.Np * p.Np);
    double* accum = cv.take<double>(2 * p.Np * p.Np);
    // numba.py:223: D = pi^2 ps / 324000 = 2 pi * (ps in radians); the panels take phases in turns
    const double ps_rad = pixel_scale * (M_PI / 648000.0);
    const int64_t ntile = (p.Np / 64) * (p.Np / 64);
    for (int64_t ch = 0; ch < p.nchunk; ++ch) {
        const int64_t k0 = ch * p.kc;
        dim3 pg((unsigned)p.kc, (unsigned)((p.Np + 127) / 128));
        dim3 gg((unsigned)ntile, (unsigned)p.nsplit, 2);
        compact_panel_kernel<double><<<pg, 128, 0, st>>>(noise_map_real, uv, K, N, p.Np, ps_rad, k0, p.kc,
                                                         reinterpret_cast<double*>(tab));
        AJ_LAUNCHED();
        compact_gemm_kernel<double><<<gg, 256, 0, st>>>(reinterpret_cast<double*>(tab), p.kc, p.Np, p.k_per_split,
                                                        partial);
        AJ_LAUNCHED();
        compact_reduce_kernel<<<blocks_for(2 * p.Np * p.Np, 256, 1024), 256, 0, st>>>(partial, p.nsplit, p.Np, accum,
                                                                                   ch == 0);
        AJ_LAUNCHED();
    }
    compact_assemble_kernel<<<blocks_for(N * (2 * N - 1), 256, 1024), 256, 0, st>>>(accum, N, p.Np, out);
    return check_launch();
}

size_t aj_w_tilde_preload_workspace_size(int64_t Y, int64_t X, int64_t K, int precision) {
    (void)precision;
    const int64_t C = 4 * Y * X;
    CosSumPlan pl = cos_sum_plan(C, K);
    Sizer s;
    s.take<double>(C);
    s.take<double>(C);
    s.take<int64_t>(C);
    s.take<double>(C);
    s.take<double>(pl.nsplit * C);
    return s.total();
}

int aj_w_tilde_preload(const double* noise_map_real, const double* uv, int64_t K, int64_t Y, int64_t X,
                       const double* grid_2d, int64_t gy, int64_t gx, double* out, void* workspace,
                       size_t workspace_bytes, int precision, void* stream) {
    if (Y < 0 || X < 0 || K < 0 || gy < Y || gx < X || (precision != AJ_FP64 && precision != AJ_MIXED))
        return AJ_ERR_ARG;
    if (Y == 0 || X == 0) return AJ_OK;
    if (!out || !grid_2d || (K > 0 && (!noise_map_real || !uv))) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(out, 0, sizeof(double) * 4 * Y * X, st) != cudaSuccess) return AJ_ERR_CUDA;
    if (K == 0) return AJ_OK;
    const int64_t C = 4 * Y * X;
    CosSumPlan pl = cos_sum_plan(C, K);
    if (!workspace || workspace_bytes < aj_w_tilde_preload_workspace_size(Y, X, K, precision)) return AJ_ERR_WORKSPACE;
    Carver cv(workspace, workspace_bytes);
    double* xo = cv.take<double>(C);
    double* yo = cv.take<double>(C);
    int64_t* dst = cv.take<int64_t>(C);
    double* vals = cv.take<double>(C);
    double* partial = cv.take<double>(pl.nsplit * C);
    preload_offsets_kernel<<<blocks_for(C, 256, 1024), 256, 0, st>>>(grid_2d, gy, gx, Y, X, xo, yo, dst);
    AJ_LAUNCHED();
    // original.py:358-361: cos(2 pi (x_off u_k0 + y_off u_k1)) weighted by noise^-2
    AJ_TRY(launch_cos_sum(xo, yo, 1, C, uv, noise_map_real, nullptr, 0, K, nullptr, vals, partial, pl, precision, st));
    scatter_valid_kernel<<<blocks_for(C, 256, 1024), 256, 0, st>>>(vals, dst, C, out);
    return check_launch();
}

size_t aj_w_tilde_data_workspace_size(int64_t M, int64_t K, int precision) {
    (void)precision;
    CosSumPlan pl = cos_sum_plan(M, K);
    Sizer s;
    s.take<double>(pl.nsplit * M);
    return s.total();
}

int aj_w_tilde_data(const double* visibilities_real, const double* noise_map_real, const double* uv,
                    const double* grid_slim, int64_t K, int64_t M, double* out, void* workspace,
                    size_t workspace_bytes, int precision, void* stream) {
    if (M < 0 || K < 0 || (precision != AJ_FP64 && precision != AJ_MIXED)) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    if (!out || !grid_slim || (K > 0 && (!noise_map_real || !uv || !visibilities_real))) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (K == 0) return cudaMemsetAsync(out, 0, sizeof(double) * M, st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    CosSumPlan pl = cos_sum_plan(M, K);
    if (!workspace || workspace_bytes < aj_w_tilde_data_workspace_size(M, K, precision)) return AJ_ERR_WORKSPACE;
    double* partial = static_cast<double*>(workspace);
    // numba.py:151: cos(g_2pi[i,1] u_k0 + g_2pi[i,0] u_k1): X = grid[:, 1], Y = grid[:, 0]
    return launch_cos_sum(grid_slim + 1, grid_slim, 2, M, uv, noise_map_real, visibilities_real, 1, K, nullptr, out,
                          partial, pl, precision, st);
}

size_t aj_dirty_image_workspace_size(int64_t M, int64_t K) {
    CosSumPlan pl = cos_sum_plan(M, K);
    Sizer s;
    s.take<double>(pl.nsplit * M);
    return s.total();
}

int aj_dirty_image(const double* visibilities, const double* noise_map_real, const double* uv,
                   const double* grid_slim, int64_t K, int64_t M, double* out, void* workspace,
                   size_t workspace_bytes, void* stream) {
    if (M < 0 || K < 0) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    if (!out || !grid_slim || (K > 0 && (!noise_map_real || !uv || !visibilities))) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (K == 0) return cudaMemsetAsync(out, 0, sizeof(double) * M, st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    CosSumPlan pl = cos_sum_plan(M, K);
    if (!workspace || workspace_bytes < aj_dirty_image_workspace_size(M, K)) return AJ_ERR_WORKSPACE;
    // phase 2 pi (x u + y v) with x = grid[:, 1], y = grid[:, 0], the w_tilde pairing (numba.py:204)
    return launch_cos_sum(grid_slim + 1, grid_slim, 2, M, uv, noise_map_real, visibilities, 2, K, nullptr, out,
                          static_cast<double*>(workspace), pl, AJ_FP64, st);
}

int aj_w_tilde_via_compact(const double* w_compact, int64_t N, const int64_t* native_index, int64_t M,
                           double* out64, float* out32, int* info, void* stream) {
    if (N <= 0 || M < 0 || !w_compact || (M > 0 && !native_index)) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    dim3 grid(blocks_for(M, 256, 64), (unsigned)(M < 65535 ? M : 65535));
    expand_kernel<true><<<grid, 256, 0, as_stream(stream)>>>(w_compact, N, 2 * N - 1, native_index, M, out64, out32,
                                                             info);
    return check_launch();
}

int aj_w_tilde_via_preload(const double* preload, int64_t py, int64_t px, const int64_t* native_index, int64_t M,
                           double* out64, float* out32, int* info, void* stream) {
    if (py <= 0 || px <= 0 || M < 0 || !preload || (M > 0 && !native_index)) return AJ_ERR_ARG;
    if (M == 0) return AJ_OK;
    dim3 grid(blocks_for(M, 256, 64), (unsigned)(M < 65535 ? M : 65535));
    expand_kernel<false><<<grid, 256, 0, as_stream(stream)>>>(preload, py, px, native_index, M, out64, out32, info);
    return check_launch();
}

}  // extern "C"
