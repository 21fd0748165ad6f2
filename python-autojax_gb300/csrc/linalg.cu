// Dense float64 linear algebra for the inversion (the solve and slogdet of
// numba.py:731, 849-850; the inverse the adjoint needs).
//
// Blocked right-looking Cholesky with NB = 32 columns per step:
//   diag kernel  — one block factors the NB x NB diagonal block in shared
//                  memory (pivot <= 0 or NaN -> info) and inverts it;
//   panel kernel — rows below: L_ik = A_ik L_kk^-T, a multiply by the stored
//                  inverse (rows independent, in place);
//   update       — lower tiles of the trailing matrix: A -= L_k L_k^T.
// Triangular inverse (L^-1): right-looking block forward substitution of
// L X = I where one launch per block row both accumulates L_ik X_k and, for
// the tiles of the next block row, applies -L_ii^-1 (tile = whole block rows).
// A^-1 = L^-T L^-1 (lower tiles, k-range starting at the tile diagonal, mirrored).
// Vector solves run one launch per block, each block recomputing the 32
// solved values it needs from the stored diagonal inverse.

#include <math.h>

#include "aj_internal.cuh"

namespace aj {

constexpr int NB = kSpdNB;

__device__ __forceinline__ void lower_tile64(int64_t t, int64_t& bi, int64_t& bj) {
    int64_t r = static_cast<int64_t>((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    bi = r;
    bj = t - r * (r + 1) / 2;
}

// ------------------------------------------------------------------ GEMM

template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
    gemm_f64_kernel(int64_t m, int64_t n, int64_t k, double alpha, const double* __restrict__ A, int64_t lda,
                    const double* __restrict__ B, int64_t ldb, double beta, double* __restrict__ C, int64_t ldc,
                    int lower_only, int tri_k, int64_t tiles_n) {
    __shared__ double As[32][33];
    __shared__ double Bs[32][33];
    int64_t ti, tj;
    if (lower_only)
        lower_tile64(blockIdx.x, ti, tj);
    else {
        ti = blockIdx.x / tiles_n;
        tj = blockIdx.x % tiles_n;
    }
    const int64_t i0 = ti * 32, j0 = tj * 32;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    const int64_t kbeg = tri_k ? (i0 > j0 ? i0 : j0) : 0;
    for (int64_t k0 = kbeg; k0 < k; k0 += 32) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * 256;
            int ii, kk;
            if (TA) {
                kk = e >> 5;
                ii = e & 31;
            } else {
                ii = e >> 5;
                kk = e & 31;
            }
            const int64_t gi = i0 + ii, gk = k0 + kk;
            double v = 0.0;
            if (gi < m && gk < k) v = TA ? A[gk * lda + gi] : A[gi * lda + gk];
            As[kk][ii] = v;
            int jj, kb;
            if (TB) {
                jj = e >> 5;
                kb = e & 31;
            } else {
                kb = e >> 5;
                jj = e & 31;
            }
            const int64_t gj = j0 + jj, gk2 = k0 + kb;
            double w = 0.0;
            if (gj < n && gk2 < k) w = TB ? B[gj * ldb + gk2] : B[gk2 * ldb + gj];
            Bs[kb][jj] = w;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 32; ++kk) {
            const double a0 = As[kk][ty * 2], a1 = As[kk][ty * 2 + 1];
            const double b0 = Bs[kk][tx * 2], b1 = Bs[kk][tx * 2 + 1];
            acc[0][0] = fma(a0, b0, acc[0][0]);
            acc[0][1] = fma(a0, b1, acc[0][1]);
            acc[1][0] = fma(a1, b0, acc[1][0]);
            acc[1][1] = fma(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int64_t gi = i0 + ty * 2 + r, gj = j0 + tx * 2 + c;
            if (gi < m && gj < n) {
                double v = alpha * acc[r][c];
                if (beta != 0.0) v = fma(beta, C[gi * ldc + gj], v);
                C[gi * ldc + gj] = v;
            }
        }
}

int gemm_f64(bool transA, bool transB, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
             const double* B, int64_t ldb, double beta, double* C, int64_t ldc, bool lower_only, cudaStream_t st) {
    if (m <= 0 || n <= 0) return AJ_OK;
    const int64_t tm = (m + 31) / 32, tn = (n + 31) / 32;
    const int64_t tiles = lower_only ? tm * (tm + 1) / 2 : tm * tn;
    const unsigned g = (unsigned)tiles;
#define AJ_GEMM_LAUNCH(ta, tb)                                                                                         \
    gemm_f64_kernel<ta, tb><<<g, 256, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower_only ? 1 : 0, 0, tn)
    if (!transA && !transB)
        AJ_GEMM_LAUNCH(false, false);
    else if (!transA && transB)
        AJ_GEMM_LAUNCH(false, true);
    else if (transA && !transB)
        AJ_GEMM_LAUNCH(true, false);
    else
        AJ_GEMM_LAUNCH(true, true);
#undef AJ_GEMM_LAUNCH
    return check_launch();
}

// ------------------------------------------------------------- transpose

template <typename T>
__global__ void transpose_kernel(const T* __restrict__ in, int64_t rows, int64_t cols, T* __restrict__ out) {
    __shared__ T tile[32][33];
    const int64_t bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t gi = by + r, gj = bx + threadIdx.x;
        if (gi < rows && gj < cols) tile[r][threadIdx.x] = in[gi * cols + gj];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t gi = bx + r, gj = by + threadIdx.x;
        if (gi < cols && gj < rows) out[gi * rows + gj] = tile[threadIdx.x][r];
    }
}

template <typename T>
int transpose(const T* in, int64_t rows, int64_t cols, T* out, cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return AJ_OK;
    dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
    transpose_kernel<T><<<grid, dim3(32, 8), 0, st>>>(in, rows, cols, out);
    return check_launch();
}
template int transpose<double>(const double*, int64_t, int64_t, double*, cudaStream_t);
template int transpose<float>(const float*, int64_t, int64_t, float*, cudaStream_t);

// -------------------------------------------------------------- Cholesky

// Factor the diagonal block at k0 in place and store its inverse in dinv (NB x NB, lower).
// One barrier a column: every thread evaluates the pivot (rsqrt) itself and the
// scaled column goes to a separate array, so the rank-1 update can read the
// unscaled one; the inverse splits each column's substitution over 8 threads.
__global__ void __launch_bounds__(256)
    chol_diag_kernel(double* __restrict__ L, int64_t S, int64_t k0, double* __restrict__ dinv, int* info) {
    __shared__ double a[NB][NB + 1];
    __shared__ double l[NB][NB + 1];
    __shared__ double inv[NB][NB + 1];
    __shared__ double rinv[NB];
    __shared__ int bad;
    const int tid = threadIdx.x;
    const int64_t nb = (S - k0) < NB ? (S - k0) : NB;
    if (tid == 0) bad = 0;
    for (int e = tid; e < NB * NB; e += 256) {
        const int i = e / NB, j = e % NB;
        double v;
        if (i < nb && j < nb)
            v = (j <= i) ? L[(k0 + i) * S + k0 + j] : 0.0;
        else
            v = (i == j) ? 1.0 : 0.0;  // identity padding past the matrix end
        a[i][j] = v;
        l[i][j] = 0.0;
        inv[i][j] = 0.0;
    }
    const int ur = tid >> 3, uq = tid & 7;
    for (int j = 0; j < NB; ++j) {
        __syncthreads();
        const double d = a[j][j];
        if (!(d > 0.0)) {
            if (tid == 0) {
                bad = 1;
                report(info, AJ_INFO_NOT_POSITIVE_DEFINITE, k0 + j);
            }
            break;
        }
        const double r = rsqrt(d);
        if (tid == 0) {
            l[j][j] = d * r;
            rinv[j] = r;
        }
        if (ur > j) {
            const double lrj = a[ur][j] * r;
            if (uq == 0) l[ur][j] = lrj;
#pragma unroll
            for (int c = uq; c < NB; c += 8)
                if (c > j && c <= ur) a[ur][c] = fma(-lrj, a[c][j] * r, a[ur][c]);
        }
    }
    __syncthreads();
    if (bad) return;
    const int c = tid >> 3, q = tid & 7;
    if (tid < NB) inv[tid][tid] = rinv[tid];
    __syncthreads();
    for (int i = 1; i < NB; ++i) {
        double part = 0.0;
        if (c < i)
            for (int p = c + q; p < i; p += 8) part = fma(l[i][p], inv[p][c], part);
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (c < i && q == 0) inv[i][c] = -part * rinv[i];
        __syncthreads();
    }
    for (int e = tid; e < NB * NB; e += 256) {
        const int i = e / NB, j = e % NB;
        if (i < nb && j < nb) L[(k0 + i) * S + k0 + j] = (j <= i) ? l[i][j] : 0.0;
        dinv[e] = inv[i][j];
    }
}

// rows r >= k0 + NB: L[r][k0 .. k0+NB) = L[r][k0 ..) * dinv^T (32 rows per block)
__global__ void __launch_bounds__(256)
    chol_panel_kernel(double* __restrict__ L, int64_t S, int64_t k0, const double* __restrict__ dinv) {
    __shared__ double x[32][NB + 1];
    __shared__ double d[NB][NB + 1];
    const int tid = threadIdx.x;
    const int64_t r0 = k0 + NB + blockIdx.x * 32;
    const int64_t nb = (S - k0) < NB ? (S - k0) : NB;
    for (int e = tid; e < 32 * NB; e += 256) {
        const int i = e / NB, j = e % NB;
        const int64_t r = r0 + i;
        x[i][j] = (r < S && j < nb) ? L[r * S + k0 + j] : 0.0;
        d[i][j] = dinv[e];
    }
    __syncthreads();
    const int i = tid >> 3, q = tid & 7;
    const int64_t r = r0 + i;
    double out[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int c = q + 8 * t;
        double s = 0.0;
        for (int p = 0; p <= c; ++p) s = fma(x[i][p], d[c][p], s);
        out[t] = s;
    }
    if (r < S)
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int c = q + 8 * t;
            if (c < nb) L[r * S + k0 + c] = out[t];
        }
}

__global__ void zero_upper_kernel(double* __restrict__ L, int64_t S) {
    for (int64_t i = blockIdx.y; i < S; i += gridDim.y)
        for (int64_t j = i + 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < S;
             j += (int64_t)gridDim.x * blockDim.x)
            L[i * S + j] = 0.0;
}

__global__ void logdet_kernel(const double* __restrict__ L, int64_t S, double* __restrict__ out, const int* info) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < S; i += blockDim.x) acc += log(L[i * S + i]);
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) *out = (info && info[0] == AJ_INFO_NOT_POSITIVE_DEFINITE) ? NAN : 2.0 * acc;
}

// --------------------------------------------------- triangular inverse

__global__ void linv_init_kernel(double* __restrict__ Li, int64_t S, const double* __restrict__ dinv, int64_t kb0) {
    const int64_t kb = kb0 + blockIdx.x;
    const int64_t k0 = kb * NB;
    for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
        const int i = e / NB, j = e % NB;
        if (k0 + i < S && k0 + j < S) Li[(k0 + i) * S + k0 + j] = dinv[kb * NB * NB + e];
    }
}

// One block row step of L X = I: tiles (ti > kb, tj <= kb) accumulate L[ti][kb] X[kb][tj] into the
// off-diagonal storage; tiles of block row kb + 1 then become -dinv[kb+1] * accumulated.
__global__ void __launch_bounds__(256)
    trtri_step_kernel(const double* __restrict__ L, double* __restrict__ Li, int64_t S, int64_t kb,
                      const double* __restrict__ dinv) {
    __shared__ double a[32][33];
    __shared__ double b[32][33];
    const int64_t nbt = (S + NB - 1) / NB;
    const int64_t ncol = kb + 1;
    const int64_t ti = kb + 1 + blockIdx.x / ncol, tj = blockIdx.x % ncol;
    if (ti >= nbt) return;
    const int tid = threadIdx.x;
    const int64_t i0 = ti * NB, j0 = tj * NB, p0 = kb * NB;
    for (int e = tid; e < NB * NB; e += 256) {
        const int r = e / NB, c = e % NB;
        a[r][c] = (i0 + r < S && p0 + c < S) ? L[(i0 + r) * S + p0 + c] : 0.0;   // L[ti][kb]
        b[r][c] = (p0 + r < S && j0 + c < S) ? Li[(p0 + r) * S + j0 + c] : 0.0;  // X[kb][tj]
    }
    __syncthreads();
    const int r = tid >> 3, q = tid & 7;
    double acc[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int c = q + 8 * t;
        double s = (i0 + r < S && j0 + c < S) ? Li[(i0 + r) * S + j0 + c] : 0.0;
        for (int p = 0; p < NB; ++p) s = fma(a[r][p], b[p][c], s);
        acc[t] = s;
    }
    if (ti != kb + 1) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int c = q + 8 * t;
            if (i0 + r < S && j0 + c < S) Li[(i0 + r) * S + j0 + c] = acc[t];
        }
        return;
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 4; ++t) a[r][q + 8 * t] = acc[t];  // reuse a as the accumulated tile
    for (int e = tid; e < NB * NB; e += 256) b[e / NB][e % NB] = dinv[(kb + 1) * NB * NB + e];
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int c = q + 8 * t;
        double s = 0.0;
        for (int p = 0; p <= r; ++p) s = fma(b[r][p], a[p][c], s);
        if (i0 + r < S && j0 + c < S) Li[(i0 + r) * S + j0 + c] = -s;
    }
}

__global__ void mirror_lower_kernel(double* __restrict__ A, int64_t S) {
    for (int64_t i = blockIdx.y; i < S; i += gridDim.y)
        for (int64_t j = i + 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < S;
             j += (int64_t)gridDim.x * blockDim.x)
            A[i * S + j] = A[j * S + i];
}

// ----------------------------------------------------------- vector solves

// forward step kb: y_kb = dinv_kb r_kb (r = running right-hand side); block 0 stores y_kb,
// blocks b >= 1 subtract L[rows of block b][kb] y_kb from r for the rows below.
__global__ void __launch_bounds__(128)
    fwd_step_kernel(const double* __restrict__ L, int64_t S, int64_t kb, const double* __restrict__ dinv,
                    double* __restrict__ r, double* __restrict__ y) {
    __shared__ double yk[NB];
    const int64_t k0 = kb * NB;
    const int tid = threadIdx.x;
    if (tid < NB) {
        double s = 0.0;
        for (int p = 0; p <= tid; ++p) {
            const double v = (k0 + p < S) ? r[k0 + p] : 0.0;
            s = fma(dinv[kb * NB * NB + tid * NB + p], v, s);
        }
        yk[tid] = s;
    }
    __syncthreads();
    if (blockIdx.x == 0) {
        if (tid < NB && k0 + tid < S) y[k0 + tid] = yk[tid];
        return;
    }
    const int64_t row = k0 + NB + (int64_t)(blockIdx.x - 1) * blockDim.x + tid;
    if (row < S) {
        double s = 0.0;
        for (int p = 0; p < NB && k0 + p < S; ++p) s = fma(L[row * S + k0 + p], yk[p], s);
        r[row] -= s;
    }
}

// backward step kb (descending): x_kb = dinv_kb^T r_kb; block 0 stores x_kb, other blocks
// subtract L[kb rows][col]^T x_kb from r for the columns left of the block.
__global__ void __launch_bounds__(128)
    bwd_step_kernel(const double* __restrict__ L, int64_t S, int64_t kb, const double* __restrict__ dinv,
                    double* __restrict__ r, double* __restrict__ x) {
    __shared__ double xk[NB];
    const int64_t k0 = kb * NB;
    const int tid = threadIdx.x;
    if (tid < NB) {
        double s = 0.0;
        for (int p = tid; p < NB; ++p) {
            const double v = (k0 + p < S) ? r[k0 + p] : 0.0;
            s = fma(dinv[kb * NB * NB + p * NB + tid], v, s);
        }
        xk[tid] = s;
    }
    __syncthreads();
    if (blockIdx.x == 0) {
        if (tid < NB && k0 + tid < S) x[k0 + tid] = xk[tid];
        return;
    }
    const int64_t col = (int64_t)(blockIdx.x - 1) * blockDim.x + tid;
    if (col < k0) {
        double s = 0.0;
        for (int p = 0; p < NB && k0 + p < S; ++p) s = fma(L[(k0 + p) * S + col], xk[p], s);
        r[col] -= s;
    }
}

// ------------------------------------------------------------ host side

size_t spd_workspace_bytes(int64_t S, bool with_inverse) {
    const int64_t nbt = (S + NB - 1) / NB;
    Sizer s;
    s.take<double>(S * S);
    if (with_inverse) s.take<double>(S * S);
    s.take<double>(nbt * NB * NB);
    s.take<double>(2 * S);
    s.take<double>(8);
    return s.total();
}

SpdWorkspace spd_carve(Carver& cv, int64_t S, bool with_inverse) {
    const int64_t nbt = (S + NB - 1) / NB;
    SpdWorkspace w;
    w.L = cv.take<double>(S * S);
    w.Linv = with_inverse ? cv.take<double>(S * S) : nullptr;
    w.dinv = cv.take<double>(nbt * NB * NB);
    w.vec = cv.take<double>(2 * S);
    w.scal = cv.take<double>(8);
    return w;
}

int spd_factor(const double* A, int64_t S, SpdWorkspace& w, double* logdet, int* info, cudaStream_t st,
               bool lookahead, bool with_inverse, double* Ainv) {
    if (with_inverse && !w.Linv) return AJ_ERR_ARG;
    if (Ainv && !with_inverse) return AJ_ERR_ARG;
    if (S <= 0) return AJ_OK;
    if (A != w.L && cudaMemcpyAsync(w.L, A, sizeof(double) * S * S, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return AJ_ERR_CUDA;
    const int64_t nbt = (S + NB - 1) / NB;
    if (!lookahead || nbt < 3) {
        if (with_inverse && cudaMemsetAsync(w.Linv, 0, sizeof(double) * S * S, st) != cudaSuccess) return AJ_ERR_CUDA;
        for (int64_t kb = 0; kb < nbt; ++kb) {
            const int64_t k0 = kb * NB;
            chol_diag_kernel<<<1, 256, 0, st>>>(w.L, S, k0, w.dinv + kb * NB * NB, info);
            AJ_LAUNCHED();
            const int64_t below = S - k0 - NB;
            if (below > 0) {
                chol_panel_kernel<<<(unsigned)((below + 31) / 32), 256, 0, st>>>(w.L, S, k0, w.dinv + kb * NB * NB);
                AJ_LAUNCHED();
                double* P = w.L + (k0 + NB) * S + k0;
                AJ_TRY(gemm_f64(false, true, below, below, NB, -1.0, P, S, P, S, 1.0, w.L + (k0 + NB) * S + k0 + NB,
                                S, true, st));
            }
        }
        if (with_inverse) {
            linv_init_kernel<<<(unsigned)nbt, 256, 0, st>>>(w.Linv, S, w.dinv, 0);
            AJ_LAUNCHED();
            for (int64_t kb = 0; kb + 1 < nbt; ++kb) {
                trtri_step_kernel<<<(unsigned)((nbt - kb - 1) * (kb + 1)), 256, 0, st>>>(w.L, w.Linv, S, kb, w.dinv);
                AJ_LAUNCHED();
            }
        }
        if (Ainv) AJ_TRY(spd_inverse_from_factor(S, w, Ainv, st));
    } else {
        // One step of lookahead on two lanes (lanes.cu): lane 0 carries the chain (the diagonal
        // block, the panel below it, and the update of the next block column alone), lane 1 the
        // rest of each step's trailing update, which then runs beside the next step's chain.  The
        // next block column also takes the previous step's bulk update, so lane 0 waits for it
        // before updating that column.
        // With the inverse, lane 2 runs L^-1's block forward substitution one step behind: its
        // step kb needs block column kb of L (final after panel kb) and the inverse of diagonal
        // block kb + 1.
        // With A^-1, lane 3 builds it up as L^-T L^-1 one block row of L^-1 at a time: once block row
        // R is final (after its diagonal block and L^-1's step R - 1), its rank-32 contribution goes
        // into every lower tile (I, J <= R).
        Lanes* lp = nullptr;
        AJ_TRY(lanes_for(st, &lp));
        Lanes& ln = *lp;
        const int nl = Ainv ? 4 : (with_inverse ? 3 : 2);
        AJ_TRY(lanes_fork(ln, st, nl));
        cudaStream_t crit = ln.s[0], bulk = ln.s[1], inv = ln.s[2], lau = ln.s[3];
        if (with_inverse && cudaMemsetAsync(w.Linv, 0, sizeof(double) * S * S, inv) != cudaSuccess)
            return AJ_ERR_CUDA;
        if (Ainv && cudaMemsetAsync(Ainv, 0, sizeof(double) * S * S, lau) != cudaSuccess) return AJ_ERR_CUDA;
        bool bulk_prev = false;
        for (int64_t kb = 0; kb < nbt; ++kb) {
            const int64_t k0 = kb * NB;
            chol_diag_kernel<<<1, 256, 0, crit>>>(w.L, S, k0, w.dinv + kb * NB * NB, info);
            AJ_LAUNCHED();
            if (with_inverse) {
                AJ_TRY(lane_signal(ln, kEvDiag, 0));
                AJ_TRY(lane_wait(ln, 2, kEvDiag));
                linv_init_kernel<<<1, 256, 0, inv>>>(w.Linv, S, w.dinv, kb);
                AJ_LAUNCHED();
                if (kb > 0) {
                    trtri_step_kernel<<<(unsigned)((nbt - kb) * kb), 256, 0, inv>>>(w.L, w.Linv, S, kb - 1, w.dinv);
                    AJ_LAUNCHED();
                }
                if (Ainv) {
                    // block row kb of L^-1 is final now
                    AJ_TRY(lane_signal(ln, kEvRow, 2));
                    AJ_TRY(lane_wait(ln, 3, kEvRow));
                    const int64_t m = (kb + 1) * NB < S ? (kb + 1) * NB : S;
                    const int64_t kr = S - k0 < NB ? S - k0 : NB;
                    const double* R = w.Linv + k0 * S;
                    AJ_TRY(gemm_f64(true, false, m, m, kr, 1.0, R, S, R, S, 1.0, Ainv, S, true, lau));
                }
            }
            const int64_t below = S - k0 - NB;
            if (below <= 0) break;
            chol_panel_kernel<<<(unsigned)((below + 31) / 32), 256, 0, crit>>>(w.L, S, k0, w.dinv + kb * NB * NB);
            AJ_LAUNCHED();
            double* P = w.L + (k0 + NB) * S + k0;
            const int64_t cw = below < NB ? below : NB;
            const int64_t rest = below - cw;
            if (rest > 0) {
                AJ_TRY(lane_signal(ln, kEvPanel, 0));
                AJ_TRY(lane_wait(ln, 1, kEvPanel));
            }
            if (bulk_prev) AJ_TRY(lane_wait(ln, 0, kEvUpdate));
            AJ_TRY(gemm_f64(false, true, below, cw, NB, -1.0, P, S, P, S, 1.0, w.L + (k0 + NB) * S + k0 + NB, S, false,
                            crit));
            if (rest > 0) {
                const int64_t c0 = k0 + NB + cw;
                AJ_TRY(gemm_f64(false, true, rest, rest, NB, -1.0, P + cw * S, S, P + cw * S, S, 1.0,
                                w.L + c0 * S + c0, S, true, bulk));
                AJ_TRY(lane_signal(ln, kEvUpdate, 1));
            }
            bulk_prev = rest > 0;
        }
        AJ_TRY(lanes_join(ln, st, nl));
        if (Ainv) {
            dim3 g(blocks_for(S, 256, 8), (unsigned)(S < 65535 ? S : 65535));
            mirror_lower_kernel<<<g, 256, 0, st>>>(Ainv, S);
            AJ_LAUNCHED();
        }
    }
    dim3 zg(blocks_for(S, 256, 8), (unsigned)(S < 65535 ? S : 65535));
    zero_upper_kernel<<<zg, 256, 0, st>>>(w.L, S);
    AJ_LAUNCHED();
    if (logdet) {
        logdet_kernel<<<1, 1024, 0, st>>>(w.L, S, logdet, info);
        AJ_LAUNCHED();
    }
    return AJ_OK;
}

int spd_invert_factor(int64_t S, SpdWorkspace& w, int* info, cudaStream_t st) {
    (void)info;
    if (S <= 0) return AJ_OK;
    if (!w.Linv) return AJ_ERR_ARG;
    const int64_t nbt = (S + NB - 1) / NB;
    if (cudaMemsetAsync(w.Linv, 0, sizeof(double) * S * S, st) != cudaSuccess) return AJ_ERR_CUDA;
    linv_init_kernel<<<(unsigned)nbt, 256, 0, st>>>(w.Linv, S, w.dinv, 0);
    AJ_LAUNCHED();
    for (int64_t kb = 0; kb + 1 < nbt; ++kb) {
        const int64_t tiles = (nbt - kb - 1) * (kb + 1);
        trtri_step_kernel<<<(unsigned)tiles, 256, 0, st>>>(w.L, w.Linv, S, kb, w.dinv);
        AJ_LAUNCHED();
    }
    return AJ_OK;
}

int spd_inverse_from_factor(int64_t S, SpdWorkspace& w, double* Ainv, cudaStream_t st) {
    if (S <= 0) return AJ_OK;
    const int64_t tm = (S + 31) / 32;
    gemm_f64_kernel<true, false><<<(unsigned)(tm * (tm + 1) / 2), 256, 0, st>>>(S, S, S, 1.0, w.Linv, S, w.Linv, S, 0.0,
                                                                               Ainv, S, 1, 1, tm);
    AJ_LAUNCHED();
    dim3 g(blocks_for(S, 256, 8), (unsigned)(S < 65535 ? S : 65535));
    mirror_lower_kernel<<<g, 256, 0, st>>>(Ainv, S);
    return check_launch();
}

int spd_solve_vec(int64_t S, SpdWorkspace& w, const double* b, double* x, int* info, cudaStream_t st) {
    (void)info;
    if (S <= 0) return AJ_OK;
    const int64_t nbt = (S + NB - 1) / NB;
    double* r = w.vec;
    double* y = w.vec + S;
    if (cudaMemcpyAsync(r, b, sizeof(double) * S, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return AJ_ERR_CUDA;
    for (int64_t kb = 0; kb < nbt; ++kb) {
        const int64_t below = S - kb * NB - NB;
        const unsigned g = 1 + (unsigned)(below > 0 ? (below + 127) / 128 : 0);
        fwd_step_kernel<<<g, 128, 0, st>>>(w.L, S, kb, w.dinv, r, y);
        AJ_LAUNCHED();
    }
    for (int64_t kb = nbt - 1; kb >= 0; --kb) {
        const int64_t left = kb * NB;
        const unsigned g = 1 + (unsigned)((left + 127) / 128);
        bwd_step_kernel<<<g, 128, 0, st>>>(w.L, S, kb, w.dinv, y, x);
        AJ_LAUNCHED();
    }
    return AJ_OK;
}

}  // namespace aj

using namespace aj;

extern "C" {

size_t aj_spd_solve_workspace_size(int64_t S) { return spd_workspace_bytes(S, false); }

int aj_spd_solve(const double* data_vector, const double* A, int64_t S, double* out, void* workspace,
                 size_t workspace_bytes, int* info, void* stream) {
    if (S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!data_vector || !A || !out) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < spd_workspace_bytes(S, false)) return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace, workspace_bytes);
    SpdWorkspace w = spd_carve(cv, S, false);
    AJ_TRY(spd_factor(A, S, w, nullptr, info, st));
    return spd_solve_vec(S, w, data_vector, out, info, st);
}

int aj_spd_logdet(const double* A, int64_t S, double* out, void* workspace, size_t workspace_bytes, int* info,
                  void* stream) {
    if (S < 0 || !out) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (S == 0) return cudaMemsetAsync(out, 0, sizeof(double), st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    if (!A) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < spd_workspace_bytes(S, false)) return AJ_ERR_WORKSPACE;
    Carver cv(workspace, workspace_bytes);
    SpdWorkspace w = spd_carve(cv, S, false);
    return spd_factor(A, S, w, out, info, st);
}

size_t aj_spd_inverse_workspace_size(int64_t S) { return spd_workspace_bytes(S, true); }

int aj_spd_inverse(const double* A, int64_t S, double* Ainv, double* logdet, void* workspace, size_t workspace_bytes,
                   int* info, void* stream) {
    if (S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!A || !Ainv) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < spd_workspace_bytes(S, true)) return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace, workspace_bytes);
    SpdWorkspace w = spd_carve(cv, S, true);
    return spd_factor(A, S, w, logdet, info, st, true, true, Ainv);
}

}  // extern "C"
