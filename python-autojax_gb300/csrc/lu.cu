// LU with partial pivoting in float64: the reference's general solve and log|det|
// (np.linalg.solve and np.linalg.slogdet, numba.py:731 and 849-850, both LAPACK
// getrf) for a curvature-plus-regularisation matrix that is not positive definite.
//
// The inversion's A = F + H is symmetric positive definite by construction, so the
// Cholesky paths serve every ordinary call; this is the fallback the Python layer
// takes when the Cholesky reports a non-positive pivot, so that an indefinite but
// non-singular A is solved, as the reference solves it, instead of rejected.
//
// Blocked right-looking factorisation, NB = 32 columns a step, row-major in place:
//   panel  — one 1024-thread block factors the S - k0 rows of the 32-column panel
//            column by column: the pivot is the first row of largest magnitude
//            (as LAPACK's idamax picks it), the panel's part of the two rows is
//            swapped, the column scaled and the rest of the panel updated;
//   swaps  — the panel's row interchanges applied to every other column, one
//            thread per column, in order;
//   U block row — the unit-lower triangle of the panel solved against the block
//            row to the right of it, one thread per column;
//   update — the trailing matrix minus L21 U12 (the float64 GEMM).
// A pivot that is exactly zero sets info to AJ_INFO_SINGULAR (LAPACK's info > 0)
// and is left unscaled.  The solve permutes b, then runs the unit-lower and upper
// substitutions column-oriented in one block; log|det A| = sum log|U_ii|.

#include <math.h>

#include "aj_internal.cuh"

namespace aj {

namespace {

constexpr int kLuNB = 32;
constexpr int kLuThreads = 1024;

__global__ void __launch_bounds__(kLuThreads)
    lu_panel_kernel(double* __restrict__ A, int64_t S, int64_t k0, int nb, int64_t* __restrict__ piv, int* info) {
    __shared__ double best_v[kLuThreads / 32];
    __shared__ int64_t best_i[kLuThreads / 32];
    __shared__ int64_t pivot_row;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int jj = 0; jj < nb; ++jj) {
        const int64_t j = k0 + jj;
        // first row of largest |A[i][j]|, i >= j
        double bv = -1.0;
        int64_t bi = S;
        for (int64_t i = j + tid; i < S; i += kLuThreads) {
            const double v = fabs(A[i * S + j]);
            if (v > bv) {
                bv = v;
                bi = i;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            best_v[wid] = bv;
            best_i[wid] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            double v = best_v[0];
            int64_t r = best_i[0];
            for (int w = 1; w < kLuThreads / 32; ++w)
                if (best_v[w] > v || (best_v[w] == v && best_i[w] < r)) {
                    v = best_v[w];
                    r = best_i[w];
                }
            if (r >= S) r = j;
            pivot_row = r;
            piv[j] = r;
            if (!(A[r * S + j] != 0.0)) report(info, AJ_INFO_SINGULAR, j);
        }
        __syncthreads();
        const int64_t p = pivot_row;
        // swap the panel's part of rows j and p
        if (p != j && tid < nb) {
            const int64_t c = k0 + tid;
            const double t = A[j * S + c];
            A[j * S + c] = A[p * S + c];
            A[p * S + c] = t;
        }
        __syncthreads();
        const double d = A[j * S + j];
        const bool ok = d != 0.0;
        // scale the column below the pivot and update the panel's remaining columns
        for (int64_t i = j + 1 + tid; i < S; i += kLuThreads) {
            double l = A[i * S + j];
            if (ok) {
                l = l / d;
                A[i * S + j] = l;
            }
            for (int c = jj + 1; c < nb; ++c) A[i * S + k0 + c] = fma(-l, A[j * S + k0 + c], A[i * S + k0 + c]);
        }
        __syncthreads();
    }
}

// The panel's interchanges (rows k0 .. k0 + nb - 1, in order) on the columns outside the panel.
__global__ void lu_swap_kernel(double* __restrict__ A, int64_t S, int64_t k0, int nb, const int64_t* __restrict__ piv) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < S - nb; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t col = c < k0 ? c : c + nb;
        for (int jj = 0; jj < nb; ++jj) {
            const int64_t j = k0 + jj, p = piv[j];
            if (p != j) {
                const double t = A[j * S + col];
                A[j * S + col] = A[p * S + col];
                A[p * S + col] = t;
            }
        }
    }
}

// U12 = L11^-1 A12 for the columns right of the panel (L11 unit lower).
__global__ void lu_trsm_kernel(double* __restrict__ A, int64_t S, int64_t k0, int nb) {
    const int64_t c0 = k0 + nb;
    for (int64_t c = c0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < S; c += (int64_t)gridDim.x * blockDim.x) {
        double u[kLuNB];
        for (int r = 0; r < nb; ++r) u[r] = A[(k0 + r) * S + c];
        for (int r = 1; r < nb; ++r) {
            double v = u[r];
            for (int q = 0; q < r; ++q) v = fma(-A[(k0 + r) * S + k0 + q], u[q], v);
            u[r] = v;
        }
        for (int r = 1; r < nb; ++r) A[(k0 + r) * S + c] = u[r];
    }
}

// x = A^-1 b from the factor: P b, then L y = P b (unit lower), then U x = y, column-oriented.
__global__ void __launch_bounds__(kLuThreads)
    lu_solve_kernel(const double* __restrict__ LU, int64_t S, const int64_t* __restrict__ piv,
                    const double* __restrict__ b, double* __restrict__ x) {
    const int tid = threadIdx.x;
    for (int64_t i = tid; i < S; i += kLuThreads) x[i] = b[i];
    __syncthreads();
    if (tid == 0)
        for (int64_t j = 0; j < S; ++j) {
            const int64_t p = piv[j];
            if (p != j) {
                const double t = x[j];
                x[j] = x[p];
                x[p] = t;
            }
        }
    __syncthreads();
    for (int64_t j = 0; j < S; ++j) {
        const double yj = x[j];
        for (int64_t i = j + 1 + tid; i < S; i += kLuThreads) x[i] = fma(-LU[i * S + j], yj, x[i]);
        __syncthreads();
    }
    for (int64_t j = S - 1; j >= 0; --j) {
        __shared__ double xj;
        if (tid == 0) {
            xj = x[j] / LU[j * S + j];
            x[j] = xj;
        }
        __syncthreads();
        const double v = xj;
        for (int64_t i = tid; i < j; i += kLuThreads) x[i] = fma(-LU[i * S + j], v, x[i]);
        __syncthreads();
    }
}

__global__ void lu_logabsdet_kernel(const double* __restrict__ LU, int64_t S, double* __restrict__ out) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < S; i += blockDim.x) acc += log(fabs(LU[i * S + i]));
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) *out = acc;
}

struct LuBufs {
    double* LU;
    int64_t* piv;
};

size_t lu_carve(Carver& cv, int64_t S, LuBufs& b) {
    b.LU = cv.take<double>(S * S);
    b.piv = cv.take<int64_t>(S);
    return cv.used;
}

}  // namespace

}  // namespace aj

using namespace aj;

extern "C" {

size_t aj_lu_solve_workspace_size(int64_t S) {
    if (S < 0) return 0;
    Carver cv(nullptr, ~size_t(0) >> 1);
    LuBufs b;
    lu_carve(cv, S, b);
    return align_up(cv.used);
}

int aj_lu_solve(const double* data_vector, const double* A, int64_t S, double* out, double* logabsdet,
                void* workspace, size_t workspace_bytes, int* info, void* stream) {
    if (S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!A || !info || (out && !data_vector)) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < aj_lu_solve_workspace_size(S)) return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace, workspace_bytes);
    LuBufs b;
    lu_carve(cv, S, b);
    if (cudaMemcpyAsync(b.LU, A, sizeof(double) * S * S, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return AJ_ERR_CUDA;
    for (int64_t k0 = 0; k0 < S; k0 += kLuNB) {
        const int nb = static_cast<int>(S - k0 < kLuNB ? S - k0 : kLuNB);
        lu_panel_kernel<<<1, kLuThreads, 0, st>>>(b.LU, S, k0, nb, b.piv, info);
        AJ_LAUNCHED();
        if (S > nb) {
            lu_swap_kernel<<<blocks_for(S - nb, 256, 4 * num_sms()), 256, 0, st>>>(b.LU, S, k0, nb, b.piv);
            AJ_LAUNCHED();
        }
        const int64_t rest = S - k0 - nb;
        if (rest > 0) {
            lu_trsm_kernel<<<blocks_for(rest, 128, 4 * num_sms()), 128, 0, st>>>(b.LU, S, k0, nb);
            AJ_LAUNCHED();
            double* L21 = b.LU + (k0 + nb) * S + k0;
            double* U12 = b.LU + k0 * S + k0 + nb;
            double* A22 = b.LU + (k0 + nb) * S + k0 + nb;
            AJ_TRY(gemm_f64(false, false, rest, rest, nb, -1.0, L21, S, U12, S, 1.0, A22, S, false, st));
        }
    }
    if (logabsdet) {
        lu_logabsdet_kernel<<<1, 1024, 0, st>>>(b.LU, S, logabsdet);
        AJ_LAUNCHED();
    }
    if (out) {
        lu_solve_kernel<<<1, kLuThreads, 0, st>>>(b.LU, S, b.piv, data_vector, out);
        AJ_LAUNCHED();
    }
    return check_launch();
}

}  // extern "C"
