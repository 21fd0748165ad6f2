// Host-side building blocks shared between the translation units.
#pragma once

#include "aj_common.cuh"

namespace aj {

// ---- linalg.cu

// columns per step of the float64 blocked Cholesky (linalg.cu); the no-allocation solve sizes its
// fixed scratch with it
constexpr int kSpdNB = 32;

// C (m x n) = alpha op(A) op(B) + beta C, row-major float64.
// lower_only: only tiles on or below the diagonal of C are touched (square C).
int gemm_f64(bool transA, bool transB, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
             const double* B, int64_t ldb, double beta, double* C, int64_t ldc, bool lower_only, cudaStream_t st);

// out (cols x rows) = in (rows x cols)^T
template <typename T>
int transpose(const T* in, int64_t rows, int64_t cols, T* out, cudaStream_t st);

// Cholesky-based SPD toolkit on a float64 S x S matrix (row-major, lower triangle used).
struct SpdWorkspace {
    double* L;        // S x S factor (lower), also holds scratch upper
    double* Linv;     // S x S inverse factor (lower) or nullptr
    double* dinv;     // nblocks x NB x NB inverses of the diagonal blocks
    double* vec;      // S scratch
    double* scal;     // 8 scratch scalars
};
size_t spd_workspace_bytes(int64_t S, bool with_inverse);
SpdWorkspace spd_carve(Carver& cv, int64_t S, bool with_inverse);
// L = chol(A) (A read, not modified); logdet written to *logdet (device); info on failure.
// With lookahead the chain and the bulk of each trailing update run on two lanes forked from st;
// with_inverse also computes Linv = L^-1 (w.Linv), on a third lane one step behind the factor, and
// with Ainv (S x S) also A^-1 = L^-T L^-1 (full symmetric), streamed on a fourth lane.
int spd_factor(const double* A, int64_t S, SpdWorkspace& w, double* logdet, int* info, cudaStream_t st,
               bool lookahead = true, bool with_inverse = false, double* Ainv = nullptr);
// Linv = L^-1 (lower)
int spd_invert_factor(int64_t S, SpdWorkspace& w, int* info, cudaStream_t st);
// x = A^-1 b using L (triangular solves); b and x may alias
int spd_solve_vec(int64_t S, SpdWorkspace& w, const double* b, double* x, int* info, cudaStream_t st);
// Ainv (S x S, full symmetric) = Linv^T Linv
int spd_inverse_from_factor(int64_t S, SpdWorkspace& w, double* Ainv, cudaStream_t st);

// ---- lanes.cu (side streams that fork from and join back into the caller's stream)

// 0: critical chain (highest priority; the others share the next), 1: bulk updates, 2: triangular inverse
// of the first matrix, 3: triangular inverse of the second, 4: A^-1 of the first; 5: a second
// factorisation running beside the first (never forked or joined by it)
constexpr int kLaneCount = 6;
enum LaneEvent {
    kEvFork = 0,
    kEvPanel,
    kEvUpdate,
    kEvDiag,
    kEvRow,      // a block row of the first matrix's L^-1 is final
    kEvPre,      // the evaluation's independent pre-work forks here ...
    kEvPreDone,  // ... and is joined here
    kEvHDone,    // H's factorisation, beside A's, is done
    kEvHReady,   // H is split and its inverse buffer zeroed
    kEvAinv,     // A^-1 is complete (its product runs beside the solve's first products)
    kEvJoin0,
    kLaneEvents = kEvJoin0 + kLaneCount
};
struct Lanes {
    cudaStream_t s[kLaneCount];
    cudaEvent_t ev[kLaneEvents];
};
// the lanes that forks from `caller` use on the current device (created on first use)
int lanes_for(cudaStream_t caller, Lanes** out);
// destroys the lanes of `caller` on the current device, if it has any
int lanes_release(cudaStream_t caller);
// lanes 0..n-1 start after the work already on st
int lanes_fork(Lanes& l, cudaStream_t st, int n);
// st continues after the work on lanes 0..n-1
int lanes_join(Lanes& l, cudaStream_t st, int n);
int lane_signal(Lanes& l, int event, int from);
int lane_wait(Lanes& l, int lane, int event);

// ---- linalg_df.cu (double-float planes: hi and lo float arrays)

struct DfSpd {
    float *Lh, *Ll;  // factor (S x S)
    float *Ih, *Il;  // inverse factor (S x S) or null
    float *dh, *dl;  // inverses of the diagonal blocks
    float *fh, *fl;  // factored diagonal blocks
    double* piv;     // the S pivots L_ii in float64
    double* vec;     // S scratch
    double* vec2;    // S scratch
    float* part;     // partial sums of the transposed triangular product
    void* tcws;      // scratch of the tensor-core L^-T L^-1 (with_ainv), or null
    size_t tcws_bytes;
};
// with_ainv: also the scratch for A^-1 = L^-T L^-1 on the tensor cores (needs with_inverse)
size_t dfspd_bytes(int64_t S, bool with_inverse, bool with_ainv = false);
DfSpd dfspd_carve(Carver& cv, int64_t S, bool with_inverse, bool with_ainv = false);
// A^-1's lower triangle (double-float planes, leading dimension S) = X^T X, X = L^-1 lower, on the
// tensor cores
size_t tc_lauum_workspace_bytes(int64_t S);
int tc_lauum(const float* Xh, const float* Xl, int64_t S, float* Ch, float* Cl, void* ws, size_t bytes,
             cudaStream_t st);
int df_split(const double* x, int64_t n, float* hi, float* lo, cudaStream_t st);
int df_mirror_lower(float* hi, float* lo, int64_t S, cudaStream_t st);
int df_join(const float* hi, const float* lo, int64_t n, double* x, cudaStream_t st);
// A = F + H (S x S) from F's lower triangle (F planes, H float64): A symmetric in full, and its
// lower triangle, upper zero, in lo_h/lo_l
int df_add_f64_sym(const float* fh, const float* fl, const double* h, int64_t S, float* ah, float* al, float* lo_h,
                   float* lo_l, cudaStream_t st);
int gemm_df(bool ta, bool tb, int64_t m, int64_t n, int64_t k, bool neg, const float* Ah, const float* Al, int64_t lda,
            const float* Bh, const float* Bl, int64_t ldb, bool accumulate, float* Ch, float* Cl, int64_t ldc,
            bool lower_only, bool tri_k, cudaStream_t st);
// Double-float Cholesky L (in w[z]) with log|A| of count = 1 or 2 independent
// S x S matrices (planes) sharing every launch; the
// first n_inverse of them also get their inverse factor L^-1 (in w->Ih/Il),
// computed alongside the factorisation as its panels complete.  With AIh/AIl
// set (planes, S x S; the first matrix's DfSpd carved with_ainv), the first
// matrix's inverse A^-1 = L^-T L^-1 follows on the tensor cores (tc_lauum).
// f32_inverse: L^-1 in plain float32 from L's hi plane (into Ih; Il keeps what it held), for a
// matrix whose L^-1 serves only a trace that enters the result scaled down (the regularisation
// matrix's tr(H^-1))
int dfspd_factor_invert_n(const float* const* Ah, const float* const* Al, int count, int n_inverse, int64_t S,
                          DfSpd* const* w, double* const* logdet, int* info, cudaStream_t st, float* AIh = nullptr,
                          float* AIl = nullptr, bool prepared = false, bool f32_inverse = false);
// x = A^-1 b refined once against A (planes), the correction through A^-1's planes when given;
// b_split: b's planes are already in w.vec; xh/xl, when set, receive x's planes; ainv_ready, when
// set, is waited for before the correction reads A^-1 (whose product may run on another stream)
int dfspd_solve_refined(int64_t S, DfSpd& w, const float* Ah, const float* Al, const double* b, double* x,
                        cudaStream_t st, const float* AIh = nullptr, const float* AIl = nullptr, bool b_split = false,
                        float* xh = nullptr, float* xl = nullptr, cudaEvent_t ainv_ready = nullptr);
int df_frob_lower(const float* h, const float* l, int64_t S, double* partial, int64_t nparts, cudaStream_t st);

// ---- wtilde_tc.cu (the mixed direct w_tilde on the tensor cores)

size_t wtilde_tc_workspace_bytes(int64_t K, int64_t M);
// ph/pl (M x M) receive the lower triangle of W = sum_k w_k cos(...) as double-float planes
int wtilde_tc(const double* sigma, const double* uv, const double* grid, int64_t K, int64_t M, float* ph, float* pl,
              void* ws, size_t bytes, cudaStream_t st);

// ---- mapping.cu

// H = 1e-8 I + c^2 L (numba.py:686-694); c read from coefficient_dev when it is not null
int regularization(double coefficient, const double* coefficient_dev, const int64_t* neighbors,
                   const int64_t* neighbors_sizes, int64_t S, int64_t P, double* out, int* info, cudaStream_t st);

// Column-compressed transpose of the sparse mapping (index, weight) rows.
struct Csc {
    int* colptr;   // S + 1
    int* rows;     // nnz capacity M * B
    double* vals;  // nnz capacity
    float2* vdf;   // the same weights as double-float (hi, lo), converted once at build
    int* keys;     // scratch: per-chunk column histograms
    int* cursor;   // scratch: per-chunk column write offsets
    int* part;     // scratch: per chunk-group column counts, then the groups' first offsets
};
enum CscMode { CSC_SUM = 0, CSC_ASSIGN = 1 };
void csc_take(Carver& cv, int64_t M, int64_t B, int64_t S, Csc& c);
size_t csc_bytes(int64_t M, int64_t B, int64_t S);
// rows stop at the first -1 unless `sizes` is given (then row m uses its first sizes[m] entries)
int csc_build(const int64_t* idx, const double* w, const int64_t* sizes, int64_t M, int64_t B, int64_t S, CscMode mode,
              Csc& c, int* info, cudaStream_t st);
// out (S x cols, ld_out) = T^T X (M x cols, ld_x) via the CSC; Tin/Tout float or double
template <typename Tin, typename Tout>
int csc_spmm_t(const Csc& c, int64_t S, const Tin* X, int64_t ld_x, int64_t cols, Tout* out, int64_t ld_out,
               cudaStream_t st);
// double-float planes: out (S x cols) = T^T X with X given as (hi, lo) planes
// (lower: only out[s][c] with c <= s is written)
int csc_spmm_t_df(const Csc& c, int64_t S, const float* Xh, const float* Xl, int64_t ld_x, int64_t cols, float* Oh,
                  float* Ol, int64_t ld_out, cudaStream_t st, bool lower = false);
// the same with the output transposed: out (cols x S, leading dimension ld_out) = (T^T X)^T, bit-identical
// to transposing csc_spmm_t_df's output; needs X rows 16-byte aligned and cols % 4 == 0
int csc_spmm_t_df_tr(const Csc& c, int64_t S, const float* Xh, const float* Xl, int64_t ld_x, int64_t cols, float* Oh,
                     float* Ol, int64_t ld_out, cudaStream_t st);
// out[s] = sum_e val[e] * x[row[e]]
int csc_spmv_t(const Csc& c, int64_t S, const double* x, double* out, cudaStream_t st);
// TW (S x M) with TW[s][m1] = sum_e val[e] * Wc(m1, row[e]) from the compact table (T float or double)
template <typename T>
int csc_compact_tw(const Csc& c, int64_t S, const double* w_compact, int64_t N, const int64_t* native, int64_t M,
                   T* TW, int* info, cudaStream_t st);

}  // namespace aj
