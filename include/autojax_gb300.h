/*
 * autojax_gb300 — C ABI of the GB300 (sm_103a) interferometer inversion kernels.
 *
 * Conventions shared by every entry point:
 *   - pointers are DEVICE pointers to C-contiguous (row-major) arrays with the
 *     reference's dtypes: double for float64, int64_t for int64, interleaved
 *     (re, im) doubles for complex128, uint8_t (0/1) for bool;
 *   - the caller owns every buffer; nothing here allocates device memory.
 *     Scratch comes from a caller-provided workspace whose size the matching
 *     *_workspace_size() function returns;
 *   - work is enqueued on `stream` (a cudaStream_t, NULL = legacy default) and
 *     nothing synchronises, so calls can be captured in CUDA graphs;
 *   - the return value reports argument and launch errors (AJ_OK or a
 *     negative AJ_ERR_*). Data-dependent failures found on the device (an
 *     out-of-range index, a non-positive-definite pivot) are written to the
 *     caller's device word `info` (0 = fine; see AJ_INFO_*), like cuSOLVER's
 *     devInfo; the caller reads it after the stream work completes;
 *   - `precision` selects AJ_FP64 (IEEE float64 throughout, the parity path)
 *     or AJ_MIXED (float64 phase reduction, pivot logarithms and final sums;
 *     the products, factorisations and inverses in double-float arithmetic,
 *     hi + lo float32 pairs with ~2^-47 rounding, on the float32 pipe).
 *
 * Each declaration names the function of ickc/python-autojax it replaces
 * (file:line in src/autojax/).
 */
#ifndef AUTOJAX_GB300_H
#define AUTOJAX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AJ_OK 0
#define AJ_ERR_ARG (-1)       /* bad size, null pointer, unknown precision */
#define AJ_ERR_CUDA (-2)      /* a launch failed; see aj_last_cuda_error() */
#define AJ_ERR_WORKSPACE (-3) /* workspace smaller than *_workspace_size() */
#define AJ_ERR_TOO_LARGE (-4) /* size above the fixed capacity of a no-allocation entry point */

#define AJ_INFO_OK 0
#define AJ_INFO_INDEX_RANGE 1       /* an index was outside [0, n) and not -1 */
#define AJ_INFO_NOT_POSITIVE_DEFINITE 2 /* Cholesky met a pivot <= 0 or NaN */
#define AJ_INFO_SINGULAR 3              /* LU met an exactly zero (or NaN) pivot */

#define AJ_FP64 0
#define AJ_MIXED 1

/* Library version string and the last CUDA error code seen by a launch. */
const char* aj_version(void);
int aj_last_cuda_error(void);
/* Kernel launches this library has issued in the process (for launch accounting). */
unsigned long long aj_launch_count(void);
/* Arithmetic-throughput probe: `blocks` x 256 threads, each running 8 independent
 * fused multiply-add chains for iters x 16 steps (fp32 or fp64); `out` holds
 * blocks * 256 elements of that type. flops = 2 * 128 * iters * blocks * 256. */
int aj_probe_fma(int precision, int64_t blocks, int iters, void* out, void* stream);
/* Number of info words a caller should provide (the first holds the code,
 * the second the failing index or pivot). */
#define AJ_INFO_WORDS 2

/* ---------------------------------------------------------------- geometry */

/* numba.py:50-86 mask_2d_circular_from (centre via numba.py:13-44).
 * mask[ny][nx] = radius^2 < ((y - cy) psy)^2 + ((x - cx) psx)^2, bit-exact. */
int aj_mask_2d_circular(int64_t ny, int64_t nx, double psy, double psx, double radius, double centre_y,
                        double centre_x, uint8_t* mask, void* stream);

/* tests.py:279-281, 304-306 (native_index_for_slim_index = argwhere(~mask),
 * grid_radians_slim = grid_2d[~mask]). Writes the unmasked count to *count
 * (device int64) and, row-major, up to max_out (row, col) pairs; grid_2d
 * (ny, nx, 2) and grid_slim (max_out, 2) may be NULL. */
int aj_slim_from_mask(const uint8_t* mask, int64_t ny, int64_t nx, const double* grid_2d, int64_t max_out,
                      int64_t* native_index, double* grid_slim, int64_t* count, void* stream);

/* ------------------------------------------------------- w_tilde family */

/* numba.py:156-207 w_tilde_curvature_interferometer_from.
 * W[i][j] = sum_k noise_k^-2 cos(2 pi ((x_i - x_j) u_k + (y_i - y_j) v_k)),
 * x = grid[:,1] with u = uv[:,0], y = grid[:,0] with v = uv[:,1].
 * Computed as the K-deep symmetric product C C^T + S S^T of the
 * sqrt(w)-scaled cos/sin panels (exact identity cos(a-b) = cos a cos b +
 * sin a sin b). out64 (M, M) is always written; out_planes (2, M, M), may
 * be NULL, receives the double-float planes (hi then lo) the mixed
 * likelihood reads. AJ_MIXED evaluates the panel in float64, cuts each value
 * into 7 exact 7-bit integer digits (48 bits) and sums the digit products on
 * the bf16 tensor cores (tcgen05, float32 accumulators holding exact integers),
 * folded into double-float; a bounded wait that expires (a fault of the
 * device, not of the data) leaves NaN in out64[0]. */
size_t aj_w_tilde_curvature_workspace_size(int64_t K, int64_t M, int precision);
int aj_w_tilde_curvature(const double* noise_map_real, const double* uv, const double* grid_slim, int64_t K,
                         int64_t M, double* out64, float* out_planes, void* workspace, size_t workspace_bytes,
                         int precision, void* stream);

/* Test probe of the tensor-core digit product behind AJ_MIXED w_tilde (no
 * reference counterpart). digits: [7][Mp][rows] bf16 integers (|d| <= 64),
 * Mp = M rounded up to 128, rows a multiple of 256. For i >= j < M writes
 * out (+)= scale * sum_{d+e<=6} 2^(-7(d+e)) sum_r digits[d][i][r] digits[e][j][r]
 * as double-float planes out_hi/out_lo (M, M); `scale` and `err` are device
 * words (err != 0 after a wait expired). */
int aj_digit_syrk_probe(const void* digits, int64_t rows, int64_t M, float* out_hi, float* out_lo,
                        const float* scale, int accumulate, int* err, void* stream);

/* numba.py:211-234 w_compact_curvature_interferometer_from.
 * out (N, 2N-1): w_c[n0][n1+N-1] = sum_k noise_k^-2 cos(D (n1 u_k - n0 v_k)),
 * D = pi^2 pixel_scale / 324000. */
size_t aj_w_compact_curvature_workspace_size(int64_t N, int64_t K, int precision);
int aj_w_compact_curvature(int64_t N, const double* noise_map_real, const double* uv, int64_t K,
                           double pixel_scale, double* out, void* workspace, size_t workspace_bytes,
                           int precision, void* stream);

/* original.py:230-403 w_tilde_curvature_preload_interferometer_from.
 * out (2Y, 2X): the four corner-offset quadrants of the (Y, X) block of
 * grid_2d (gy, gx, 2), gy >= Y, gx >= X. Row Y and column X stay zero. */
size_t aj_w_tilde_preload_workspace_size(int64_t Y, int64_t X, int64_t K, int precision);
int aj_w_tilde_preload(const double* noise_map_real, const double* uv, int64_t K, int64_t Y, int64_t X,
                       const double* grid_2d, int64_t gy, int64_t gx, double* out, void* workspace,
                       size_t workspace_bytes, int precision, void* stream);

/* numba.py:95-152 w_tilde_data_interferometer_from.
 * out[i] = sum_k (noise_k^2 / vis_k)^2 cos(2 pi (g_i1 u_k + g_i0 v_k)). */
size_t aj_w_tilde_data_workspace_size(int64_t M, int64_t K, int precision);
int aj_w_tilde_data(const double* visibilities_real, const double* noise_map_real, const double* uv,
                    const double* grid_slim, int64_t K, int64_t M, double* out, void* workspace,
                    size_t workspace_bytes, int precision, void* stream);

/* Tile policy of the double-float factorisation (no reference counterpart).
 * A step of the trailing update or of L^-1 runs in 64 x 64 output tiles when
 * it has at least this many of them (per matrix), else in 32 x 32 tiles.
 * Results do not depend on the choice; speed does. Process-wide; set between
 * calls (a captured graph keeps the choice made at capture).
 * autojax_gb300.tune picks the values by timing. */
int aj_set_tile_policy(int update_min_tiles, int inverse_min_tiles);
int aj_get_tile_policy(int* out2);

/* Dirty image (no reference function; the reference reads it from its
 * dataset, tests.py:424-426): out[i] = sum_k noise_k^-2 (Re V_k cos t - Im V_k
 * sin t), t = 2 pi (x_i u_k + y_i v_k), x = grid[:,1], y = grid[:,0]; the
 * adjoint of the DFT, consistent with the chi^2 expansion the likelihood uses.
 * visibilities (K,) complex128. Float64 throughout. */
size_t aj_dirty_image_workspace_size(int64_t M, int64_t K);
int aj_dirty_image(const double* visibilities, const double* noise_map_real, const double* uv,
                   const double* grid_slim, int64_t K, int64_t M, double* out, void* workspace,
                   size_t workspace_bytes, void* stream);

/* numba.py:238-255 w_tilde_via_compact_from. out64/out32 (M, M), either may be NULL.
 * Offsets outside the table set info = AJ_INFO_INDEX_RANGE and write 0. */
int aj_w_tilde_via_compact(const double* w_compact, int64_t N, const int64_t* native_index, int64_t M,
                           double* out64, float* out32, int* info, void* stream);

/* numba.py:259-290 w_tilde_via_preload_from: W[i][j] = preload[y_j - y_i][x_j - x_i]
 * with negative indices wrapping once, as NumPy indexing does. */
int aj_w_tilde_via_preload(const double* preload, int64_t py, int64_t px, const int64_t* native_index, int64_t M,
                           double* out64, float* out32, int* info, void* stream);

/* ------------------------------------------------------ mapping matrix */

/* numba.py:294-376 mapping_matrix_from: out (M, S) dense; rows stop at the
 * first -1; a repeated index keeps the last weight. */
int aj_mapping_matrix(const int64_t* pix_indexes, const double* pix_weights, int64_t M, int64_t B, int64_t S,
                      double* out, int* info, void* stream);

/* numba.py:380-406 data_vector_from: out (S,) = dirty_image (M,) @ mapping (M, S). */
int aj_data_vector(const double* mapping_matrix, const double* dirty_image, int64_t M, int64_t S, double* out,
                   void* stream);

/* numba.py:410-435 curvature_matrix_via_w_tilde_from: out (S, S) = T^T W T
 * (dense T (M, S), dense W (M, M)); workspace holds W T. */
size_t aj_curvature_dense_workspace_size(int64_t M, int64_t S);
int aj_curvature_dense(const double* w_tilde, const double* mapping_matrix, int64_t M, int64_t S, double* out,
                       void* workspace, size_t workspace_bytes, void* stream);

/* Sparse (index, weight) mapping products. The workspace holds the
 * column-compressed transpose of T built on the device. */
size_t aj_sparse_workspace_size(int64_t M, int64_t B, int64_t S, int64_t cols);

/* numba.py:553-587 sparse_mapping_matrix_transpose_matmul: out (S, cols) = T^T matrix (M, cols). */
int aj_sparse_mapping_matrix_transpose_matmul(const double* matrix, int64_t M, int64_t cols,
                                              const int64_t* pix_indexes, const double* pix_weights, int64_t B,
                                              int64_t S, double* out, void* workspace, size_t workspace_bytes,
                                              int* info, void* stream);

/* numba.py:591-614 curvature_matrix_via_w_wilde_sparse_mapping_matrix_from:
 * out (S, S) = T^T (T^T W)^T. */
int aj_curvature_w_tilde_sparse(const double* w_tilde, int64_t M, const int64_t* pix_indexes,
                                const double* pix_weights, int64_t B, int64_t S, double* out, void* workspace,
                                size_t workspace_bytes, int* info, void* stream);

/* numba.py:591-614 curvature_matrix_via_w_wilde_sparse_mapping_matrix_from in double-float:
 * the two gathers the AJ_MIXED likelihood runs (Omega = (T^T W)^T, then F = T^T Omega) from
 * W's double-float planes (hi, lo; see aj_split_f64), joined to float64 in out (S, S). */
size_t aj_curvature_w_tilde_sparse_mixed_workspace_size(int64_t M, int64_t B, int64_t S);
int aj_curvature_w_tilde_sparse_mixed(const float* w_tilde_hi, const float* w_tilde_lo, int64_t M,
                                      const int64_t* pix_indexes, const double* pix_weights, int64_t B, int64_t S,
                                      double* out, void* workspace, size_t workspace_bytes, int* info, void* stream);

/* numba.py:500-549 _w_compact_matmul_sparse_mapping_matrix_from: out (M, S) = W T
 * with W gathered from the compact table (N, 2N-1) on the fly. */
int aj_w_compact_matmul_sparse(const double* w_compact, int64_t N, const int64_t* native_index, int64_t M,
                               const int64_t* pix_indexes, const double* pix_weights, int64_t B, int64_t S,
                               double* out, void* workspace, size_t workspace_bytes, int* info, void* stream);

/* numba.py:618-647 curvature_matrix_via_w_compact_sparse_mapping_matrix_from
 * (= numba.py:651-653 curvature_matrix_via_w_tilde_curvature_preload_interferometer_from,
 *  and the result of numba.py:439-496 ..._direct_from): out (S, S). */
int aj_curvature_w_compact_sparse(const double* w_compact, int64_t N, const int64_t* native_index, int64_t M,
                                  const int64_t* pix_indexes, const double* pix_weights, int64_t B, int64_t S,
                                  double* out, void* workspace, size_t workspace_bytes, int* info, void* stream);

/* original.py:600-700 curvature_matrix_via_w_tilde_curvature_preload_interferometer_from:
 * F from the (2Y, 2X) preload table with original.py's pix_size rows. */
size_t aj_curvature_preload_original_workspace_size(int64_t M, int64_t B, int64_t S);
int aj_curvature_preload_original(const double* preload, int64_t py, int64_t px, const int64_t* pix_indexes,
                                  const int64_t* pix_sizes, const double* pix_weights, int64_t B,
                                  const int64_t* native_index, int64_t M, int64_t S, double* out,
                                  void* workspace, size_t workspace_bytes, int* info, void* stream);

/* original.py:453-545 mapping_matrix_from (accumulating, sub-gridded form). */
int aj_mapping_matrix_original(const int64_t* pix_indexes, const int64_t* pix_sizes, const double* pix_weights,
                               int64_t n_sub, int64_t B, int64_t S, int64_t M, const int64_t* slim_index,
                               const double* sub_fraction, double* out, int* info, void* stream);

/* -------------------------------------------------- regularisation, solve */

/* numba.py:657-695 constant_regularization_matrix_from: out (S, S). */
int aj_constant_regularization(double coefficient, const int64_t* neighbors, const int64_t* neighbors_sizes,
                               int64_t S, int64_t P, double* out, int* info, void* stream);

/* numba.py:699-731 reconstruction_positive_negative_from: out (S,) = A^-1 D by
 * a blocked FP64 Cholesky (A symmetric positive definite; an indefinite A sets
 * AJ_INFO_NOT_POSITIVE_DEFINITE, and aj_lu_solve then solves it as the
 * reference's LU does). */
size_t aj_spd_solve_workspace_size(int64_t S);
int aj_spd_solve(const double* data_vector, const double* A, int64_t S, double* out, void* workspace,
                 size_t workspace_bytes, int* info, void* stream);

/* The solve of aj_spd_solve for callers that cannot allocate device memory
 * (a plugin or foreign-function host that only receives device pointers, or
 * code whose allocator belongs to someone else): no workspace argument, and no
 * cudaMalloc, cudaFree or allocating library call. No counterpart in the
 * reference. Scratch is one file-scope __device__ array sized for
 * S <= AJ_NOALLOC_SOLVE_MAX_S (about 8.3 MB); larger S returns
 * AJ_ERR_TOO_LARGE. The driver places the array when it loads the library's
 * device code into a context, which under lazy module loading (the CUDA
 * default) is this entry point's first call in each context: that first call
 * can fail for lack of device memory, so make it early and before any stream
 * capture. The array then stays until the context ends. `info` is required
 * (NULL returns AJ_ERR_ARG): a non-positive-definite A is reported only there.
 * All calls in a context share the array: calls whose GPU work overlaps race. */
#define AJ_NOALLOC_SOLVE_MAX_S 1024
int aj_spd_solve_noalloc(const double* data_vector, const double* A, int64_t S, double* out, int* info, void* stream);

/* numba.py:731 np.linalg.solve and numba.py:849-850 np.linalg.slogdet(...)[1] for
 * any non-singular A: blocked float64 LU with partial pivoting (the first row of
 * largest magnitude, as LAPACK getrf). out (S,) = A^-1 D and *logabsdet =
 * log|det A|, either may be NULL; an exactly zero pivot sets AJ_INFO_SINGULAR
 * (the reference raises LinAlgError there). */
size_t aj_lu_solve_workspace_size(int64_t S);
int aj_lu_solve(const double* data_vector, const double* A, int64_t S, double* out, double* logabsdet,
                void* workspace, size_t workspace_bytes, int* info, void* stream);

/* log|det A| of a symmetric positive definite A (the slogdet of numba.py:849-850). */
int aj_spd_logdet(const double* A, int64_t S, double* out, void* workspace, size_t workspace_bytes, int* info,
                  void* stream);

/* A^-1 (S, S, full symmetric) of a symmetric positive definite A via its
 * Cholesky factor: L^-1 by block forward substitution, then L^-T L^-1.
 * The adjoint of numba.py:849 (d log|A| = tr(A^-1 dA)) needs it; no counterpart. */
size_t aj_spd_inverse_workspace_size(int64_t S);
int aj_spd_inverse(const double* A, int64_t S, double* Ainv, double* logdet, void* workspace, size_t workspace_bytes,
                   int* info, void* stream);

/* The same as aj_spd_inverse in double-float arithmetic on the float32 pipe
 * (A and A^-1 stay float64 in memory; ~2^-47 relative rounding per operation). */
size_t aj_spd_inverse_mixed_workspace_size(int64_t S);
int aj_spd_inverse_mixed(const double* A, int64_t S, double* Ainv, double* logdet, void* workspace,
                         size_t workspace_bytes, int* info, void* stream);

/* numba.py:735-752 noise_normalization_complex_from: *out = 2 (K log 2pi + sum log|Re| + sum log|Im|). */
int aj_noise_normalization(const double* noise_map_c128, int64_t K, double* out, void* stream);

/* ------------------------------------------------------------ likelihood */

/* Split float64 values into double-float planes: hi = float(x), lo = float(x - hi). */
int aj_split_f64(const double* x, int64_t n, float* hi, float* lo, void* stream);

/* Dimensions and inputs of one log-evidence evaluation. The shared W (M, M)
 * is w_tilde64, and for AJ_MIXED also its double-float planes w_tilde_hi /
 * w_tilde_lo (split once with aj_split_f64, 16-byte aligned; without them the mixed
 * path splits w_tilde64 on every call); for the compact variant w_compact (N, 2N-1) and
 * native_index (M, 2) replace it. */
typedef struct aj_problem {
    int64_t M, K, S, B, P, N;
    const double* dirty_image;       /* (M,) */
    const double* data;              /* (K,) complex128 */
    const double* noise_map;         /* (K,) complex128 */
    const double* w_tilde64;         /* (M, M) or NULL */
    const float* w_tilde_hi;         /* (M, M) double-float planes of w_tilde for AJ_MIXED */
    const float* w_tilde_lo;         /* (hi + lo = w_tilde; see aj_split_f64), or NULL */
    const double* w_compact;         /* (N, 2N-1) or NULL */
    const int64_t* native_index;     /* (M, 2) or NULL */
    const int64_t* pix_indexes;      /* (M, B) */
    const double* pix_weights;       /* (M, B) */
    const int64_t* neighbors;        /* (S, P) */
    const int64_t* neighbors_sizes;  /* (S,) */
    double coefficient;              /* regularisation coefficient c, lambda = c^2 */
    const double* coefficient_dev;   /* optional device copy of c (read instead of `coefficient` when set,
                                        so a captured CUDA graph can be replayed with new values) */
} aj_problem;

/* Outputs (device): out[0] = logE; with gradients out[1] = dlogE/dlambda and
 * grad_weights (M, B) = dlogE/dpix_weights (zero where a weight does not
 * reach the mapping matrix). reconstruction (S,) may be NULL. */
size_t aj_log_evidence_workspace_size(const aj_problem* p, int precision, int with_grad);

/* numba.py:761-857 log_likelihood_function_via_w_tilde_from (w_tilde set) and
 * numba.py:866-967 log_likelihood_function_via_w_compact_from (w_compact set);
 * `coefficient` generalises the reference's hard-coded 1.0 (numba.py:819). */
int aj_log_evidence(const aj_problem* p, int precision, int with_grad, double* out, double* grad_weights,
                    double* reconstruction, void* workspace, size_t workspace_bytes, int* info, void* stream);

/* Mapping-weight builder (no reference counterpart: the reference takes
 * pix_indexes / pix_weights as likelihood inputs, numba.py:294-376, built by
 * PyAutoLens).  Coordinates are (y, x) pairs in one angular unit (arcsec).
 *
 * aj_sis_trace: beta = theta - theta_E theta / |theta|, an SIS at the origin;
 * theta_E is read from einstein_radius_dev when that is not NULL.
 * aj_sis_trace_vjp: dL/dtheta_E (one device double) from dL/dbeta (M, 2). */
int aj_sis_trace(const double* theta, int64_t M, double einstein_radius, const double* einstein_radius_dev,
                 double* beta, void* stream);
int aj_sis_trace_vjp(const double* theta, int64_t M, const double* grad_beta, double* grad_einstein_radius,
                     void* stream);

/* Barycentric weights of the traced points in the triangulation (simplices,
 * (T, 3) vertex indices into points (S, 2)): pix_indexes / pix_weights
 * (M, 3).  A point maps to the first (lowest-index) triangle containing it,
 * decided in float64 without contraction; outside the hull it maps to its
 * nearest vertex with weight 1 and the row is -1 padded.  A simplex entry out
 * of range sets AJ_INFO_INDEX_RANGE. */
int aj_delaunay_weights(const double* beta, int64_t M, const double* points, int64_t S, const int64_t* simplices,
                        int64_t T, int64_t* pix_indexes, double* pix_weights, int* info, void* stream);
/* dL/dpoints (S, 2) and dL/dbeta (M, 2) from dL/dpix_weights (M, 3); rows
 * outside the hull contribute nothing. */
int aj_delaunay_weights_vjp(const double* beta, int64_t M, const double* points, int64_t S,
                            const int64_t* pix_indexes, const double* grad_weights, double* grad_points,
                            double* grad_beta, void* stream);

/* Bilinear weights (M, 4) on the n x n rectangular mesh over [-hw, hw]^2,
 * rows growing downwards in y, and dL/dbeta from dL/dpix_weights. */
int aj_bilinear_weights(const double* beta, int64_t M, int64_t n, double half_width, int64_t* pix_indexes,
                        double* pix_weights, void* stream);
int aj_bilinear_weights_vjp(const double* beta, int64_t M, int64_t n, double half_width, const double* grad_weights,
                            double* grad_beta, void* stream);

/* Batched log-evidence: n independent lens-model evaluations in one call (no
 * reference counterpart; the reference evaluates one model per call of
 * numba.py:761-857).  problems[i] usually share dirty_image, data, noise_map
 * and w_tilde (or w_compact); S, mapping, neighbours and coefficient are per
 * evaluation.  out is (n, 2) and info (n, 2); grad_weights[i] (M, B),
 * reconstruction[i] (S_i,) (the array may be NULL) and workspaces[i], of at
 * least aj_log_evidence_workspace_size(&problems[i], ...) bytes, are per
 * evaluation.  The evaluations run as up to AJ_BATCH_BRANCHES concurrent
 * branches forked from `stream` and joined back into it; every problem is
 * validated before anything is enqueued. */
#define AJ_BATCH_BRANCHES 16
int aj_log_evidence_batched(const aj_problem* problems, int64_t n, int precision, int with_grad, double* out,
                            double* const* grad_weights, double* const* reconstruction, void* const* workspaces,
                            const size_t* workspace_bytes, int* info, void* stream);

/* Frees the side streams and events the library created for `stream` on the
 * current device (the factorisation lanes, and for batches the branch streams
 * with their lanes); they are otherwise kept until the process exits, one set
 * per caller stream. Call it when no work issued through `stream` is in
 * flight or being captured; a later call on the stream creates a fresh set.
 * No reference counterpart. */
int aj_release_stream(void* stream);

/* CUDA-graph capture of library calls (no reference counterpart: the
 * reference evaluates eagerly).  Everything enqueued on `stream` between
 * aj_graph_begin and aj_graph_end is recorded, including the work the library
 * forks onto its own prioritised side streams, and instantiated so that
 * replays keep those priorities.  `stream` must not be the legacy default
 * stream.  Make one uncaptured call of the same work on the same stream
 * first: the side streams are created then. */
int aj_graph_begin(void* stream);
int aj_graph_end(void* stream, void** graph_exec);
int aj_graph_launch(void* graph_exec, void* stream);
int aj_graph_destroy(void* graph_exec);

#ifdef __cplusplus
}
#endif

#endif /* AUTOJAX_GB300_H */
