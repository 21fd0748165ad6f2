// Double-float (float32 hi + lo) linear algebra for the mixed-precision path.
//
// GB300 issues ~62x more float32 than float64 operations per clock, so the
// S^3 work of the evaluation (two Cholesky factorisations, two triangular
// inverses) runs as double-float on the float32 pipe: ~11-15 float32
// operations per multiply-add with ~2^-47 relative rounding (float64 keeps
// 2^-53; the inversion's conditioning needs better than float32's 2^-24, see
// the mixed-precision notes in the design document).  A^-1 = L^-T L^-1 runs on
// the tensor cores as exact digit products (wtilde_tc.cu).
//
// Matrices are row-major S x S with separate hi and lo float planes.
// Blocked algorithms use NB = 32; the diagonal block of every step is
// factored (and inverted) redundantly by every block of the panel kernel, so
// one launch per step both factors the pivot block and solves the rows below.

#include <math.h>

#include "aj_internal.cuh"
#include "df32.cuh"

namespace aj {

constexpr int DNB = 32;

// Up to two independent matrices factored or inverted by the same launches
// (blockIdx.y picks one).  The evaluation factors A and H separately, H on
// lanes of its own beside A's (likelihood.cu), so each launch carries one.
struct DfMats {
    float* Lh[2];
    float* Ll[2];
    float* Ih[2];
    float* Il[2];
    float* dh[2];
    float* dl[2];
    float* fh[2];  // factored diagonal blocks (copied into L after the last panel)
    float* fl[2];
    double* piv[2];
    int ninv;  // matrices z < ninv also get L^-1: the panel writes its diagonal block
};

// element z of a kernel-parameter pair without indexing it dynamically (which
// would copy the parameter block to the stack)
template <typename T>
__device__ __forceinline__ T pick(T const (&a)[2], int z) {
    return z ? a[1] : a[0];
}

// tile t of the lower triangle, row-major: (bi, bj) with bj <= bi.  The float
// square root is exact enough for a first guess (t < 2^24); the loops fix it.
__device__ __forceinline__ void lower_tile_df(int64_t t, int64_t& bi, int64_t& bj) {
    int64_t r = static_cast<int64_t>((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    bi = r;
    bj = t - r * (r + 1) / 2;
}

// ----------------------------------------------------------------- planes

__global__ void split_kernel(const double* __restrict__ x, int64_t n, float* __restrict__ hi, float* __restrict__ lo) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const df v = df_from(x[t]);
        hi[t] = v.hi;
        lo[t] = v.lo;
    }
}

__global__ void join_kernel(const float* __restrict__ hi, const float* __restrict__ lo, int64_t n,
                            double* __restrict__ x) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        x[t] = (double)hi[t] + (double)lo[t];
}

// ------------------------------------------------------------------- GEMM

// C (m x n) = (neg ? -1 : 1) op(A) op(B) (+ C when accumulate), double-float planes.
// 64 x 64 tiles, 256 threads with 4 x 4 accumulators each; the k loop runs in
// 32-deep slabs staged through shared memory with the next slab prefetched
// into registers, products accumulate lazily (renormalised every 8 k).
constexpr int GBK = 32;

template <bool TA, bool TB>
__device__ __forceinline__ void gemm_df_load(const float* __restrict__ Ah, const float* __restrict__ Al, int64_t lda,
                                             const float* __restrict__ Bh, const float* __restrict__ Bl, int64_t ldb,
                                             int64_t m, int64_t n, int64_t k, int64_t i0, int64_t j0, int64_t k0,
                                             int tid, float (&ra)[16], float (&rb)[16]) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int e = tid + q * 256;  // 2048 = 64 x 32 elements per operand slab
        int ii, kk;
        if (TA) {
            kk = e >> 6;
            ii = e & 63;
        } else {
            ii = e >> 5;
            kk = e & 31;
        }
        const int64_t gi = i0 + ii, gk = k0 + kk;
        float vh = 0.f, vl = 0.f;
        if (gi < m && gk < k) {
            const int64_t off = TA ? gk * lda + gi : gi * lda + gk;
            vh = Ah[off];
            vl = Al[off];
        }
        ra[2 * q] = vh;
        ra[2 * q + 1] = vl;
        int jj, kb;
        if (TB) {
            jj = e >> 5;
            kb = e & 31;
        } else {
            kb = e >> 6;
            jj = e & 63;
        }
        const int64_t gj = j0 + jj, gk2 = k0 + kb;
        float wh = 0.f, wl = 0.f;
        if (gj < n && gk2 < k) {
            const int64_t off = TB ? gj * ldb + gk2 : gk2 * ldb + gj;
            wh = Bh[off];
            wl = Bl[off];
        }
        rb[2 * q] = wh;
        rb[2 * q + 1] = wl;
    }
}

template <bool TA, bool TB>
__device__ __forceinline__ void gemm_df_store(float (*sAh)[68], float (*sAl)[68], float (*sBh)[68], float (*sBl)[68],
                                              int tid, const float (&ra)[16], const float (&rb)[16]) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int e = tid + q * 256;
        int ii, kk, jj, kb;
        if (TA) {
            kk = e >> 6;
            ii = e & 63;
        } else {
            ii = e >> 5;
            kk = e & 31;
        }
        if (TB) {
            jj = e >> 5;
            kb = e & 31;
        } else {
            kb = e >> 6;
            jj = e & 63;
        }
        sAh[kk][ii] = ra[2 * q];
        sAl[kk][ii] = ra[2 * q + 1];
        sBh[kb][jj] = rb[2 * q];
        sBl[kb][jj] = rb[2 * q + 1];
    }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
    gemm_df_kernel(int64_t m, int64_t n, int64_t k, int neg, const float* __restrict__ Ah, const float* __restrict__ Al,
                   int64_t lda, const float* __restrict__ Bh, const float* __restrict__ Bl, int64_t ldb, int accumulate,
                   float* __restrict__ Ch, float* __restrict__ Cl, int64_t ldc, int lower_only, int tri_k,
                   int64_t tiles_n) {
    __shared__ float sAh[GBK][68], sAl[GBK][68], sBh[GBK][68], sBl[GBK][68];
    int64_t ti, tj;
    if (lower_only)
        lower_tile_df(blockIdx.x, ti, tj);
    else {
        ti = blockIdx.x / tiles_n;
        tj = blockIdx.x % tiles_n;
    }
    const int64_t i0 = ti * 64, j0 = tj * 64;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    df acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = {0.f, 0.f};
    const int64_t kbeg = tri_k ? (i0 > j0 ? i0 : j0) : 0;
    float ra[16], rb[16];
    if (kbeg < k) gemm_df_load<TA, TB>(Ah, Al, lda, Bh, Bl, ldb, m, n, k, i0, j0, kbeg, tid, ra, rb);
    for (int64_t k0 = kbeg; k0 < k; k0 += GBK) {
        gemm_df_store<TA, TB>(sAh, sAl, sBh, sBl, tid, ra, rb);
        __syncthreads();
        if (k0 + GBK < k) gemm_df_load<TA, TB>(Ah, Al, lda, Bh, Bl, ldb, m, n, k, i0, j0, k0 + GBK, tid, ra, rb);
#pragma unroll
        for (int k8 = 0; k8 < GBK; k8 += 8) {
#pragma unroll
            for (int kk = k8; kk < k8 + 8; ++kk) {
                df a[4], b[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) a[r] = {sAh[kk][ty * 4 + r], sAl[kk][ty * 4 + r]};
#pragma unroll
                for (int c = 0; c < 4; ++c) b[c] = {sBh[kk][tx * 4 + c], sBl[kk][tx * 4 + c]};
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c) df_fma_lazy(acc[r][c], a[r], b[c]);
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) df_renorm(acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int64_t gi = i0 + ty * 4 + r, gj = j0 + tx * 4 + c;
            if (gi < m && gj < n) {
                df v = neg ? df_neg(acc[r][c]) : acc[r][c];
                if (accumulate) v = df_add(v, {Ch[gi * ldc + gj], Cl[gi * ldc + gj]});
                Ch[gi * ldc + gj] = v.hi;
                Cl[gi * ldc + gj] = v.lo;
            }
        }
}

int gemm_df(bool ta, bool tb, int64_t m, int64_t n, int64_t k, bool neg, const float* Ah, const float* Al, int64_t lda,
            const float* Bh, const float* Bl, int64_t ldb, bool accumulate, float* Ch, float* Cl, int64_t ldc,
            bool lower_only, bool tri_k, cudaStream_t st) {
    if (m <= 0 || n <= 0) return AJ_OK;
    const int64_t tm = (m + 63) / 64, tn = (n + 63) / 64;
    const unsigned g = (unsigned)(lower_only ? tm * (tm + 1) / 2 : tm * tn);
#define AJ_DF_GEMM(a, b)                                                                                          \
    gemm_df_kernel<a, b><<<g, 256, 0, st>>>(m, n, k, neg ? 1 : 0, Ah, Al, lda, Bh, Bl, ldb, accumulate ? 1 : 0, Ch, \
                                            Cl, ldc, lower_only ? 1 : 0, tri_k ? 1 : 0, tn)
    if (!ta && !tb)
        AJ_DF_GEMM(false, false);
    else if (!ta && tb)
        AJ_DF_GEMM(false, true);
    else if (ta && !tb)
        AJ_DF_GEMM(true, false);
    else
        AJ_DF_GEMM(true, true);
#undef AJ_DF_GEMM
    return check_launch();
}

// -------------------------------------------------------------- Cholesky

// Factor the diagonal block at k0 (every block, redundantly) and, in block
// b >= 1, solve the 64 panel rows k0 + 32 + 64 (b - 1) .. for L's columns
// (rows <- A_rows L_kk^-T) in the same column loop.  Block 0 stores L_kk (in
// the factored-block buffer, not in L: blocks of the same launch may start
// late and must still read the unfactored block from L), the pivots and
// L_kk^-1, which it computes while the other blocks store their rows.
// Latency matters more than work here (one launch per 32 columns sits on the
// critical path), so the column loop takes one barrier a column and lets each
// finished column's warp drop out.
// With `pre` set the kernel first applies the previous step's update to its
// own block column (A_kk -= P_k P_k^T, rows -= P_r P_k^T with P the previous
// panel's rows), so the critical chain is one launch per step; the rest of
// each trailing update runs on another lane.
constexpr int PANEL_THREADS = 1024;
constexpr int PANEL_SP = 8;  // sub-panel width of the panel factorisation
static_assert(PANEL_THREADS >= 3 * 32 && PANEL_THREADS % 128 == 0 && DNB % PANEL_SP == 0,
              "a thread per solved row; whole warps on each sub-partition; whole sub-panels");
constexpr int PRE_DIGITS = 6;  // 8-bit digits per double-float value in the tensor-core pre-update
constexpr int PRE_LEVELS = 7;  // digit-product levels i + j kept
constexpr int PRE_KS = DNB + 8;  // bf16 row stride of the digit planes: conflict-free fragment loads
// Panel rows a block solves besides the pivot block.  A panel block holds a whole SM while most of
// its threads wait on the pivot chain: 128 rows (half the blocks) measured 2.604 against 2.462 ms
// an evaluation (the chain's steps grow) and 608 against 596 evaluations/s batched.
constexpr int PANEL_ROWS = 64;
constexpr int PANEL_NROW = DNB + PANEL_ROWS;  // a block's rows: the pivot block's, then its panel rows
static_assert(PANEL_NROW >= 3 * DNB, "block 0 keeps L_kk^-1 and a scratch block in the panel-row space");
// previous-panel rows as (hi, lo) pairs (the pivot block's 32 and this block's panel rows), then
// their digit planes
constexpr size_t PANEL_DYN_SMEM =
    sizeof(float2) * PANEL_NROW * (DNB + 1) + sizeof(uint16_t) * PRE_DIGITS * PANEL_NROW * PRE_KS;

// x 2^k for k <= 252, exact unless the result leaves the normal range (two power-of-two factors
// built from their exponent bits, each within the float range)
__device__ __forceinline__ float scale2(float x, int k) {
    if (k < -252) return x * 0.f;  // below the float range either way
    const int k1 = k / 2;
    return x * __int_as_float((k1 + 127) << 23) * __int_as_float((k - k1 + 127) << 23);
}

// d (16 x 8, float32) += a (16 x 16, bf16, row-major) b (16 x 8, bf16, column-major): one warp-wide
// mma.sync; a thread holds a = {A[g][2t..], A[g+8][2t..], A[g][2t+8..], A[g+8][2t+8..]},
// b = {B[2t..][g], B[2t+8..][g]} and d = {D[g][2t], D[g][2t+1], D[g+8][2t], D[g+8][2t+1]},
// g = lane / 4, t = lane % 4, pairs packed low element first
__device__ __forceinline__ void mma_bf16_16816(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(PANEL_THREADS)
    dfchol_panel_kernel(DfMats mats, int64_t S, int64_t k0, int pre, int* info) {
    const int z = blockIdx.y;
    float* __restrict__ Lh = pick(mats.Lh, z);
    float* __restrict__ Ll = pick(mats.Ll, z);
    const int64_t kb = k0 / DNB;
    float* __restrict__ dh = pick(mats.dh, z) + kb * DNB * DNB;
    float* __restrict__ dl = pick(mats.dl, z) + kb * DNB * DNB;
    float* __restrict__ fh = pick(mats.fh, z) + kb * DNB * DNB;
    float* __restrict__ fl = pick(mats.fl, z) + kb * DNB * DNB;
    double* __restrict__ piv = pick(mats.piv, z);
    // the block's rows: 0 .. 31 the pivot block (lower triangle), then PANEL_ROWS panel rows
    __shared__ float ph[PANEL_NROW][DNB + 1], pl[PANEL_NROW][DNB + 1];
    __shared__ float rh[DNB], rl[DNB];
    extern __shared__ float2 panel_dyn[];
    float2(*pdf)[DNB + 1] = reinterpret_cast<float2(*)[DNB + 1]>(panel_dyn);                    // P_k: 32 rows
    float2(*prf)[DNB + 1] = reinterpret_cast<float2(*)[DNB + 1]>(panel_dyn + DNB * (DNB + 1));  // P_r
    uint16_t* xd = reinterpret_cast<uint16_t*>(panel_dyn + PANEL_NROW * (DNB + 1));  // digits [i][row][k]
    __shared__ int pexp[PANEL_NROW];  // row scales 2^e of the pre-update
    __shared__ int bad;
    const int tid = threadIdx.x;
    const bool rows = blockIdx.x > 0;
    const int nrow = rows ? PANEL_NROW : DNB;
    const int64_t nb = (S - k0) < DNB ? (S - k0) : DNB;
    const int64_t kp = k0 - DNB;  // the previous panel's first column (pre only)
    if (tid == 0) bad = 0;
    for (int e = tid; e < DNB * DNB; e += PANEL_THREADS) {
        const int i = e / DNB, j = e % DNB;
        float vh, vl;
        if (i < nb && j < nb) {
            const int64_t off = (k0 + i) * S + k0 + j;
            vh = j <= i ? Lh[off] : 0.f;
            vl = j <= i ? Ll[off] : 0.f;
        } else {
            vh = i == j ? 1.f : 0.f;
            vl = 0.f;
        }
        ph[i][j] = vh;
        pl[i][j] = vl;
        if (pre) {
            const bool pin = i < nb;
            pdf[i][j] = pin ? make_float2(Lh[(k0 + i) * S + kp + j], Ll[(k0 + i) * S + kp + j]) : make_float2(0.f, 0.f);
        }
    }
    // panel rows are loaded up front so their latency overlaps the factorisation
    const int64_t r0 = k0 + DNB + (int64_t)(blockIdx.x - 1) * PANEL_ROWS;
    if (rows) {
        for (int e = tid; e < PANEL_ROWS * DNB; e += PANEL_THREADS) {
            const int i = e / DNB, j = e % DNB;
            const int64_t r = r0 + i;
            const bool in = r < S && j < nb;
            ph[DNB + i][j] = in ? Lh[r * S + k0 + j] : 0.f;
            pl[DNB + i][j] = in ? Ll[r * S + k0 + j] : 0.f;
            if (pre) prf[i][j] = r < S ? make_float2(Lh[r * S + kp + j], Ll[r * S + kp + j]) : make_float2(0.f, 0.f);
        }
    }
    __syncthreads();
    if (pre) {
        // A_kk (lower) -= P_k P_k^T and rows -= P_r P_k^T, i.e. C = X Y^T with X = [P_k; P_r] (the
        // previous panel's columns in this block's rows) and Y = P_k, on the tensor cores.  Each
        // row of X is scaled by a power of two, |x| < 2^e, and cut into six signed 8-bit digits
        // (x = 2^(e - 7) sum_i d_i 2^(-8 i), |d_i| <= 128, exact in bf16); the digit products of
        // level L = i + j sum exactly in float32 (at most 6 x 32 x 2^14 < 2^24) and levels 0 .. 6
        // fold back into double-float.  What is dropped is below 2^-43 of 2^(e_r + e_c), the
        // rounding of a 32-term double-float dot product.
        const int w = tid >> 5, lane = tid & 31;
        for (int r = w; r < nrow; r += PANEL_THREADS / 32) {
            const float2 v = r < DNB ? pdf[r][lane] : prf[r - DNB][lane];
            float m = fabsf(v.x);
#pragma unroll
            for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            // e with m < 2^e from m's exponent bits (a subnormal or zero m takes the smallest)
            const int be = (int)((__float_as_uint(m) >> 23) & 0xffu);
            const int e = m > 0.f ? (be > 0 ? be - 126 : -126) : 0;
            if (lane == 0) pexp[r] = e;
            df t = {scale2(v.x, 7 - e), scale2(v.y, 7 - e)};
#pragma unroll
            for (int i = 0; i < PRE_DIGITS; ++i) {
                const float d = rintf(t.hi);  // an integer of at most 8 bits: its bf16 is the top half
                xd[(i * PANEL_NROW + r) * PRE_KS + lane] = (uint16_t)(__float_as_uint(d) >> 16);
                float hs, he;
                two_sum(t.hi - d, t.lo, hs, he);
                t = {hs * 256.f, he * 256.f};
            }
        }
        __syncthreads();
        // 16 x 8 output tiles spread over the warps: rows R0 .., columns C0 ..
        for (int tile = w; tile < (nrow / 16) * (DNB / 8); tile += PANEL_THREADS / 32) {
            const int R0 = (tile / (DNB / 8)) * 16, C0 = (tile % (DNB / 8)) * 8;
            const int g = lane >> 2, tq = lane & 3;
            float acc[PRE_LEVELS][4];
#pragma unroll
            for (int L = 0; L < PRE_LEVELS; ++L)
#pragma unroll
                for (int o = 0; o < 4; ++o) acc[L][o] = 0.f;
#pragma unroll
            for (int i = 0; i < PRE_DIGITS; ++i)
#pragma unroll
                for (int j = 0; j < PRE_DIGITS; ++j) {
                    if (i + j >= PRE_LEVELS) continue;
                    const uint16_t* A = xd + i * PANEL_NROW * PRE_KS;
                    const uint16_t* Bm = xd + j * PANEL_NROW * PRE_KS;
#pragma unroll
                    for (int ks = 0; ks < DNB; ks += 16) {
                        uint32_t a[4], b[2];
                        a[0] = *reinterpret_cast<const uint32_t*>(A + (R0 + g) * PRE_KS + ks + 2 * tq);
                        a[1] = *reinterpret_cast<const uint32_t*>(A + (R0 + g + 8) * PRE_KS + ks + 2 * tq);
                        a[2] = *reinterpret_cast<const uint32_t*>(A + (R0 + g) * PRE_KS + ks + 2 * tq + 8);
                        a[3] = *reinterpret_cast<const uint32_t*>(A + (R0 + g + 8) * PRE_KS + ks + 2 * tq + 8);
                        b[0] = *reinterpret_cast<const uint32_t*>(Bm + (C0 + g) * PRE_KS + ks + 2 * tq);
                        b[1] = *reinterpret_cast<const uint32_t*>(Bm + (C0 + g) * PRE_KS + ks + 2 * tq + 8);
                        mma_bf16_16816(acc[i + j], a, b);
                    }
                }
            // accumulator o holds (R0 + g (+ 8 for o >= 2), C0 + 2 tq + (o & 1))
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const int r = R0 + g + (o >= 2 ? 8 : 0), c = C0 + 2 * tq + (o & 1);
                // levels 3 .. 6 are below 2^-24 of level 0, so their float sum rounds at the
                // 2^-48 level; levels 0 .. 2 and that tail add as double-float
                float tail = 0.f;
#pragma unroll
                for (int L = PRE_LEVELS - 1; L >= 3; --L) tail += acc[L][o] * __int_as_float((127 - 8 * L) << 23);
                df sum = {tail, 0.f};
#pragma unroll
                for (int L = 2; L >= 0; --L) sum = df_add(sum, {acc[L][o] * __int_as_float((127 - 8 * L) << 23), 0.f});
                const int sc = pexp[r] + pexp[c] - 14;
                sum = {scale2(sum.hi, sc), scale2(sum.lo, sc)};
                if (r >= DNB || (c <= r && r < nb && c < nb)) {
                    const df v = df_add({ph[r][c], pl[r][c]}, df_neg(sum));
                    ph[r][c] = v.hi;
                    pl[r][c] = v.lo;
                }
            }
        }
    }
    // Factor the pivot block and solve the panel rows for L's columns, 8 columns (a sub-panel)
    // at a time, in three phases a sub-panel:
    //  A. Warp 0 factors the sub-panel's 8 x 8 diagonal block in lanes 0 .. 7 (one row a lane).
    //     Meanwhile the warps on the other three SM sub-partitions (warp w runs on sub-partition
    //     w mod 4) apply the previous sub-panel to the columns past this one.  The pivot chain is
    //     latency-bound: alone on its sub-partition it takes ~290 cycles a pivot, beside seven
    //     busy warps ~1,800, so the warps that share warp 0's sub-partition sit this phase out.
    //  B. One thread a row solves the rows below the diagonal block (the pivot block's and the
    //     panel's) against it.
    //  C. All warps apply the sub-panel to the next sub-panel's columns.
    // Every value is computed by the same operations in the same order as a single chain that
    // carries all rows through the pivots together, so the factor does not depend on this split.
    const int w = tid >> 5, lane = tid & 31;
    // a[x][c] -= sum_t l[x][p0 + t] l[c][p0 + t] over the block's rows x (the pivot block's only
    // on and below the diagonal) and the columns c0 <= c < c1; work items t0, t0 + nt, ...
    auto rank_update = [&](int p0, int c0, int c1, int t0, int nt) {
        const int nc = c1 - c0;
        for (int e = t0; e < nrow * nc; e += nt) {
            const int x = e / nc, c = c0 + e % nc;
            if (x < DNB && x < c) continue;
            df acc = {0.f, 0.f};
#pragma unroll
            for (int t = 0; t < PANEL_SP; ++t)
                df_fma_lazy(acc, {ph[x][p0 + t], pl[x][p0 + t]}, {ph[c][p0 + t], pl[c][p0 + t]});
            const df v = df_add({ph[x][c], pl[x][c]}, df_neg(df_norm(acc)));
            ph[x][c] = v.hi;
            pl[x][c] = v.lo;
        }
    };
    constexpr int kSideWarps = (PANEL_THREADS / 32) * 3 / 4;  // warps off sub-partition 0
    __syncthreads();  // the pre-update's writes
    for (int J = 0; J < DNB / PANEL_SP; ++J) {
        const int j0 = J * PANEL_SP;
        if (w == 0) {
            df dv[PANEL_SP];
#pragma unroll
            for (int t = 0; t < PANEL_SP; ++t)
                dv[t] = lane < PANEL_SP ? df{ph[j0 + lane][j0 + t], pl[j0 + lane][j0 + t]} : df{0.f, 0.f};
            // No branch inside the pivot loop, so the compiler schedules it as one block (the
            // next pivot's column ahead of this pivot's later ones).  A failed pivot (the same in
            // every lane) is acted on after the loop; the NaNs it leaves are never stored.  Lane t
            // keeps pivot t's r = 1 / L_tt for the stores after the loop.
            int fail = PANEL_SP;
            df my_r = {0.f, 0.f};
#pragma unroll
            for (int t = 0; t < PANEL_SP; ++t) {
                const df d = {__shfl_sync(0xffffffffu, dv[t].hi, t), __shfl_sync(0xffffffffu, dv[t].lo, t)};
                fail = (fail == PANEL_SP && !(d.hi > 0.f)) ? t : fail;
                const df r = dfrsqrt(d);
                dv[t] = lane == t ? dfmul(d, r) : dfmul(dv[t], r);
                my_r = lane == t ? r : my_r;
#pragma unroll
                for (int u = t + 1; u < PANEL_SP; ++u) {
                    const df lu = {__shfl_sync(0xffffffffu, dv[t].hi, u), __shfl_sync(0xffffffffu, dv[t].lo, u)};
                    df_fms_acc(dv[u], dv[t], lu);
                }
            }
            if (fail < PANEL_SP) {
                if (lane == 0) {
                    bad = 1;
                    if (blockIdx.x == 0) report(info, AJ_INFO_NOT_POSITIVE_DEFINITE, k0 + j0 + fail);
                }
            } else if (lane < PANEL_SP) {
                df l_tt = dv[0];
#pragma unroll
                for (int t = 1; t < PANEL_SP; ++t) l_tt = lane == t ? dv[t] : l_tt;
                rh[j0 + lane] = my_r.hi;
                rl[j0 + lane] = my_r.lo;
                if (blockIdx.x == 0 && j0 + lane < nb) piv[k0 + j0 + lane] = df_to(l_tt);
#pragma unroll
                for (int t = 0; t < PANEL_SP; ++t) {
                    ph[j0 + lane][j0 + t] = dv[t].hi;
                    pl[j0 + lane][j0 + t] = dv[t].lo;
                }
            }
        } else if ((w & 3) != 0 && J > 0) {
            rank_update(j0 - PANEL_SP, j0 + PANEL_SP, DNB, (w - (w >> 2) - 1) * 32 + lane, kSideWarps * 32);
        }
        __syncthreads();
        if (bad) return;
        {
            // rows j0 + 8 .. 31 of the pivot block, then the panel rows
            const int npiv = DNB - j0 - PANEL_SP;
            if (tid < npiv + (rows ? PANEL_ROWS : 0)) {
                const int x = tid < npiv ? j0 + PANEL_SP + tid : DNB + (tid - npiv);
                df y[PANEL_SP];
#pragma unroll
                for (int t = 0; t < PANEL_SP; ++t) y[t] = {ph[x][j0 + t], pl[x][j0 + t]};
#pragma unroll
                for (int t = 0; t < PANEL_SP; ++t) {
                    y[t] = dfmul(y[t], {rh[j0 + t], rl[j0 + t]});
#pragma unroll
                    for (int u = t + 1; u < PANEL_SP; ++u)
                        df_fms_acc(y[u], y[t], {ph[j0 + u][j0 + t], pl[j0 + u][j0 + t]});
                }
#pragma unroll
                for (int t = 0; t < PANEL_SP; ++t) {
                    ph[x][j0 + t] = y[t].hi;
                    pl[x][j0 + t] = y[t].lo;
                }
            }
        }
        __syncthreads();
        if (J + 1 < DNB / PANEL_SP) {
            rank_update(j0, j0 + PANEL_SP, j0 + 2 * PANEL_SP, tid, PANEL_THREADS);
            __syncthreads();
        }
    }
    if (blockIdx.x == 0) {
        // L_kk^-1 by recursive doubling while the other blocks store their rows: at level b the
        // 32 / (2b) pairs of b x b diagonal blocks (A above C, B the block of L between them) get
        // their off-diagonal block -C^-1 (B A^-1), through T = B A^-1
        float(*ih)[DNB + 1] = ph + DNB;  // the block has no panel rows: their space holds L_kk^-1
        float(*il)[DNB + 1] = pl + DNB;
        float* th = &ph[2 * DNB][0];
        float* tl = &pl[2 * DNB][0];
        for (int e = tid; e < DNB * DNB; e += PANEL_THREADS) {
            const int i = e / DNB, j = e % DNB;
            ih[i][j] = i == j ? rh[i] : 0.f;
            il[i][j] = i == j ? rl[i] : 0.f;
        }
        __syncthreads();
        for (int b = 1; b < DNB; b <<= 1) {
            const int n = (DNB / 2) * b;  // outputs of this level: pairs x b^2
            const int pair = tid / (b * b), rem = tid % (b * b), r = rem / b, c = rem % b;
            const int i0 = 2 * b * pair;
            if (tid < n) {
                df acc = {0.f, 0.f};
                for (int q = c; q < b; ++q)
                    df_fma_acc(acc, {ph[i0 + b + r][i0 + q], pl[i0 + b + r][i0 + q]},
                               {ih[i0 + q][i0 + c], il[i0 + q][i0 + c]});
                th[tid] = acc.hi;
                tl[tid] = acc.lo;
            }
            __syncthreads();
            if (tid < n) {
                df acc = {0.f, 0.f};
                for (int q = 0; q <= r; ++q)
                    df_fma_acc(acc, {ih[i0 + b + r][i0 + b + q], il[i0 + b + r][i0 + b + q]},
                               {th[pair * b * b + q * b + c], tl[pair * b * b + q * b + c]});
                ih[i0 + b + r][i0 + c] = -acc.hi;
                il[i0 + b + r][i0 + c] = -acc.lo;
            }
            __syncthreads();
        }
        float* __restrict__ Ih = z < mats.ninv ? pick(mats.Ih, z) : nullptr;
        float* __restrict__ Il = z < mats.ninv ? pick(mats.Il, z) : nullptr;
        for (int e = tid; e < DNB * DNB; e += PANEL_THREADS) {
            const int i = e / DNB, j = e % DNB;
            if (Ih && i < nb && j < nb) {
                const int64_t off = (k0 + i) * S + k0 + j;
                Ih[off] = ih[i][j];
                Il[off] = il[i][j];
            }
            fh[e] = j <= i ? ph[i][j] : 0.f;
            fl[e] = j <= i ? pl[i][j] : 0.f;
            dh[e] = ih[i][j];
            dl[e] = il[i][j];
        }
        return;
    }
    for (int e = tid; e < PANEL_ROWS * DNB; e += PANEL_THREADS) {
        const int i = e / DNB, j = e % DNB;
        const int64_t r = r0 + i;
        if (r < S && j < nb) {
            Lh[r * S + k0 + j] = ph[DNB + i][j];
            Ll[r * S + k0 + j] = pl[DNB + i][j];
        }
    }
}

// Trailing update of one Cholesky step past the next block column (which the
// next panel kernel updates itself): C (lower 32 x 32 tiles of the trailing
// matrix, tile columns >= 1) -= P P^T with P the solved panel.  128 threads,
// 8 outputs each, operands as (hi, lo) pairs (6 shared loads per 8
// multiply-adds); small register and shared footprint so several blocks share
// an SM and the late, small steps still fill the GPU.
__global__ void __launch_bounds__(128)
    dfsyrk_update_kernel(DfMats mats, int64_t S, int64_t k0) {
    float* __restrict__ Lh = pick(mats.Lh, blockIdx.y);
    float* __restrict__ Ll = pick(mats.Ll, blockIdx.y);
    __shared__ float2 pi[32][33], pj[32][33];  // (hi, lo) of the panel rows of tile rows i and j
    const int64_t r0 = k0 + DNB;
    int64_t ti, tj;
    lower_tile_df(blockIdx.x, ti, tj);
    ++ti;
    ++tj;
    const int64_t i0 = r0 + ti * 32, j0 = r0 + tj * 32;
    const int tid = threadIdx.x;
    const int ty = tid >> 3, tx = tid & 7;  // rows ty, ty+16; columns tx, tx+8, tx+16, tx+24
    // the outputs' current values are fetched first so their latency overlaps the tile loads
    df cur[2][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int64_t gi = i0 + ty + 16 * a, gj = j0 + tx + 8 * b;
            const bool in = gi < S && gj < S && gj <= gi;
            cur[a][b] = in ? df{Lh[gi * S + gj], Ll[gi * S + gj]} : df{0.f, 0.f};
        }
    for (int e = tid; e < 32 * 32; e += 128) {
        const int a = e >> 5, b = e & 31;
        const bool ii = i0 + a < S, jj = j0 + a < S;
        pi[a][b] = ii ? make_float2(Lh[(i0 + a) * S + k0 + b], Ll[(i0 + a) * S + k0 + b]) : make_float2(0.f, 0.f);
        pj[a][b] = jj ? make_float2(Lh[(j0 + a) * S + k0 + b], Ll[(j0 + a) * S + k0 + b]) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    df acc[2][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = {0.f, 0.f};
#pragma unroll
    for (int k8 = 0; k8 < 32; k8 += 8) {
#pragma unroll
        for (int k = k8; k < k8 + 8; ++k) {
            const float2 x0 = pi[ty][k], x1 = pi[ty + 16][k];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const float2 y = pj[tx + 8 * b][k];
                df_fma_lazy(acc[0][b], {x0.x, x0.y}, {y.x, y.y});
                df_fma_lazy(acc[1][b], {x1.x, x1.y}, {y.x, y.y});
            }
        }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) df_renorm(acc[a][b]);
    }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int64_t gi = i0 + ty + 16 * a, gj = j0 + tx + 8 * b;
            if (gi < S && gj < S && gj <= gi) {
                const df v = df_add(cur[a][b], df_neg(acc[a][b]));
                Lh[gi * S + gj] = v.hi;
                Ll[gi * S + gj] = v.lo;
            }
        }
}

// L's diagonal blocks from the factored-block buffer; grid (blocks, matrices)
__global__ void df_store_diag_kernel(DfMats mats, int64_t S) {
    float* __restrict__ Lh = pick(mats.Lh, blockIdx.y);
    float* __restrict__ Ll = pick(mats.Ll, blockIdx.y);
    const float* __restrict__ fh = pick(mats.fh, blockIdx.y);
    const float* __restrict__ fl = pick(mats.fl, blockIdx.y);
    const int64_t kb = blockIdx.x, k0 = kb * DNB;
    for (int e = threadIdx.x; e < DNB * DNB; e += blockDim.x) {
        const int i = e / DNB, j = e % DNB;
        if (k0 + i < S && k0 + j < S) {
            Lh[(k0 + i) * S + k0 + j] = fh[kb * DNB * DNB + e];
            Ll[(k0 + i) * S + k0 + j] = fl[kb * DNB * DNB + e];
        }
    }
}

__global__ void df_zero_upper_kernel(float* __restrict__ h, float* __restrict__ l, int64_t S) {
    for (int64_t i = blockIdx.y; i < S; i += gridDim.y)
        for (int64_t j = i + 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < S;
             j += (int64_t)gridDim.x * blockDim.x) {
            h[i * S + j] = 0.f;
            l[i * S + j] = 0.f;
        }
}

// log|A_z| = 2 sum_i log(pivot_i) for matrix z = blockIdx.x (out_z null: skipped)
__global__ void df_logdet_kernel(const double* __restrict__ piv0, const double* __restrict__ piv1, int64_t S,
                                 double* __restrict__ out0, double* __restrict__ out1, const int* info) {
    __shared__ double red[32];
    const double* piv = blockIdx.x == 0 ? piv0 : piv1;
    double* out = blockIdx.x == 0 ? out0 : out1;
    if (!out) return;
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < S; i += blockDim.x) acc += log(piv[i]);
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) *out = (info && info[0] == AJ_INFO_NOT_POSITIVE_DEFINITE) ? NAN : 2.0 * acc;
}

// ---------------------------------------------------- triangular inverse

// see trtri_step_kernel (linalg.cu): accumulate L[ti][kb] X[kb][tj]; block row kb + 1 applies -dinv.
// 256 threads, 4 outputs each (row r, columns q + 8t): the L^-1 steps trail the factorisation one
// a panel, so a step's latency counts as much as its throughput (128 threads with 8 outputs each
// measured 2.605 against 2.532 ms an evaluation).  Operands as (hi, lo) pairs in shared memory.
// Each output adds over k in the order and with the renormalisation points of df_trtri64_kernel,
// so the two give the same bits.  Block row kb + 1 then multiplies by the diagonal block's inverse
// (lower triangular: the terms past the diagonal are exact zeros), unrolled, one lazy chain per
// output.
__global__ void __launch_bounds__(256)
    df_trtri_step_kernel(DfMats mats, int64_t S, int64_t kb) {
    const float* __restrict__ Lh = pick(mats.Lh, blockIdx.y);
    const float* __restrict__ Ll = pick(mats.Ll, blockIdx.y);
    float* __restrict__ Ih = pick(mats.Ih, blockIdx.y);
    float* __restrict__ Il = pick(mats.Il, blockIdx.y);
    const float* __restrict__ dh = pick(mats.dh, blockIdx.y);
    const float* __restrict__ dl = pick(mats.dl, blockIdx.y);
    __shared__ float2 as[32][33], bs[32][33];  // as[r][k] = L[i0 + r][p0 + k], bs[k][c] = X[p0 + k][j0 + c]
    const int64_t nbt = (S + DNB - 1) / DNB;
    const int64_t ncol = kb + 1;
    const int64_t ti = kb + 1 + blockIdx.x / ncol, tj = blockIdx.x % ncol;
    if (ti >= nbt) return;
    const int tid = threadIdx.x;
    const int64_t i0 = ti * DNB, j0 = tj * DNB, p0 = kb * DNB;
    const int r = tid >> 3, q = tid & 7;
    df acc[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int64_t gi = i0 + r, gj = j0 + q + 8 * t;
        const bool in = gi < S && gj < S;
        acc[t] = in ? df{Ih[gi * S + gj], Il[gi * S + gj]} : df{0.f, 0.f};
    }
    for (int e = tid; e < DNB * DNB; e += 256) {
        const int rr = e / DNB, c = e % DNB;
        const bool ina = i0 + rr < S && p0 + c < S, inb = p0 + rr < S && j0 + c < S;
        as[rr][c] = ina ? make_float2(Lh[(i0 + rr) * S + p0 + c], Ll[(i0 + rr) * S + p0 + c]) : make_float2(0.f, 0.f);
        bs[rr][c] = inb ? make_float2(Ih[(p0 + rr) * S + j0 + c], Il[(p0 + rr) * S + j0 + c]) : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int k8 = 0; k8 < DNB; k8 += 8) {
#pragma unroll
        for (int k = k8; k < k8 + 8; ++k) {
            const float2 x = as[r][k];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const float2 y = bs[k][q + 8 * t];
                df_fma_lazy(acc[t], {x.x, x.y}, {y.x, y.y});
            }
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) df_renorm(acc[t]);
    }
    if (ti != kb + 1) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int64_t gi = i0 + r, gj = j0 + q + 8 * t;
            if (gi < S && gj < S) {
                Ih[gi * S + gj] = acc[t].hi;
                Il[gi * S + gj] = acc[t].lo;
            }
        }
        return;
    }
    // X[kb + 1 block][tj] = -dinv_{kb+1} acc: acc to shared memory (as), dinv into bs
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 4; ++t) as[r][q + 8 * t] = make_float2(acc[t].hi, acc[t].lo);
    for (int e = tid; e < DNB * DNB; e += 256)
        bs[e / DNB][e % DNB] = make_float2(dh[(kb + 1) * DNB * DNB + e], dl[(kb + 1) * DNB * DNB + e]);
    __syncthreads();
    df out[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
    for (int p8 = 0; p8 < DNB; p8 += 8) {
#pragma unroll
        for (int p = p8; p < p8 + 8; ++p) {
            const float2 d = bs[r][p];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const float2 y = as[p][q + 8 * t];
                df_fma_lazy(out[t], {d.x, d.y}, {y.x, y.y});
            }
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) df_renorm(out[t]);
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int64_t gi = i0 + r, gj = j0 + q + 8 * t;
        if (gi < S && gj < S) {
            Ih[gi * S + gj] = -out[t].hi;
            Il[gi * S + gj] = -out[t].lo;
        }
    }
}

// ------------------------------------------------- 64 x 64 tile updates
//
// The large steps of the trailing update and of L^-1 use 64 x 64 output
// tiles: 256 threads with 4 x 4 outputs each (rows ty + 16a,
// columns tx + 16b) read k-major (hi, lo) pairs from shared memory, half a
// shared load per double-float multiply-add against ~1.5 for the 32 x 32
// kernels.  The order over k, the operand order and the renormalisation
// points are those of the 32 x 32 kernels, so a step gives the same bits
// whichever tile size runs it.
constexpr int T64 = 64;

struct Tile64 {
    float2 a[DNB][T64 + 1];  // a[k][row of the output tile]
    float2 b[DNB][T64 + 1];  // b[k][column of the output tile]
};

// acc[a][b] += sum_k A[k][ty + 16a] B[k][tx + 16b], lazy, renormalised every 8 k
__device__ __forceinline__ void tile64_mac(const Tile64& t, df acc[4][4], int ty, int tx) {
#pragma unroll
    for (int k8 = 0; k8 < DNB; k8 += 8) {
#pragma unroll 2
        for (int k = k8; k < k8 + 8; ++k) {
            float2 av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = t.a[k][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = t.b[k][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) df_fma_lazy(acc[i][j], {av[i].x, av[i].y}, {bv[j].x, bv[j].y});
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) df_renorm(acc[i][j]);
    }
}

// t.a[k][r] = M[(r0 + r) * S + c0 + k] for r < 64, k < 32 (rows r0.. of a 32-column block; zero outside S)
__device__ __forceinline__ void load_rows_kmajor(float2 (*dst)[T64 + 1], const float* __restrict__ h,
                                                 const float* __restrict__ l, int64_t S, int64_t r0, int64_t c0) {
    for (int e = threadIdx.x; e < T64 * DNB; e += blockDim.x) {
        const int r = e / DNB, k = e % DNB;
        const bool in = r0 + r < S && c0 + k < S;
        const int64_t off = (r0 + r) * S + c0 + k;
        dst[k][r] = in ? make_float2(h[off], l[off]) : make_float2(0.f, 0.f);
    }
}

// t.b[k][c] = M[(r0 + k) * S + c0 + c] for k < 32, c < 64 (32 rows, 64 columns; zero outside S)
__device__ __forceinline__ void load_cols(float2 (*dst)[T64 + 1], const float* __restrict__ h,
                                          const float* __restrict__ l, int64_t S, int64_t r0, int64_t c0) {
    for (int e = threadIdx.x; e < T64 * DNB; e += blockDim.x) {
        const int k = e / T64, c = e % T64;
        const bool in = r0 + k < S && c0 + c < S;
        const int64_t off = (r0 + k) * S + c0 + c;
        dst[k][c] = in ? make_float2(h[off], l[off]) : make_float2(0.f, 0.f);
    }
}

// Trailing update of step k0 past the next block column, 64 x 64 tiles from c1 = k0 + 64:
// C -= P_i P_j^T (lower tiles; a diagonal tile writes its lower half)
__global__ void __launch_bounds__(256)
    dfsyrk_update64_kernel(DfMats mats, int64_t S, int64_t k0) {
    float* __restrict__ Lh = pick(mats.Lh, blockIdx.y);
    float* __restrict__ Ll = pick(mats.Ll, blockIdx.y);
    __shared__ Tile64 t;
    int64_t ti, tj;
    lower_tile_df(blockIdx.x, ti, tj);
    const int64_t c1 = k0 + 2 * DNB;
    const int64_t i0 = c1 + ti * T64, j0 = c1 + tj * T64;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    df cur[4][4], acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t gi = i0 + ty + 16 * i, gj = j0 + tx + 16 * j;
            const bool in = gi < S && gj < S && gj <= gi;
            cur[i][j] = in ? df{Lh[gi * S + gj], Ll[gi * S + gj]} : df{0.f, 0.f};
            acc[i][j] = {0.f, 0.f};
        }
    load_rows_kmajor(t.a, Lh, Ll, S, i0, k0);
    load_rows_kmajor(t.b, Lh, Ll, S, j0, k0);
    __syncthreads();
    tile64_mac(t, acc, ty, tx);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t gi = i0 + ty + 16 * i, gj = j0 + tx + 16 * j;
            if (gi < S && gj < S && gj <= gi) {
                const df v = df_add(cur[i][j], df_neg(acc[i][j]));
                Lh[gi * S + gj] = v.hi;
                Ll[gi * S + gj] = v.lo;
            }
        }
}

// L^-1 step kb for the rows past the next block row: X[i][j] += L[i][kb-block] X[kb-block][j]
// over rows i >= (kb + 2) 32 and columns j < (kb + 1) 32, in 64 x 64 tiles (the next block row,
// which also applies the diagonal inverse, stays with df_trtri_step_kernel)
__global__ void __launch_bounds__(256)
    df_trtri64_kernel(DfMats mats, int64_t S, int64_t kb) {
    const float* __restrict__ Lh = pick(mats.Lh, blockIdx.y);
    const float* __restrict__ Ll = pick(mats.Ll, blockIdx.y);
    float* __restrict__ Ih = pick(mats.Ih, blockIdx.y);
    float* __restrict__ Il = pick(mats.Il, blockIdx.y);
    __shared__ Tile64 t;
    const int64_t ncol = (kb + 1) * DNB;  // columns of X that are nonzero in block row kb
    const int64_t nJ = (ncol + T64 - 1) / T64;
    const int64_t I = blockIdx.x / nJ, J = blockIdx.x % nJ;
    const int64_t i0 = (kb + 2) * DNB + I * T64, j0 = J * T64, p0 = kb * DNB;
    if (i0 >= S) return;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    df acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t gi = i0 + ty + 16 * i, gj = j0 + tx + 16 * j;
            const bool in = gi < S && gj < ncol;
            acc[i][j] = in ? df{Ih[gi * S + gj], Il[gi * S + gj]} : df{0.f, 0.f};
        }
    load_rows_kmajor(t.a, Lh, Ll, S, i0, p0);
    load_cols(t.b, Ih, Il, S, p0, j0);
    __syncthreads();
    tile64_mac(t, acc, ty, tx);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t gi = i0 + ty + 16 * i, gj = j0 + tx + 16 * j;
            if (gi < S && gj < ncol) {
                Ih[gi * S + gj] = acc[i][j].hi;
                Il[gi * S + gj] = acc[i][j].lo;
            }
        }
}

// ------------------------------------------------- L^-1 in float32
//
// The same two L^-1 steps in plain float32, from L's hi plane, into X's hi plane (its lo plane is
// left as it is).  For a matrix whose L^-1 serves only a trace that enters its result scaled down:
// the regularisation matrix's tr(H^-1) enters dlogE/dlambda as 1e-8 tr(H^-1) / lambda against
// S / lambda, and H is deflated (condition ~1e3), so float32's ~1e-6 on the trace moves dlogE/dlambda
// by ~1e-12 relative at the K=1e6 configuration, for 1 float32 instruction a multiply-add instead of
// 11.

__global__ void __launch_bounds__(256)
    f32_trtri_step_kernel(DfMats mats, int64_t S, int64_t kb) {
    const float* __restrict__ Lh = pick(mats.Lh, blockIdx.y);
    float* __restrict__ Ih = pick(mats.Ih, blockIdx.y);
    const float* __restrict__ dh = pick(mats.dh, blockIdx.y);
    __shared__ float as[32][33], bs[32][33];  // as[r][k] = L[i0 + r][p0 + k], bs[k][c] = X[p0 + k][j0 + c]
    const int64_t nbt = (S + DNB - 1) / DNB;
    const int64_t ncol = kb + 1;
    const int64_t ti = kb + 1 + blockIdx.x / ncol, tj = blockIdx.x % ncol;
    if (ti >= nbt) return;
    const int tid = threadIdx.x;
    const int64_t i0 = ti * DNB, j0 = tj * DNB, p0 = kb * DNB;
    const int r = tid >> 3, q = tid & 7;
    float acc[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int64_t gi = i0 + r, gj = j0 + q + 8 * t;
        acc[t] = gi < S && gj < S ? Ih[gi * S + gj] : 0.f;
    }
    for (int e = tid; e < DNB * DNB; e += 256) {
        const int rr = e / DNB, c = e % DNB;
        as[rr][c] = i0 + rr < S && p0 + c < S ? Lh[(i0 + rr) * S + p0 + c] : 0.f;
        bs[rr][c] = p0 + rr < S && j0 + c < S ? Ih[(p0 + rr) * S + j0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < DNB; ++k) {
        const float x = as[r][k];
#pragma unroll
        for (int t = 0; t < 4; ++t) acc[t] = fmaf(x, bs[k][q + 8 * t], acc[t]);
    }
    if (ti != kb + 1) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int64_t gi = i0 + r, gj = j0 + q + 8 * t;
            if (gi < S && gj < S) Ih[gi * S + gj] = acc[t];
        }
        return;
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 4; ++t) as[r][q + 8 * t] = acc[t];
    for (int e = tid; e < DNB * DNB; e += 256) bs[e / DNB][e % DNB] = dh[(kb + 1) * DNB * DNB + e];
    __syncthreads();
    float out[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int p = 0; p < DNB; ++p) {
        const float d = bs[r][p];
#pragma unroll
        for (int t = 0; t < 4; ++t) out[t] = fmaf(d, as[p][q + 8 * t], out[t]);
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int64_t gi = i0 + r, gj = j0 + q + 8 * t;
        if (gi < S && gj < S) Ih[gi * S + gj] = -out[t];
    }
}

__global__ void __launch_bounds__(256)
    f32_trtri64_kernel(DfMats mats, int64_t S, int64_t kb) {
    const float* __restrict__ Lh = pick(mats.Lh, blockIdx.y);
    float* __restrict__ Ih = pick(mats.Ih, blockIdx.y);
    __shared__ float a[DNB][T64 + 1], b[DNB][T64 + 1];  // a[k][row], b[k][column]
    const int64_t ncol = (kb + 1) * DNB;
    const int64_t nJ = (ncol + T64 - 1) / T64;
    const int64_t I = blockIdx.x / nJ, J = blockIdx.x % nJ;
    const int64_t i0 = (kb + 2) * DNB + I * T64, j0 = J * T64, p0 = kb * DNB;
    if (i0 >= S) return;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t gi = i0 + ty + 16 * i, gj = j0 + tx + 16 * j;
            acc[i][j] = gi < S && gj < ncol ? Ih[gi * S + gj] : 0.f;
        }
    for (int e = tid; e < T64 * DNB; e += 256) {
        const int rr = e / DNB, k = e % DNB;  // a: rows of L's block column kb
        a[k][rr] = i0 + rr < S && p0 + k < S ? Lh[(i0 + rr) * S + p0 + k] : 0.f;
        const int k2 = e / T64, c = e % T64;  // b: block row kb of X
        b[k2][c] = p0 + k2 < S && j0 + c < S ? Ih[(p0 + k2) * S + j0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < DNB; ++k) {
        float av[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) av[i] = a[k][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = b[k][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t gi = i0 + ty + 16 * i, gj = j0 + tx + 16 * j;
            if (gi < S && gj < ncol) Ih[gi * S + gj] = acc[i][j];
        }
}

__global__ void df_mirror_lower_kernel(float* __restrict__ h, float* __restrict__ l, int64_t S) {
    for (int64_t i = blockIdx.y; i < S; i += gridDim.y)
        for (int64_t j = i + 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < S;
             j += (int64_t)gridDim.x * blockDim.x) {
            h[i * S + j] = h[j * S + i];
            l[i * S + j] = l[j * S + i];
        }
}

// Output of a matrix-vector product: float64 and, when yh is set, double-float planes;
// with add the product is added to y (read first) and the sum is stored.
__device__ __forceinline__ void store_y(double v, int64_t i, double* y, float* yh, float* yl, bool add = false) {
    if (add) v = y[i] + v;
    if (y) y[i] = v;
    if (yh) {
        const df d = df_from(v);
        yh[i] = d.hi;
        yl[i] = d.lo;
    }
}

// y = Li x for lower-triangular Li; x as double-float planes (converted once,
// not per row).  One warp per row, four independent accumulators per lane so
// several loads are in flight.
__global__ void __launch_bounds__(256)
    df_trmv_kernel(const float* __restrict__ Lh, const float* __restrict__ Ll, int64_t S,
                   const float* __restrict__ xh, const float* __restrict__ xl, double* __restrict__ y,
                   float* __restrict__ yh, float* __restrict__ yl) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (i >= S) return;
    df acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    const float* rh = Lh + i * S;
    const float* rl = Ll + i * S;
    int64_t j = lane;
    for (; j + 96 <= i; j += 128)
#pragma unroll
        for (int u = 0; u < 4; ++u) df_fma_acc(acc[u], {rh[j + 32 * u], rl[j + 32 * u]}, {xh[j + 32 * u], xl[j + 32 * u]});
    for (; j <= i; j += 32) df_fma_acc(acc[0], {rh[j], rl[j]}, {xh[j], xl[j]});
    const double v = warp_sum(df_to(df_add(df_add(acc[0], acc[1]), df_add(acc[2], acc[3]))));
    if (lane == 0) store_y(v, i, y, yh, yl);
}

// y = Li^T x: y[i] = sum_{j >= i} Li[j][i] x[j], in two passes.  Pass 1: block
// (i-group of 32 columns, j-chunk of TRMV_ROWS rows) reads its tile row by row
// (one coalesced 128-byte line per row and plane), its 8 warps split the rows
// and meet in shared memory; the chunk's partial sums go to part[chunk][i].
// Pass 2 adds the chunks in order, so the result does not depend on timing.
constexpr int TRMV_ROWS = 64;

__global__ void __launch_bounds__(256)
    df_trmv_t_part_kernel(const float* __restrict__ Lh, const float* __restrict__ Ll, int64_t S,
                          const float* __restrict__ xh, const float* __restrict__ xl, float* __restrict__ ph,
                          float* __restrict__ pl) {
    __shared__ float sh[8][32], sl[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t i0 = (int64_t)blockIdx.x * 32, i = i0 + lane;
    const int64_t j0 = (int64_t)blockIdx.y * TRMV_ROWS;
    df acc = {0.f, 0.f};
    if (j0 + TRMV_ROWS > i0) {  // otherwise the whole tile is above the diagonal
        for (int r = warp; r < TRMV_ROWS; r += 8) {
            const int64_t j = j0 + r;
            if (j < S && i < S && j >= i) df_fma_acc(acc, {Lh[j * S + i], Ll[j * S + i]}, {xh[j], xl[j]});
        }
    }
    sh[warp][lane] = acc.hi;
    sl[warp][lane] = acc.lo;
    __syncthreads();
    if (warp == 0 && i < S) {
        df tot = {sh[0][lane], sl[0][lane]};
        for (int w = 1; w < 8; ++w) tot = df_add(tot, {sh[w][lane], sl[w][lane]});
        ph[blockIdx.y * S + i] = tot.hi;
        pl[blockIdx.y * S + i] = tot.lo;
    }
}

__global__ void df_trmv_t_sum_kernel(const float* __restrict__ ph, const float* __restrict__ pl, int64_t S,
                                     int64_t nchunk, double* __restrict__ y, float* __restrict__ yh,
                                     float* __restrict__ yl, int add) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S; i += (int64_t)gridDim.x * blockDim.x) {
        df tot = {0.f, 0.f};
        for (int64_t c = i / TRMV_ROWS; c < nchunk; ++c) tot = df_add(tot, {ph[c * S + i], pl[c * S + i]});
        store_y(df_to(tot), i, y, yh, yl, add != 0);
    }
}

// y = A x, y = b - A x when b is set, or y += A x with add, for a full
// double-float A (x as planes; b, y float64, y also as planes when yh is set);
// one warp per row, four independent accumulators per lane.  With 16-byte rows
// the loads are float4, three a lane and operand in flight (the refined solve's
// last product sits on the evaluation's tail)
__global__ void __launch_bounds__(256)
    df_gemv_kernel(const float* __restrict__ Ah, const float* __restrict__ Al, int64_t S,
                   const float* __restrict__ xh, const float* __restrict__ xl, const double* __restrict__ b,
                   double* __restrict__ y, float* __restrict__ yh, float* __restrict__ yl, int add) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (i >= S) return;
    df acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    const float* rh = Ah + i * S;
    const float* rl = Al + i * S;
    const uintptr_t bits = reinterpret_cast<uintptr_t>(rh) | reinterpret_cast<uintptr_t>(rl) |
                           reinterpret_cast<uintptr_t>(xh) | reinterpret_cast<uintptr_t>(xl);
    if ((S & 3) == 0 && (bits & 15) == 0) {
        // 16-byte loads, three a lane and operand in flight; accumulator u takes component u
        const float4* h4 = reinterpret_cast<const float4*>(rh);
        const float4* l4 = reinterpret_cast<const float4*>(rl);
        const float4* xh4 = reinterpret_cast<const float4*>(xh);
        const float4* xl4 = reinterpret_cast<const float4*>(xl);
        const int64_t n4 = S / 4;
        int64_t q = lane;
        for (; q + 64 < n4; q += 96) {
            float4 a[3], b[3], c[3], d[3];
#pragma unroll
            for (int u = 0; u < 3; ++u) {
                a[u] = h4[q + 32 * u];
                b[u] = l4[q + 32 * u];
                c[u] = xh4[q + 32 * u];
                d[u] = xl4[q + 32 * u];
            }
#pragma unroll
            for (int u = 0; u < 3; ++u) {
                df_fma_acc(acc[0], {a[u].x, b[u].x}, {c[u].x, d[u].x});
                df_fma_acc(acc[1], {a[u].y, b[u].y}, {c[u].y, d[u].y});
                df_fma_acc(acc[2], {a[u].z, b[u].z}, {c[u].z, d[u].z});
                df_fma_acc(acc[3], {a[u].w, b[u].w}, {c[u].w, d[u].w});
            }
        }
        for (; q < n4; q += 32) {
            const float4 a = h4[q], b = l4[q], c = xh4[q], d = xl4[q];
            df_fma_acc(acc[0], {a.x, b.x}, {c.x, d.x});
            df_fma_acc(acc[1], {a.y, b.y}, {c.y, d.y});
            df_fma_acc(acc[2], {a.z, b.z}, {c.z, d.z});
            df_fma_acc(acc[3], {a.w, b.w}, {c.w, d.w});
        }
    } else {
        int64_t j = lane;
        for (; j + 96 < S; j += 128)
#pragma unroll
            for (int u = 0; u < 4; ++u)
                df_fma_acc(acc[u], {rh[j + 32 * u], rl[j + 32 * u]}, {xh[j + 32 * u], xl[j + 32 * u]});
        for (; j < S; j += 32) df_fma_acc(acc[0], {rh[j], rl[j]}, {xh[j], xl[j]});
    }
    const double v = warp_sum(df_to(df_add(df_add(acc[0], acc[1]), df_add(acc[2], acc[3]))));
    if (lane == 0) store_y(b ? b[i] - v : v, i, y, yh, yl, add != 0);
}

// partial sums of squares of a lower-triangular double-float matrix
__global__ void df_frob_lower_kernel(const float* __restrict__ h, const float* __restrict__ l, int64_t S,
                                     double* __restrict__ partial) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int64_t i = blockIdx.x; i < S; i += gridDim.x)
        for (int64_t j = threadIdx.x; j <= i; j += blockDim.x) {
            const double v = (double)h[i * S + j] + (double)l[i * S + j];
            acc = fma(v, v, acc);
        }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// ------------------------------------------------------------ host side

size_t dfspd_bytes(int64_t S, bool with_inverse, bool with_ainv) {
    const int64_t nbt = (S + DNB - 1) / DNB;
    Sizer s;
    if (with_inverse && with_ainv) s.take<char>(tc_lauum_workspace_bytes(S));
    s.take<float>(2 * S * S);  // L planes
    if (with_inverse) s.take<float>(2 * S * S);
    s.take<float>(2 * nbt * DNB * DNB);  // diagonal-block inverses
    s.take<float>(2 * nbt * DNB * DNB);  // factored diagonal blocks
    s.take<double>(S);  // pivots
    s.take<double>(S);  // vector scratch
    s.take<double>(S);  // vector scratch
    s.take<float>(2 * ((S + TRMV_ROWS - 1) / TRMV_ROWS) * S);  // transposed-product partial sums
    return s.total();
}

DfSpd dfspd_carve(Carver& cv, int64_t S, bool with_inverse, bool with_ainv) {
    const int64_t nbt = (S + DNB - 1) / DNB;
    DfSpd w;
    if (with_inverse && with_ainv) {
        w.tcws_bytes = tc_lauum_workspace_bytes(S);
        w.tcws = cv.take<char>(w.tcws_bytes);
    } else {
        w.tcws = nullptr;
        w.tcws_bytes = 0;
    }
    float* L = cv.take<float>(2 * S * S);
    w.Lh = L;
    w.Ll = L ? L + S * S : nullptr;
    if (with_inverse) {
        float* I = cv.take<float>(2 * S * S);
        w.Ih = I;
        w.Il = I ? I + S * S : nullptr;
    } else {
        w.Ih = w.Il = nullptr;
    }
    float* d = cv.take<float>(2 * nbt * DNB * DNB);
    w.dh = d;
    w.dl = d ? d + nbt * DNB * DNB : nullptr;
    float* f = cv.take<float>(2 * nbt * DNB * DNB);
    w.fh = f;
    w.fl = f ? f + nbt * DNB * DNB : nullptr;
    w.piv = cv.take<double>(S);
    w.vec = cv.take<double>(S);
    w.vec2 = cv.take<double>(S);
    w.part = cv.take<float>(2 * ((S + TRMV_ROWS - 1) / TRMV_ROWS) * S);
    return w;
}

int df_mirror_lower(float* hi, float* lo, int64_t S, cudaStream_t st) {
    dim3 g(blocks_for(S, 256, 8), (unsigned)(S < 65535 ? S : 65535));
    df_mirror_lower_kernel<<<g, 256, 0, st>>>(hi, lo, S);
    return check_launch();
}

int df_split(const double* x, int64_t n, float* hi, float* lo, cudaStream_t st) {
    split_kernel<<<blocks_for(n, 256, 8 * num_sms()), 256, 0, st>>>(x, n, hi, lo);
    return check_launch();
}

int df_join(const float* hi, const float* lo, int64_t n, double* x, cudaStream_t st) {
    join_kernel<<<blocks_for(n, 256, 8 * num_sms()), 256, 0, st>>>(hi, lo, n, x);
    return check_launch();
}

// A = F + H from F's lower triangle, one 32 x 32 tile pair per block: lower tile (I, J), J <= I,
// goes to A and to lo (the factorisation's starting copy); its transpose to A's tile (J, I) and
// zeros to lo's.  A diagonal tile mirrors its own lower triangle.  So A is exactly symmetric.
__global__ void __launch_bounds__(256)
    add_df_f64_sym_kernel(const float* __restrict__ fh, const float* __restrict__ fl, const double* __restrict__ h,
                          int64_t S, float* __restrict__ ah, float* __restrict__ al, float* __restrict__ lo_h,
                          float* __restrict__ lo_l) {
    __shared__ float th[32][33], tl[32][33];
    int64_t ti, tj;
    lower_tile_df(blockIdx.x, ti, tj);
    const int64_t i0 = ti * 32, j0 = tj * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const bool diag = ti == tj;
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + r, j = j0 + tx;
        df v = {0.f, 0.f};
        if (i < S && j < S && (!diag || tx <= r)) v = df_add({fh[i * S + j], fl[i * S + j]}, df_from(h[i * S + j]));
        th[r][tx] = v.hi;
        tl[r][tx] = v.lo;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + r, j = j0 + tx;
        if (i < S && j < S) {
            const bool low = !diag || tx <= r;
            const float vh = low ? th[r][tx] : th[tx][r];
            const float vl = low ? tl[r][tx] : tl[tx][r];
            ah[i * S + j] = vh;
            al[i * S + j] = vl;
            lo_h[i * S + j] = low ? vh : 0.f;
            lo_l[i * S + j] = low ? vl : 0.f;
        }
    }
    if (!diag)
        for (int r = ty; r < 32; r += 8) {
            const int64_t i = j0 + r, j = i0 + tx;
            if (i < S && j < S) {
                ah[i * S + j] = th[tx][r];
                al[i * S + j] = tl[tx][r];
                lo_h[i * S + j] = 0.f;
                lo_l[i * S + j] = 0.f;
            }
        }
}

int df_add_f64_sym(const float* fh, const float* fl, const double* h, int64_t S, float* ah, float* al, float* lo_h,
                   float* lo_l, cudaStream_t st) {
    if (S <= 0) return AJ_OK;
    const int64_t nt = (S + 31) / 32;
    add_df_f64_sym_kernel<<<(unsigned)(nt * (nt + 1) / 2), 256, 0, st>>>(fh, fl, h, S, ah, al, lo_h, lo_l);
    return check_launch();
}

static DfMats mats_of(DfSpd* const* w, int count) {
    DfMats m{};
    for (int z = 0; z < 2; ++z) {
        DfSpd* x = w[z < count ? z : 0];
        m.Lh[z] = x->Lh;
        m.Ll[z] = x->Ll;
        m.Ih[z] = x->Ih;
        m.Il[z] = x->Il;
        m.dh[z] = x->dh;
        m.dl[z] = x->dl;
        m.fh[z] = x->fh;
        m.fl[z] = x->fl;
        m.piv[z] = x->piv;
    }
    return m;
}

// When a step switches from 32 x 32 to 64 x 64 tiles: the minimum number of
// 64 x 64 output tiles per matrix (below it the 32 x 32 kernels, with 4x the
// blocks, fill the GPU better).  Set by aj_set_tile_policy (the autotuner).
static int g_tile64_min[2] = {128, 128};  // trailing update, L^-1 step

// L (in w[z]) = chol(A[z]) for z < count (1 or 2), and L^-1 for z < n_inverse; A given as planes
// (copied unless it is w's own L).  With `prepared` the caller has already put each A's lower
// triangle, upper triangle zero, in w[z]'s L and zeroed the L^-1 and A^-1 buffers.
//
// Three lanes forked from st (lanes.cu).  Lane 0 carries the critical chain:
// the pivot panel of step k, then the update of block column k + 1 alone, so
// panel k + 1 can start at once.  Lane 1 applies the rest of step k's trailing
// update meanwhile; lane 0 waits for it before touching column k + 2.  Lane 2
// runs the block forward substitution for L^-1: its step k needs block column
// k of L and the diagonal inverse of block k + 1, both final once panel k + 1
// is done, so it trails the factorisation by one panel.
int dfspd_factor_invert_n(const float* const* Ah, const float* const* Al, int count, int n_inverse, int64_t S,
                          DfSpd* const* w, double* const* logdet, int* info, cudaStream_t st, float* AIh,
                          float* AIl, bool prepared, bool f32_inverse) {
    if (S <= 0) return AJ_OK;
    if (count < 1 || count > 2 || n_inverse < 0 || n_inverse > count) return AJ_ERR_ARG;
    if ((AIh || AIl) && (!AIh || !AIl || n_inverse < 1)) return AJ_ERR_ARG;
    dim3 zg(blocks_for(S, 256, 8), (unsigned)(S < 65535 ? S : 65535));
    for (int z = 0; z < count && !prepared; ++z) {
        if (Ah[z] != w[z]->Lh) {
            if (cudaMemcpyAsync(w[z]->Lh, Ah[z], sizeof(float) * S * S, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
                cudaMemcpyAsync(w[z]->Ll, Al[z], sizeof(float) * S * S, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                return AJ_ERR_CUDA;
        }
        // the factorisation reads and writes only the lower triangle
        df_zero_upper_kernel<<<zg, 256, 0, st>>>(w[z]->Lh, w[z]->Ll, S);
        AJ_LAUNCHED();
    }
    for (int z = 0; z < n_inverse; ++z) {
        if (!w[z]->Ih) return AJ_ERR_ARG;
        if (!prepared && cudaMemsetAsync(w[z]->Ih, 0, sizeof(float) * 2 * S * S, st) != cudaSuccess)
            return AJ_ERR_CUDA;
    }
    if (AIh && !prepared &&
        (cudaMemsetAsync(AIh, 0, sizeof(float) * S * S, st) != cudaSuccess ||
         cudaMemsetAsync(AIl, 0, sizeof(float) * S * S, st) != cudaSuccess))
        return AJ_ERR_CUDA;
    DfMats m = mats_of(w, count);
    m.ninv = n_inverse;
    Lanes* lanes = nullptr;
    AJ_TRY(lanes_for(st, &lanes));
    Lanes& ln = *lanes;
    // A^-1 = L^-T L^-1 on the tensor cores once the lanes have joined (the product streamed by
    // 256-row slabs of L^-1 beside the factorisation measured slower in the batch, 572 against 596
    // evaluations/s, and no faster alone: its CTAs, one an SM, crowd the panels)
    if (AIh && !w[0]->tcws) return AJ_ERR_ARG;
    const int nlanes = 2 + n_inverse;  // lanes 2 .. 1 + n_inverse for L^-1
    AJ_TRY(lanes_fork(ln, st, nlanes));
    cudaStream_t crit = ln.s[0], bulk = ln.s[1];
    // each matrix's L^-1 on its own lane: a view of m whose slot 0 is matrix z
    DfMats one[2] = {m, m};
    for (int z = 0; z < 2; ++z) {
        one[z].Lh[0] = one[z].Lh[1] = m.Lh[z];
        one[z].Ll[0] = one[z].Ll[1] = m.Ll[z];
        one[z].Ih[0] = one[z].Ih[1] = m.Ih[z];
        one[z].Il[0] = one[z].Il[1] = m.Il[z];
        one[z].dh[0] = one[z].dh[1] = m.dh[z];
        one[z].dl[0] = one[z].dl[1] = m.dl[z];
    }
    const int64_t nbt = (S + DNB - 1) / DNB;
    static bool panel_attr[64] = {};
    {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
        if (dev < 64 && !panel_attr[dev]) {
            if (cudaFuncSetAttribute(dfchol_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)PANEL_DYN_SMEM) != cudaSuccess)
                return AJ_ERR_CUDA;
            panel_attr[dev] = true;
        }
    }
    auto panel = [&](int64_t kb) {
        const int64_t k0 = kb * DNB;
        const int64_t below = S - k0 - DNB;
        const unsigned g = 1 + (unsigned)(below > 0 ? (below + PANEL_ROWS - 1) / PANEL_ROWS : 0);
        dfchol_panel_kernel<<<dim3(g, count), PANEL_THREADS, PANEL_DYN_SMEM, crit>>>(m, S, k0, kb > 0 ? 1 : 0, info);
        return check_launch();
    };
    // Step kb: panel kb + 1 applies panel kb's update to its own block column,
    // so it only has to wait for the bulk update of step kb - 1 (which reached
    // that column); the bulk update of step kb covers the columns after it.
    AJ_TRY(panel(0));
    bool rest_prev = false;
    for (int64_t kb = 0; kb + 1 < nbt; ++kb) {
        const int64_t k0 = kb * DNB;
        const int64_t tb = (S - k0 - DNB + 31) / 32;  // trailing tile rows (>= 1 here)
        // wait for the previous bulk update before kEvUpdate is recorded again
        if (rest_prev) AJ_TRY(lane_wait(ln, 0, kEvUpdate));
        if (tb > 1) {
            AJ_TRY(lane_signal(ln, kEvPanel, 0));
            AJ_TRY(lane_wait(ln, 1, kEvPanel));
            const int64_t n64 = (S - k0 - 2 * DNB + T64 - 1) / T64;
            const int64_t t64 = n64 * (n64 + 1) / 2;
            if (t64 >= g_tile64_min[0])
                dfsyrk_update64_kernel<<<dim3((unsigned)t64, count), 256, 0, bulk>>>(m, S, k0);
            else
                dfsyrk_update_kernel<<<dim3((unsigned)((tb - 1) * tb / 2), count), 128, 0, bulk>>>(m, S, k0);
            AJ_LAUNCHED();
            AJ_TRY(lane_signal(ln, kEvUpdate, 1));
        }
        rest_prev = tb > 1;
        AJ_TRY(panel(kb + 1));
        if (n_inverse > 0) {
            AJ_TRY(lane_signal(ln, kEvDiag, 0));
            // rows past the next block row in 64 x 64 tiles when there are enough of them; the
            // next block row (which applies the diagonal inverse) always in 32 x 32 tiles
            const int64_t nI = (S - (kb + 2) * DNB + T64 - 1) / T64, nJ = ((kb + 1) * DNB + T64 - 1) / T64;
            const bool big = nI > 0 && nI * nJ >= g_tile64_min[1];
            const int64_t tiles = (big ? 1 : nbt - kb - 1) * (kb + 1);
            for (int z = 0; z < n_inverse; ++z) {
                AJ_TRY(lane_wait(ln, 2 + z, kEvDiag));
                if (f32_inverse)
                    f32_trtri_step_kernel<<<(unsigned)tiles, 256, 0, ln.s[2 + z]>>>(one[z], S, kb);
                else
                    df_trtri_step_kernel<<<(unsigned)tiles, 256, 0, ln.s[2 + z]>>>(one[z], S, kb);
                AJ_LAUNCHED();
                if (big) {
                    if (f32_inverse)
                        f32_trtri64_kernel<<<(unsigned)(nI * nJ), 256, 0, ln.s[2 + z]>>>(one[z], S, kb);
                    else
                        df_trtri64_kernel<<<(unsigned)(nI * nJ), 256, 0, ln.s[2 + z]>>>(one[z], S, kb);
                    AJ_LAUNCHED();
                }
            }
        }
    }
    df_store_diag_kernel<<<dim3((unsigned)nbt, count), 256, 0, crit>>>(m, S);
    AJ_LAUNCHED();
    // the log-determinants need only the pivots: on the bulk lane, idle by now, beside the tails
    // of the other lanes
    if (logdet && (logdet[0] || (count > 1 && logdet[1]))) {
        AJ_TRY(lane_signal(ln, kEvPanel, 0));
        AJ_TRY(lane_wait(ln, 1, kEvPanel));
        df_logdet_kernel<<<(unsigned)count, 1024, 0, bulk>>>(w[0]->piv, count > 1 ? w[1]->piv : nullptr, S, logdet[0],
                                                             count > 1 ? logdet[1] : nullptr, info);
        AJ_LAUNCHED();
    }
    AJ_TRY(lanes_join(ln, st, nlanes));
    if (AIh) AJ_TRY(tc_lauum(w[0]->Ih, w[0]->Il, S, AIh, AIl, w[0]->tcws, w[0]->tcws_bytes, st));
    return AIh ? df_mirror_lower(AIh, AIl, S, st) : AJ_OK;
}

// x = Li^T (Li b) with the inverse factor, b given as planes bh (S hi floats,
// then S lo floats); uh is 2 S floats of scratch.  x's planes go to xh/xl when
// xh is set; with add, the product is added to x instead of replacing it.
// (Two triangular products split the conditioning between two factors of
// sqrt(cond A); one product with an explicit A^-1 would lose cond(A) at once.)
static int df_trsolve(int64_t S, DfSpd& w, const float* bh, float* uh, double* x, float* xh, float* xl, bool add,
                      cudaStream_t st) {
    if (!w.Ih) return AJ_ERR_ARG;
    df_trmv_kernel<<<blocks_for(S * 32, 256), 256, 0, st>>>(w.Ih, w.Il, S, bh, bh + S, nullptr, uh, uh + S);
    AJ_LAUNCHED();
    const int64_t nchunk = (S + TRMV_ROWS - 1) / TRMV_ROWS;
    float* ph = w.part;
    float* pl = w.part + nchunk * S;
    df_trmv_t_part_kernel<<<dim3((unsigned)((S + 31) / 32), (unsigned)nchunk), 256, 0, st>>>(w.Ih, w.Il, S, uh,
                                                                                           uh + S, ph, pl);
    AJ_LAUNCHED();
    df_trmv_t_sum_kernel<<<blocks_for(S, 256, 64), 256, 0, st>>>(ph, pl, S, nchunk, x, xh, xl, add ? 1 : 0);
    return check_launch();
}

// x = A^-1 b with one step of iterative refinement against A (planes).  The
// correction A^-1 r goes through A^-1's planes (one row-wise product) when
// they are given: r is already small, so the explicit inverse's cond(A) loss
// applies to a correction, not to the solution.  Five launches: each product
// also writes the planes the next one reads, the residual never exists in
// float64, and the last product adds the correction to x in place.
// b_split: b's planes are already in w.vec (S hi floats, then S lo floats).
// xh/xl, when set, receive the planes of the final x.
int dfspd_solve_refined(int64_t S, DfSpd& w, const float* Ah, const float* Al, const double* b, double* x,
                        cudaStream_t st, const float* AIh, const float* AIl, bool b_split, float* xh, float* xl,
                        cudaEvent_t ainv_ready) {
    if (!w.Ih) return AJ_ERR_ARG;
    float* v1 = reinterpret_cast<float*>(w.vec);   // b's planes, then x0's
    float* v2 = reinterpret_cast<float*>(w.vec2);  // L^-1 b's planes, then r's
    if (!b_split) AJ_TRY(df_split(b, S, v1, v1 + S, st));
    AJ_TRY(df_trsolve(S, w, v1, v2, x, v1, v1 + S, false, st));
    const unsigned g = blocks_for(S * 32, 256);
    df_gemv_kernel<<<g, 256, 0, st>>>(Ah, Al, S, v1, v1 + S, b, nullptr, v2, v2 + S, 0);
    AJ_LAUNCHED();
    if (AIh) {
        if (ainv_ready && cudaStreamWaitEvent(st, ainv_ready, 0) != cudaSuccess) return AJ_ERR_CUDA;
        df_gemv_kernel<<<g, 256, 0, st>>>(AIh, AIl, S, v2, v2 + S, nullptr, x, xh, xl, 1);
        return check_launch();
    }
    return df_trsolve(S, w, v2, v1, x, xh, xl, true, st);
}

int df_frob_lower(const float* h, const float* l, int64_t S, double* partial, int64_t nparts, cudaStream_t st) {
    df_frob_lower_kernel<<<(unsigned)nparts, 256, 0, st>>>(h, l, S, partial);
    return check_launch();
}

}  // namespace aj

using namespace aj;

extern "C" {

int aj_set_tile_policy(int update_min_tiles, int inverse_min_tiles) {
    if (update_min_tiles < 1 || inverse_min_tiles < 1) return AJ_ERR_ARG;
    aj::g_tile64_min[0] = update_min_tiles;
    aj::g_tile64_min[1] = inverse_min_tiles;
    return AJ_OK;
}

int aj_get_tile_policy(int* out2) {
    if (!out2) return AJ_ERR_ARG;
    for (int i = 0; i < 2; ++i) out2[i] = aj::g_tile64_min[i];
    return AJ_OK;
}

size_t aj_spd_inverse_mixed_workspace_size(int64_t S) {
    Sizer s;
    s.take<float>(2 * S * S);  // A planes
    s.take<float>(2 * S * S);  // A^-1 planes
    s.take<char>(dfspd_bytes(S, true, true));
    return s.total();
}

int aj_spd_inverse_mixed(const double* A, int64_t S, double* Ainv, double* logdet, void* workspace,
                         size_t workspace_bytes, int* info, void* stream) {
    if (S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!A || !Ainv) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < aj_spd_inverse_mixed_workspace_size(S)) return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace, workspace_bytes);
    float* Ap = cv.take<float>(2 * S * S);
    float* Ip = cv.take<float>(2 * S * S);
    char* sub = cv.take<char>(dfspd_bytes(S, true, true));
    Carver sc(sub, dfspd_bytes(S, true, true));
    DfSpd w = dfspd_carve(sc, S, true, true);
    AJ_TRY(df_split(A, S * S, Ap, Ap + S * S, st));
    const float* ah[1] = {Ap};
    const float* al[1] = {Ap + S * S};
    DfSpd* ws[1] = {&w};
    double* ld[1] = {logdet};
    AJ_TRY(dfspd_factor_invert_n(ah, al, 1, 1, S, ws, ld, info, st, Ip, Ip + S * S));
    return df_join(Ip, Ip + S * S, S * S, Ainv, st);
}

}  // extern "C"
