// The trailing update of the double-float Cholesky on the tensor cores.
//
// Step k of the blocked factorisation subtracts X X^T from the lower trailing
// matrix, X the panel's 32 finished columns of the rows below (the S^3/6 bulk
// of the factorisation: numba.py:731's solve and 849-850's log-determinant by
// way of the Cholesky factor).  Each row of X, as the exact float64 sum of its
// double-float planes, is scaled by its own power of two to [-1, 1] and cut into
// 7 integer digits of 7 bits (48 bits; the scheme of the mixed w_tilde product,
// wtilde_tc.cu): x_ik = 2^e_i sum_d delta_d 2^-(6+7d).  Then
//
//   sum_k x_ik x_jk = 2^(e_i + e_j - 12) sum_L 2^-7L sum_{d+e=L} sum_k delta_d(i,k) delta_e(j,k),
//
// where every level sum (L + 1 <= 7 digit pairs over 32 columns, products of
// at most 2^12) is an integer below 2^20, exact in a float32 TMEM accumulator.
// Levels above 6 are dropped: below 2^-48 of the two rows' scales a term, the
// rounding of a 32-term double-float dot product.  The epilogue folds the
// levels into double-float by TwoSum, scales by the exact power of two and
// subtracts from the trailing matrix's planes.
//
// One CTA per 128 x 64 tile of the lower trailing triangle: one thread issues
// the two TMA loads (all 7 digits of the tile's 128 and 64 rows, 64-byte
// swizzled rows of 32 columns; rows past the matrix read as zeros), allocates
// 512 TMEM columns after issuing them (so a CTA waiting for another's TMEM has
// its operands in flight), waits, issues the 2 x 28 MMAs and commits; then
// all 8 warps read the 7 level accumulators (warps w and w + 4 share TMEM
// lanes 32 (w mod 4), one 32-column half each).  Every wait is bounded; an
// expired one reports AJ_INFO_DEVICE_TIMEOUT in the factorisation's info word.

#include <cuda_bf16.h>
#include <math.h>

#include <mutex>

#include "aj_internal.cuh"
#include "df32.cuh"
#include "tc_common.cuh"

namespace aj {

namespace dftc {

using namespace tc;

constexpr int kDigits = 7;
constexpr int kDigitBits = 7;
constexpr int kFirstBits = 6;
constexpr int BM = 128, BN = 64, BK = 32;
constexpr int kStageA = kDigits * BM * BK * 2;
constexpr int kStageB = kDigits * BN * BK * 2;
constexpr int kThreads = 256;
constexpr int kTmemCols = 512;
constexpr size_t kSmemBytes = size_t(kStageA + kStageB) + 1024 + 128;
constexpr uint32_t kIdesc = idesc_bf16(BM, BN);

static_assert(kDigits * BN <= kTmemCols, "level accumulators exceed TMEM");
static_assert(kDigits * BK * (1 << (2 * (kDigitBits - 1))) < (1 << 23), "level sums must stay exact");

struct Shared {
    uint64_t full;
    uint64_t mmadone;
    uint32_t tmem_base;
    int abort;
    int expired;  // this CTA's own timeout word (each CTA runs one stage; none waits on another)
    int exp_j[BN];
};

// Digits of rows r0 .. S-1 of the panel columns k0 .. k0+31: D[d][r - r0][k] (bf16), E[r - r0] = e_r.
// One warp a row, lane k on column k.
__global__ void __launch_bounds__(256)
    df_digits_kernel(const float* __restrict__ Lh, const float* __restrict__ Ll, int64_t S, int64_t k0, int64_t r0,
                     __nv_bfloat16* __restrict__ D, int* __restrict__ E) {
    const int lane = threadIdx.x & 31;
    const int64_t n = S - r0;
    const int64_t r = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= n) return;
    const int64_t row = r0 + r, col = k0 + lane;
    const double x = col < S ? (double)Lh[row * S + col] + (double)Ll[row * S + col] : 0.0;
    double m = fabs(x);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    int e = 0;
    if (m > 0.0 && m == m) {
        const double f = frexp(m, &e);  // m = f 2^e, f in [0.5, 1)
        if (f == 0.5) e -= 1;            // a power of two: 2^e = m
    }
    double y = ldexp(x, kFirstBits - e);
    const int64_t plane = n * BK;
#pragma unroll
    for (int d = 0; d < kDigits; ++d) {
        const double q = rint(y);
        D[d * plane + r * BK + lane] = __float2bfloat16_rn(static_cast<float>(q));
        y = (y - q) * (double)(1 << kDigitBits);
    }
    if (lane == 0) E[r] = e;
}

// lower 128 x 64 tile t of an n x n triangle (J <= 2I + 1, J < nJ), row-major
__device__ __forceinline__ void tile_of(int64_t t, int64_t nJ, int64_t& I, int64_t& J) {
    int64_t i = 0;
    for (;;) {
        const int64_t w = min(2 * i + 2, nJ);
        if (t < w) break;
        t -= w;
        ++i;
    }
    I = i;
    J = t;
}

__global__ void __launch_bounds__(kThreads, 2)
    df_tc_update_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                        const int* __restrict__ E, float* __restrict__ Lh, float* __restrict__ Ll, int64_t S,
                        int64_t r0, int* info) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    Shared* sh = reinterpret_cast<Shared*>(base + kStageA + kStageB);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t n = S - r0;
    const int64_t nJ = (n + BN - 1) / BN;
    int64_t I, J;
    tile_of(blockIdx.x, nJ, I, J);
    if (threadIdx.x == 0) {
        mbar_init(&sh->full, 1);
        mbar_init(&sh->mmadone, 1);
        sh->abort = 0;
        sh->expired = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_expect_tx(&sh->full, kStageA + kStageB);
        tma_load_3d(base, &map_a, 0, static_cast<int>(I * BM), 0, &sh->full);
        tma_load_3d(base + kStageA, &map_b, 0, static_cast<int>(J * BN), 0, &sh->full);
    }
    if (threadIdx.x < BN) {
        const int64_t j = J * BN + threadIdx.x;
        sh->exp_j[threadIdx.x] = j < n ? E[j] : 0;
    }
    if (warp == 0) tmem_alloc(&sh->tmem_base, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;
    volatile int* abort = &sh->abort;
    if (threadIdx.x == 0) {
        if (mbar_wait(&sh->full, 0, abort, &sh->expired)) {
            tc_fence_after();
            const uint32_t sa = smem_u32(base), sb = sa + kStageA;
#pragma unroll
            for (int ks = 0; ks < BK / 16; ++ks)
#pragma unroll
                for (int L = 0; L < kDigits; ++L)
#pragma unroll
                    for (int d = 0; d <= L; ++d) {
                        const uint64_t ad = desc_sw64(sa + d * (BM * BK * 2) + ks * 32);
                        const uint64_t bd = desc_sw64(sb + (L - d) * (BN * BK * 2) + ks * 32);
                        tc_mma(tmem + static_cast<uint32_t>(L * BN), ad, bd, kIdesc, (ks == 0 && d == 0) ? 0u : 1u);
                    }
        }
        tc_commit(&sh->mmadone);
    }
    __syncwarp();
    const bool ok = mbar_wait(&sh->mmadone, 0, abort, &sh->expired);
    tc_fence_after();
    if (ok && !*abort) {
        const int q = warp & 3, half = warp >> 2;
        const int64_t ri = I * BM + q * 32 + lane;  // row within the trailing matrix
        const uint32_t taddr = tmem + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(half * 32);
        float h[32], l[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            h[j] = 0.f;
            l[j] = 0.f;
        }
#pragma unroll 1
        for (int L = kDigits - 1; L >= 0; --L) {
            float v[32];
            tc_ld32(taddr + static_cast<uint32_t>(L * BN), v);
            const float sc = ldexpf(1.0f, -kDigitBits * L);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const float c = v[j] * sc;
                const float s = h[j] + c;
                const float bb = s - h[j];
                l[j] += (h[j] - (s - bb)) + (c - bb);
                h[j] = s;
            }
        }
        if (ri < n) {
            const int64_t gi = r0 + ri;
            const int ei = E[ri];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int64_t cj = J * BN + half * 32 + j;
                const int64_t gj = r0 + cj;
                if (cj >= n || gj > gi) continue;
                const int sh2 = ei + sh->exp_j[half * 32 + j] - 2 * kFirstBits;
                const df p = df_norm({ldexpf(h[j], sh2), ldexpf(l[j], sh2)});
                const df cur = {Lh[gi * S + gj], Ll[gi * S + gj]};
                const df v = df_add(cur, df_neg(p));
                Lh[gi * S + gj] = v.hi;
                Ll[gi * S + gj] = v.lo;
            }
        }
    }
    if (!ok && threadIdx.x == 0) report(info, AJ_INFO_DEVICE_TIMEOUT, r0);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static std::mutex mu;
    static EncodeTiledFn fn = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// [kDigits][n][32] bf16 digits as boxes of {32 columns, rows, kDigits}; rows past n read as zeros
int make_map(CUtensorMap* map, const void* D, int64_t n, int rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return AJ_ERR_CUDA;
    const cuuint64_t dims[3] = {BK, static_cast<cuuint64_t>(n), kDigits};
    const cuuint64_t strides[2] = {BK * 2, static_cast<cuuint64_t>(n) * BK * 2};
    const cuuint32_t box[3] = {BK, static_cast<cuuint32_t>(rows), kDigits};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(D), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? AJ_OK : AJ_ERR_CUDA;
}

int set_smem_attr() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return AJ_OK;
    if (cudaFuncSetAttribute(df_tc_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kSmemBytes)) != cudaSuccess)
        return AJ_ERR_CUDA;
    if (dev >= 0 && dev < 64) done[dev] = true;
    return AJ_OK;
}

}  // namespace dftc

size_t df_tc_digit_bytes(int64_t S) { return size_t(dftc::kDigits) * S * dftc::BK * 2; }

// L (planes Lh/Ll, S x S) -= X X^T on the lower triangle of rows and columns r0 .. S-1, X = L[r0:, k0:k0+32].
int df_tc_update(float* Lh, float* Ll, int64_t S, int64_t k0, int64_t r0, void* digits, int* exps, int* info,
                 cudaStream_t st) {
    using namespace dftc;
    const int64_t n = S - r0;
    if (n <= 0) return AJ_OK;
    if (reinterpret_cast<uintptr_t>(digits) % 16 != 0) return AJ_ERR_ARG;
    auto* D = static_cast<__nv_bfloat16*>(digits);
    df_digits_kernel<<<static_cast<unsigned>((n + 7) / 8), 256, 0, st>>>(Lh, Ll, S, k0, r0, D, exps);
    AJ_LAUNCHED();
    CUtensorMap ma, mb;
    AJ_TRY(make_map(&ma, D, n, BM));
    AJ_TRY(make_map(&mb, D, n, BN));
    AJ_TRY(set_smem_attr());
    const int64_t nI = (n + BM - 1) / BM, nJ = (n + BN - 1) / BN;
    int64_t tiles = 0;
    for (int64_t i = 0; i < nI; ++i) tiles += (2 * i + 2 < nJ ? 2 * i + 2 : nJ);
    df_tc_update_kernel<<<static_cast<unsigned>(tiles), kThreads, kSmemBytes, st>>>(ma, mb, exps, Lh, Ll, S, r0,
                                                                                    info);
    return check_launch();
}

}  // namespace aj
