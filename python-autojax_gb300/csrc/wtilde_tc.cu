// Mixed-precision direct w_tilde on the Blackwell tensor cores (numba.py:156-207).
//
// W = P^T P with P[r][i] = sqrt(w_k) {cos, sin}(2 pi t_ik) (the cos rows, then the
// sin rows, of one chunk of visibilities).  The float64 panel values are cut into
// exact integer digits and the product runs as a sum of exact digit products on
// the bf16 tensor pipe (an Ozaki-style split):
//
//   y = P / s in [-1, 1] (s a power of two >= max sqrt(w_k)),
//   y = sum_d delta_d 2^-(B0 + B d),  delta_d integers, |delta_d| <= 2^(B-1),
//
// with B = 7 bits a digit (B0 = 6 for the first), kDigits = 7 digits: 48 bits,
// the residual below 2^-48 of s.  A digit is exact in bf16, and a product of two
// is an integer of at most 2^12; the products of one "level" L = d + e share
// the scale 2^-(2 B0 + B L), so for every level a tcgen05.mma (M = 128, N = 64,
// K = 16) sums the digit products of its L + 1 pairs into one float32 TMEM
// accumulator.  Over a group of kGroupRows rows a level sum stays below
// (L + 1) kGroupRows 2^12 <= 7 * 256 * 4096 = 2^22.8, so every partial sum is an
// integer the float32 accumulator holds exactly.  Levels above kDigits - 1 are
// dropped: they are below 2^-48 of s^2 per term, the panel's own rounding.
// After each group the epilogue warps read the level sums out of TMEM and fold
// them, scaled by powers of two (exact), into double-float accumulators with
// TwoSum (error-free but for the low word's rounding, ~2^-48 relative).
//
// Layout: the digit panel is [kDigits][Mp][Rc] bf16 (k fastest), loaded by TMA as
// one 3-D box per operand and stage (all digits of a 32-row k slab, 64-byte
// rows, 64-byte swizzle), the canonical K-major layout the shared-memory matrix
// descriptors name.  One CTA computes one 128 x 64 tile of the lower block
// triangle over the whole chunk: warp 0 issues the TMA loads, warp 1 (one
// thread) the MMAs and owns the TMEM allocation, warps 2-5 run the epilogue.
// Every wait on an mbarrier is bounded (seconds, by the global timer): on
// expiry the CTA sets an error word, drains what it issued and frees its TMEM.

#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <mutex>

#include "aj_internal.cuh"
#include "df32.cuh"
#include "tc_common.cuh"

namespace aj {

namespace tc {

constexpr int kDigits = 7;                  // digits a value in the w_tilde product
constexpr int kInvDigits = 8;               // digits a value in L^-T L^-1 (below)
constexpr int kDigitBits = 7;
constexpr int kFirstBits = 6;  // y in [-1, 1]: the first digit rint(y 2^6) lies in [-64, 64]
constexpr int BM = 128, BN = 64, BK = 32;   // tile rows, tile columns, k rows a stage
constexpr int kGroupRows = 256;             // rows summed in TMEM between epilogue folds
constexpr int kStagesPerGroup = kGroupRows / BK;
constexpr int kStages = 2;
constexpr int kTmemCols = 512;              // >= levels * BN, a power of two
constexpr int kThreads = 192;

// Sizes for ND digits a value: ND levels 0 .. ND - 1, each an N = 64 TMEM accumulator.  Level L
// sums L + 1 <= ND digit pairs, so a level sum over a group stays within ND kGroupRows 2^12 <= 2^23,
// an integer float32 holds exactly.
template <int ND>
struct Cut {
    static constexpr int kStageA = ND * BM * BK * 2;  // bytes
    static constexpr int kStageB = ND * BN * BK * 2;
    static constexpr int kStageBytes = kStageA + kStageB;
    static constexpr size_t kSmemBytes = size_t(kStages) * kStageBytes + 1024 + 256;
    static_assert(ND * BN <= kTmemCols, "level accumulators exceed TMEM");
    static_assert(ND * kGroupRows * (1 << (2 * (kDigitBits - 1))) <= (1 << 23), "level sums must stay exact");
    static_assert(kSmemBytes <= 232448, "shared memory");
};
static_assert(kGroupRows % BK == 0, "group of whole stages");

struct Shared {
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t accfull;
    uint64_t accempty;
    uint64_t mmadone;
    uint32_t tmem_base;
    int abort;
};

// kind::f16 instruction descriptor: float32 accumulator, bf16 A and B, both K-major, M = 128, N = 64.
constexpr uint32_t kIdesc = idesc_bf16(BM, BN);

// Lower block-triangle tile t -> (row tile I of 128 rows, column tile J of 64 columns), J <= 2I + 1.
// Tiles go in bands of kBand row tiles, column-major inside a band, so the CTAs resident at once
// share both operands' rows (a band's A rows and a run of B rows) in L2 instead of each reading a
// B tile of its own.
constexpr int64_t kBand = 8;
__device__ __forceinline__ void tile_of(int64_t t, int64_t nI, int64_t& I, int64_t& J) {
    int64_t i0 = 0;
    for (;;) {
        const int64_t i1 = min(nI, i0 + kBand);
        const int64_t n = (i1 - i0) * (i0 + i1 + 1);  // sum over I in [i0, i1) of 2I + 2
        if (t < n || i1 >= nI) break;
        t -= n;
        i0 = i1;
    }
    const int64_t i1 = min(nI, i0 + kBand);
    for (int64_t j = 0;; ++j) {
        const int64_t ilo = max(i0, j / 2);  // the rows of this band with 2I + 1 >= j
        const int64_t cnt = i1 > ilo ? i1 - ilo : 0;
        if (t < cnt) {
            I = ilo + t;
            J = j;
            return;
        }
        t -= cnt;
    }
}

__device__ __forceinline__ void two_sum_into(float& hi, float& lo, float c) {
    const float s = hi + c;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (c - bb);
    hi = s;
    lo += e;
}

// x 2^k, exact while the result stays in the normal range (two power-of-two factors, each a float)
__device__ __forceinline__ float times_pow2(float x, int k) {
    k = max(-252, min(252, k));
    const int k1 = k / 2;
    return x * __int_as_float((k1 + 127) << 23) * __int_as_float((k - k1 + 127) << 23);
}

// Out (+)= scale 2^(e_i + e_j) acc on the lower triangle of one 128 x 64 tile (e = 0 without exps).
__device__ __forceinline__ void store_row(float* __restrict__ oh, float* __restrict__ ol, int64_t ld, int64_t M,
                                          int64_t gi, int64_t gj0, const float (&h)[BN], const float (&l)[BN],
                                          float scale, const int* __restrict__ exps, int accumulate) {
    if (gi >= M) return;
    const int ei = exps ? exps[gi] : 0;
#pragma unroll
    for (int j = 0; j < BN; ++j) {
        const int64_t gj = gj0 + j;
        if (gj > gi || gj >= M) continue;
        float ah = h[j] * scale, al = l[j] * scale;
        if (exps) {
            const int k = ei + exps[gj];
            ah = times_pow2(ah, k);
            al = times_pow2(al, k);
        }
        if (accumulate) {
            const float bh = oh[gi * ld + gj], bl = ol[gi * ld + gj];
            const float s = ah + bh;
            const float bb = s - ah;
            float e = (ah - (s - bb)) + (bh - bb);
            e += al + bl;
            ah = s + e;
            al = e - (ah - s);
        } else {
            const float s = ah + al;
            al = al - (s - ah);
            ah = s;
        }
        oh[gi * ld + gj] = ah;
        ol[gi * ld + gj] = al;
    }
}

// One CTA per lower tile; Rc rows of digits (a multiple of kGroupRows).  The product is scaled by
// *scale_dev (s^2 2^-(2 first bits)) and, with exps, by 2^(e_i + e_j) per entry (digits of column
// i cut at its own power of two).  With tri, a digit row k is zero for k < i (the panel is an upper
// triangle, as the transpose of L^-1 is): a tile starts at the group holding its first row.  The
// tiles of the first split_rows row tiles (the ones with the most groups then) are split in two:
// their CTA sums the first half of the groups into out, and one of split_rows (split_rows + 1)
// extra CTAs, launched ahead of the nI (nI + 1) tiles, the second half into out2 (the caller adds
// out2 to out).
template <int ND>
__global__ void __launch_bounds__(kThreads, 1)
    digit_syrk_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                      int64_t Rc, int64_t M, int64_t Mp, float* __restrict__ out_h, float* __restrict__ out_l,
                      int64_t ld, const float* __restrict__ scale_dev, const int* __restrict__ exps, int tri,
                      int split_rows, float* __restrict__ out2_h, float* __restrict__ out2_l, int accumulate,
                      int* __restrict__ err) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    Shared* sh = reinterpret_cast<Shared*>(base + size_t(kStages) * Cut<ND>::kStageBytes);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t I, J;
    const int64_t nI = Mp / BM;
    // The split tiles' second halves come first: with one CTA an SM the grid runs in about one and
    // a half waves, and the second halves are among the longest CTAs (the first row tiles sum the
    // most groups), so they start in the first wave and the short tiles fill in behind them.
    const int64_t nsecond = static_cast<int64_t>(split_rows) * (split_rows + 1);
    int part = 0;  // 1: the second half of a split tile
    if (blockIdx.x >= nsecond) {
        tile_of(blockIdx.x - nsecond, nI, I, J);
    } else {
        int64_t e = blockIdx.x;  // split tiles in row-major order: 2I + 2 in row tile I
        I = 0;
        while (e >= 2 * I + 2) {
            e -= 2 * I + 2;
            ++I;
        }
        J = e;
        part = 1;
    }
    int g0 = tri ? static_cast<int>(max(I * BM, J * BN) / kGroupRows) : 0;
    int gend = static_cast<int>(Rc / kGroupRows);
    if (I < split_rows) {
        const int gmid = g0 + (gend - g0) / 2;
        if (part)
            g0 = gmid;
        else
            gend = gmid;
    }
    float* __restrict__ oh = part ? out2_h : out_h;
    float* __restrict__ ol = part ? out2_l : out_l;
    const int ngroups = gend - g0;  // groups this CTA sums, from g0
    const int nstages = ngroups * kStagesPerGroup;
    const int it0 = g0 * kStagesPerGroup;  // the first stage's k slab

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->empty[s], 1);
        }
        mbar_init(&sh->accfull, 1);
        mbar_init(&sh->accempty, 4);
        mbar_init(&sh->mmadone, 1);
        sh->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(&sh->tmem_base, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;
    volatile int* abort = &sh->abort;

    if (warp == 0) {
        if (lane == 0) {
            // producer: every stage holds all digits of one 32-row slab of both operands
            int issued = 0;
            for (int it = 0; it < nstages; ++it) {
                const int s = it % kStages;
                if (it >= kStages && !mbar_wait(&sh->empty[s], ((it / kStages) & 1) ^ 1, abort, err)) break;
                unsigned char* sa = base + size_t(s) * Cut<ND>::kStageBytes;
                mbar_expect_tx(&sh->full[s], Cut<ND>::kStageBytes);
                tma_load_3d(sa, &map_a, (it0 + it) * BK, static_cast<int>(I * BM), 0, &sh->full[s]);
                tma_load_3d(sa + Cut<ND>::kStageA, &map_b, (it0 + it) * BK, static_cast<int>(J * BN), 0, &sh->full[s]);
                ++issued;
            }
            // drain: every issued load lands before the CTA may leave (a no-op on the normal path,
            // where the MMA thread consumed them all)
            for (int it = (issued > kStages ? issued - kStages : 0); it < issued && *abort; ++it) {
                const int s = it % kStages;
                unsigned long long t0 = global_ns();
                while (!mbar_try_wait(&sh->full[s], (it / kStages) & 1) && global_ns() - t0 < kWaitNs) {
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t sbase = smem_u32(base);
            for (int g = 0; g < ngroups && !*abort; ++g) {
                if (g > 0 && !mbar_wait(&sh->accempty, (g - 1) & 1, abort, err)) break;
                tc_fence_after();
                bool ok = true;
                for (int sg = 0; sg < kStagesPerGroup; ++sg) {
                    const int it = g * kStagesPerGroup + sg;
                    const int s = it % kStages;
                    if (!mbar_wait(&sh->full[s], (it / kStages) & 1, abort, err)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = sbase + static_cast<uint32_t>(s * Cut<ND>::kStageBytes);
                    const uint32_t sb = sa + Cut<ND>::kStageA;
                    // A digit d meets B digits e = 0 .. 6 - d back to back, so A stays in the
                    // collector buffer across them; the d = 0 sweep writes every level first
#pragma unroll
                    for (int ks = 0; ks < BK / 16; ++ks) {
#pragma unroll
                        for (int d = 0; d < ND; ++d) {
                            const uint64_t ad = desc_sw64(sa + d * (BM * BK * 2) + ks * 32);
                            const uint32_t acc = (sg == 0 && ks == 0 && d == 0) ? 0u : 1u;
#pragma unroll
                            for (int e = 0; e < ND - d; ++e) {
                                const uint64_t bd = desc_sw64(sb + e * (BN * BK * 2) + ks * 32);
                                const uint32_t dst = tmem + static_cast<uint32_t>((d + e) * BN);
                                if (ND - d == 1)
                                    tc_mma(dst, ad, bd, kIdesc, acc);
                                else if (e == 0)
                                    tc_mma_collect<ACollect::kFill>(dst, ad, bd, kIdesc, acc);
                                else if (e == ND - d - 1)
                                    tc_mma_collect<ACollect::kLastUse>(dst, ad, bd, kIdesc, acc);
                                else
                                    tc_mma_collect<ACollect::kUse>(dst, ad, bd, kIdesc, acc);
                            }
                        }
                    }
                    tc_commit(&sh->empty[s]);
                }
                if (!ok) break;
                tc_commit(&sh->accfull);
            }
            // every MMA this thread issued completes before the TMEM is freed
            tc_commit(&sh->mmadone);
            const unsigned long long t0 = global_ns();
            while (!mbar_try_wait(&sh->mmadone, 0) && global_ns() - t0 < kWaitNs) {
            }
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) ..
        const int q = warp & 3;
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(q * 32) << 16);
        float h[BN], l[BN];
#pragma unroll
        for (int j = 0; j < BN; ++j) {
            h[j] = 0.f;
            l[j] = 0.f;
        }
        for (int g = 0; g < ngroups; ++g) {
            if (!mbar_wait(&sh->accfull, g & 1, abort, err)) break;
            tc_fence_after();
#pragma unroll 1
            for (int L = ND - 1; L >= 0; --L) {
                const float sc = ldexpf(1.0f, -kDigitBits * L);
#pragma unroll
                for (int half = 0; half < BN / 32; ++half) {
                    float v[32];
                    tc_ld32(lane_addr + static_cast<uint32_t>(L * BN + half * 32), v);
#pragma unroll
                    for (int j = 0; j < 32; ++j) two_sum_into(h[half * 32 + j], l[half * 32 + j], v[j] * sc);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&sh->accempty);
#pragma unroll
            for (int j = 0; j < BN; ++j) {
                const float s = h[j] + l[j];
                l[j] = l[j] - (s - h[j]);
                h[j] = s;
            }
        }
        if (!*abort) {
            const int64_t gi = I * BM + q * 32 + lane;
            store_row(oh, ol, ld, M, gi, J * BN, h, l, *scale_dev, exps, accumulate);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// The largest sqrt(w_k) = 1 / |sigma_k| as the bits of a positive double (they order as integers).
__global__ void max_inv_sigma_kernel(const double* __restrict__ sigma, int64_t K,
                                     unsigned long long* __restrict__ max_bits) {
    unsigned long long m = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < K; k += (int64_t)gridDim.x * blockDim.x) {
        const double v = 1.0 / fabs(sigma[k]);
        const unsigned long long b = (v == v && v < INFINITY) ? __double_as_longlong(v) : 0ull;
        m = b > m ? b : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
        m = x > m ? x : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(max_bits, m);
}

// s = 2^e >= max sqrt(w); the product's scale s^2 2^-(2 kFirstBits) as a float.
__global__ void digit_scale_kernel(const unsigned long long* __restrict__ max_bits, int* __restrict__ e_out,
                                   float* __restrict__ scale_out) {
    const double m = __longlong_as_double(static_cast<long long>(*max_bits));
    int e = 0;
    if (m > 0.0) {
        const double f = frexp(m, &e);  // m = f 2^e, f in [0.5, 1): 2^e > m
        if (f == 0.5) e -= 1;            // m is a power of two: s = m
    }
    *e_out = e;
    *scale_out = ldexpf(1.0f, 2 * e - 2 * kFirstBits);
}

// Digits of y = sqrt(w_k) {cos, sin}(2 pi t_ik) / s: D[d][i][kk] (cos) and D[d][i][kc + kk] (sin)
// for k = k0 + kk; zero for k >= K or i >= M (padding).  Phase and sincospi in float64, digits
// by exact float64 steps.
__global__ void wtilde_digits_kernel(const double* __restrict__ sigma, const double* __restrict__ uv,
                                     const double* __restrict__ grid, int64_t K, int64_t M, int64_t k0, int64_t kc,
                                     int64_t Mp, const int* __restrict__ e_dev, __nv_bfloat16* __restrict__ D) {
    const int64_t kk = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (kk >= kc) return;
    const int64_t k = k0 + kk;
    for (int64_t i = blockIdx.y; i < Mp; i += gridDim.y) {
    double yc = 0.0, ys = 0.0;
    if (k < K && i < M) {
        const double u = uv[2 * k], v = uv[2 * k + 1];
        const double t = fma(grid[2 * i + 1], u, grid[2 * i] * v);
        const double sw = 1.0 / fabs(sigma[k]);
        double sd, cd;
        sincospi(2.0 * t, &sd, &cd);
        const int e = *e_dev;
        yc = ldexp(cd * sw, kFirstBits - e);
        ys = ldexp(sd * sw, kFirstBits - e);
    }
    const int64_t Rc = 2 * kc;
    const int64_t plane = Mp * Rc;
    __nv_bfloat16* dc = D + i * Rc + kk;
    __nv_bfloat16* ds = dc + kc;
#pragma unroll
    for (int d = 0; d < kDigits; ++d) {
        const double qc = rint(yc), qs = rint(ys);
        dc[d * plane] = __float2bfloat16_rn(static_cast<float>(qc));
        ds[d * plane] = __float2bfloat16_rn(static_cast<float>(qs));
        yc = (yc - qc) * (double)(1 << kDigitBits);
        ys = (ys - qs) * (double)(1 << kDigitBits);
    }
    }
}

__global__ void poison_on_error_kernel(const int* __restrict__ err, float* __restrict__ out) {
    if (*err) out[0] = __int_as_float(0x7fc00000);
}

// ------------------------------------------------------------------ host

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

// the [nd][Mp][Rc] bf16 panel seen as boxes of {BK k, rows, nd}
int make_map(CUtensorMap* map, const void* D, int64_t Rc, int64_t Mp, int rows, int nd) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return AJ_ERR_CUDA;
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(Rc), static_cast<cuuint64_t>(Mp), static_cast<cuuint64_t>(nd)};
    const cuuint64_t strides[2] = {static_cast<cuuint64_t>(Rc) * 2, static_cast<cuuint64_t>(Mp * Rc) * 2};
    const cuuint32_t box[3] = {BK, static_cast<cuuint32_t>(rows), static_cast<cuuint32_t>(nd)};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(D), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? AJ_OK : AJ_ERR_CUDA;
}

template <int ND>
int set_smem_attr() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return AJ_OK;
    if (cudaFuncSetAttribute(digit_syrk_kernel<ND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(Cut<ND>::kSmemBytes)) != cudaSuccess)
        return AJ_ERR_CUDA;
    if (dev >= 0 && dev < 64) done[dev] = true;
    return AJ_OK;
}

// The lower block triangle of sum_L 2^-7L sum_{d+e=L} D_d D_e^T over the panel's Rc rows, for ND
// (kDigits or kInvDigits) digit planes.
template <int ND>
int launch_syrk(const void* D, int64_t Rc, int64_t M, int64_t Mp, float* oh, float* ol, int64_t ld,
                const float* scale_dev, const int* exps, int tri, int accumulate, int* err, cudaStream_t st,
                int split_rows = 0, float* o2h = nullptr, float* o2l = nullptr) {
    if (Rc <= 0 || Rc % kGroupRows != 0 || Mp % BM != 0 || Mp < M) return AJ_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(D) % 16 != 0) return AJ_ERR_ARG;
    CUtensorMap ma, mb;
    AJ_TRY(make_map(&ma, D, Rc, Mp, BM, ND));
    AJ_TRY(make_map(&mb, D, Rc, Mp, BN, ND));
    AJ_TRY(set_smem_attr<ND>());
    const int64_t nI = Mp / BM;
    if (split_rows < 0 || split_rows > nI || (split_rows > 0 && (!o2h || !o2l))) return AJ_ERR_ARG;
    const int64_t tiles = nI * (nI + 1) + static_cast<int64_t>(split_rows) * (split_rows + 1);
    digit_syrk_kernel<ND><<<static_cast<unsigned>(tiles), kThreads, Cut<ND>::kSmemBytes, st>>>(
        ma, mb, Rc, M, Mp, oh, ol, ld, scale_dev, exps, tri, split_rows, o2h, o2l, accumulate, err);
    return check_launch();
}

}  // namespace tc

// ------------------------------------------------ the mixed direct w_tilde

struct WtildeTcPlan {
    int64_t Mp, kc, Rc, nchunk;
    size_t digit_bytes;
};

WtildeTcPlan wtilde_tc_plan(int64_t K, int64_t M) {
    WtildeTcPlan p;
    p.Mp = (M + tc::BM - 1) / tc::BM * tc::BM;
    if (p.Mp == 0) p.Mp = tc::BM;
    // visibilities a chunk: the panel ([digits][Mp][2 kc] bf16) within 2 GiB, kc a multiple of half a group
    // (chunks of equal size, so the last one is not mostly padding)
    const int64_t half = tc::kGroupRows / 2;
    int64_t kmax = static_cast<int64_t>((size_t(2) << 30) / (size_t(tc::kDigits) * p.Mp * 2 * 2));
    kmax = kmax / half * half;
    if (kmax < half) kmax = half;
    const int64_t Kpos = K > 0 ? K : 1;
    p.nchunk = (Kpos + kmax - 1) / kmax;
    const int64_t per = (Kpos + p.nchunk - 1) / p.nchunk;
    p.kc = (per + half - 1) / half * half;
    p.Rc = 2 * p.kc;
    p.digit_bytes = size_t(tc::kDigits) * p.Mp * p.Rc * 2;
    return p;
}

size_t wtilde_tc_workspace_bytes(int64_t K, int64_t M) {
    WtildeTcPlan p = wtilde_tc_plan(K, M);
    Sizer s;
    s.take<char>(p.digit_bytes);
    s.take<unsigned long long>(1);
    s.take<int>(2);
    s.take<float>(1);
    return s.total();
}

// ph/pl (M x M, leading dimension M) receive the lower triangle of W as double-float planes.
int wtilde_tc(const double* sigma, const double* uv, const double* grid, int64_t K, int64_t M, float* ph, float* pl,
              void* ws, size_t bytes, cudaStream_t st) {
    WtildeTcPlan p = wtilde_tc_plan(K, M);
    if (bytes < wtilde_tc_workspace_bytes(K, M)) return AJ_ERR_WORKSPACE;
    Carver cv(ws, bytes);
    auto* D = cv.take<__nv_bfloat16>(p.digit_bytes / 2);
    auto* maxbits = cv.take<unsigned long long>(1);
    int* ints = cv.take<int>(2);  // [0] the scale exponent, [1] the error word
    float* scale = cv.take<float>(1);
    if (cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), st) != cudaSuccess ||
        cudaMemsetAsync(ints, 0, 2 * sizeof(int), st) != cudaSuccess)
        return AJ_ERR_CUDA;
    tc::max_inv_sigma_kernel<<<blocks_for(K, 256, 4 * num_sms()), 256, 0, st>>>(sigma, K, maxbits);
    AJ_LAUNCHED();
    tc::digit_scale_kernel<<<1, 1, 0, st>>>(maxbits, ints, scale);
    AJ_LAUNCHED();
    for (int64_t ch = 0; ch < p.nchunk; ++ch) {
        dim3 g(static_cast<unsigned>((p.kc + 255) / 256), static_cast<unsigned>(p.Mp < 65535 ? p.Mp : 65535));
        tc::wtilde_digits_kernel<<<g, 256, 0, st>>>(sigma, uv, grid, K, M, ch * p.kc, p.kc, p.Mp, ints, D);
        AJ_LAUNCHED();
        AJ_TRY(tc::launch_syrk<tc::kDigits>(D, p.Rc, M, p.Mp, ph, pl, M, scale, nullptr, 0, ch > 0 ? 1 : 0, ints + 1, st));
    }
    tc::poison_on_error_kernel<<<1, 1, 0, st>>>(ints + 1, ph);
    return check_launch();
}

// ------------------------------------------- A^-1 = L^-T L^-1 on the tensor cores
//
// With X = L^-1 (lower, double-float planes), A^-1[i][j] = sum_k X[k][i] X[k][j]: the product
// above with "pixels" the columns of X and the reduction over its rows.  Column i is cut into
// kInvDigits = 8 digits (55 bits) at its own power of two 2^e_i > max_k |X[k][i]|; a column of X
// has 2-norm sqrt(A^-1_ii), so an entry's truncation error stays below the double-float rounding
// of sum_k |X[k][i] X[k][j]|.  Rows k < i of X are zero, so a tile starts at the group holding its
// first row.

namespace tc {

struct LauumPlan {
    int64_t Sp, Rc;
};

LauumPlan lauum_plan(int64_t S) {
    LauumPlan p;
    p.Sp = (S + BM - 1) / BM * BM;
    p.Rc = (S + kGroupRows - 1) / kGroupRows * kGroupRows;  // >= Sp: every tile has a group to sum
    return p;
}

// colmax[i] = the bits of max_k |Xh[k][i]| (non-negative floats order as their bits)
__global__ void col_absmax_kernel(const float* __restrict__ Xh, int64_t S, unsigned* __restrict__ colmax) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= S) return;
    unsigned m = 0;
    for (int64_t k = blockIdx.y; k < S; k += gridDim.y) m = max(m, __float_as_uint(fabsf(Xh[k * S + i])));
    atomicMax(&colmax[i], m);
}

// 2^e > |x| for every x of a column whose largest |hi| has the bits m (0 for a zero column)
__device__ __forceinline__ int col_exp(unsigned m) {
    if (m == 0u) return 0;
    const int be = static_cast<int>((m >> 23) & 0xffu);
    return be > 0 ? be - 126 : -126;
}

// D[d][i][k] = digit d of X[k][i] 2^(kFirstBits - e_i) for k < Rc, i < Sp (zero outside S x S),
// through a 32 x 32 shared-memory transpose; blocks (0, y) also write e_i, block (0, 0) the scale.
__global__ void __launch_bounds__(256)
    lauum_digits_kernel(const float* __restrict__ Xh, const float* __restrict__ Xl, int64_t S, int64_t Sp, int64_t Rc,
                        const unsigned* __restrict__ colmax, int* __restrict__ exps, float* __restrict__ scale,
                        __nv_bfloat16* __restrict__ D) {
    __shared__ float th[32][33], tl[32][33];
    const int64_t k0 = blockIdx.x * 32ll, i0 = blockIdx.y * 32ll;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int64_t k = k0 + ty + 8 * r, i = i0 + tx;
        const bool in = k < S && i < S;
        th[ty + 8 * r][tx] = in ? Xh[k * S + i] : 0.f;
        tl[ty + 8 * r][tx] = in ? Xl[k * S + i] : 0.f;
    }
    if (blockIdx.x == 0 && ty == 0) {
        const int64_t i = i0 + tx;
        exps[i] = i < S ? col_exp(colmax[i]) : 0;
        if (blockIdx.y == 0 && tx == 0) *scale = ldexpf(1.0f, -2 * kFirstBits);
    }
    __syncthreads();
    const int64_t plane = Sp * Rc;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int il = ty + 8 * r;
        const int64_t i = i0 + il, k = k0 + tx;
        const int e = i < S ? col_exp(colmax[i]) : 0;
        // y = x 2^(kFirstBits - e), |y| < 2^kFirstBits; each digit leaves an exact remainder
        float yh = times_pow2(th[tx][il], kFirstBits - e), yl = times_pow2(tl[tx][il], kFirstBits - e);
        __nv_bfloat16* dst = D + i * Rc + k;
#pragma unroll
        for (int d = 0; d < kInvDigits; ++d) {
            const float q = rintf(yh);
            dst[d * plane] = __float2bfloat16_rn(q);
            float sh, se;
            two_sum(yh - q, yl, sh, se);
            yh = sh * static_cast<float>(1 << kDigitBits);
            yl = se * static_cast<float>(1 << kDigitBits);
        }
    }
}

// C += C2 on row i's lower triangle (j <= i), as double-float: the split tiles' second halves
__global__ void add_lower_kernel(const float* __restrict__ c2h, const float* __restrict__ c2l, int64_t S,
                                 float* __restrict__ ch, float* __restrict__ cl) {
    const int64_t i = blockIdx.y;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j > i) return;
    const int64_t o = i * S + j;
    const df v = df_add({ch[o], cl[o]}, {c2h[o], c2l[o]});
    ch[o] = v.hi;
    cl[o] = v.lo;
}

}  // namespace tc

size_t tc_lauum_workspace_bytes(int64_t S) {
    const tc::LauumPlan p = tc::lauum_plan(S);
    Sizer s;
    s.take<__nv_bfloat16>(size_t(tc::kInvDigits) * p.Sp * p.Rc);
    s.take<float>(2 * S * S);  // the second halves of the split tiles
    s.take<unsigned>(p.Sp);
    s.take<int>(p.Sp);
    s.take<int>(1);
    s.take<float>(1);
    return s.total();
}

// C's lower triangle (double-float planes, leading dimension S) = X^T X for the lower-triangular
// X; the upper triangle is left alone.  An expired wait inside the product leaves NaN in C[0][0].
int tc_lauum(const float* Xh, const float* Xl, int64_t S, float* Ch, float* Cl, void* ws, size_t bytes,
             cudaStream_t st) {
    if (S <= 0) return AJ_OK;
    if (bytes < tc_lauum_workspace_bytes(S)) return AJ_ERR_WORKSPACE;
    const tc::LauumPlan p = tc::lauum_plan(S);
    Carver cv(ws, bytes);
    auto* D = cv.take<__nv_bfloat16>(size_t(tc::kInvDigits) * p.Sp * p.Rc);
    float* C2 = cv.take<float>(2 * S * S);
    unsigned* colmax = cv.take<unsigned>(p.Sp);
    int* exps = cv.take<int>(p.Sp);
    int* err = cv.take<int>(1);
    float* scale = cv.take<float>(1);
    if (cudaMemsetAsync(colmax, 0, sizeof(unsigned) * p.Sp, st) != cudaSuccess ||
        cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess)
        return AJ_ERR_CUDA;
    const unsigned rows_split = static_cast<unsigned>(S < 64 ? S : 64);
    tc::col_absmax_kernel<<<dim3(static_cast<unsigned>((S + 255) / 256), rows_split), 256, 0, st>>>(Xh, S, colmax);
    AJ_LAUNCHED();
    tc::lauum_digits_kernel<<<dim3(static_cast<unsigned>(p.Rc / 32), static_cast<unsigned>(p.Sp / 32)), 256, 0, st>>>(
        Xh, Xl, S, p.Sp, p.Rc, colmax, exps, scale, D);
    AJ_LAUNCHED();
    // row tile I sums Rc / 256 - floor(I / 2) groups; the row tiles with 3 or more are split in two, so
    // the longest CTA sums about half the longest tile's groups (S = 1,500: 3 of 6 groups, 228 CTAs)
    const int64_t nI = p.Sp / tc::BM, ng = p.Rc / tc::kGroupRows;
    const int split_rows = static_cast<int>(std::min<int64_t>(nI, std::max<int64_t>(0, 2 * (ng - 3) + 2)));
    AJ_TRY(tc::launch_syrk<tc::kInvDigits>(D, p.Rc, S, p.Sp, Ch, Cl, S, scale, exps, 1, 0, err, st, split_rows, C2,
                                           C2 + S * S));
    if (split_rows > 0) {
        const int64_t rows = std::min<int64_t>(S, static_cast<int64_t>(split_rows) * tc::BM);
        tc::add_lower_kernel<<<dim3(static_cast<unsigned>((rows + 255) / 256), static_cast<unsigned>(rows)), 256, 0,
                               st>>>(C2, C2 + S * S, S, Ch, Cl);
        AJ_LAUNCHED();
    }
    tc::poison_on_error_kernel<<<1, 1, 0, st>>>(err, Ch);
    return check_launch();
}

}  // namespace aj

using namespace aj;

extern "C" {

int aj_digit_syrk_probe(const void* digits, int64_t rows, int64_t M, float* out_hi, float* out_lo,
                        const float* scale, int accumulate, int* err, void* stream) {
    if (!digits || !out_hi || !out_lo || !scale || !err || M <= 0 || rows <= 0) return AJ_ERR_ARG;
    const int64_t Mp = (M + tc::BM - 1) / tc::BM * tc::BM;
    return tc::launch_syrk<tc::kDigits>(digits, rows, M, Mp, out_hi, out_lo, M, scale, nullptr, 0, accumulate, err,
                           as_stream(stream));
}

}  // extern "C"
