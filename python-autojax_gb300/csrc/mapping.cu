// Mapping matrix, sparse mapping products and the regularisation matrix
// (numba.py:294-695, original.py:453-545, 600-700).
//
// The sparse (index, weight) rows of the mapping T (M x S, B entries a row)
// are turned on the device into a column-compressed transpose: for every
// source pixel s the list of (image pixel m, weight) that reference it,
// sorted by (m, b) so every sum runs in the reference's loop order.  Products
// with T^T then gather whole rows of the dense operand, coalesced, with no
// atomics.  Two row semantics exist in the reference and both are kept:
//   CSC_SUM    — every entry before the first -1 contributes (the sparse
//                products, numba.py:580-586, 543-548);
//   CSC_ASSIGN — a repeated index keeps only its last weight (the dense
//                mapping_matrix_from, numba.py:369-375).

#include "aj_internal.cuh"
#include "df32.cuh"

namespace aj {

// ------------------------------------------------------------- dense T

__global__ void mapping_dense_kernel(const int64_t* __restrict__ idx, const double* __restrict__ w, int64_t M,
                                     int64_t B, int64_t S, double* __restrict__ out, int* info) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t b = 0; b < B; ++b) {
            const int64_t s = idx[m * B + b];
            if (s == -1) break;
            if (s < 0 || s >= S) {
                report(info, AJ_INFO_INDEX_RANGE, m * B + b);
                continue;
            }
            out[m * S + s] = w[m * B + b];
        }
    }
}

// original.py:527-543: T[slim[i]][idx] += sub_fraction[slim[i]] * w over the first sizes[i] entries
__global__ void mapping_original_kernel(const int64_t* __restrict__ idx, const int64_t* __restrict__ sizes,
                                        const double* __restrict__ w, int64_t n_sub, int64_t B, int64_t S, int64_t M,
                                        const int64_t* __restrict__ slim, const double* __restrict__ frac,
                                        double* __restrict__ out, int* info) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_sub; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = slim[i];
        if (r < 0 || r >= M) {
            report(info, AJ_INFO_INDEX_RANGE, i);
            continue;
        }
        const int64_t nb = sizes[i] < B ? sizes[i] : B;
        for (int64_t b = 0; b < nb; ++b) {
            const int64_t s = idx[i * B + b];
            if (s < 0 || s >= S) {
                report(info, AJ_INFO_INDEX_RANGE, i * B + b);
                continue;
            }
            atomicAdd(&out[r * S + s], frac[r] * w[i * B + b]);
        }
    }
}

// D[s] = sum_m dirty[m] T[m][s]: 32 columns per block, 8 row groups, fixed-order reduction.
__global__ void data_vector_dense_kernel(const double* __restrict__ T, const double* __restrict__ d, int64_t M,
                                         int64_t S, double* __restrict__ out) {
    __shared__ double part[8][32];
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int64_t s = blockIdx.x * 32 + lane;
    double acc = 0.0;
    if (s < S)
        for (int64_t m = g; m < M; m += 8) acc = fma(d[m], T[m * S + s], acc);
    part[g][lane] = acc;
    __syncthreads();
    if (g == 0 && s < S) {
        double v = 0.0;
        for (int q = 0; q < 8; ++q) v += part[q][lane];
        out[s] = v;
    }
}

// ------------------------------------------------------------------ CSC

__device__ __forceinline__ bool csc_entry(const int64_t* idx, const int64_t* sizes, int64_t m, int64_t b, int64_t B,
                                          int64_t S, CscMode mode, int64_t& s, int* info) {
    const int64_t* row = idx + m * B;
    if (sizes) {
        const int64_t nb = sizes[m] < B ? sizes[m] : B;
        if (b >= nb) return false;
    } else {
        for (int64_t q = 0; q <= b; ++q)
            if (row[q] == -1) return false;
    }
    s = row[b];
    if (s < 0 || s >= S) {
        report(info, AJ_INFO_INDEX_RANGE, m * B + b);
        return false;
    }
    if (mode == CSC_ASSIGN) {
        const int64_t nb = sizes ? (sizes[m] < B ? sizes[m] : B) : B;
        for (int64_t q = b + 1; q < nb; ++q) {
            if (!sizes && row[q] == -1) break;
            if (row[q] == s) return false;  // overwritten by a later entry
        }
    }
    return true;
}

// Stable counting sort of the kept entries by source index, entries taken in
// (m, b) order: chunk c of CSC_CHUNK consecutive entries histograms its
// columns, a scan over (column, chunk) gives every chunk its write offset in
// each column, and each chunk then writes its entries in order.  Columns come
// out sorted by (m, b) — the reference's loop order — with no atomics on the
// output and no per-column sort, whatever the column lengths.
constexpr int CSC_CHUNK = 256;

__global__ void __launch_bounds__(256)
    csc_hist_kernel(const int64_t* __restrict__ idx, const int64_t* __restrict__ sizes, int64_t M, int64_t B,
                    int64_t S, CscMode mode, int* __restrict__ hist, int* info) {
    // hist[chunk][s]
    const int64_t c = blockIdx.x;
    const int64_t e0 = c * CSC_CHUNK, e1 = min(M * B, e0 + CSC_CHUNK);
    int* h = hist + c * S;
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        int64_t s;
        if (csc_entry(idx, sizes, e / B, e % B, B, S, mode, s, info)) atomicAdd(&h[s], 1);
    }
}

// colptr[s] = sum of all counts of columns < s; off[chunk][s] = colptr[s] + counts of earlier chunks
// Column pointers and per-chunk write offsets from the per-chunk histograms, in three passes so the
// long sums over chunks run spread over the GPU: per chunk-group column counts (part[g][s]), one
// block's exclusive scan over the columns (colptr, and each group's first offset back into part),
// then each group's chunks' offsets (off[c][s]).
constexpr int CSC_GROUPS = 8;

__global__ void csc_group_count_kernel(const int* __restrict__ hist, int64_t nchunk, int64_t S, int* __restrict__ part) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int64_t g = blockIdx.y, per = (nchunk + CSC_GROUPS - 1) / CSC_GROUPS;
    const int64_t c0 = g * per, c1 = min(nchunk, c0 + per);
    int t = 0;
    for (int64_t c = c0; c < c1; ++c) t += hist[c * S + s];
    part[g * S + s] = t;
}

__global__ void csc_scan_kernel(int64_t S, int* __restrict__ part, int* __restrict__ colptr) {
    __shared__ int warp_tot[32];
    __shared__ int base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t s0 = 0; s0 < S; s0 += blockDim.x) {
        const int64_t s = s0 + threadIdx.x;
        int cnt[CSC_GROUPS];
        int tot = 0;
#pragma unroll
        for (int g = 0; g < CSC_GROUPS; ++g) {
            cnt[g] = s < S ? part[g * S + s] : 0;
            tot += cnt[g];
        }
        int x = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        int before = 0;
        for (int w = 0; w < wid; ++w) before += warp_tot[w];
        if (s < S) {
            int run = base + before + x - tot;
            colptr[s] = run;
#pragma unroll
            for (int g = 0; g < CSC_GROUPS; ++g) {
                part[g * S + s] = run;
                run += cnt[g];
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < nw; ++w) t += warp_tot[w];
            base += t;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) colptr[S] = base;
}

__global__ void csc_group_offsets_kernel(const int* __restrict__ hist, int64_t nchunk, int64_t S,
                                         const int* __restrict__ part, int* __restrict__ off) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int64_t g = blockIdx.y, per = (nchunk + CSC_GROUPS - 1) / CSC_GROUPS;
    const int64_t c0 = g * per, c1 = min(nchunk, c0 + per);
    int run = part[g * S + s];
    for (int64_t c = c0; c < c1; ++c) {
        off[c * S + s] = run;
        run += hist[c * S + s];
    }
}

// one warp per chunk walks its entries in order; equal columns inside a
// 32-entry group are ranked with a match mask so writes stay in (m, b) order
__global__ void csc_place_kernel(const int64_t* __restrict__ idx, const double* __restrict__ w,
                                 const int64_t* __restrict__ sizes, int64_t M, int64_t B, int64_t S, CscMode mode,
                                 int* __restrict__ off, int* __restrict__ rows, double* __restrict__ vals,
                                 float2* __restrict__ vdf) {
    const int64_t c = blockIdx.x;
    const int lane = threadIdx.x;
    const int64_t e0 = c * CSC_CHUNK, e1 = min(M * B, e0 + CSC_CHUNK);
    int* cur = off + c * S;
    for (int64_t g = e0; g < e1; g += 32) {
        const int64_t e = g + lane;
        int64_t s = -1;
        const bool ok = e < e1 && csc_entry(idx, sizes, e / B, e % B, B, S, mode, s, nullptr);
        const int key = ok ? (int)s : -1 - lane;  // unique negative keys for skipped lanes
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        const int leader = __ffs(peers) - 1;
        int basepos = 0;
        if (ok && lane == leader) basepos = cur[s];
        basepos = __shfl_sync(0xffffffffu, basepos, leader);
        if (ok) {
            const double v = w[e];
            const df d = df_from(v);
            rows[basepos + rank] = static_cast<int>(e / B);
            vals[basepos + rank] = v;
            vdf[basepos + rank] = make_float2(d.hi, d.lo);
        }
        __syncwarp();
        if (ok && lane == leader) cur[s] = basepos + __popc(peers);
        __syncwarp();
    }
}

// out[s][c] = sum_e val[e] X[row[e]][c]; grid (S, column blocks), V columns per thread
template <typename Tin, typename Tout, int V>
__global__ void __launch_bounds__(256)
    csc_spmm_t_kernel(const int* __restrict__ colptr, const int* __restrict__ rows, const double* __restrict__ vals,
                      const Tin* __restrict__ X, int64_t ld_x, int64_t cols, Tout* __restrict__ out, int64_t ld_out) {
    using Acc = typename std::conditional<sizeof(Tin) == 8 || sizeof(Tout) == 8, double, float>::type;
    const int64_t s = blockIdx.x;
    const int64_t c0 = (blockIdx.y * (int64_t)blockDim.x + threadIdx.x) * V;
    if (c0 >= cols) return;
    const int b = colptr[s], e = colptr[s + 1];
    Acc acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = 0;
    const bool full = c0 + V <= cols;
    for (int q = b; q < e; ++q) {
        const Tin* xr = X + (int64_t)rows[q] * ld_x + c0;
        const Acc a = static_cast<Acc>(vals[q]);
        if (full) {
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v] = fma(a, static_cast<Acc>(__ldg(xr + v)), acc[v]);
        } else {
            for (int v = 0; v < V && c0 + v < cols; ++v) acc[v] = fma(a, static_cast<Acc>(__ldg(xr + v)), acc[v]);
        }
    }
    Tout* o = out + s * ld_out + c0;
    for (int v = 0; v < V && c0 + v < cols; ++v) o[v] = static_cast<Tout>(acc[v]);
}

// float4 fast path of the hot W T product: X rows 16-byte aligned, cols % 4 == 0
__global__ void __launch_bounds__(256)
    csc_spmm_t_f32x4_kernel(const int* __restrict__ colptr, const int* __restrict__ rows,
                            const float2* __restrict__ vdf, const float* __restrict__ X, int64_t ld_x, int64_t cols,
                            float* __restrict__ out, int64_t ld_out) {
    const int64_t s = blockIdx.x;
    const int64_t c0 = (blockIdx.y * (int64_t)blockDim.x + threadIdx.x) * 4;
    if (c0 >= cols) return;
    const int b = colptr[s], e = colptr[s + 1];
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int q = b; q < e; ++q) {
        const float4 x = __ldg(reinterpret_cast<const float4*>(X + (int64_t)rows[q] * ld_x + c0));
        const float a = vdf[q].x;
        acc.x = fmaf(a, x.x, acc.x);
        acc.y = fmaf(a, x.y, acc.y);
        acc.z = fmaf(a, x.z, acc.z);
        acc.w = fmaf(a, x.w, acc.w);
    }
    *reinterpret_cast<float4*>(out + s * ld_out + c0) = acc;
}

// double-float version for unaligned X or odd column counts: 4 consecutive
// columns per thread, scalar loads
__global__ void __launch_bounds__(256)
    csc_spmm_t_df_kernel(const int* __restrict__ colptr, const int* __restrict__ rows, const float2* __restrict__ vdf,
                         const float* __restrict__ Xh, const float* __restrict__ Xl, int64_t ld_x, int64_t cols,
                         float* __restrict__ Oh, float* __restrict__ Ol, int64_t ld_out, int lower) {
    const int64_t s = blockIdx.x;
    const int64_t c0 = (blockIdx.y * (int64_t)blockDim.x + threadIdx.x) * 4;
    if (c0 >= cols || (lower && c0 > s)) return;
    const int b = colptr[s], e = colptr[s + 1];
    df acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int q = b; q < e; ++q) {
        const float2 w = vdf[q];
        const df a = {w.x, w.y};
        const int64_t off = (int64_t)rows[q] * ld_x + c0;
        for (int v = 0; v < 4 && c0 + v < cols; ++v) df_fma_acc(acc[v], a, {__ldg(Xh + off + v), __ldg(Xl + off + v)});
    }
    for (int v = 0; v < 4 && c0 + v < cols; ++v) {
        Oh[s * ld_out + c0 + v] = acc[v].hi;
        Ol[s * ld_out + c0 + v] = acc[v].lo;
    }
}

// The float4 fast path of the double-float gather (X rows 16-byte aligned,
// cols % 4 == 0).  The block first stages its source pixel's entries (row and
// weight) in shared memory, so a row load waits on no index load; entries then
// go four at a time.  A group running past the column's end reads the segment's
// first row with weight 0, which adds exactly nothing.  Accumulation is lazy,
// renormalised every 8 entries, in entry order.  The one-pixel kernel keeps no
// second group of rows in flight: at 64 registers, 8 blocks an SM hide the
// latency better (measured 7 us per evaluation faster than the double-buffered
// form at 120 registers); the transposed kernel keeps it.
constexpr int kGatherStage = 128;  // entries staged per pass (a multiple of 8)

__device__ __forceinline__ void gather_group(const int* __restrict__ srow, const float2* __restrict__ sw,
                                             const float* __restrict__ Xh, const float* __restrict__ Xl,
                                             int64_t ld_x, int64_t c0, int q, int n, float4* h, float4* l,
                                             float2* a) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const bool in = q + u < n;
        const int qq = in ? q + u : 0;
        const int64_t off = (int64_t)srow[qq] * ld_x + c0;
        h[u] = __ldg(reinterpret_cast<const float4*>(Xh + off));
        l[u] = __ldg(reinterpret_cast<const float4*>(Xl + off));
        a[u] = in ? sw[qq] : make_float2(0.f, 0.f);
    }
}

__global__ void __launch_bounds__(128, 8)
    csc_spmm_t_df_vec_kernel(const int* __restrict__ colptr, const int* __restrict__ rows,
                             const float2* __restrict__ vdf, const float* __restrict__ Xh,
                             const float* __restrict__ Xl, int64_t ld_x, int64_t cols, float* __restrict__ Oh,
                             float* __restrict__ Ol, int64_t ld_out, int lower) {
    __shared__ int srow[kGatherStage];
    __shared__ float2 sw[kGatherStage];
    const int64_t s = blockIdx.x;
    if (lower && (int64_t)blockIdx.y * blockDim.x * 4 > s) return;  // the whole chunk is above the diagonal
    const int64_t c0 = (blockIdx.y * (int64_t)blockDim.x + threadIdx.x) * 4;
    const bool live = c0 < cols && (!lower || c0 <= s);
    const int b = colptr[s], e = colptr[s + 1];
    df acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    int group = 0;
    for (int seg = b; seg < e; seg += kGatherStage) {
        const int n = min(kGatherStage, e - seg);
        if (seg != b) __syncthreads();  // the previous pass's reads are done
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            srow[t] = rows[seg + t];
            sw[t] = vdf[seg + t];
        }
        __syncthreads();
        if (!live) continue;
        for (int q = 0; q < n; q += 4) {
            float4 h[4], l[4];
            float2 a[4];
            gather_group(srow, sw, Xh, Xl, ld_x, c0, q, n, h, l, a);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const df w = {a[u].x, a[u].y};
                df_fma_lazy(acc[0], w, {h[u].x, l[u].x});
                df_fma_lazy(acc[1], w, {h[u].y, l[u].y});
                df_fma_lazy(acc[2], w, {h[u].z, l[u].z});
                df_fma_lazy(acc[3], w, {h[u].w, l[u].w});
            }
            if (++group % 2 == 0)
#pragma unroll
                for (int v = 0; v < 4; ++v) df_renorm(acc[v]);
        }
    }
    if (!live) return;
#pragma unroll
    for (int v = 0; v < 4; ++v) df_renorm(acc[v]);
    *reinterpret_cast<float4*>(Oh + s * ld_out + c0) = make_float4(acc[0].hi, acc[1].hi, acc[2].hi, acc[3].hi);
    *reinterpret_cast<float4*>(Ol + s * ld_out + c0) = make_float4(acc[0].lo, acc[1].lo, acc[2].lo, acc[3].lo);
}

// The same gather with the output transposed (out[c][s], e.g. Omega = (T^T W)^T): a block takes
// 2 source pixels over one 512-column chunk, one pixel after another with the entry order, the
// grouping and the renormalisation of csc_spmm_t_df_vec_kernel (so each sum is bit-identical),
// keeps the results in shared memory and stores 2 consecutive pixels (8 bytes) per output row.
// With the grid pixel-fastest, (threads in flight x 4 columns x 2 pixels) / S columns of X are
// live at once, inside L2; 8 pixels a block (32-byte stores) kept 126 MB live at M = 9,504,
// S = 1,500 and read X 1.95 times from DRAM, 60 us slower per evaluation.
//
// The rows are latency-bound loads (long-scoreboard stalls, 24% warps active with a group of
// four entries double-buffered in registers).  Each thread instead streams its own 16-byte pieces
// of the next kTrDepth groups into a private ring in shared memory with cp.async (no registers
// held while they fly, no barrier: a thread reads only what it copied), so kTrDepth x 128 bytes a
// thread are in flight.  With the ring, 2 pixels a block (5 blocks an SM by shared memory)
// measured faster than 4 (4 blocks an SM).
constexpr int kTrPix = 2;
constexpr int kTrCols = 512;
constexpr int kTrThreads = kTrCols / 4;
constexpr int kTrDepth = 2;  // groups of four entries in flight a thread

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(smem))),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// ring[((slot * 4 + u) * 2 + plane) * kTrThreads + thread]: a warp's pieces of one entry and
// plane are 512 contiguous bytes
template <int D>
constexpr size_t tr_ring_bytes() {
    return sizeof(float4) * D * 4 * 2 * kTrThreads;
}

template <int D>
__global__ void __launch_bounds__(kTrThreads)
    csc_spmm_t_df_tr_kernel(const int* __restrict__ colptr, const int* __restrict__ rows,
                            const float2* __restrict__ vdf, const float* __restrict__ Xh,
                            const float* __restrict__ Xl, int64_t ld_x, int64_t cols, int64_t S,
                            float* __restrict__ Oh, float* __restrict__ Ol, int64_t ld_out) {
    extern __shared__ float4 ring[];
    __shared__ int srow[kGatherStage];
    __shared__ float2 sw[kGatherStage];
    __shared__ float th[kTrPix][kTrCols], tl[kTrPix][kTrCols];
    const int64_t s0 = (int64_t)blockIdx.x * kTrPix;
    const int64_t cbase = (int64_t)blockIdx.y * kTrCols;
    const int tid = threadIdx.x;
    const int cl = tid * 4;
    const int64_t c0 = cbase + cl;
    const bool live = c0 < cols;
    // copies group q's four entries (a group past the column's end repeats the segment's first
    // row, which then meets weight 0) into ring slot q % D
    auto issue = [&](int q, int n) {
        float4* base = ring + (q % D) * 4 * 2 * kTrThreads + tid;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int qq = q * 4 + u < n ? q * 4 + u : 0;
            const int64_t off = (int64_t)srow[qq] * ld_x + c0;
            cp_async16(base + (u * 2 + 0) * kTrThreads, Xh + off);
            cp_async16(base + (u * 2 + 1) * kTrThreads, Xl + off);
        }
    };
    for (int sp = 0; sp < kTrPix; ++sp) {
        const int64_t s = s0 + sp;
        if (s >= S) break;
        df acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        const int b = colptr[s], e = colptr[s + 1];
        int group = 0;
        for (int seg = b; seg < e; seg += kGatherStage) {
            const int n = min(kGatherStage, e - seg);
            __syncthreads();  // the previous pass's reads of the staged entries are done
            for (int t = tid; t < n; t += blockDim.x) {
                srow[t] = rows[seg + t];
                sw[t] = vdf[seg + t];
            }
            __syncthreads();
            if (!live) continue;
            const int ng = (n + 3) / 4;
#pragma unroll
            for (int q = 0; q < D; ++q) {
                if (q < ng) issue(q, n);
                cp_async_commit();  // one group a step, empty or not, so the wait counts stay fixed
            }
            for (int q = 0; q < ng; ++q) {
                cp_async_wait<D - 1>();  // this thread's copies of group q have landed
                const float4* base = ring + (q % D) * 4 * 2 * kTrThreads + tid;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4 h = base[(u * 2 + 0) * kTrThreads];
                    const float4 l = base[(u * 2 + 1) * kTrThreads];
                    const float2 a2 = q * 4 + u < n ? sw[q * 4 + u] : make_float2(0.f, 0.f);
                    const df w = {a2.x, a2.y};
                    df_fma_lazy(acc[0], w, {h.x, l.x});
                    df_fma_lazy(acc[1], w, {h.y, l.y});
                    df_fma_lazy(acc[2], w, {h.z, l.z});
                    df_fma_lazy(acc[3], w, {h.w, l.w});
                }
                if (++group % 2 == 0)
#pragma unroll
                    for (int v = 0; v < 4; ++v) df_renorm(acc[v]);
                // the slot's values are in registers and consumed: refill it
                if (q + D < ng) issue(q + D, n);
                cp_async_commit();
            }
        }
        if (live) {
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                df_renorm(acc[v]);
                th[sp][cl + v] = acc[v].hi;
                tl[sp][cl + v] = acc[v].lo;
            }
        }
    }
    cp_async_wait<0>();
    __syncthreads();
    const int np = (int)(S - s0 < kTrPix ? S - s0 : kTrPix);
    const bool vec = np == kTrPix && ld_out % 2 == 0 && s0 % 2 == 0;
    for (int r = tid; r < kTrCols; r += blockDim.x) {
        const int64_t c = cbase + r;
        if (c >= cols) break;
        float* oh = Oh + c * ld_out + s0;
        float* ol = Ol + c * ld_out + s0;
        if (vec) {
            reinterpret_cast<float2*>(oh)[0] = make_float2(th[0][r], th[1][r]);
            reinterpret_cast<float2*>(ol)[0] = make_float2(tl[0][r], tl[1][r]);
        } else {
            for (int sp = 0; sp < np; ++sp) {
                oh[sp] = th[sp][r];
                ol[sp] = tl[sp][r];
            }
        }
    }
}

__global__ void csc_spmv_t_kernel(const int* __restrict__ colptr, const int* __restrict__ rows,
                                  const double* __restrict__ vals, int64_t S, const double* __restrict__ x,
                                  double* __restrict__ out) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < S; s += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int q = colptr[s]; q < colptr[s + 1]; ++q) acc = fma(vals[q], x[rows[q]], acc);
        out[s] = acc;
    }
}

// TW[s][m1] = sum_e val[e] Wc(m1, m2 = row[e]) with the compact lookup of numba.py:538-541.
// Persistent over (s, 1024-column chunk) items so each block loads the table once.
template <typename T, bool SMEM>
__global__ void __launch_bounds__(256)
    csc_compact_tw_kernel(const int* __restrict__ colptr, const int* __restrict__ rows,
                          const double* __restrict__ vals, int64_t S, const double* __restrict__ wc, int64_t N,
                          const int64_t* __restrict__ nat, int64_t M, T* __restrict__ TW, int* info) {
    extern __shared__ unsigned char smem_raw[];
    T* tab = reinterpret_cast<T*>(smem_raw);
    const int64_t W = 2 * N - 1;
    const T* tsrc;
    if constexpr (SMEM) {
        for (int64_t t = threadIdx.x; t < N * W; t += blockDim.x) tab[t] = static_cast<T>(wc[t]);
        __syncthreads();
        tsrc = tab;
    }
    const int64_t chunks = (M + 1023) / 1024;
    const int64_t items = S * chunks;
    for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        const int64_t s = it / chunks, ch = it - s * chunks;
        int64_t r1[4], c1[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int64_t m1 = ch * 1024 + v * 256 + threadIdx.x;
            r1[v] = m1 < M ? nat[2 * m1] : 0;
            c1[v] = m1 < M ? nat[2 * m1 + 1] : 0;
        }
        T acc[4] = {0, 0, 0, 0};
        for (int q = colptr[s]; q < colptr[s + 1]; ++q) {
            const int64_t m2 = rows[q];
            const int64_t r2 = nat[2 * m2], c2 = nat[2 * m2 + 1];
            const T a = static_cast<T>(vals[q]);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const int64_t n1 = r1[v] - r2;
                const int64_t n2 = (n1 >= 0 ? c1[v] - c2 : c2 - c1[v]) + (N - 1);
                const int64_t ar = n1 < 0 ? -n1 : n1;
                T wv = 0;
                if (ar < N && n2 >= 0 && n2 < W) {
                    if constexpr (SMEM)
                        wv = tsrc[ar * W + n2];
                    else
                        wv = static_cast<T>(__ldg(wc + ar * W + n2));
                } else if (ch * 1024 + v * 256 + threadIdx.x < M) {
                    report(info, AJ_INFO_INDEX_RANGE, m2);
                }
                acc[v] = fma(a, wv, acc[v]);
            }
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int64_t m1 = ch * 1024 + v * 256 + threadIdx.x;
            if (m1 < M) TW[s * M + m1] = acc[v];
        }
    }
}

// symmetric expansion of original.py's preload pairs: W[i][j] = preload[yb - ya][xb - xa], (a, b) = (min, max)
__global__ void expand_preload_sym_kernel(const double* __restrict__ pre, int64_t py, int64_t px,
                                          const int64_t* __restrict__ nat, int64_t M, double* __restrict__ out,
                                          int* info) {
    for (int64_t i = blockIdx.y; i < M; i += gridDim.y) {
        for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
            const int64_t a = i < j ? i : j, b = i < j ? j : i;
            int64_t r = nat[2 * b] - nat[2 * a], c = nat[2 * b + 1] - nat[2 * a + 1];
            if (r < 0) r += py;
            if (c < 0) c += px;
            double v = 0.0;
            if (r >= 0 && r < py && c >= 0 && c < px)
                v = pre[r * px + c];
            else
                report(info, AJ_INFO_INDEX_RANGE, i * M + j);
            out[i * M + j] = v;
        }
    }
}

// -------------------------------------------------------- regularisation

// numba.py:686-694: diag(1e-8 + c^2 n_i), then H[i][k] -= c^2 along the row until -1
__global__ void regularization_kernel(double coef, const double* __restrict__ coef_dev, const int64_t* __restrict__ nb,
                                      const int64_t* __restrict__ nsz, int64_t S, int64_t P, double* __restrict__ H,
                                      int* info) {
    const double c = coef_dev ? *coef_dev : coef;
    const double c2 = c * c;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S; i += (int64_t)gridDim.x * blockDim.x) {
        H[i * S + i] = __dadd_rn(1e-8, __dmul_rn(c2, (double)nsz[i]));
        for (int64_t j = 0; j < P; ++j) {
            const int64_t k = nb[i * P + j];
            if (k == -1) break;
            if (k < 0 || k >= S) {
                report(info, AJ_INFO_INDEX_RANGE, i * P + j);
                continue;
            }
            H[i * S + k] = __dsub_rn(H[i * S + k], c2);
        }
    }
}

// ------------------------------------------------------------ host side

int regularization(double coefficient, const double* coefficient_dev, const int64_t* neighbors,
                   const int64_t* neighbors_sizes, int64_t S, int64_t P, double* out, int* info, cudaStream_t st) {
    if (cudaMemsetAsync(out, 0, sizeof(double) * S * S, st) != cudaSuccess) return AJ_ERR_CUDA;
    regularization_kernel<<<blocks_for(S, 128, 8 * num_sms()), 128, 0, st>>>(coefficient, coefficient_dev, neighbors,
                                                                           neighbors_sizes, S, P, out, info);
    return check_launch();
}

inline int64_t csc_chunks(int64_t M, int64_t B) { return (M * B + CSC_CHUNK - 1) / CSC_CHUNK; }

size_t csc_bytes(int64_t M, int64_t B, int64_t S) {
    const int64_t nch = csc_chunks(M, B) > 0 ? csc_chunks(M, B) : 1;
    Sizer s;
    s.take<int>(S + 1);
    s.take<int>(M * B);
    s.take<double>(M * B);
    s.take<float2>(M * B);
    s.take<int>(nch * S);  // hist
    s.take<int>(nch * S);  // offsets / cursors
    s.take<int>(CSC_GROUPS * S);  // chunk-group counts / offsets
    return s.total();
}

void csc_take(Carver& cv, int64_t M, int64_t B, int64_t S, Csc& c) {
    const int64_t nch = csc_chunks(M, B) > 0 ? csc_chunks(M, B) : 1;
    c.colptr = cv.take<int>(S + 1);
    c.rows = cv.take<int>(M * B);
    c.vals = cv.take<double>(M * B);
    c.vdf = cv.take<float2>(M * B);
    c.keys = cv.take<int>(nch * S);
    c.cursor = cv.take<int>(nch * S);
    c.part = cv.take<int>(CSC_GROUPS * S);
}

int csc_build(const int64_t* idx, const double* w, const int64_t* sizes, int64_t M, int64_t B, int64_t S, CscMode mode,
              Csc& c, int* info, cudaStream_t st) {
    const int64_t nch = csc_chunks(M, B);
    if (nch == 0) return cudaMemsetAsync(c.colptr, 0, sizeof(int) * (S + 1), st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    int* hist = c.keys;
    int* off = c.cursor;
    if (cudaMemsetAsync(hist, 0, sizeof(int) * nch * S, st) != cudaSuccess) return AJ_ERR_CUDA;
    csc_hist_kernel<<<(unsigned)nch, 256, 0, st>>>(idx, sizes, M, B, S, mode, hist, info);
    AJ_LAUNCHED();
    const dim3 gg(static_cast<unsigned>((S + 127) / 128), CSC_GROUPS);
    csc_group_count_kernel<<<gg, 128, 0, st>>>(hist, nch, S, c.part);
    AJ_LAUNCHED();
    csc_scan_kernel<<<1, 1024, 0, st>>>(S, c.part, c.colptr);
    AJ_LAUNCHED();
    csc_group_offsets_kernel<<<gg, 128, 0, st>>>(hist, nch, S, c.part, off);
    AJ_LAUNCHED();
    csc_place_kernel<<<(unsigned)nch, 32, 0, st>>>(idx, w, sizes, M, B, S, mode, off, c.rows, c.vals, c.vdf);
    return check_launch();
}

template <typename Tin, typename Tout>
int csc_spmm_t(const Csc& c, int64_t S, const Tin* X, int64_t ld_x, int64_t cols, Tout* out, int64_t ld_out,
               cudaStream_t st) {
    if (S == 0 || cols == 0) return AJ_OK;
    if constexpr (sizeof(Tin) == 4 && sizeof(Tout) == 4) {
        const bool aligned = (cols % 4 == 0) && (ld_x % 4 == 0) && (ld_out % 4 == 0) &&
                             (reinterpret_cast<uintptr_t>(X) % 16 == 0) && (reinterpret_cast<uintptr_t>(out) % 16 == 0);
        if (aligned) {
            dim3 grid((unsigned)S, (unsigned)((cols / 4 + 255) / 256));
            csc_spmm_t_f32x4_kernel<<<grid, 256, 0, st>>>(c.colptr, c.rows, c.vdf, X, ld_x, cols, out, ld_out);
            return check_launch();
        }
    }
    constexpr int V = 2;
    dim3 grid((unsigned)S, (unsigned)((cols + 256 * V - 1) / (256 * V)));
    csc_spmm_t_kernel<Tin, Tout, V><<<grid, 256, 0, st>>>(c.colptr, c.rows, c.vals, X, ld_x, cols, out, ld_out);
    return check_launch();
}

template int csc_spmm_t<double, double>(const Csc&, int64_t, const double*, int64_t, int64_t, double*, int64_t,
                                        cudaStream_t);
template int csc_spmm_t<float, float>(const Csc&, int64_t, const float*, int64_t, int64_t, float*, int64_t,
                                      cudaStream_t);
template int csc_spmm_t<float, double>(const Csc&, int64_t, const float*, int64_t, int64_t, double*, int64_t,
                                       cudaStream_t);

int csc_spmm_t_df(const Csc& c, int64_t S, const float* Xh, const float* Xl, int64_t ld_x, int64_t cols, float* Oh,
                  float* Ol, int64_t ld_out, cudaStream_t st, bool lower) {
    if (S == 0 || cols == 0) return AJ_OK;
    // 512-column chunks: under 3% idle threads at both M = 9,504 and S = 1,500, and a chunk's
    // rows of X (M x 512 x 8 bytes) stay in L2 while every source pixel gathers from them
    dim3 grid((unsigned)S, (unsigned)((cols / 4 + 1 + 127) / 128));
    const bool vec = (cols % 4 == 0) && (ld_x % 4 == 0) && (ld_out % 4 == 0) &&
                     (reinterpret_cast<uintptr_t>(Xh) % 16 == 0) && (reinterpret_cast<uintptr_t>(Xl) % 16 == 0) &&
                     (reinterpret_cast<uintptr_t>(Oh) % 16 == 0) && (reinterpret_cast<uintptr_t>(Ol) % 16 == 0);
    if (vec)
        csc_spmm_t_df_vec_kernel<<<grid, 128, 0, st>>>(c.colptr, c.rows, c.vdf, Xh, Xl, ld_x, cols, Oh, Ol, ld_out,
                                                       lower ? 1 : 0);
    else
        csc_spmm_t_df_kernel<<<grid, 128, 0, st>>>(c.colptr, c.rows, c.vdf, Xh, Xl, ld_x, cols, Oh, Ol, ld_out,
                                                   lower ? 1 : 0);
    return check_launch();
}

int csc_spmm_t_df_tr(const Csc& c, int64_t S, const float* Xh, const float* Xl, int64_t ld_x, int64_t cols, float* Oh,
                     float* Ol, int64_t ld_out, cudaStream_t st) {
    if (S == 0 || cols == 0) return AJ_OK;
    const bool vec = (cols % 4 == 0) && (ld_x % 4 == 0) && (reinterpret_cast<uintptr_t>(Xh) % 16 == 0) &&
                     (reinterpret_cast<uintptr_t>(Xl) % 16 == 0) && (reinterpret_cast<uintptr_t>(Oh) % 16 == 0) &&
                     (reinterpret_cast<uintptr_t>(Ol) % 16 == 0);
    if (!vec) return AJ_ERR_ARG;
    static bool attr[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    if (dev < 64 && !attr[dev]) {
        if (cudaFuncSetAttribute(csc_spmm_t_df_tr_kernel<kTrDepth>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tr_ring_bytes<kTrDepth>()) != cudaSuccess)
            return AJ_ERR_CUDA;
        attr[dev] = true;
    }
    dim3 grid((unsigned)((S + kTrPix - 1) / kTrPix), (unsigned)((cols + kTrCols - 1) / kTrCols));
    csc_spmm_t_df_tr_kernel<kTrDepth><<<grid, kTrThreads, tr_ring_bytes<kTrDepth>(), st>>>(
        c.colptr, c.rows, c.vdf, Xh, Xl, ld_x, cols, S, Oh, Ol, ld_out);
    return check_launch();
}

int csc_spmv_t(const Csc& c, int64_t S, const double* x, double* out, cudaStream_t st) {
    csc_spmv_t_kernel<<<blocks_for(S, 256, 4 * num_sms()), 256, 0, st>>>(c.colptr, c.rows, c.vals, S, x, out);
    return check_launch();
}

template <typename T>
int csc_compact_tw(const Csc& c, int64_t S, const double* w_compact, int64_t N, const int64_t* native, int64_t M,
                   T* TW, int* info, cudaStream_t st) {
    const size_t tab_bytes = sizeof(T) * N * (2 * N - 1);
    const int64_t items = S * ((M + 1023) / 1024);
    const size_t smem_cap = 200 * 1024;
    if (tab_bytes <= smem_cap) {
        static bool set[2][64] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 64 && !set[sizeof(T) == 8][dev]) {
            if (cudaFuncSetAttribute(csc_compact_tw_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem_cap) != cudaSuccess)
                return AJ_ERR_CUDA;
            set[sizeof(T) == 8][dev] = true;
        }
        const int per_sm = tab_bytes <= 100 * 1024 ? 2 : 1;
        int64_t g = (int64_t)num_sms() * per_sm;
        if (g > items) g = items;
        csc_compact_tw_kernel<T, true><<<(unsigned)g, 256, tab_bytes, st>>>(c.colptr, c.rows, c.vals, S, w_compact, N,
                                                                            native, M, TW, info);
    } else {
        int64_t g = (int64_t)num_sms() * 4;
        if (g > items) g = items;
        csc_compact_tw_kernel<T, false><<<(unsigned)g, 256, 0, st>>>(c.colptr, c.rows, c.vals, S, w_compact, N, native,
                                                                     M, TW, info);
    }
    return check_launch();
}

template int csc_compact_tw<double>(const Csc&, int64_t, const double*, int64_t, const int64_t*, int64_t, double*, int*,
                                    cudaStream_t);
template int csc_compact_tw<float>(const Csc&, int64_t, const double*, int64_t, const int64_t*, int64_t, float*, int*,
                                   cudaStream_t);

}  // namespace aj

using namespace aj;

namespace {

// F = T^T (T^T X^T)^T for a symmetric-or-not M x M X: TW = T^T X, Omega = TW^T, F = T^T Omega.
int curvature_from_square(const Csc& c, int64_t S, const double* X, int64_t M, double* TW, double* Om, double* out,
                          cudaStream_t st) {
    AJ_TRY(csc_spmm_t<double, double>(c, S, X, M, M, TW, M, st));
    AJ_TRY(transpose<double>(TW, S, M, Om, st));
    return csc_spmm_t<double, double>(c, S, Om, S, S, out, S, st);
}

}  // namespace

extern "C" {

int aj_mapping_matrix(const int64_t* pix_indexes, const double* pix_weights, int64_t M, int64_t B, int64_t S,
                      double* out, int* info, void* stream) {
    if (M < 0 || B < 0 || S < 0) return AJ_ERR_ARG;
    if (M == 0 || S == 0) return AJ_OK;
    if (!out || (B > 0 && (!pix_indexes || !pix_weights))) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(out, 0, sizeof(double) * M * S, st) != cudaSuccess) return AJ_ERR_CUDA;
    if (B == 0) return AJ_OK;
    mapping_dense_kernel<<<blocks_for(M, 128, 8 * num_sms()), 128, 0, st>>>(pix_indexes, pix_weights, M, B, S, out,
                                                                          info);
    return check_launch();
}

int aj_mapping_matrix_original(const int64_t* pix_indexes, const int64_t* pix_sizes, const double* pix_weights,
                               int64_t n_sub, int64_t B, int64_t S, int64_t M, const int64_t* slim_index,
                               const double* sub_fraction, double* out, int* info, void* stream) {
    if (n_sub < 0 || B < 0 || S < 0 || M < 0) return AJ_ERR_ARG;
    if (M == 0 || S == 0) return AJ_OK;
    if (!out) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(out, 0, sizeof(double) * M * S, st) != cudaSuccess) return AJ_ERR_CUDA;
    if (n_sub == 0 || B == 0) return AJ_OK;
    if (!pix_indexes || !pix_sizes || !pix_weights || !slim_index || !sub_fraction) return AJ_ERR_ARG;
    mapping_original_kernel<<<blocks_for(n_sub, 128, 8 * num_sms()), 128, 0, st>>>(
        pix_indexes, pix_sizes, pix_weights, n_sub, B, S, M, slim_index, sub_fraction, out, info);
    return check_launch();
}

int aj_data_vector(const double* mapping_matrix, const double* dirty_image, int64_t M, int64_t S, double* out,
                   void* stream) {
    if (M < 0 || S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!out || (M > 0 && (!mapping_matrix || !dirty_image))) return AJ_ERR_ARG;
    data_vector_dense_kernel<<<blocks_for(S, 32), 256, 0, as_stream(stream)>>>(mapping_matrix, dirty_image, M, S, out);
    return check_launch();
}

size_t aj_curvature_dense_workspace_size(int64_t M, int64_t S) { return align_up(sizeof(double) * M * S); }

int aj_curvature_dense(const double* w_tilde, const double* mapping_matrix, int64_t M, int64_t S, double* out,
                       void* workspace, size_t workspace_bytes, void* stream) {
    if (M < 0 || S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!out || (M > 0 && (!w_tilde || !mapping_matrix))) return AJ_ERR_ARG;
    if (workspace_bytes < aj_curvature_dense_workspace_size(M, S) || (M > 0 && !workspace)) return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    double* WT = static_cast<double*>(workspace);
    // numba.py:435: T^T (W T)
    AJ_TRY(gemm_f64(false, false, M, S, M, 1.0, w_tilde, M, mapping_matrix, S, 0.0, WT, S, false, st));
    return gemm_f64(true, false, S, S, M, 1.0, mapping_matrix, S, WT, S, 0.0, out, S, false, st);
}

size_t aj_sparse_workspace_size(int64_t M, int64_t B, int64_t S, int64_t cols) {
    Sizer s;
    s.take<char>(csc_bytes(M, B, S));
    s.take<double>(S * (cols > M ? cols : M));  // TW
    s.take<double>((M > S ? M : S) * (cols > S ? cols : S));  // Omega / transposes
    return s.total();
}

int aj_sparse_mapping_matrix_transpose_matmul(const double* matrix, int64_t M, int64_t cols,
                                              const int64_t* pix_indexes, const double* pix_weights, int64_t B,
                                              int64_t S, double* out, void* workspace, size_t workspace_bytes,
                                              int* info, void* stream) {
    if (M < 0 || cols < 0 || B < 0 || S < 0) return AJ_ERR_ARG;
    if (S == 0 || cols == 0) return AJ_OK;
    if (!out || (M > 0 && (!matrix || (B > 0 && (!pix_indexes || !pix_weights))))) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < csc_bytes(M, B, S)) return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace, workspace_bytes);
    Csc c;
    csc_take(cv, M, B, S, c);
    AJ_TRY(csc_build(pix_indexes, pix_weights, nullptr, M, B, S, CSC_SUM, c, info, st));
    return csc_spmm_t<double, double>(c, S, matrix, cols, cols, out, cols, st);
}

int aj_curvature_w_tilde_sparse(const double* w_tilde, int64_t M, const int64_t* pix_indexes,
                                const double* pix_weights, int64_t B, int64_t S, double* out, void* workspace,
                                size_t workspace_bytes, int* info, void* stream) {
    if (M < 0 || B < 0 || S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!out || (M > 0 && (!w_tilde || !pix_indexes || !pix_weights))) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < aj_sparse_workspace_size(M, B, S, M)) return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace, workspace_bytes);
    Csc c;
    csc_take(cv, M, B, S, c);
    double* TW = cv.take<double>(S * M);
    double* Om = cv.take<double>(M * S);
    AJ_TRY(csc_build(pix_indexes, pix_weights, nullptr, M, B, S, CSC_SUM, c, info, st));
    return curvature_from_square(c, S, w_tilde, M, TW, Om, out, st);
}

int aj_w_compact_matmul_sparse(const double* w_compact, int64_t N, const int64_t* native_index, int64_t M,
                               const int64_t* pix_indexes, const double* pix_weights, int64_t B, int64_t S,
                               double* out, void* workspace, size_t workspace_bytes, int* info, void* stream) {
    if (N <= 0 || M < 0 || B < 0 || S < 0) return AJ_ERR_ARG;
    if (M == 0 || S == 0) return AJ_OK;
    if (!out || !w_compact || !native_index || !pix_indexes || !pix_weights) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < aj_sparse_workspace_size(M, B, S, M)) return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Carver cv(workspace, workspace_bytes);
    Csc c;
    csc_take(cv, M, B, S, c);
    double* TW = cv.take<double>(S * M);
    AJ_TRY(csc_build(pix_indexes, pix_weights, nullptr, M, B, S, CSC_SUM, c, info, st));
    AJ_TRY(csc_compact_tw<double>(c, S, w_compact, N, native_index, M, TW, info, st));
    return transpose<double>(TW, S, M, out, st);
}

int aj_curvature_w_compact_sparse(const double* w_compact, int64_t N, const int64_t* native_index, int64_t M,
                                  const int64_t* pix_indexes, const double* pix_weights, int64_t B, int64_t S,
                                  double* out, void* workspace, size_t workspace_bytes, int* info, void* stream) {
    if (N <= 0 || M < 0 || B < 0 || S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!out) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (M == 0) return cudaMemsetAsync(out, 0, sizeof(double) * S * S, st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    if (!w_compact || !native_index || !pix_indexes || !pix_weights) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < aj_sparse_workspace_size(M, B, S, M)) return AJ_ERR_WORKSPACE;
    Carver cv(workspace, workspace_bytes);
    Csc c;
    csc_take(cv, M, B, S, c);
    double* TW = cv.take<double>(S * M);
    double* Om = cv.take<double>(M * S);
    AJ_TRY(csc_build(pix_indexes, pix_weights, nullptr, M, B, S, CSC_SUM, c, info, st));
    AJ_TRY(csc_compact_tw<double>(c, S, w_compact, N, native_index, M, TW, info, st));
    AJ_TRY(transpose<double>(TW, S, M, Om, st));
    return csc_spmm_t<double, double>(c, S, Om, S, S, out, S, st);
}

size_t aj_curvature_preload_original_workspace_size(int64_t M, int64_t B, int64_t S) {
    Sizer need;
    need.take<char>(aj_sparse_workspace_size(M, B, S, M));
    need.take<double>(M * M);
    return need.total();
}

int aj_curvature_preload_original(const double* preload, int64_t py, int64_t px, const int64_t* pix_indexes,
                                  const int64_t* pix_sizes, const double* pix_weights, int64_t B,
                                  const int64_t* native_index, int64_t M, int64_t S, double* out,
                                  void* workspace, size_t workspace_bytes, int* info, void* stream) {
    if (py <= 0 || px <= 0 || M < 0 || B < 0 || S < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!out) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (M == 0) return cudaMemsetAsync(out, 0, sizeof(double) * S * S, st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    if (!preload || !native_index || !pix_indexes || !pix_sizes || !pix_weights) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < aj_curvature_preload_original_workspace_size(M, B, S)) return AJ_ERR_WORKSPACE;
    Carver cv(workspace, workspace_bytes);
    Csc c;
    csc_take(cv, M, B, S, c);
    double* TW = cv.take<double>(S * M);
    double* Om = cv.take<double>(M * S);
    double* W = cv.take<double>(M * M);
    AJ_TRY(csc_build(pix_indexes, pix_weights, pix_sizes, M, B, S, CSC_SUM, c, info, st));
    // original.py's upper pairs + mirror + diagonal == T^T W_sym T with W_sym[i][j] = preload[yb-ya][xb-xa]
    dim3 grid(blocks_for(M, 256, 64), (unsigned)(M < 65535 ? M : 65535));
    expand_preload_sym_kernel<<<grid, 256, 0, st>>>(preload, py, px, native_index, M, W, info);
    AJ_LAUNCHED();
    return curvature_from_square(c, S, W, M, TW, Om, out, st);
}

int aj_constant_regularization(double coefficient, const int64_t* neighbors, const int64_t* neighbors_sizes,
                               int64_t S, int64_t P, double* out, int* info, void* stream) {
    if (S < 0 || P < 0) return AJ_ERR_ARG;
    if (S == 0) return AJ_OK;
    if (!out || !neighbors_sizes || (P > 0 && !neighbors)) return AJ_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(out, 0, sizeof(double) * S * S, st) != cudaSuccess) return AJ_ERR_CUDA;
    regularization_kernel<<<blocks_for(S, 128, 8 * num_sms()), 128, 0, st>>>(coefficient, nullptr, neighbors,
                                                                           neighbors_sizes, S, P, out, info);
    return check_launch();
}

}  // extern "C"
