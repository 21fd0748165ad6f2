// The log-evidence of one lens-model evaluation and its adjoint
// (numba.py:761-857, 866-967; the gradient has no reference counterpart).
//
//   logE = -1/2 [ chi.chi - s.D + log|A| - log|H| + norm ],  A = F + H,
//   F = T^T W T,  D = T^T dirty,  s = A^-1 D,  H = 1e-8 I + lambda L.
// With Omega = W T:
//   dlogE/dlambda  = -1/2 [ s^T L s + tr(A^-1 L) - tr(H^-1 L) ],
//                     tr(H^-1 L) = (S - 1e-8 tr(H^-1)) / lambda  (H^-1 L = (I - 1e-8 H^-1) / lambda),
//   dlogE/dT[m, j] = dirty_m s_j - (Omega s)_m s_j - (Omega A^-1)[m, j],
// read on the sparse pattern of the weights.  The w_tilde likelihood builds
// both F and D from the dense mapping (a repeated index keeps its last
// weight, numba.py:824-841); the compact one builds F from the summed sparse
// rows and D from the dense mapping (numba.py:928-951) — both are kept.
//
// Dataset terms (chi.chi and sum log|noise|) are recomputed on every call;
// sum log|x| is evaluated as log of frexp-normalised products of 32 values
// plus the exponent sum, so the float64 pipe does one log per 32 inputs.

#include <math.h>

#include "aj_internal.cuh"
#include "df32.cuh"

namespace aj {

constexpr int KT_THREADS = 256;
constexpr int KT_PER_THREAD = 32;

// partial[b] = (sum chi^2, sum log|noise|) over this block's chunk of the 2K reals
__global__ void __launch_bounds__(KT_THREADS)
    k_terms_kernel(const double* __restrict__ data, const double* __restrict__ noise, int64_t n2,
                   double* __restrict__ partial) {
    __shared__ double red[32];
    const int64_t base = ((int64_t)blockIdx.x * KT_THREADS + threadIdx.x) * KT_PER_THREAD;
    double chi2 = 0.0, mant = 1.0;
    int64_t ex = 0;
    for (int q = 0; q < KT_PER_THREAD; ++q) {
        const int64_t t = base + q;
        if (t < n2) {
            const double x = noise[t];
            const double r = data[t] / x;
            chi2 = fma(r, r, chi2);
            int e;
            const double m = frexp(fabs(x), &e);
            mant *= m;
            ex += e;
        }
    }
    double lg = log(mant) + (double)ex * 0.69314718055994530942;
    chi2 = block_sum(chi2, red);
    lg = block_sum(lg, red);
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = chi2;
        partial[2 * blockIdx.x + 1] = lg;
    }
}

// out[0] = logE from the partials, s.D, log|A|, log|H| (numba.py:846-857)
__global__ void assemble_kernel(const double* __restrict__ partial, int64_t nblk, int64_t K,
                                const double* __restrict__ s, const double* __restrict__ D, int64_t S,
                                const double* __restrict__ logdets, const double* __restrict__ shift,
                                double* __restrict__ out) {
    __shared__ double red[32];
    double chi2 = 0.0, lg = 0.0, sd = 0.0;
    for (int64_t b = threadIdx.x; b < nblk; b += blockDim.x) {
        chi2 += partial[2 * b];
        lg += partial[2 * b + 1];
    }
    for (int64_t i = threadIdx.x; i < S; i += blockDim.x) sd = fma(s[i], D[i], sd);
    chi2 = block_sum(chi2, red);
    lg = block_sum(lg, red);
    sd = block_sum(sd, red);
    if (threadIdx.x == 0) {
        const double norm = 2.0 * ((double)K * 1.8378770664093454836 + lg);  // log(2 pi)
        const double sh = shift ? shift[0] : 0.0;
        const double logH = logdets[1] + (sh > 0.0 ? log(1e-8) - log(1e-8 + sh) : 0.0);
        out[0] = -0.5 * (chi2 - sd + logdets[0] - logH + norm);
    }
}

__global__ void add_kernel(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c,
                           int64_t n) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        c[t] = a[t] + b[t];
}

// partial sums of squares of a lower-triangular matrix (tr(H^-1) = ||L_H^-1||_F^2)
__global__ void frob_lower_kernel(const double* __restrict__ Li, int64_t S, double* __restrict__ partial) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int64_t i = blockIdx.x; i < S; i += gridDim.x)
        for (int64_t j = threadIdx.x; j <= i; j += blockDim.x) {
            const double v = Li[i * S + j];
            acc = fma(v, v, acc);
        }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// out[1] = dlogE/dlambda.  L's entries follow numba.py:688-694: diag(n), -1 per neighbour entry.
// A^-1 entry (i, j) from float64 storage, or from double-float planes when Ainv is null
__device__ __forceinline__ double ainv_at(const double* Ainv, const float* AIh, const float* AIl, int64_t S, int64_t i,
                                          int64_t j) {
    return Ainv ? Ainv[i * S + j] : (double)AIh[i * S + j] + (double)AIl[i * S + j];
}

__global__ void dlam_kernel(const int64_t* __restrict__ nb, const int64_t* __restrict__ nsz, int64_t S, int64_t P,
                            const double* __restrict__ s, const double* __restrict__ Ainv,
                            const float* __restrict__ AIh, const float* __restrict__ AIl,
                            const double* __restrict__ frob_partial, int64_t nfrob, double coef,
                            const double* __restrict__ coef_dev, const double* __restrict__ shift,
                            double* __restrict__ out) {
    const double c = coef_dev ? *coef_dev : coef;
    const double lam = c * c;
    __shared__ double red[32];
    double sls = 0.0, tra = 0.0, trl = 0.0, trh = 0.0;
    for (int64_t i = threadIdx.x; i < S; i += blockDim.x) {
        const double ni = (double)nsz[i];
        sls = fma(ni, s[i] * s[i], sls);
        tra = fma(ni, ainv_at(Ainv, AIh, AIl, S, i, i), tra);
        trl += ni;
        for (int64_t j = 0; j < P; ++j) {
            const int64_t k = nb[i * P + j];
            if (k == -1) break;
            if (k < 0 || k >= S) continue;
            sls -= s[i] * s[k];
            tra -= ainv_at(Ainv, AIh, AIl, S, k, i);
            if (k == i) trl -= 1.0;
        }
    }
    for (int64_t b = threadIdx.x; b < nfrob; b += blockDim.x) trh += frob_partial[b];
    sls = block_sum(sls, red);
    tra = block_sum(tra, red);
    trl = block_sum(trl, red);
    trh = block_sum(trh, red);
    if (threadIdx.x == 0) {
        const double sh = shift ? shift[0] : 0.0;
        if (sh > 0.0) trh += 1.0 / 1e-8 - 1.0 / (1e-8 + sh);
        // tr(H^-1 L): (S - eps tr(H^-1)) / lambda, or tr(L) / eps when lambda = 0 (H = eps I)
        const double trHL = lam != 0.0 ? ((double)S - 1e-8 * trh) / lam : trl / 1e-8;
        out[1] = -0.5 * (sls + tra - trHL);
    }
}

// grad[m][b] for the weights; one warp per image pixel m
__global__ void __launch_bounds__(256)
    weight_grad_kernel(const int64_t* __restrict__ idx, int64_t M, int64_t B, int64_t S,
                       const double* __restrict__ Om, const double* __restrict__ Ainv, const double* __restrict__ s,
                       const double* __restrict__ dirty, int compact_mode, double* __restrict__ grad) {
    const int lane = threadIdx.x & 31;
    const int64_t m = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (m >= M) return;
    const double* om = Om + m * S;
    double oms = 0.0;
    for (int64_t j = lane; j < S; j += 32) oms = fma(om[j], s[j], oms);
    oms = warp_sum(oms);
    const int64_t* row = idx + m * B;
    bool ended = false;
    for (int64_t b = 0; b < B; ++b) {
        const int64_t sp = row[b];
        if (sp == -1) ended = true;
        double g = 0.0;
        if (!ended && sp >= 0 && sp < S) {
            bool last = true;  // not overwritten by a later entry (dense-mapping semantics)
            for (int64_t q = b + 1; q < B; ++q) {
                if (row[q] == -1) break;
                if (row[q] == sp) last = false;
            }
            const bool keepD = last;
            const bool keepF = compact_mode ? true : last;
            double oa = 0.0;
            if (keepF) {
                const double* ar = Ainv + sp * S;
                for (int64_t j = lane; j < S; j += 32) oa = fma(om[j], ar[j], oa);
                oa = warp_sum(oa);
            }
            if (keepD) g += dirty[m] * s[sp];
            if (keepF) g -= oms * s[sp] + oa;
        }
        if (lane == 0) grad[m * B + b] = g;
    }
}

// Which terms of the weight gradient mapping entry b of a row takes (dense-mapping semantics: a
// later duplicate of the same source pixel overwrites an earlier one, and the row ends at -1).
// Returns false when the entry contributes nothing.
__device__ __forceinline__ bool wg_entry(const int64_t* row, int64_t B, int64_t b, int64_t S, int compact_mode,
                                         int64_t& sp, bool& keepD, bool& keepF) {
    for (int64_t q = 0; q <= b; ++q)
        if (row[q] == -1) return false;
    sp = row[b];
    if (sp < 0 || sp >= S) return false;
    bool last = true;
    for (int64_t q = b + 1; q < B; ++q) {
        if (row[q] == -1) break;
        if (row[q] == sp) last = false;
    }
    keepD = last;
    keepF = compact_mode ? true : last;
    return true;
}

// The same gradient on the mixed path, from the double-float planes of Omega
// (M x S) and A^-1 (S x S) and of s: the dot products run as double-float on
// the float32 pipe, with no float64 copies of Omega or A^-1.  One block per
// image pixel m: each thread reads its slices of Omega's row once and forms
// Omega_m . s and up to kWgDots products Omega_m . A^-1_sp side by side (16-byte
// loads when every row is 16-byte aligned), so a thread's dependent chain is
// S / kWgThreads steps long; a block reduction in fixed order finishes them.
// (of 32, 64, 96, 128, 256 and 384 threads, 64 measured best for many evaluations at once and within
// 0.5% of the best, 32, for a single one)
constexpr int kWgThreads = 64;
constexpr int kWgDots = 4;

__global__ void __launch_bounds__(kWgThreads)
    weight_grad_df_kernel(const int64_t* __restrict__ idx, int64_t M, int64_t B, int64_t S,
                          const float* __restrict__ Omh, const float* __restrict__ Oml, const float* __restrict__ AIh,
                          const float* __restrict__ AIl, const float* __restrict__ sh, const float* __restrict__ sl,
                          const double* __restrict__ s, const double* __restrict__ dirty, int compact_mode, int vec4,
                          double* __restrict__ grad) {
    __shared__ double red[kWgThreads / 32][1 + kWgDots];
    __shared__ double tot[1 + kWgDots];
    const int64_t m = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float* oh = Omh + m * S;
    const float* ol = Oml + m * S;
    const int64_t* row = idx + m * B;
    double oms = 0.0;
    for (int64_t b0 = 0; b0 < B; b0 += kWgDots) {
        const bool first = b0 == 0;
        const float* ah[kWgDots];
        const float* al[kWgDots];
#pragma unroll
        for (int u = 0; u < kWgDots; ++u) {
            int64_t sp;
            bool kd, kf;
            const bool use = b0 + u < B && wg_entry(row, B, b0 + u, S, compact_mode, sp, kd, kf) && kf;
            ah[u] = use ? AIh + sp * S : nullptr;
            al[u] = use ? AIl + sp * S : nullptr;
        }
        df acc[1 + kWgDots];
#pragma unroll
        for (int u = 0; u <= kWgDots; ++u) acc[u] = {0.f, 0.f};
        if (vec4) {
            for (int64_t t = threadIdx.x; t < S / 4; t += kWgThreads) {
                const float4 h = reinterpret_cast<const float4*>(oh)[t];
                const float4 l = reinterpret_cast<const float4*>(ol)[t];
                if (first) {
                    const float4 xh = reinterpret_cast<const float4*>(sh)[t];
                    const float4 xl = reinterpret_cast<const float4*>(sl)[t];
                    df_fma_lazy(acc[0], {h.x, l.x}, {xh.x, xl.x});
                    df_fma_lazy(acc[0], {h.y, l.y}, {xh.y, xl.y});
                    df_fma_lazy(acc[0], {h.z, l.z}, {xh.z, xl.z});
                    df_fma_lazy(acc[0], {h.w, l.w}, {xh.w, xl.w});
                    df_renorm(acc[0]);
                }
#pragma unroll
                for (int u = 0; u < kWgDots; ++u) {
                    if (!ah[u]) continue;
                    const float4 xh = reinterpret_cast<const float4*>(ah[u])[t];
                    const float4 xl = reinterpret_cast<const float4*>(al[u])[t];
                    df_fma_lazy(acc[1 + u], {h.x, l.x}, {xh.x, xl.x});
                    df_fma_lazy(acc[1 + u], {h.y, l.y}, {xh.y, xl.y});
                    df_fma_lazy(acc[1 + u], {h.z, l.z}, {xh.z, xl.z});
                    df_fma_lazy(acc[1 + u], {h.w, l.w}, {xh.w, xl.w});
                    df_renorm(acc[1 + u]);
                }
            }
        } else {
            for (int64_t t = threadIdx.x; t < S; t += kWgThreads) {
                const df o = {oh[t], ol[t]};
                if (first) df_fma_acc(acc[0], o, {sh[t], sl[t]});
#pragma unroll
                for (int u = 0; u < kWgDots; ++u)
                    if (ah[u]) df_fma_acc(acc[1 + u], o, {ah[u][t], al[u][t]});
            }
        }
        // block sums in a fixed order: lanes (warp_sum), then warps 0, 1, ...
#pragma unroll
        for (int u = 0; u <= kWgDots; ++u) {
            const double v = warp_sum(df_to(acc[u]));
            if (lane == 0) red[warp][u] = v;
        }
        __syncthreads();
        if (threadIdx.x <= kWgDots) {
            double v = 0.0;
            for (int w = 0; w < kWgThreads / 32; ++w) v += red[w][threadIdx.x];
            tot[threadIdx.x] = v;
        }
        __syncthreads();
        if (first) oms = tot[0];
        if (threadIdx.x < kWgDots && b0 + threadIdx.x < B) {
            const int64_t b = b0 + threadIdx.x;
            int64_t sp;
            bool keepD = false, keepF = false;
            double g = 0.0;
            if (wg_entry(row, B, b, S, compact_mode, sp, keepD, keepF)) {
                if (keepD) g += dirty[m] * s[sp];
                if (keepF) g -= oms * s[sp] + tot[1 + threadIdx.x];
            }
            grad[m * B + b] = g;
        }
        __syncthreads();  // red and tot are reused by the next pass
    }
}

// Deflation of H's constant mode for the double-float factorisation.
// When the neighbour lists describe a graph Laplacian (sizes equal to the
// entries before -1, no self-loops, every entry mirrored with the same
// multiplicity), H 1 = 1e-8 1 exactly, so H~ = H + (c/S) 1 1^T only moves that
// eigenvalue from 1e-8 to 1e-8 + c and
//   log|H| = log|H~| + log(1e-8) - log(1e-8 + c),
//   tr(H^-1) = tr(H~^-1) + 1/1e-8 - 1/(1e-8 + c).
// With c = lambda * mean(n) H~ is as well conditioned as lambda L on the
// complement of the constant vector, where 48-bit arithmetic suffices.
// Lists that are not a Laplacian get c = 0 (no deflation).
__global__ void laplacian_shift_kernel(const int64_t* __restrict__ nb, const int64_t* __restrict__ nsz, int64_t S,
                                       int64_t P, double coef, const double* __restrict__ coef_dev,
                                       double* __restrict__ shift) {
    __shared__ int ok_s;
    __shared__ double red[32];
    if (threadIdx.x == 0) ok_s = 1;
    __syncthreads();
    int ok = 1;
    double nsum = 0.0;
    for (int64_t i = threadIdx.x; i < S; i += blockDim.x) {
        const int64_t* row = nb + i * P;
        int64_t cnt = 0;
        for (int64_t j = 0; j < P; ++j) {
            const int64_t k = row[j];
            if (k == -1) break;
            ++cnt;
            if (k < 0 || k >= S || k == i) {
                ok = 0;
                continue;
            }
            int64_t m_ik = 0, m_ki = 0;
            for (int64_t q = 0; q < P && row[q] != -1; ++q) m_ik += row[q] == k;
            const int64_t* rk = nb + k * P;
            for (int64_t q = 0; q < P && rk[q] != -1; ++q) m_ki += rk[q] == i;
            if (m_ik != m_ki) ok = 0;
        }
        if (cnt != nsz[i]) ok = 0;
        nsum += (double)nsz[i];
    }
    if (!ok) atomicAnd(&ok_s, 0);
    nsum = block_sum(nsum, red);
    __syncthreads();
    if (threadIdx.x == 0) {
        const double c = coef_dev ? *coef_dev : coef;
        const double lam = c * c;
        const double sh = ok_s ? lam * (nsum / (double)S) : 0.0;
        shift[0] = sh > 0.0 ? sh : 0.0;
    }
}

// (hi, lo) planes of H + shift[0] / S
__global__ void split_shifted_kernel(const double* __restrict__ H, int64_t S, const double* __restrict__ shift,
                                     float* __restrict__ hi, float* __restrict__ lo) {
    const double add = shift[0] / (double)S;
    const int64_t n = S * S;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const df v = t % S <= t / S ? df_from(H[t] + add) : df{0.f, 0.f};  // lower triangle only
        hi[t] = v.hi;
        lo[t] = v.lo;
    }
}

// single-block noise normalisation for the standalone drop-in call
__global__ void noise_norm_kernel(const double* __restrict__ x, int64_t n2, int64_t K, double* __restrict__ out) {
    __shared__ double red[32];
    double lg = 0.0, mant = 1.0;
    int64_t ex = 0;
    int cnt = 0;
    for (int64_t t = threadIdx.x; t < n2; t += blockDim.x) {
        int e;
        mant *= frexp(fabs(x[t]), &e);
        ex += e;
        if (++cnt == KT_PER_THREAD) {
            lg += log(mant);
            mant = 1.0;
            cnt = 0;
        }
    }
    lg += log(mant) + (double)ex * 0.69314718055994530942;
    lg = block_sum(lg, red);
    if (threadIdx.x == 0) *out = 2.0 * ((double)K * 1.8378770664093454836 + lg);
}

struct EvidenceBufs {
    Csc ca{}, cs{};
    SpdWorkspace wa{}, wh{};          // float64 path
    DfSpd da{}, dh{};                 // mixed path
    double *TW, *Om, *F, *H, *A, *Ainv, *D, *s, *kpart, *fpart, *logdets;
    float *Wh, *Wl;                   // w_tilde planes when split per call
    float *TWh, *TWl, *Omh, *Oml, *Fh, *Fl, *Ah, *Al, *AIh, *AIl, *sh, *sl;
    int64_t nk_blocks, nfrob;
    bool compact, grad, mixed;
};

// One routine both sizes (base == nullptr) and carves the workspace, so the two never disagree.
size_t evidence_carve(const aj_problem* p, bool mixed, bool with_grad, void* base, size_t bytes, EvidenceBufs& b) {
    const int64_t M = p->M, S = p->S, B = p->B;
    b = EvidenceBufs{};
    b.compact = p->w_compact != nullptr;
    b.grad = with_grad;
    b.mixed = mixed;
    b.nk_blocks = (2 * p->K + (int64_t)KT_THREADS * KT_PER_THREAD - 1) / ((int64_t)KT_THREADS * KT_PER_THREAD);
    if (b.nk_blocks < 1) b.nk_blocks = 1;
    b.nfrob = 2 * (int64_t)num_sms();
    Carver cv(base, base ? bytes : ~size_t(0) >> 1);
    auto sub = [&](size_t n) {
        char* at = cv.take<char>(n);
        return Carver(at, n);
    };
    {
        Carver c = sub(csc_bytes(M, B, S));
        csc_take(c, M, B, S, b.ca);
    }
    if (b.compact) {
        Carver c = sub(csc_bytes(M, B, S));
        csc_take(c, M, B, S, b.cs);
    } else {
        b.cs = b.ca;
    }
    b.H = cv.take<double>(S * S);
    b.D = cv.take<double>(S);
    b.s = cv.take<double>(S);
    b.kpart = cv.take<double>(2 * b.nk_blocks);
    b.fpart = cv.take<double>(b.nfrob);
    b.logdets = cv.take<double>(8);
    if (!mixed) {
        b.TW = cv.take<double>(S * M);
        b.Om = cv.take<double>(M * S);
        b.F = cv.take<double>(S * S);
        b.A = cv.take<double>(S * S);
        {
            Carver c = sub(spd_workspace_bytes(S, with_grad));
            b.wa = spd_carve(c, S, with_grad);
        }
        {
            Carver c = sub(spd_workspace_bytes(S, with_grad));
            b.wh = spd_carve(c, S, with_grad);
        }
        b.Ainv = with_grad ? cv.take<double>(S * S) : nullptr;
    } else {
        if (!b.compact && !(p->w_tilde_hi && p->w_tilde_lo)) {
            b.Wh = cv.take<float>(M * M);
            b.Wl = cv.take<float>(M * M);
        }
        if (b.compact) {
            b.TW = cv.take<double>(S * M);
            b.TWh = cv.take<float>(S * M);
            b.TWl = cv.take<float>(S * M);
        } else if (M % 4 != 0) {
            // the transposed Omega gather stores 4 columns (16 bytes) a row: other M gather T^T W
            // row-major, then transpose
            b.TWh = cv.take<float>(S * M);
            b.TWl = cv.take<float>(S * M);
        }
        b.Omh = cv.take<float>(M * S);
        b.Oml = cv.take<float>(M * S);
        b.Fh = cv.take<float>(S * S);
        b.Fl = cv.take<float>(S * S);
        b.Ah = cv.take<float>(S * S);
        b.Al = cv.take<float>(S * S);
        {
            Carver c = sub(dfspd_bytes(S, true, with_grad));
            b.da = dfspd_carve(c, S, true, with_grad);
        }
        {
            Carver c = sub(dfspd_bytes(S, with_grad));
            b.dh = dfspd_carve(c, S, with_grad);
        }
        if (with_grad) {
            b.AIh = cv.take<float>(S * S);
            b.AIl = cv.take<float>(S * S);
            b.sh = cv.take<float>(S);
            b.sl = cv.take<float>(S);
        }
    }
    return align_up(cv.used);
}

int check_problem(const aj_problem* p) {
    if (!p) return AJ_ERR_ARG;
    if (p->M < 0 || p->K < 0 || p->S <= 0 || p->B < 0 || p->P < 0) return AJ_ERR_ARG;
    if (!p->dirty_image || !p->pix_indexes || !p->pix_weights || !p->neighbors_sizes) return AJ_ERR_ARG;
    if (p->P > 0 && !p->neighbors) return AJ_ERR_ARG;
    if (p->K > 0 && (!p->data || !p->noise_map)) return AJ_ERR_ARG;
    if (p->w_compact) {
        if (p->N <= 0 || !p->native_index) return AJ_ERR_ARG;
    } else if (!p->w_tilde64) {
        return AJ_ERR_ARG;
    }
    return AJ_OK;
}

}  // namespace aj

using namespace aj;

extern "C" {

int aj_noise_normalization(const double* noise_map_c128, int64_t K, double* out, void* stream) {
    if (K < 0 || !out || (K > 0 && !noise_map_c128)) return AJ_ERR_ARG;
    noise_norm_kernel<<<1, 1024, 0, as_stream(stream)>>>(noise_map_c128, 2 * K, K, out);
    return check_launch();
}

size_t aj_log_evidence_workspace_size(const aj_problem* p, int precision, int with_grad) {
    if (check_problem(p) != AJ_OK) return 0;
    EvidenceBufs b;
    return evidence_carve(p, precision == AJ_MIXED, with_grad != 0, nullptr, 0, b);
}

int aj_split_f64(const double* x, int64_t n, float* hi, float* lo, void* stream) {
    if (n < 0 || (n > 0 && (!x || !hi || !lo))) return AJ_ERR_ARG;
    if (n == 0) return AJ_OK;
    return df_split(x, n, hi, lo, as_stream(stream));
}

int aj_log_evidence(const aj_problem* p, int precision, int with_grad, double* out, double* grad_weights,
                    double* reconstruction, void* workspace, size_t workspace_bytes, int* info, void* stream) {
    AJ_TRY(check_problem(p));
    if (precision != AJ_FP64 && precision != AJ_MIXED) return AJ_ERR_ARG;
    if (!out || (with_grad && !grad_weights)) return AJ_ERR_ARG;
    const bool mixed = precision == AJ_MIXED;
    EvidenceBufs b;
    const size_t need = evidence_carve(p, mixed, with_grad != 0, nullptr, 0, b);
    if (!workspace || workspace_bytes < need) return AJ_ERR_WORKSPACE;
    evidence_carve(p, mixed, with_grad != 0, workspace, workspace_bytes, b);
    cudaStream_t st = as_stream(stream);
    const int64_t M = p->M, S = p->S, B = p->B, K = p->K;

    // sparse mapping: dense-mapping semantics for D (and for F of the w_tilde likelihood)
    AJ_TRY(csc_build(p->pix_indexes, p->pix_weights, nullptr, M, B, S, CSC_ASSIGN, b.ca, info, st));
    if (b.compact) AJ_TRY(csc_build(p->pix_indexes, p->pix_weights, nullptr, M, B, S, CSC_SUM, b.cs, info, st));
    // Work that does not depend on w_tilde runs on a side lane while the w_tilde
    // products run here: D = T^T dirty, H (and its split, mixed), the chi^2 and
    // log-noise sums.
    Lanes* lanes = nullptr;
    AJ_TRY(lanes_for(st, &lanes));
    Lanes& ln = *lanes;
    cudaStream_t pre = ln.s[2];
    if (cudaEventRecord(ln.ev[kEvPre], st) != cudaSuccess || cudaStreamWaitEvent(pre, ln.ev[kEvPre], 0) != cudaSuccess)
        return AJ_ERR_CUDA;
    {
        int rc = csc_spmv_t(b.ca, S, p->dirty_image, b.D, pre);
        if (rc == AJ_OK)
            rc = regularization(p->coefficient, p->coefficient_dev, p->neighbors, p->neighbors_sizes, S, p->P, b.H,
                                info, pre);
        if (rc == AJ_OK && mixed) {
            laplacian_shift_kernel<<<1, 1024, 0, pre>>>(p->neighbors, p->neighbors_sizes, S, p->P, p->coefficient,
                                                         p->coefficient_dev, b.logdets + 4);
            rc = check_launch();
            if (rc == AJ_OK) {
                // straight into H's factorisation workspace, and the inverse buffers zeroed here too,
                // so the factorisation starts without copies
                split_shifted_kernel<<<blocks_for(S * S, 256, 8 * num_sms()), 256, 0, pre>>>(b.H, S, b.logdets + 4,
                                                                                             b.dh.Lh, b.dh.Ll);
                rc = check_launch();
                if (rc == AJ_OK &&
                    (cudaMemsetAsync(b.da.Ih, 0, sizeof(float) * 2 * S * S, pre) != cudaSuccess ||
                     (with_grad && (cudaMemsetAsync(b.dh.Ih, 0, sizeof(float) * 2 * S * S, pre) != cudaSuccess ||
                                    cudaMemsetAsync(b.AIh, 0, sizeof(float) * S * S, pre) != cudaSuccess ||
                                    cudaMemsetAsync(b.AIl, 0, sizeof(float) * S * S, pre) != cudaSuccess))))
                    rc = AJ_ERR_CUDA;
            }
        }
        // H's factorisation (below) can start here, before the chi^2 and log-noise sums
        if (cudaEventRecord(ln.ev[kEvHReady], pre) != cudaSuccess) return AJ_ERR_CUDA;
        if (rc == AJ_OK) {
            if (K > 0) {
                k_terms_kernel<<<(unsigned)b.nk_blocks, KT_THREADS, 0, pre>>>(p->data, p->noise_map, 2 * K, b.kpart);
                rc = check_launch();
            } else if (cudaMemsetAsync(b.kpart, 0, sizeof(double) * 2 * b.nk_blocks, pre) != cudaSuccess) {
                rc = AJ_ERR_CUDA;
            }
            // D's planes for the solve, in A's solve scratch (which its factorisation leaves alone)
            if (rc == AJ_OK && mixed) {
                float* dp = reinterpret_cast<float*>(b.da.vec);
                rc = df_split(b.D, S, dp, dp + S, pre);
            }
        }
        // joined even after a failed enqueue, so st never runs ahead of the side lane
        if (cudaEventRecord(ln.ev[kEvPreDone], pre) != cudaSuccess) return AJ_ERR_CUDA;
        if (rc != AJ_OK) {
            cudaStreamWaitEvent(st, ln.ev[kEvPreDone], 0);
            return rc;
        }
        if (!mixed) {
            // H's float64 chain beside A's on lane 5: the factor, then (with the gradient) L^-1 and
            // tr(H^-1)'s partial sums; A's factor, solve and inverse stay on this stream
            cudaStream_t hlane = ln.s[5];
            if (cudaStreamWaitEvent(hlane, ln.ev[kEvHReady], 0) != cudaSuccess) return AJ_ERR_CUDA;
            rc = spd_factor(b.H, S, b.wh, b.logdets + 1, info, hlane, true, with_grad);
            if (rc == AJ_OK && with_grad) {
                frob_lower_kernel<<<(unsigned)b.nfrob, 256, 0, hlane>>>(b.wh.Linv, S, b.fpart);
                rc = check_launch();
            }
            if (cudaEventRecord(ln.ev[kEvHDone], hlane) != cudaSuccess) return AJ_ERR_CUDA;
            if (rc != AJ_OK) {
                cudaStreamWaitEvent(st, ln.ev[kEvHDone], 0);
                return rc;
            }
        }
        if (mixed) {
            // H's factorisation (and, with the gradient, its L^-1 for tr(H^-1)) beside A's, from
            // lane 5 (which A's factorisation never forks or joins), on lanes of its own
            cudaStream_t hlane = ln.s[5];
            if (cudaStreamWaitEvent(hlane, ln.ev[kEvHReady], 0) != cudaSuccess) return AJ_ERR_CUDA;
            const float* hh[1] = {b.dh.Lh};
            const float* hl[1] = {b.dh.Ll};
            DfSpd* hw[1] = {&b.dh};
            double* hld[1] = {b.logdets + 1};
            // (L^-1 of H in float32: tr(H^-1) enters dlogE/dlambda as 1e-8 tr(H^-1) / lambda against
            // S / lambda, and the deflated H is well conditioned, so float32 moves it by ~1e-12)
            rc = dfspd_factor_invert_n(hh, hl, 1, with_grad ? 1 : 0, S, hw, hld, info, hlane, nullptr, nullptr, true,
                                       true);
            // tr(H^-1)'s partial sums for dlogE/dlambda here too, long before the evaluation's tail
            if (rc == AJ_OK && with_grad) rc = df_frob_lower(b.dh.Ih, b.dh.Il, S, b.fpart, b.nfrob, hlane);
            if (cudaEventRecord(ln.ev[kEvHDone], hlane) != cudaSuccess) return AJ_ERR_CUDA;
            if (rc != AJ_OK) {
                cudaStreamWaitEvent(st, ln.ev[kEvHDone], 0);
                return rc;
            }
        }
    }
    auto join_pre = [&]() {
        return cudaStreamWaitEvent(st, ln.ev[kEvPreDone], 0) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    };

    if (!mixed) {
        // Omega = W T (via TW = T^T W, W symmetric), F = T^T Omega, A = F + H
        if (b.compact)
            AJ_TRY(csc_compact_tw<double>(b.cs, S, p->w_compact, p->N, p->native_index, M, b.TW, info, st));
        else
            AJ_TRY(csc_spmm_t<double, double>(b.cs, S, p->w_tilde64, M, M, b.TW, M, st));
        AJ_TRY(transpose<double>(b.TW, S, M, b.Om, st));
        AJ_TRY(csc_spmm_t<double, double>(b.cs, S, b.Om, S, S, b.F, S, st));
        AJ_TRY(join_pre());
        add_kernel<<<blocks_for(S * S, 256, 8 * num_sms()), 256, 0, st>>>(b.F, b.H, b.A, S * S);
        AJ_LAUNCHED();
        AJ_TRY(spd_factor(b.A, S, b.wa, b.logdets + 0, info, st, true, with_grad, with_grad ? b.Ainv : nullptr));
        AJ_TRY(spd_solve_vec(S, b.wa, b.D, b.s, info, st));
    } else {
        // the same chain in double-float on the float32 pipe
        const float *Wh = p->w_tilde_hi, *Wl = p->w_tilde_lo;
        if (b.compact) {
            AJ_TRY(csc_compact_tw<double>(b.cs, S, p->w_compact, p->N, p->native_index, M, b.TW, info, st));
            AJ_TRY(df_split(b.TW, S * M, b.TWh, b.TWl, st));
        } else {
            if (!Wh || !Wl) {
                AJ_TRY(df_split(p->w_tilde64, M * M, b.Wh, b.Wl, st));
                Wh = b.Wh;
                Wl = b.Wl;
            }
            if (M % 4 == 0) {
                // Omega = (T^T W)^T straight from the gather (the planes must be 16-byte aligned)
                AJ_TRY(csc_spmm_t_df_tr(b.cs, S, Wh, Wl, M, M, b.Omh, b.Oml, S, st));
            } else {
                AJ_TRY(csc_spmm_t_df(b.cs, S, Wh, Wl, M, M, b.TWh, b.TWl, M, st));
            }
        }
        if (b.compact || M % 4 != 0) {
            AJ_TRY(transpose<float>(b.TWh, S, M, b.Omh, st));
            AJ_TRY(transpose<float>(b.TWl, S, M, b.Oml, st));
        }
        // F's lower triangle (F is symmetric); A in full for the refinement's residual and its
        // lower triangle for the factorisation
        AJ_TRY(csc_spmm_t_df(b.cs, S, b.Omh, b.Oml, S, S, b.Fh, b.Fl, S, st, true));
        AJ_TRY(join_pre());
        AJ_TRY(df_add_f64_sym(b.Fh, b.Fl, b.H, S, b.Ah, b.Al, b.da.Lh, b.da.Ll, st));
        // A's factorisation, L^-1 and (with the gradient) A^-1 on this stream's lanes; H's runs
        // beside it from the side lane
        const float* fh[1] = {b.da.Lh};
        const float* fl[1] = {b.da.Ll};
        DfSpd* fw[1] = {&b.da};
        double* ld[1] = {b.logdets + 0};
        AJ_TRY(dfspd_factor_invert_n(fh, fl, 1, 1, S, fw, ld, info, st, nullptr, nullptr, true));
        // with the gradient, A^-1 = L^-T L^-1 on the tensor cores on lane 4, beside the solve's first
        // products (which need only L^-1); the solve waits for it before its correction
        cudaEvent_t ainv_ready = nullptr;
        if (with_grad) {
            cudaStream_t lau = ln.s[4];
            if (cudaEventRecord(ln.ev[kEvAinv], st) != cudaSuccess ||
                cudaStreamWaitEvent(lau, ln.ev[kEvAinv], 0) != cudaSuccess)
                return AJ_ERR_CUDA;
            AJ_TRY(tc_lauum(b.da.Ih, b.da.Il, S, b.AIh, b.AIl, b.da.tcws, b.da.tcws_bytes, lau));
            AJ_TRY(df_mirror_lower(b.AIh, b.AIl, S, lau));
            if (cudaEventRecord(ln.ev[kEvAinv], lau) != cudaSuccess) return AJ_ERR_CUDA;
            ainv_ready = ln.ev[kEvAinv];
        }
        // (with the gradient, s's planes for the adjoint come out of the solve's last product)
        AJ_TRY(dfspd_solve_refined(S, b.da, b.Ah, b.Al, b.D, b.s, st, with_grad ? b.AIh : nullptr,
                                   with_grad ? b.AIl : nullptr, true, with_grad ? b.sh : nullptr,
                                   with_grad ? b.sl : nullptr, ainv_ready));
    }
    // H's chain (log|H|, and tr(H^-1)'s partial sums with the gradient) joins before the assembly
    if (cudaStreamWaitEvent(st, ln.ev[kEvHDone], 0) != cudaSuccess) return AJ_ERR_CUDA;

    // logE from the chi^2 and log-noise sums (side lane), s.D and the log-determinants; on the
    // mixed path with the gradient it runs on the side lane beside the weight gradient
    const bool side_assemble = mixed && with_grad;
    if (!side_assemble) {
        assemble_kernel<<<1, 1024, 0, st>>>(b.kpart, b.nk_blocks, K, b.s, b.D, S, b.logdets,
                                            mixed ? b.logdets + 4 : nullptr, out);
        AJ_LAUNCHED();
    }
    if (reconstruction &&
        cudaMemcpyAsync(reconstruction, b.s, sizeof(double) * S, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return AJ_ERR_CUDA;
    if (!with_grad) return AJ_OK;

    // adjoint
    // dlogE/dlambda (and, mixed, the assembly) on the side lane while st computes the weight
    // gradient; both read only finished data
    if (cudaEventRecord(ln.ev[kEvPre], st) != cudaSuccess || cudaStreamWaitEvent(pre, ln.ev[kEvPre], 0) != cudaSuccess)
        return AJ_ERR_CUDA;
    {
        int rc = AJ_OK;
        if (side_assemble) {
            assemble_kernel<<<1, 1024, 0, pre>>>(b.kpart, b.nk_blocks, K, b.s, b.D, S, b.logdets, b.logdets + 4, out);
            rc = check_launch();
        }
        if (rc == AJ_OK) {
            dlam_kernel<<<1, 1024, 0, pre>>>(p->neighbors, p->neighbors_sizes, S, p->P, b.s, mixed ? nullptr : b.Ainv,
                                             b.AIh, b.AIl, b.fpart, b.nfrob, p->coefficient, p->coefficient_dev,
                                             mixed ? b.logdets + 4 : nullptr, out);
            rc = check_launch();
        }
        if (cudaEventRecord(ln.ev[kEvPreDone], pre) != cudaSuccess) return AJ_ERR_CUDA;
        if (rc != AJ_OK) {
            cudaStreamWaitEvent(st, ln.ev[kEvPreDone], 0);
            return rc;
        }
    }
    if (M > 0 && B > 0) {
        if (mixed)
            weight_grad_df_kernel<<<(unsigned)M, kWgThreads, 0, st>>>(
                p->pix_indexes, M, B, S, b.Omh, b.Oml, b.AIh, b.AIl, b.sh, b.sl, b.s, p->dirty_image,
                b.compact ? 1 : 0,
                S % 4 == 0 && aligned16(b.Omh, b.Oml, b.AIh, b.AIl, b.sh, b.sl) ? 1 : 0, grad_weights);
        else
            weight_grad_kernel<<<blocks_for(M * 32, 256), 256, 0, st>>>(p->pix_indexes, M, B, S, b.Om, b.Ainv, b.s,
                                                                        p->dirty_image, b.compact ? 1 : 0,
                                                                        grad_weights);
        AJ_LAUNCHED();
    }
    return join_pre();
}

size_t aj_curvature_w_tilde_sparse_mixed_workspace_size(int64_t M, int64_t B, int64_t S) {
    if (M < 0 || B < 0 || S <= 0) return 0;
    Sizer z;
    z.take<char>(csc_bytes(M, B, S));
    z.take<float>(M * S);
    z.take<float>(M * S);
    z.take<float>(M * S);
    z.take<float>(M * S);
    z.take<float>(S * S);
    z.take<float>(S * S);
    return z.total();
}

int aj_curvature_w_tilde_sparse_mixed(const float* w_tilde_hi, const float* w_tilde_lo, int64_t M,
                                      const int64_t* pix_indexes, const double* pix_weights, int64_t B, int64_t S,
                                      double* out, void* workspace, size_t workspace_bytes, int* info, void* stream) {
    if (M < 0 || B < 0 || S <= 0 || !out) return AJ_ERR_ARG;
    if (M > 0 && (!w_tilde_hi || !w_tilde_lo || (B > 0 && (!pix_indexes || !pix_weights)))) return AJ_ERR_ARG;
    if (!workspace || workspace_bytes < aj_curvature_w_tilde_sparse_mixed_workspace_size(M, B, S))
        return AJ_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    if (M == 0 || B == 0) return cudaMemsetAsync(out, 0, sizeof(double) * S * S, st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
    Carver cv(workspace, workspace_bytes);
    Csc c;
    {
        char* at = cv.take<char>(csc_bytes(M, B, S));
        Carver sub(at, csc_bytes(M, B, S));
        csc_take(sub, M, B, S, c);
    }
    float* TWh = cv.take<float>(M * S);
    float* TWl = cv.take<float>(M * S);
    float* Omh = cv.take<float>(M * S);
    float* Oml = cv.take<float>(M * S);
    float* Fh = cv.take<float>(S * S);
    float* Fl = cv.take<float>(S * S);
    AJ_TRY(csc_build(pix_indexes, pix_weights, nullptr, M, B, S, CSC_SUM, c, info, st));
    // the likelihood's own two gathers: Omega = (T^T W)^T, then F's lower triangle = T^T Omega
    const bool tr = M % 4 == 0 && reinterpret_cast<uintptr_t>(w_tilde_hi) % 16 == 0 &&
                    reinterpret_cast<uintptr_t>(w_tilde_lo) % 16 == 0;
    if (tr) {
        AJ_TRY(csc_spmm_t_df_tr(c, S, w_tilde_hi, w_tilde_lo, M, M, Omh, Oml, S, st));
    } else {
        AJ_TRY(csc_spmm_t_df(c, S, w_tilde_hi, w_tilde_lo, M, M, TWh, TWl, M, st));
        AJ_TRY(transpose<float>(TWh, S, M, Omh, st));
        AJ_TRY(transpose<float>(TWl, S, M, Oml, st));
    }
    AJ_TRY(csc_spmm_t_df(c, S, Omh, Oml, S, S, Fh, Fl, S, st, true));
    AJ_TRY(df_mirror_lower(Fh, Fl, S, st));
    return df_join(Fh, Fl, S * S, out, st);
}

}  // extern "C"
