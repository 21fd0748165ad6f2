// A solve entry point that allocates nothing and takes no workspace.
//
// Some callers cannot allocate device memory: a plugin or foreign-function
// host that only receives device pointers from its embedding application, or
// code running where the allocator is owned by someone else.  This variant of
// aj_spd_solve keeps its scratch (the Cholesky factor, the diagonal-block
// inverses and two vectors) in one file-scope __device__ array sized for
// S <= AJ_NOALLOC_SOLVE_MAX_S, so the caller passes only inputs and outputs.
//
// The array is placed in a GPU's memory when the driver loads this library's
// device code into a context.  Under lazy module loading (the default since
// CUDA 12.2) that happens on the first call of this entry point in each
// context, so that first call can fail with an out-of-memory error on a full
// device: make it early, and before any stream capture.  The array then stays
// until the context is destroyed (normally at process exit).  On the host the
// array's name is only a stand-in: its device address belongs to one context,
// so it is looked up per context (cudaGetSymbolAddress, with that context
// current) and cached under the context's unique id, which survives neither a
// cudaDeviceReset nor a switch to another context.  All calls in a context
// share the one array, so two calls whose GPU work overlaps (on different
// streams, or from different threads) race on it.

#include <cuda.h>

#include <mutex>

#include "aj_internal.cuh"

namespace aj {

namespace {

constexpr int64_t kMaxS = AJ_NOALLOC_SOLVE_MAX_S;
constexpr int kCacheSlots = 64;

// sized with the same Sizer sequence as spd_workspace_bytes(kMaxS, false)
constexpr size_t noalloc_bytes() {
    const int64_t nbt = (kMaxS + kSpdNB - 1) / kSpdNB;
    size_t used = 0;
    auto take = [&](size_t bytes) { used = (used + 255) / 256 * 256 + bytes; };
    take(sizeof(double) * kMaxS * kMaxS);
    take(sizeof(double) * nbt * kSpdNB * kSpdNB);
    take(sizeof(double) * 2 * kMaxS);
    take(sizeof(double) * 8);
    return (used + 255) / 256 * 256;
}

__device__ __align__(256) unsigned char g_solve_scratch[noalloc_bytes()];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

std::mutex g_mu;
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
unsigned long long g_ids[kCacheSlots] = {};
void* g_addrs[kCacheSlots] = {};
int g_next = 0;

// Unique id of the calling thread's current context (0 when there is none yet).
int current_context_id(unsigned long long* id) {
    *id = 0;
    if (!g_ctx_current || !g_ctx_id) {
        cudaDriverEntryPointQueryResult q1{}, q2{};
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return AJ_ERR_CUDA;
        g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS) return AJ_ERR_CUDA;
    if (ctx && g_ctx_id(ctx, id) != CUDA_SUCCESS) return AJ_ERR_CUDA;
    return AJ_OK;
}

// Device address of the scratch in the current context.
int scratch_address(void** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    unsigned long long id = 0;
    AJ_TRY(current_context_id(&id));
    if (id != 0) {
        for (int i = 0; i < kCacheSlots; ++i)
            if (g_ids[i] == id) {
                *out = g_addrs[i];
                return AJ_OK;
            }
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_solve_scratch);
    if (e != cudaSuccess || !p) {
        g_last_cuda_error = static_cast<int>(e);
        return AJ_ERR_CUDA;
    }
    // the lookup makes the device's primary context current when there was none
    if (id == 0) AJ_TRY(current_context_id(&id));
    if (id != 0) {
        g_ids[g_next] = id;
        g_addrs[g_next] = p;
        g_next = (g_next + 1) % kCacheSlots;
    }
    *out = p;
    return AJ_OK;
}

}  // namespace

}  // namespace aj

using namespace aj;

extern "C" {

int aj_spd_solve_noalloc(const double* data_vector, const double* A, int64_t S, double* out, int* info, void* stream) {
    if (S < 0) return AJ_ERR_ARG;
    if (S > kMaxS) return AJ_ERR_TOO_LARGE;
    if (S == 0) return AJ_OK;
    // a non-positive-definite A is reported only through info, so it is required
    if (!data_vector || !A || !out || !info) return AJ_ERR_ARG;
    static_assert(noalloc_bytes() >= sizeof(double) * kMaxS * kMaxS, "scratch size");
    if (spd_workspace_bytes(S, false) > noalloc_bytes()) return AJ_ERR_TOO_LARGE;
    void* base = nullptr;
    AJ_TRY(scratch_address(&base));
    cudaStream_t st = as_stream(stream);
    // every scratch word is written before it is read: L is a copy of A, the
    // diagonal-block inverses and vectors are produced by the factorisation and solve
    Carver cv(base, noalloc_bytes());
    SpdWorkspace w = spd_carve(cv, S, false);
    // on the caller's stream alone (no side streams are created for it)
    AJ_TRY(spd_factor(A, S, w, nullptr, info, st, false));
    return spd_solve_vec(S, w, data_vector, out, info, st);
}

}  // extern "C"
