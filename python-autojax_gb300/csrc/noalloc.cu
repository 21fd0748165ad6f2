// A solve entry point that allocates nothing and takes no workspace.
//
// Some callers cannot allocate device memory: a plugin or foreign-function
// host that only receives device pointers from its embedding application, or
// code running where the allocator is owned by someone else.  This variant of
// aj_spd_solve keeps its scratch (the Cholesky factor, the diagonal-block
// inverses and two vectors) in one file-scope __device__ array sized for
// S <= AJ_NOALLOC_SOLVE_MAX_S, so the caller passes only inputs and outputs.
//
// The array lives in every GPU's memory from the moment the library is loaded
// until the process exits.  On the host its name is only a stand-in: the
// device address is obtained once per device with cudaGetSymbolAddress, with
// that device current, on the first call made on that device.  All calls on a
// device share the one array, so two calls whose GPU work overlaps (on
// different streams, or from different threads) race on it.

#include <mutex>

#include "aj_internal.cuh"

namespace aj {

namespace {

constexpr int64_t kMaxS = AJ_NOALLOC_SOLVE_MAX_S;
constexpr int kMaxDevices = 64;

// sized with the same Sizer sequence as spd_workspace_bytes(kMaxS, false)
constexpr size_t noalloc_bytes() {
    const int64_t nbt = (kMaxS + 31) / 32;
    size_t used = 0;
    auto take = [&](size_t bytes) { used = (used + 255) / 256 * 256 + bytes; };
    take(sizeof(double) * kMaxS * kMaxS);
    take(sizeof(double) * nbt * 32 * 32);
    take(sizeof(double) * 2 * kMaxS);
    take(sizeof(double) * 8);
    return (used + 255) / 256 * 256;
}

__device__ __align__(256) unsigned char g_solve_scratch[noalloc_bytes()];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of the scratch on the current device (resolved once per device).
int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return AJ_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_solve_scratch);
        if (e != cudaSuccess || !p) {
            g_last_cuda_error = static_cast<int>(e);
            return AJ_ERR_CUDA;
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
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
    if (!data_vector || !A || !out) return AJ_ERR_ARG;
    static_assert(noalloc_bytes() >= 1, "scratch size");
    if (spd_workspace_bytes(S, false) > noalloc_bytes()) return AJ_ERR_TOO_LARGE;
    void* base = nullptr;
    AJ_TRY(scratch_address(&base));
    cudaStream_t st = as_stream(stream);
    // every scratch word is written before it is read: L is a copy of A, the
    // diagonal-block inverses and vectors are produced by the factorisation and solve
    Carver cv(base, noalloc_bytes());
    SpdWorkspace w = spd_carve(cv, S, false);
    AJ_TRY(spd_factor(A, S, w, nullptr, info, st));
    return spd_solve_vec(S, w, data_vector, out, info, st);
}

}  // extern "C"
