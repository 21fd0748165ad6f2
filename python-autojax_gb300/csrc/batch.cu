// Many lens-model evaluations against one dataset in a single call.
//
// An MCMC or nested sampler evaluates many lens models (each with its own
// source-pixel count S, mapping, neighbours and regularisation coefficient)
// against one observation: the dirty image, visibilities, noise and w_tilde
// are shared and stay resident.  One evaluation is a chain of small,
// latency-bound launches (the blocked factorisations); run alone it leaves
// most of the GPU idle.  The batch therefore forks the caller's stream into
// branch streams, enqueues the evaluations over the branches (balanced, below), and
// joins them back, so the chains of different evaluations fill each other's
// gaps.  Captured into one CUDA graph (aj_graph_begin/end), a whole batch is a
// single graph launch whose branches the GPU runs concurrently.  The models go
// to the branches longest first, each onto the branch with the least work so far.
//
// Branch streams are created once per (device, caller stream) on first use,
// like the factorisation lanes, which are in turn keyed by branch stream, so
// every evaluation in flight has its own lanes.

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "aj_internal.cuh"

namespace aj {

namespace {

constexpr int kBranches = AJ_BATCH_BRANCHES;

struct Branches {
    cudaStream_t s[kBranches];
    cudaEvent_t fork;
    cudaEvent_t join[kBranches];
};

std::mutex g_branch_mu;
std::map<std::pair<int, cudaStream_t>, Branches*> g_branches;

int branches_for(cudaStream_t caller, Branches** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_branch_mu);
    auto it = g_branches.find({dev, caller});
    if (it == g_branches.end()) {
        Branches* b = new Branches{};
        bool ok = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
        for (int i = 0; ok && i < kBranches; ++i)
            ok = cudaStreamCreateWithFlags(&b->s[i], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) == cudaSuccess;
        if (!ok) {
            g_last_cuda_error = static_cast<int>(cudaGetLastError());
            delete b;  // handles created before the failure stay with the context
            return AJ_ERR_CUDA;
        }
        it = g_branches.emplace(std::make_pair(dev, caller), b).first;
    }
    *out = it->second;
    return AJ_OK;
}

}  // namespace

}  // namespace aj

using namespace aj;

extern "C" {

int aj_release_stream(void* stream) {
    cudaStream_t st = as_stream(stream);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    Branches* br = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_branch_mu);
        auto it = g_branches.find({dev, st});
        if (it != g_branches.end()) {
            br = it->second;
            g_branches.erase(it);
        }
    }
    int rc = AJ_OK;
    if (br) {
        for (int b = 0; b < kBranches; ++b) {
            // each branch stream carries lanes of its own
            if (lanes_release(br->s[b]) != AJ_OK) rc = AJ_ERR_CUDA;
            if (cudaStreamDestroy(br->s[b]) != cudaSuccess || cudaEventDestroy(br->join[b]) != cudaSuccess)
                rc = AJ_ERR_CUDA;
        }
        if (cudaEventDestroy(br->fork) != cudaSuccess) rc = AJ_ERR_CUDA;
        delete br;
    }
    if (lanes_release(st) != AJ_OK) rc = AJ_ERR_CUDA;
    return rc;
}

int aj_log_evidence_batched(const aj_problem* problems, int64_t n, int precision, int with_grad, double* out,
                            double* const* grad_weights, double* const* reconstruction, void* const* workspaces,
                            const size_t* workspace_bytes, int* info, void* stream) {
    if (n < 0) return AJ_ERR_ARG;
    if (n == 0) return AJ_OK;
    if (!problems || !out || !workspaces || !workspace_bytes || !info) return AJ_ERR_ARG;
    if (precision != AJ_FP64 && precision != AJ_MIXED) return AJ_ERR_ARG;
    if (with_grad && !grad_weights) return AJ_ERR_ARG;
    // every evaluation is validated before anything is enqueued
    for (int64_t i = 0; i < n; ++i) {
        const size_t need = aj_log_evidence_workspace_size(&problems[i], precision, with_grad);
        if (need == 0) return AJ_ERR_ARG;
        if (!workspaces[i] || workspace_bytes[i] < need) return AJ_ERR_WORKSPACE;
        if (with_grad && !grad_weights[i]) return AJ_ERR_ARG;
    }
    cudaStream_t st = as_stream(stream);
    Branches* br = nullptr;
    AJ_TRY(branches_for(st, &br));
    const int nb = n < kBranches ? static_cast<int>(n) : kBranches;
    if (cudaEventRecord(br->fork, st) != cudaSuccess) return AJ_ERR_CUDA;
    for (int b = 0; b < nb; ++b)
        if (cudaStreamWaitEvent(br->s[b], br->fork, 0) != cudaSuccess) return AJ_ERR_CUDA;
    // Longest first onto the least-loaded branch: an evaluation's work grows as S^3 (its factorisations)
    // plus M S (its gathers), and the branches run concurrently, so balancing their loads shortens the
    // batch.  A model's kernels and their order are the same on any branch, so results do not depend on
    // the assignment.
    std::vector<int64_t> order(n);
    for (int64_t i = 0; i < n; ++i) order[i] = i;
    auto cost = [&](int64_t i) {
        const double S = (double)problems[i].S;
        return S * S * S + 64.0 * (double)problems[i].M * S;
    };
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return cost(a) > cost(b); });
    std::vector<double> load(nb, 0.0);
    int rc = AJ_OK;
    for (int64_t k = 0; k < n && rc == AJ_OK; ++k) {
        const int64_t i = order[k];
        int b = 0;
        for (int c = 1; c < nb; ++c)
            if (load[c] < load[b]) b = c;
        load[b] += cost(i);
        rc = aj_log_evidence(&problems[i], precision, with_grad, out + 2 * i, with_grad ? grad_weights[i] : nullptr,
                             reconstruction ? reconstruction[i] : nullptr, workspaces[i], workspace_bytes[i],
                             info + 2 * i, br->s[b]);
    }
    // join even after a failed enqueue, so the caller's stream never runs ahead of a branch
    for (int b = 0; b < nb; ++b) {
        if (cudaEventRecord(br->join[b], br->s[b]) != cudaSuccess ||
            cudaStreamWaitEvent(st, br->join[b], 0) != cudaSuccess)
            return AJ_ERR_CUDA;
    }
    return rc;
}

}  // extern "C"
