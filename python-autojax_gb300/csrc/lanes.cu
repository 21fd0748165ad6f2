// Side streams for work that forks from, and joins back into, the caller's stream.
//
// The blocked factorisations are chains of small, latency-bound launches.  They
// run faster as concurrent chains: the critical one (the pivot panels) on the
// highest-priority stream, and at one lower priority the bulk of each trailing
// update and the triangular inverses, which need only finished panels (one lane
// per matrix); the float64 path's A^-1 = L^-T L^-1 also streams on a lane, as
// rows of L^-1 finish.
// (Ranking the bulk lane below or above the others measured 23 us and 5 us
// slower per evaluation at K = 1e6.)  Every fork starts
// with an event recorded on the caller's stream and every join ends with the
// caller's stream waiting on each lane, so the caller sees one ordered stream,
// and stream capture records the same dependencies as graph edges.
//
// Streams and events are created once per (device, caller stream) on first
// use and live until aj_release_stream(caller) or process exit (a caller that
// makes a fresh stream per call should release each one when its work is
// done; a later stream that happens to get the same handle value reuses the
// set, which is harmless once the first stream's work has finished).
// Keying by the caller's stream keeps concurrent callers apart: evaluations
// enqueued on different streams (or
// captured as parallel branches of one graph) each fork onto lanes of their
// own, so their chains stay concurrent and never share an event.

#include <map>
#include <mutex>

#include "aj_internal.cuh"

namespace aj {

namespace {

std::mutex g_lanes_mu;
std::map<std::pair<int, cudaStream_t>, Lanes*> g_lanes;

// Every set the same, including one forked from another set's lane (H's factorisation beside
// A's): its panel chain at the top priority too measured 9 us per evaluation faster than at the
// side priority, and 87 us faster than at the lowest.
int create_lanes(Lanes& l) {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return AJ_ERR_CUDA;
    const int mid = greatest < least ? greatest + 1 : least;
    const int prio[kLaneCount] = {greatest, mid, mid, mid, mid, mid};
    for (int i = 0; i < kLaneCount; ++i)
        if (cudaStreamCreateWithPriority(&l.s[i], cudaStreamNonBlocking, prio[i]) != cudaSuccess) return AJ_ERR_CUDA;
    for (int i = 0; i < kLaneEvents; ++i)
        if (cudaEventCreateWithFlags(&l.ev[i], cudaEventDisableTiming) != cudaSuccess) return AJ_ERR_CUDA;
    return AJ_OK;
}

}  // namespace

int lanes_for(cudaStream_t caller, Lanes** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_lanes_mu);
    auto it = g_lanes.find({dev, caller});
    if (it == g_lanes.end()) {
        Lanes* l = new Lanes{};
        const int rc = create_lanes(*l);
        if (rc != AJ_OK) {
            g_last_cuda_error = static_cast<int>(cudaGetLastError());
            delete l;  // streams or events created before the failure stay with the context
            return rc;
        }
        it = g_lanes.emplace(std::make_pair(dev, caller), l).first;
    }
    *out = it->second;
    return AJ_OK;
}

int lanes_release(cudaStream_t caller) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
    Lanes* l = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_lanes_mu);
        auto it = g_lanes.find({dev, caller});
        if (it == g_lanes.end()) return AJ_OK;
        l = it->second;
        g_lanes.erase(it);
    }
    bool ok = true;
    for (int i = 0; i < kLaneCount; ++i) ok &= cudaStreamDestroy(l->s[i]) == cudaSuccess;
    for (int i = 0; i < kLaneEvents; ++i) ok &= cudaEventDestroy(l->ev[i]) == cudaSuccess;
    delete l;
    return ok ? AJ_OK : AJ_ERR_CUDA;
}

int lanes_fork(Lanes& l, cudaStream_t st, int n) {
    if (cudaEventRecord(l.ev[kEvFork], st) != cudaSuccess) return AJ_ERR_CUDA;
    for (int i = 0; i < n; ++i)
        if (cudaStreamWaitEvent(l.s[i], l.ev[kEvFork], 0) != cudaSuccess) return AJ_ERR_CUDA;
    return AJ_OK;
}

int lanes_join(Lanes& l, cudaStream_t st, int n) {
    for (int i = 0; i < n; ++i) {
        if (cudaEventRecord(l.ev[kEvJoin0 + i], l.s[i]) != cudaSuccess) return AJ_ERR_CUDA;
        if (cudaStreamWaitEvent(st, l.ev[kEvJoin0 + i], 0) != cudaSuccess) return AJ_ERR_CUDA;
    }
    return AJ_OK;
}

int lane_signal(Lanes& l, int event, int from) {
    return cudaEventRecord(l.ev[event], l.s[from]) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int lane_wait(Lanes& l, int lane, int event) {
    return cudaStreamWaitEvent(l.s[lane], l.ev[event], 0) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

}  // namespace aj
