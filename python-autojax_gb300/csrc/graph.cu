// CUDA-graph capture and replay of work enqueued through this library.
//
// The evaluation forks its factorisation onto prioritised lanes (lanes.cu):
// the pivot panels must run ahead of the bulk trailing updates.  Stream
// capture records each kernel's stream priority on its graph node, but a
// graph honours those priorities only when it is instantiated with
// cudaGraphInstantiateFlagUseNodePriority; otherwise every node runs at the
// priority of the stream the graph is launched into and the bulk updates
// delay the critical chain.  These entry points capture with that flag set.

#include "aj_internal.cuh"

using namespace aj;

extern "C" {

int aj_graph_begin(void* stream) {
    if (!stream) return AJ_ERR_ARG;  // the legacy default stream cannot be captured
    const cudaError_t e = cudaStreamBeginCapture(as_stream(stream), cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        g_last_cuda_error = static_cast<int>(e);
        return AJ_ERR_CUDA;
    }
    return AJ_OK;
}

int aj_graph_end(void* stream, void** graph_exec) {
    if (!stream || !graph_exec) return AJ_ERR_ARG;
    *graph_exec = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(as_stream(stream), &g);
    if (e != cudaSuccess || !g) {
        g_last_cuda_error = static_cast<int>(e);
        if (g) cudaGraphDestroy(g);
        return AJ_ERR_CUDA;
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiateWithFlags(&exec, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        g_last_cuda_error = static_cast<int>(e);
        return AJ_ERR_CUDA;
    }
    *graph_exec = exec;
    return AJ_OK;
}

int aj_graph_launch(void* graph_exec, void* stream) {
    if (!graph_exec) return AJ_ERR_ARG;
    const cudaError_t e = cudaGraphLaunch(static_cast<cudaGraphExec_t>(graph_exec), as_stream(stream));
    if (e != cudaSuccess) {
        g_last_cuda_error = static_cast<int>(e);
        return AJ_ERR_CUDA;
    }
    return AJ_OK;
}

int aj_graph_destroy(void* graph_exec) {
    if (!graph_exec) return AJ_OK;
    return cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graph_exec)) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

}  // extern "C"
