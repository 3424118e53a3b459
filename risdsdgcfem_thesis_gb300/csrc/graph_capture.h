// graph_capture.h -- a conditional node (IF or WHILE) added during stream
// capture, its body captured from a side stream: the step graphs of the
// batch (batch.cu) and of the solid (solid.cu) loop on the device this way.
#pragma once
#include <cuda_runtime.h>

namespace femgb {

// Adds a conditional node (IF or WHILE on `h`) after the current capture
// point of `s`, captures `body` into its body graph on a side stream, and
// makes the node the new capture point of `s`.
template <typename F>
inline cudaError_t capture_conditional(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                                F&& body)
{
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaGraph_t g = nullptr;
    cudaStreamCaptureStatus cs;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = type;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp);
    if (e != cudaSuccess) return e;
    cudaStream_t bs = nullptr;
    e = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCaptureToGraph(bs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
        const cudaError_t eb = body(bs, cp.conditional.phGraph_out[0]);
        cudaGraph_t out = nullptr;
        e = cudaStreamEndCapture(bs, &out);
        if (eb != cudaSuccess) e = eb;
    }
    cudaStreamDestroy(bs);
    if (e != cudaSuccess) return e;
    return cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

}  // namespace femgb
