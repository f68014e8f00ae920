// Conditional graph nodes for the iterative solves (see graph_loop.hpp).
#include <map>
#include <string>

#include "device.hpp"
#include "graph_loop.hpp"

namespace sysu {
namespace {

__global__ void k_loop_tail(cudaGraphConditionalHandle h, const int *stop, int *count, int bound) {
    const int c = *count + 1;
    *count = c;
    cudaGraphSetConditional(h, (*stop == 0 && c < bound) ? 1u : 0u);
}

// self-test body: sets the stop flag once `stop_at` bodies have run
__global__ void k_loop_stop_at(int *stop, const int *bodies, int stop_at) {
    if (*bodies >= stop_at) *stop = 1;
}

__global__ void k_if_flag(cudaGraphConditionalHandle h, const int *flag) {
    cudaGraphSetConditional(h, *flag != 0 ? 1u : 0u);
}

}  // namespace

bool stream_capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    SYSU_CUDA(cudaStreamIsCapturing(st, &cs));
    return cs == cudaStreamCaptureStatusActive;
}

cudaGraphConditionalHandle graph_cond_handle(cudaStream_t st, unsigned default_value) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    SYSU_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
    if (cs != cudaStreamCaptureStatusActive || !g) throw CaseError{"graph_cond_handle: the stream is not capturing"};
    cudaGraphConditionalHandle h;
    SYSU_CUDA(cudaGraphConditionalHandleCreate(&h, g, default_value, cudaGraphCondAssignDefault));
    return h;
}

void graph_cond_node(cudaStream_t st, cudaStream_t side, cudaGraphConditionalHandle h,
                     cudaGraphConditionalNodeType type, const std::function<void(cudaStream_t)> &body) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t ndeps = 0;
    SYSU_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &ndeps));
    if (cs != cudaStreamCaptureStatusActive || !g) throw CaseError{"graph_cond_node: the stream is not capturing"};
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = type;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    SYSU_CUDA(cudaGraphAddNode(&node, g, deps, edges, ndeps, &p));
    cudaGraph_t bodyg = p.conditional.phGraph_out[0];
    SYSU_CUDA(cudaStreamBeginCaptureToGraph(side, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    try {
        body(side);
    } catch (...) {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(side, &junk);
        throw;
    }
    cudaGraph_t out = nullptr;
    SYSU_CUDA(cudaStreamEndCapture(side, &out));
    SYSU_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
}

void graph_loop_tail(cudaGraphConditionalHandle h, const int *stop, int *count, int bound, cudaStream_t st) {
    k_loop_tail<<<1, 1, 0, st>>>(h, stop, count, bound);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void graph_if_flag(cudaGraphConditionalHandle h, const int *flag, cudaStream_t st) {
    k_if_flag<<<1, 1, 0, st>>>(h, flag);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

namespace {
__global__ void k_loop_body_count(int *bodies) { *bodies += 1; }
}  // namespace

int graph_loop_selftest(int bound, int stop_at, cudaStream_t st) {
    if (bound < 1) throw CaseError{"graph_loop_selftest: bound must be >= 1"};
    DevBuf<int> d(3);  // stop flag, loop count, bodies run
    d.zero(st);
    cudaGraph_t g;
    SYSU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
        cudaGraphConditionalHandle h = graph_cond_handle(st, 1);
        graph_cond_node(st, graph_side_stream(), h, cudaGraphCondTypeWhile, [&](cudaStream_t s) {
            k_loop_body_count<<<1, 1, 0, s>>>(d.get() + 2);
            if (stop_at > 0) k_loop_stop_at<<<1, 1, 0, s>>>(d.get(), d.get() + 2, stop_at);
            graph_loop_tail(h, d.get(), d.get() + 1, bound, s);
        });
    } catch (...) {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(st, &junk);
        if (junk) cudaGraphDestroy(junk);
        throw;
    }
    SYSU_CUDA(cudaStreamEndCapture(st, &g));
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    SYSU_CUDA(e);
    int h[3] = {0, 0, 0};
    e = cudaGraphLaunch(exec, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d.get(), sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaGraphExecDestroy(exec);
    SYSU_CUDA(e);
    return h[2];
}

cudaStream_t graph_side_stream() {
    thread_local std::map<int, cudaStream_t> streams;
    int dev = 0;
    SYSU_CUDA(cudaGetDevice(&dev));
    auto it = streams.find(dev);
    if (it != streams.end()) return it->second;
    cudaStream_t s;
    SYSU_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    streams[dev] = s;
    return s;
}

}  // namespace sysu
