// CUDA-graph plumbing of the time step: conditional nodes inserted into an ongoing stream
// capture, and the kernel tally of what a captured step launches.
//
// A time step is captured once per regime and replayed with one cudaGraphLaunch.  The CG
// loop of a quasi-static solve is a conditional WHILE node whose body is one iteration; the
// iteration's last kernel decides on the device whether the loop goes on
// (cudaGraphSetConditional), so a solve needs no host round trip.  The reliable update of
// the mixed-precision solver is a conditional IF node inside that body.
#include "model.h"
#include <cstdlib>
#include <cstring>

namespace eqc {

thread_local int64_t* g_count_target = nullptr;
static thread_local int64_t g_tally = 0;

void capture_counting(bool on) {
    g_tally = 0;
    g_count_target = on ? &g_tally : nullptr;
}
int64_t capture_tally() { return g_tally; }

cudaGraphConditionalHandle cond_handle(Handle& h, unsigned dflt) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    EQC_CUDA(cudaStreamGetCaptureInfo(h.stream, &st, nullptr, &g, nullptr, nullptr, nullptr));
    if (st != cudaStreamCaptureStatusActive) throw Error(EQC_E_STATE, "conditional handle outside a capture");
    cudaGraphConditionalHandle c;
    // reset to dflt at every launch; a kernel upstream of (or inside) the node sets the value
    EQC_CUDA(cudaGraphConditionalHandleCreate(&c, g, dflt, cudaGraphCondAssignDefault));
    return c;
}

void cond_begin(Handle& h, cudaGraphConditionalNodeType type, cudaGraphConditionalHandle c) {
    const size_t depth = h.stream_stack.size();
    if (depth >= 4) throw Error(EQC_E_STATE, "conditional nodes nested too deeply");
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    EQC_CUDA(cudaStreamGetCaptureInfo(h.stream, &st, nullptr, &g, &deps, nullptr, &nd));
    if (st != cudaStreamCaptureStatusActive) throw Error(EQC_E_STATE, "conditional node outside a capture");
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = c;
    p.conditional.type = type;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    EQC_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    EQC_CUDA(cudaStreamUpdateCaptureDependencies(h.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    if (!h.cap_streams[depth]) EQC_CUDA(cudaStreamCreateWithFlags(&h.cap_streams[depth], cudaStreamNonBlocking));
    cudaStream_t bs = h.cap_streams[depth];
    EQC_CUDA(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    h.stream_stack.push_back(h.stream);
    h.stream = bs;
}

void abort_capture(Handle& h) {
    while (!h.stream_stack.empty()) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(h.stream, &g);
        h.stream = h.stream_stack.back();
        h.stream_stack.pop_back();
    }
    cudaStreamCaptureStatus st;
    if (cudaStreamIsCapturing(h.stream, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(h.stream, &g);
        if (g) cudaGraphDestroy(g);
    }
    cudaGetLastError();
    h.stream = h.own_stream;
    h.pdl_off = false;
    capture_counting(false);
}

static bool own_kernel(cudaGraphNode_t n) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(n, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) return false;
    cudaKernelNodeParams p{};
    if (cudaGraphKernelNodeGetParams(n, &p) != cudaSuccess || !p.func) return false;
    cudaLaunchAttributeValue cl{};   // cluster launches keep ordinary edges
    if (cudaGraphKernelNodeGetAttribute(n, cudaLaunchAttributeClusterDimension, &cl) == cudaSuccess &&
        (size_t)cl.clusterDim.x * cl.clusterDim.y * cl.clusterDim.z > 1)
        return false;
    const char* name = nullptr;
    if (cudaFuncGetName(&name, p.func) != cudaSuccess || !name) return false;
    return std::strncmp(name, "_ZN3eqc", 7) == 0 || std::strstr(name, "eqc::") != nullptr;
}

int64_t make_programmatic(cudaGraph_t g) {
    if (std::getenv("EQC_NO_PDL") || !g) return 0;
    size_t n = 0;
    EQC_CUDA(cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &n));
    if (n == 0) return 0;
    std::vector<cudaGraphNode_t> from(n), to(n);
    std::vector<cudaGraphEdgeData> ed(n);
    EQC_CUDA(cudaGraphGetEdges(g, from.data(), to.data(), ed.data(), &n));
    std::unordered_map<cudaGraphNode_t, int> indeg;
    for (size_t i = 0; i < n; ++i) indeg[to[i]] += 1;
    int64_t changed = 0;
    for (size_t i = 0; i < n; ++i) {
        if (ed[i].type != cudaGraphDependencyTypeDefault || ed[i].from_port != cudaGraphKernelNodePortDefault) continue;
        if (indeg[to[i]] != 1 || !own_kernel(from[i]) || !own_kernel(to[i])) continue;
        EQC_CUDA(cudaGraphRemoveDependencies(g, &from[i], &to[i], &ed[i], 1));
        cudaGraphEdgeData pe{};
        pe.from_port = cudaGraphKernelNodePortLaunchCompletion;
        pe.type = cudaGraphDependencyTypeProgrammatic;
        EQC_CUDA(cudaGraphAddDependencies(g, &from[i], &to[i], &pe, 1));
        ++changed;
    }
    return changed;
}

void cond_end(Handle& h) {
    if (h.stream_stack.empty()) throw Error(EQC_E_STATE, "cond_end without cond_begin");
    cudaGraph_t g = nullptr;
    EQC_CUDA(cudaStreamEndCapture(h.stream, &g));
    if (!h.pdl_off) h.pdl_edges += make_programmatic(g);
    h.stream = h.stream_stack.back();
    h.stream_stack.pop_back();
}

}  // namespace eqc
