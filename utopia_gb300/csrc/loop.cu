// Device-side iteration loop: a CUDA graph whose single node is a conditional WHILE
// node.  The body is one solver iteration captured from the stream; its last kernel
// sets the loop condition from the solver's stop flag.  One graph launch runs the
// whole solve with the exact iteration count and no host round trip per iteration.
// A device counter caps the number of body executions (the solver's own max_it stops
// it first); hitting the cap records an error flag the host checks afterwards.
#include "abi_util.cuh"
#include "solver.cuh"

namespace ugpu {

namespace {
__global__ void k_loop_tail(cudaGraphConditionalHandle handle, const int *done, int *count, int cap, int *overrun) {
    const int c = *count + 1;
    *count = c;
    unsigned int go = (*done == 0) ? 1u : 0u;
    if (go && c >= cap) {
        *overrun = 1;
        go = 0u;
    }
    cudaGraphSetConditional(handle, go);
}
}  // namespace

DeviceLoop::~DeviceLoop() { reset(); }

void DeviceLoop::reset() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    kernels = 0;
}

void DeviceLoop::build(Context &ctx, const std::function<void()> &body, const int *done, int cap) {
    reset();
    if (!state.ptr) state.alloc(sizeof(int) * 2);
    UGPU_CUDA(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle handle;
    UGPU_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = handle;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    UGPU_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &p));
    cudaGraph_t bodyg = p.conditional.phGraph_out[0];
    const int64_t l0 = ctx.launches;
    UGPU_CUDA(cudaStreamBeginCaptureToGraph(ctx.stream, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    try {
        body();
        k_loop_tail<<<1, 1, 0, ctx.stream>>>(handle, done, state.as<int>(), cap, state.as<int>() + 1);
        ctx.launches++;
        UGPU_LAUNCH_CHECK();
    } catch (...) {
        cudaGraph_t g;
        cudaStreamEndCapture(ctx.stream, &g);
        reset();
        throw;
    }
    UGPU_CUDA(cudaStreamEndCapture(ctx.stream, &bodyg));
    UGPU_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    kernels = ctx.launches - l0;
    ctx.launches = l0;
}

// runs the loop; returns the number of body executions (synchronises)
int DeviceLoop::run(Context &ctx) {
    UGPU_CHECK(exec, UGPU_ERR_STATE, "device loop not built");
    UGPU_CUDA(cudaMemsetAsync(state.ptr, 0, sizeof(int) * 2, ctx.stream));
    UGPU_CUDA(cudaGraphLaunch(exec, ctx.stream));
    int h[2] = {0, 0};
    UGPU_CUDA(cudaMemcpyAsync(h, state.ptr, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx.stream));
    UGPU_CUDA(cudaStreamSynchronize(ctx.stream));
    ctx.launches += kernels * h[0];
    UGPU_CHECK(!h[1], UGPU_ERR_INTERNAL, "device loop reached its iteration cap without the stop flag");
    return h[0];
}

}  // namespace ugpu
