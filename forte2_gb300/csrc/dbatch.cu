// Many Davidson-Liu solves in one graph launch (see DavBatch in dgraph.cuh).
#include <set>
#include <string>

#include "dgraph.cuh"

namespace f2g {

// End of one loop body: keep looping while the solve runs and the loop count is below the limit.
__global__ void k_dg_continue(cudaGraphConditionalHandle h, const DGState* __restrict__ st, int32_t* loops,
                              int max_loops) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const int c = ++loops[0];
        cudaGraphSetConditional(h, (st->status == kDGRunning && c < max_loops) ? 1u : 0u);
    }
}

DavBatch::DavBatch(DavGraph* const* graphs, int count) {
    if (count < 1)
        throw Error(2, "dgraph batch: at least one solve");
    std::set<const SigmaBuilder*> builders;
    for (int i = 0; i < count; ++i) {
        if (!graphs[i])
            throw Error(2, "dgraph batch: NULL graph");
        if (!builders.insert(graphs[i]->sb).second)
            throw Error(2, "dgraph batch: every solve needs its own sigma builder");
    }
    g.assign(graphs, graphs + count);
    loops.reserve((size_t)count);
    build();
}

void DavBatch::build() {
    if (exec)
        cudaGraphExecDestroy(exec);
    exec = nullptr;
    serials.clear();
    for (DavGraph* d : g) {
        if (!d->exec)
            d->capture(); // the solve's set-up (scratch, FP32 tables) and its own graph
        d->prepare();     // current kernel variants' scratch (they may have changed since)
        serials.push_back(d->serial);
    }
    std::unique_lock<std::mutex> lock;
    cudaStream_t cap = capture_stream(lock);
    cudaGraph_t parent = nullptr;
    F2G_CUDA(cudaGraphCreate(&parent, 0));
    int count = 0;
    try {
        for (size_t i = 0; i < g.size(); ++i) {
            DavGraph& d = *g[i];
            cudaMemsetParams mp{};
            mp.dst = loops.get() + i;
            mp.value = 0;
            mp.elementSize = sizeof(int32_t);
            mp.width = 1;
            mp.height = 1;
            cudaGraphNode_t ms = nullptr;
            F2G_CUDA(cudaGraphAddMemsetNode(&ms, parent, nullptr, 0, &mp));
            cudaGraphConditionalHandle h{};
            F2G_CUDA(cudaGraphConditionalHandleCreate(&h, parent, 1, cudaGraphCondAssignDefault));
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t cn = nullptr;
            F2G_CUDA(cudaGraphAddNode(&cn, parent, &ms, nullptr, 1, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            F2G_CUDA(cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            try {
                d.iteration(cap);
                k_dg_continue<<<1, 32, 0, cap>>>(h, d.state_dev(), loops.get() + i, d.P.maxiter_cap + 2);
                F2G_LAUNCH("k_dg_continue");
            } catch (...) {
                cudaGraph_t dropped = nullptr;
                cudaStreamEndCapture(cap, &dropped);
                cudaGetLastError();
                throw;
            }
            cudaGraph_t captured = nullptr;
            F2G_CUDA(cudaStreamEndCapture(cap, &captured));
            size_t nb = 0;
            F2G_CUDA(cudaGraphGetNodes(body, nullptr, &nb));
            cudaGraphNode_t mc = nullptr;
            F2G_CUDA(cudaGraphAddMemcpyNode1D(&mc, parent, &cn, 1, d.host_state, d.state_dev(), sizeof(DGState),
                                              cudaMemcpyDeviceToHost));
            count += (int)nb + 2;
        }
        const cudaError_t e = cudaGraphInstantiate(&exec, parent, 0);
        if (e != cudaSuccess) {
            exec = nullptr;
            cudaGetLastError();
            throw Error(3, std::string("dgraph batch: graph instantiation failed: ") + cudaGetErrorString(e));
        }
    } catch (...) {
        cudaGraphDestroy(parent);
        throw;
    }
    cudaGraphDestroy(parent);
    nodes = count;
}

void DavBatch::launch(cudaStream_t s) {
    for (size_t i = 0; i < g.size(); ++i) {
        if (g[i]->serial != serials[i]) {
            build();
            break;
        }
    }
    F2G_CUDA(cudaGraphLaunch(exec, s));
}

} // namespace f2g
