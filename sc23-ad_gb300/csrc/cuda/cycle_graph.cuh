// One FGMRES restart cycle as one CUDA graph, with the convergence test on the
// device.
//
// FGMRESflex::Solve / FGMRES<T>::Solve (gmres.hpp:237-262, 56-80) stop the
// Arnoldi loop at the first step j whose |e_{j+1}| meets the tolerance.  The
// batched engines keep that decision per pair in device memory; the graph
// built here holds step 0 and then, for j = 1 .. m-1, a conditional (IF) node
// whose body is step j.  The last kernel of step j-1 sets the node's
// condition when some pair is still active, so a cycle needs no host round
// trip between steps: skipped bodies launch nothing, and the host reads the
// pairs' state once after the cycle.  Conditions reset to 0 at every launch
// of the graph.
#pragma once
#include <vector>

#include "../sagb_internal.hpp"
#include "common.cuh"

namespace sagb {

// condition of the next step's node: set when the step left any pair active
static __global__ void k_cycle_next(const int *__restrict__ n_active, cudaGraphConditionalHandle next) {
    pdl_trigger();
    pdl_wait();
    if (*n_active > 0) cudaGraphSetConditional(next, 1u);
}

struct CycleGraph {
    cudaGraphExec_t exec = nullptr;
    int m = 0;
    bool pdl = true;
    bool refused = false;                // the driver refused this form: per-step graphs instead
    std::vector<long long> step_launches;  // kernels of step j (for the launch count)
    void clear() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        step_launches.clear();
        m = 0;
    }
    ~CycleGraph() { clear(); }
};

// step(j, next, has_next) enqueues Arnoldi step j on c.stream and, when
// has_next, ends with k_cycle_next(..., next).  Returns false (and marks the
// form refused) when capture or instantiation of the conditional graph fails;
// the stream is then out of capture and the error cleared.
template <typename Step>
bool build_cycle_graph(Ctx &c, int m, CycleGraph &cg, Step &&step) {
    cg.clear();
    cudaStream_t main = c.stream, side = nullptr;
    cudaGraph_t g = nullptr;
    const long long before = c.launches;
    bool capturing = false;
    try {
        SAGB_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
        SAGB_CUDA(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal));
        capturing = true;
        cudaStreamCaptureStatus st;
        cudaGraph_t cap = nullptr;
        const cudaGraphNode_t *deps = nullptr;
        size_t nd = 0;
        SAGB_CUDA(cudaStreamGetCaptureInfo(main, &st, nullptr, &cap, &deps, nullptr, &nd));
        std::vector<cudaGraphConditionalHandle> h(m + 1, 0);
        for (int j = 1; j < m; j++) SAGB_CUDA(cudaGraphConditionalHandleCreate(&h[j], cap, 0, cudaGraphCondAssignDefault));
        long long l0 = c.launches;
        step(0, h[1], m > 1);
        cg.step_launches.push_back(c.launches - l0);
        for (int j = 1; j < m; j++) {
            SAGB_CUDA(cudaStreamGetCaptureInfo(main, &st, nullptr, &cap, &deps, nullptr, &nd));
            cudaGraphNodeParams cp = {};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = h[j];
            cp.conditional.type = cudaGraphCondTypeIf;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            SAGB_CUDA(cudaGraphAddNode(&node, cap, deps, nullptr, nd, &cp));
            SAGB_CUDA(cudaStreamUpdateCaptureDependencies(main, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            c.stream = side;
            SAGB_CUDA(cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            l0 = c.launches;
            try {
                step(j, h[j + 1], j + 1 < m);
            } catch (...) {
                cudaGraph_t tmp = nullptr;
                cudaStreamEndCapture(side, &tmp);
                throw;
            }
            cg.step_launches.push_back(c.launches - l0);
            SAGB_CUDA(cudaStreamEndCapture(side, &body));
            c.stream = main;
        }
        capturing = false;
        SAGB_CUDA(cudaStreamEndCapture(main, &g));
        SAGB_CUDA(cudaGraphInstantiate(&cg.exec, g, 0));
        cudaGraphDestroy(g);
        g = nullptr;
    } catch (const CudaError &) {
        c.stream = main;
        if (capturing) {
            cudaGraph_t tmp = nullptr;
            cudaStreamEndCapture(main, &tmp);
            if (tmp) cudaGraphDestroy(tmp);
        }
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        cg.clear();
        cg.refused = true;
    }
    c.stream = main;
    if (side) cudaStreamDestroy(side);
    c.launches = before;
    if (cg.exec) {
        cg.m = m;
        cg.pdl = c.use_pdl;
    }
    return cg.exec != nullptr;
}

}  // namespace sagb
