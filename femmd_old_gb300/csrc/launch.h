// launch.h -- one code path for direct stream launches and CUDA-graph
// construction.  Every kernel of the timestep is issued through
// Launch::kernel(); with graph == nullptr it is a plain <<<>>> launch on the
// context stream, otherwise it becomes a kernel node depending on the
// previous node (a linear chain), and begin_if() opens a conditional IF node
// whose body is filled by a child Launch.
#pragma once
#include <cuda_runtime.h>
#include <tuple>
#include <utility>
#include <vector>

namespace femmd {

struct Launch {
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    std::vector<cudaGraphNode_t> deps;
    // direct-mode timing of the force kernel: event pairs appended per launch
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> *force_events = nullptr;
    std::vector<cudaEvent_t> *event_pool = nullptr;
    long long kernels = 0;

    template <typename... KArgs, typename... Args>
    cudaError_t kernel(void (*k)(KArgs...), dim3 g, dim3 b, size_t smem, Args &&...args) {
        if (g.x == 0 || g.y == 0 || g.z == 0) return cudaSuccess;
        kernels++;
        if (!graph) {
            k<<<g, b, smem, stream>>>(std::forward<Args>(args)...);
            return cudaGetLastError();
        }
        std::tuple<KArgs...> store(std::forward<Args>(args)...);
        void *ptrs[sizeof...(KArgs) > 0 ? sizeof...(KArgs) : 1];
        fill(ptrs, store, std::index_sequence_for<KArgs...>{});
        cudaKernelNodeParams p = {};
        p.func = (void *)k;
        p.gridDim = g;
        p.blockDim = b;
        p.sharedMemBytes = (unsigned)smem;
        p.kernelParams = ptrs;
        p.extra = nullptr;
        cudaGraphNode_t n;
        cudaError_t e = cudaGraphAddKernelNode(&n, graph, deps.empty() ? nullptr : deps.data(), deps.size(), &p);
        if (e != cudaSuccess) return e;
        deps.assign(1, n);
        return cudaSuccess;
    }

    // Record an event on the stream (direct mode only) from the pool.
    cudaEvent_t mark() {
        if (graph || !event_pool) return nullptr;
        cudaEvent_t ev;
        if (event_pool->empty()) {
            if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
        } else {
            ev = event_pool->back();
            event_pool->pop_back();
        }
        cudaEventRecord(ev, stream);
        return ev;
    }

    // Open an IF node (condition set on the device by cudaGraphSetConditional);
    // 'body' receives the body graph.  Graph mode only.
    cudaError_t begin_if(cudaGraphConditionalHandle h, Launch &body) {
        cudaGraphNodeParams p = {};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeIf;
        p.conditional.size = 1;
        cudaGraphNode_t n;
        cudaError_t e = cudaGraphAddNode(&n, graph, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &p);
        if (e != cudaSuccess) return e;
        deps.assign(1, n);
        body.stream = stream;
        body.graph = p.conditional.phGraph_out[0];
        body.deps.clear();
        return cudaSuccess;
    }

    // Open a WHILE node (the body runs while the condition, set on the
    // device, is nonzero); 'body' receives the body graph.  Graph mode only.
    cudaError_t begin_while(cudaGraphConditionalHandle h, Launch &body) {
        cudaGraphNodeParams p = {};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t n;
        cudaError_t e = cudaGraphAddNode(&n, graph, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &p);
        if (e != cudaSuccess) return e;
        deps.assign(1, n);
        body.stream = stream;
        body.graph = p.conditional.phGraph_out[0];
        body.deps.clear();
        return cudaSuccess;
    }

    // Mark the last kernel node cooperative (all its blocks co-resident).
    cudaError_t cooperative_last() {
        if (!graph || deps.empty()) return cudaErrorInvalidValue;
        cudaLaunchAttributeValue v = {};
        v.cooperative = 1;
        return cudaGraphKernelNodeSetAttribute(deps.back(), cudaLaunchAttributeCooperative, &v);
    }

  private:
    template <typename Tup, size_t... I>
    static void fill(void **ptrs, Tup &t, std::index_sequence<I...>) {
        ((ptrs[I] = (void *)&std::get<I>(t)), ...);
    }
};

}  // namespace femmd
