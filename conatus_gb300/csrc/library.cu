// Library-wide C-ABI entry points: errors, version, device queries.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "common.cuh"
#include "conatus_gb300.h"

namespace cng {
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
}  // namespace cng

extern "C" {

const char* cng_last_error(void) { return cng::g_last_error.c_str(); }

const char* cng_version(void) { return "conatus_gb300 0.1.0 (sm_103a)"; }

int cng_cuda_available(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n > 0 ? 1 : 0;
}

int cng_device_name(int dev, char* buf, int buflen) {
    cudaDeviceProp p;
    cudaError_t e = cudaGetDeviceProperties(&p, dev);
    if (e != cudaSuccess) {
        cng::set_error(cudaGetErrorString(e));
        return cng::CNG_ECUDA;
    }
    if (buf && buflen > 0) {
        std::strncpy(buf, p.name, buflen - 1);
        buf[buflen - 1] = 0;
    }
    return 0;
}

int cng_mem_info(uint64_t* free_bytes, uint64_t* total_bytes) {
    size_t f = 0, t = 0;
    cudaError_t e = cudaMemGetInfo(&f, &t);
    if (e != cudaSuccess) {
        cng::set_error(cudaGetErrorString(e));
        return cng::CNG_ECUDA;
    }
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return 0;
}

struct cng_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

int cng_graph_begin(void* stream) {
    CNG_TRY({
        if (!stream) throw cng::InvalidArgument("graph capture needs a non-default stream");
        CNG_CUDA(cudaStreamBeginCapture(static_cast<cudaStream_t>(stream), cudaStreamCaptureModeThreadLocal));
    })
}

int cng_graph_end(void* stream, cng_graph** out) {
    CNG_TRY({
        if (!out) throw cng::InvalidArgument("null output");
        *out = nullptr;
        auto* g = new cng_graph();
        cudaError_t e = cudaStreamEndCapture(static_cast<cudaStream_t>(stream), &g->graph);
        if (e != cudaSuccess) {
            delete g;
            CNG_CUDA(e);
        }
        e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g->graph);
            delete g;
            CNG_CUDA(e);
        }
        *out = g;
    })
}

int cng_graph_launch(cng_graph* g, void* stream) {
    CNG_TRY({
        if (!g) throw cng::InvalidArgument("null graph");
        CNG_CUDA(cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)));
    })
}

int cng_graph_destroy(cng_graph* g) {
    CNG_TRY({
        if (g) {
            if (g->exec) cudaGraphExecDestroy(g->exec);
            if (g->graph) cudaGraphDestroy(g->graph);
            delete g;
        }
    })
}

}  // extern "C"
