// Library-wide C-ABI entry points: errors, version, device queries.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>

#include "common.cuh"
#include "conatus_gb300.h"

namespace cng {
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

namespace {
struct Pool {
    std::mutex mu;
    std::unordered_map<void*, size_t> bytes;
    uint64_t live = 0, n_alloc = 0;
};
// never destroyed: handles may still be released while the process exits
Pool& pool() {
    static Pool* p = new Pool;
    return *p;
}
}  // namespace

void* dev_alloc(size_t bytes) {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw CudaFailure(std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes failed: " +
                          cudaGetErrorString(e));
    }
    Pool& p = pool();
    try {
        std::lock_guard<std::mutex> lock(p.mu);
        p.bytes[q] = bytes;
        p.live += bytes;
        ++p.n_alloc;
    } catch (...) {
        cudaFree(q);
        throw;
    }
    return q;
}

void dev_free(void* q) {
    if (!q) return;
    {
        Pool& p = pool();
        std::lock_guard<std::mutex> lock(p.mu);
        auto it = p.bytes.find(q);
        if (it != p.bytes.end()) {
            p.live -= it->second;
            p.bytes.erase(it);
        }
    }
    cudaFree(q);
}

void pool_counters(uint64_t* live_bytes, uint64_t* n_alloc) {
    Pool& p = pool();
    std::lock_guard<std::mutex> lock(p.mu);
    if (live_bytes) *live_bytes = p.live;
    if (n_alloc) *n_alloc = p.n_alloc;
}
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

int cng_pool_stats(uint64_t* live_bytes, uint64_t* cached_bytes, uint64_t* n_alloc, uint64_t* n_reuse) {
    CNG_TRY({
        cng::pool_counters(live_bytes, n_alloc);
        if (cached_bytes) *cached_bytes = 0;       // freed memory goes back to the driver at once
        if (n_reuse) *n_reuse = 0;
    })
}

int cng_pool_trim(void) { return 0; }

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

// FP64 arithmetic rate probe: every thread runs `iters` rounds of 8 independent fused multiply-adds
// on registers (8 chains hide the pipe's latency), then folds them into one store so that nothing
// is removed. 16 flops per thread and round.
namespace cng {
__global__ void k_dfma_probe(long long iters, double a, double b, double* __restrict__ sink) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (threadIdx.x + k) * 1e-3;
    for (long long i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == 12345.6789) sink[0] = s;          // never true for the probe's inputs; keeps the chains
}
}  // namespace cng

extern "C" int cng_dfma_probe(int64_t iters, int blocks_per_sm, void* sink, double* flops, void* stream) {
    CNG_TRY({
        if (iters <= 0 || blocks_per_sm <= 0 || !sink || !flops) throw cng::InvalidArgument("dfma_probe: bad argument");
        const int blocks = cng::sm_count() * blocks_per_sm, threads = 256;
        cng::k_dfma_probe<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(iters, 0.999999, 1e-7,
                                                                                      static_cast<double*>(sink));
        CNG_LAUNCH("k_dfma_probe");
        *flops = 16.0 * (double)iters * (double)blocks * threads;
    })
}

