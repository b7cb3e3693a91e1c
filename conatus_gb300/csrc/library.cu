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

}  // extern "C"
