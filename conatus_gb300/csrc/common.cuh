// Shared helpers of the conatus_gb300 CUDA library: complex arithmetic, error reporting through a
// thread-local message (the C-ABI returns an int status), launch checks.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <set>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace cng {

// Status codes of the C-ABI (0 = success).
enum Status : int {
    CNG_OK = 0,
    CNG_EINVAL = 1,      // invalid argument (ValueError on the Python side)
    CNG_ERUNTIME = 2,    // numerical or runtime failure (RuntimeError), e.g. "singular"
    CNG_ECUDA = 3,       // CUDA error
    CNG_ENOMEM = 4,      // allocation failed
};

struct InvalidArgument : std::invalid_argument {
    using std::invalid_argument::invalid_argument;
};
struct RuntimeFailure : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct CudaFailure : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void set_error(const std::string& msg);

// Device memory held by the library's handles (banded factors, evaluator buffers): cudaMalloc and
// cudaFree with live-byte and allocation counters (the counters of the reference core's pool).
// dev_free also takes pointers that dev_alloc did not return (they are freed, not counted).
void* dev_alloc(size_t bytes);
void dev_free(void* p);
void pool_counters(uint64_t* live_bytes, uint64_t* n_alloc);

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        throw CudaFailure(std::string(what) + ": " + cudaGetErrorString(e));
}
#define CNG_CUDA(call) ::cng::cuda_check((call), #call)
#define CNG_LAUNCH(what) ::cng::cuda_check(cudaGetLastError(), what)

// Raise a kernel's dynamic shared-memory limit to `bytes` on the current device, once per (kernel,
// device): the attribute belongs to the device's context, so a second device needs its own call.
inline void ensure_smem_attr(const void* fn, int bytes) {
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({fn, dev})) return;
    cuda_check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
               "cudaFuncSetAttribute(MaxDynamicSharedMemorySize)");
    done.insert({fn, dev});
}

// Grouped launches: one launch runs a kernel body over up to kMaxGrp argument sets (problems of
// different sizes), each over its own range of blocks [start[k], start[k + 1]). The body sees its
// block index and block count within its range. Passed as a __grid_constant__ kernel parameter.
constexpr int kMaxGrp = 8;
template <class A>
struct Grp {
    int n = 0;
    unsigned start[kMaxGrp + 1] = {};
    A a[kMaxGrp];
    __device__ __forceinline__ int find(unsigned b) const {
        int k = 0;
        while (k + 1 < n && b >= start[k + 1]) ++k;
        return k;
    }
};

// Launch fn(table, total blocks) over `args` (blocks[i] blocks each; empty entries dropped), in as
// few launches as kMaxGrp entries per launch allow.
template <class A, class Fn>
void launch_groups(const std::vector<A>& args, const std::vector<unsigned>& blocks, Fn fn) {
    Grp<A> g{};
    unsigned total = 0;
    for (size_t i = 0; i < args.size(); ++i) {
        if (blocks[i] == 0) continue;
        if (blocks[i] > 0x7fffffffu - total) throw InvalidArgument("grouped launch: too many blocks");
        g.start[g.n] = total;
        g.a[g.n] = args[i];
        total += blocks[i];
        g.start[++g.n] = total;
        if (g.n == kMaxGrp) {
            fn(g, total);
            g = Grp<A>{};
            total = 0;
        }
    }
    if (g.n) fn(g, total);
}

// Two timing events, destroyed on every exit path (a failed second creation frees the first).
struct EventPair {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    EventPair() {
        cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
        const cudaError_t e = cudaEventCreate(&e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cuda_check(e, "cudaEventCreate");
        }
    }
    ~EventPair() {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    EventPair(const EventPair&) = delete;
    EventPair& operator=(const EventPair&) = delete;
};

// ---- complex double with explicit operations (no library dependency in device code) ----------
struct alignas(16) zd {
    double re, im;
    __host__ __device__ zd() : re(0), im(0) {}
    __host__ __device__ zd(double r) : re(r), im(0) {}
    __host__ __device__ zd(double r, double i) : re(r), im(i) {}
};
__host__ __device__ inline zd operator+(zd a, zd b) { return zd(a.re + b.re, a.im + b.im); }
__host__ __device__ inline zd operator-(zd a, zd b) { return zd(a.re - b.re, a.im - b.im); }
__host__ __device__ inline zd operator-(zd a) { return zd(-a.re, -a.im); }
__host__ __device__ inline zd operator*(zd a, zd b) {
    return zd(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__host__ __device__ inline zd operator*(double s, zd a) { return zd(s * a.re, s * a.im); }
// v - a b and v + a b with two fused multiply-adds per component (four FP64 instructions, where
// v - (a * b) takes six: two multiplies, two fused multiply-adds and two subtractions)
__host__ __device__ inline zd cfms(zd v, zd a, zd b) {
    return zd(fma(a.im, b.im, fma(-a.re, b.re, v.re)), fma(-a.im, b.re, fma(-a.re, b.im, v.im)));
}
__host__ __device__ inline zd cfma(zd v, zd a, zd b) {
    return zd(fma(-a.im, b.im, fma(a.re, b.re, v.re)), fma(a.im, b.re, fma(a.re, b.im, v.im)));
}
// a / b by Smith's method (overflow-safe scaling of the denominator).
__host__ __device__ inline zd operator/(zd a, zd b) {
    if (fabs(b.re) >= fabs(b.im)) {
        double r = b.im / b.re, d = b.re + b.im * r;
        return zd((a.re + a.im * r) / d, (a.im - a.re * r) / d);
    }
    double r = b.re / b.im, d = b.im + b.re * r;
    return zd((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
__host__ __device__ inline bool operator==(zd a, zd b) { return a.re == b.re && a.im == b.im; }
__host__ __device__ inline bool operator!=(zd a, zd b) { return !(a == b); }

// ---- complex float (FP32 factors of the mixed-precision solve) --------------------------------
struct alignas(8) zf {
    float re, im;
    __host__ __device__ zf() : re(0), im(0) {}
    __host__ __device__ zf(float r) : re(r), im(0) {}
    __host__ __device__ zf(double r) : re((float)r), im(0) {}
    __host__ __device__ zf(float r, float i) : re(r), im(i) {}
};
__host__ __device__ inline zf operator+(zf a, zf b) { return zf(a.re + b.re, a.im + b.im); }
__host__ __device__ inline zf operator-(zf a, zf b) { return zf(a.re - b.re, a.im - b.im); }
__host__ __device__ inline zf operator-(zf a) { return zf(-a.re, -a.im); }
__host__ __device__ inline zf operator*(zf a, zf b) {
    return zf(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__host__ __device__ inline zf cfms(zf v, zf a, zf b) {
    return zf(fmaf(a.im, b.im, fmaf(-a.re, b.re, v.re)), fmaf(-a.im, b.re, fmaf(-a.re, b.im, v.im)));
}
__host__ __device__ inline zf cfma(zf v, zf a, zf b) {
    return zf(fmaf(-a.im, b.im, fmaf(a.re, b.re, v.re)), fmaf(a.im, b.re, fmaf(a.re, b.im, v.im)));
}
__host__ __device__ inline zf operator/(zf a, zf b) {
    if (fabsf(b.re) >= fabsf(b.im)) {
        float r = b.im / b.re, d = b.re + b.im * r;
        return zf((a.re + a.im * r) / d, (a.im - a.re * r) / d);
    }
    float r = b.re / b.im, d = b.im + b.re * r;
    return zf((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
__host__ __device__ inline bool is_zero(zf x) { return x.re == 0.0f && x.im == 0.0f; }
__device__ inline zf shfl_xor(zf v, int m) {
    return zf(__shfl_xor_sync(0xffffffffu, v.re, m), __shfl_xor_sync(0xffffffffu, v.im, m));
}
__host__ __device__ inline zf to_zf(zd a) { return zf((float)a.re, (float)a.im); }

// Magnitudes: |.| of LAPACK's pivot search (i?amax: |re| + |im| for complex) and the modulus.
__host__ __device__ inline double abs1(double x) { return fabs(x); }
__host__ __device__ inline double abs1(zd x) { return fabs(x.re) + fabs(x.im); }
__host__ __device__ inline double absval(double x) { return fabs(x); }
__host__ __device__ inline double absval(zd x) { return hypot(x.re, x.im); }
__host__ __device__ inline bool is_zero(double x) { return x == 0.0; }
__host__ __device__ inline bool is_zero(zd x) { return x.re == 0.0 && x.im == 0.0; }
__host__ __device__ inline bool finite_val(double x) { return isfinite(x); }
__host__ __device__ inline bool finite_val(zd x) { return isfinite(x.re) && isfinite(x.im); }

template <class T> __host__ __device__ inline T one();
template <> __host__ __device__ inline double one<double>() { return 1.0; }
template <> __host__ __device__ inline zd one<zd>() { return zd(1.0, 0.0); }
template <> __host__ __device__ inline zf one<zf>() { return zf(1.0f, 0.0f); }

// Warp shuffle of either type.
__device__ inline double shfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ inline zd shfl(zd v, int src) {
    return zd(__shfl_sync(0xffffffffu, v.re, src), __shfl_sync(0xffffffffu, v.im, src));
}
__device__ inline double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ inline double shfl_down_r(double v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ inline float shfl_down_r(float v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ inline zd shfl_xor(zd v, int m) {
    return zd(__shfl_xor_sync(0xffffffffu, v.re, m), __shfl_xor_sync(0xffffffffu, v.im, m));
}
template <class T>
__device__ inline T warp_sum(T v) {
    for (int m = 16; m > 0; m >>= 1) v = v + shfl_xor(v, m);
    return v;
}

// Body of a C-ABI function: exceptions become a status code and the thread-local message.
#define CNG_TRY(...)                                                                   \
    try {                                                                              \
        __VA_ARGS__;                                                                   \
        return ::cng::CNG_OK;                                                          \
    } catch (const ::cng::InvalidArgument& e) {                                        \
        ::cng::set_error(e.what());                                                    \
        return ::cng::CNG_EINVAL;                                                      \
    } catch (const ::cng::RuntimeFailure& e) {                                         \
        ::cng::set_error(e.what());                                                    \
        return ::cng::CNG_ERUNTIME;                                                    \
    } catch (const ::cng::CudaFailure& e) {                                            \
        ::cng::set_error(e.what());                                                    \
        return ::cng::CNG_ECUDA;                                                       \
    } catch (const std::bad_alloc&) {                                                  \
        ::cng::set_error("host allocation failed");                                    \
        return ::cng::CNG_ENOMEM;                                                      \
    } catch (const std::exception& e) {                                                \
        ::cng::set_error(e.what());                                                    \
        return ::cng::CNG_ERUNTIME;                                                    \
    }

inline int ceil_div(long long a, long long b) { return static_cast<int>((a + b - 1) / b); }

// Streaming multiprocessors of the current device (read once per device).
inline int sm_count() {
    static int cached[32] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 32) return 152;
    if (cached[dev] <= 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = v > 0 ? v : 152;
    }
    return cached[dev];
}

}  // namespace cng
