// Batched bordered-banded factor and solves on the GPU (FP64 real and complex).
//
// A tau system is banded except for its r boundary ("border") rows. With the border rows moved to
// the top (row permutation P), P A = B + U V^T where B equals P A with each border row i replaced by
// s_i e_i (s_i = max |row i|, 1 for a zero row), U = [e_0 .. e_{r-1}] and V^T = border rows - diag(s).
// B is factored by LU with partial pivoting inside the band (the LAPACK gbtf2 algorithm and pivot
// rule), then W = B^{-1} U and the capacitance S = I + V^T W (LU, 1-norm condition). A solve is
// y = B^{-1} P b, z = S^{-1} V^T y, x = y - W z (Woodbury). This is the algorithm of the reference's
// core/include/conatus/banded.hpp:1-27,170-478 and of its GPU batch (core/src/cuda/banded.cu); the
// kernels below are this library's own design.
//
// GPU layout (one handle = one batch of systems of equal n, common band kl/ku):
//   ab   [batch][n][ldab]   LAPACK band storage per system, column j at ab + j*ldab, A(i,j) at row
//                           kv + i - j (kv = kl + ku); LU factors after the factorization
//   ipiv [batch][n]         0-based pivot rows
//   vt   [batch][r][n]      V^T rows;  w [batch][r][n]  columns of W stored as rows
//   slu  [batch][r][r]      LU of S (column-major), spiv [batch][r]
// One warp owns one system in every kernel: the band recurrences are sequential along n and each
// column's band entries are spread over the lanes; the working vector lives in shared memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "conatus_gb300.h"

namespace cng {

static constexpr int kWarpsPerBlock = 4;
static constexpr size_t kMaxSolveSmem = 200 * 1024;   // bytes of shared memory for the y vectors

template <class T>
struct BandView {
    int batch, n, r, kl, ku, ldab, pivot;
    T* ab;
    int* ipiv;
    T* vt;
    T* w;
    T* slu;
    int* spiv;
    const int* perm;      // n entries, shared by the batch (border rows first)
    int* info;            // per system: 0 ok, j+1 singular band pivot j, -1 singular capacitance,
                          // -2 non-finite capacitance condition
    double* cond;         // per system: 1-norm condition of S (1 when r = 0)
    // transposed Woodbury data (built on demand)
    T* wt;                // [batch][r][n]
    T* stlu;              // [batch][r][r]
    int* stpiv;           // [batch][r]
};

// ------------------------------------------------------------------------------------------------
// device building blocks (one warp, lane = threadIdx.x & 31)

template <class T>
__device__ inline T band_at(const T* ab, int ldab, int kv, int i, int j) {
    return ab[(size_t)j * ldab + (kv + i - j)];
}

// In-place LU of the band (LAPACK gbtf2 order). Returns 0 or j+1 of the first zero pivot.
template <class T>
__device__ int warp_gbtf2(T* ab, int* ipiv, int n, int kl, int ku, int ldab, int pivot) {
    const int lane = threadIdx.x & 31;
    const int kv = kl + ku;
    int ju = 0, info = 0;
    for (int j = 0; j < n; ++j) {
        const int km = min(kl, n - 1 - j);
        T* colj = ab + (size_t)j * ldab;
        // pivot: largest |.|_1 among rows j..j+km, first index on ties (i?amax)
        int jp = 0;
        if (pivot) {
            double best = -1.0;
            int bi = 0;
            for (int t = lane; t <= km; t += 32) {
                double a = abs1(colj[kv + t]);
                if (a > best) { best = a; bi = t; }
            }
            for (int m = 16; m > 0; m >>= 1) {
                double ob = __shfl_xor_sync(0xffffffffu, best, m);
                int oi = __shfl_xor_sync(0xffffffffu, bi, m);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            jp = bi;
        }
        if (lane == 0) ipiv[j] = j + jp;
        const T piv = colj[kv + jp];
        if (!is_zero(piv)) {
            ju = max(ju, min(j + ku + jp, n - 1));
            if (jp != 0) {
                for (int c = j + lane; c <= ju; c += 32) {
                    T* cc = ab + (size_t)c * ldab;
                    T a = cc[kv + j + jp - c], b = cc[kv + j - c];
                    cc[kv + j + jp - c] = b;
                    cc[kv + j - c] = a;
                }
                __syncwarp();
            }
            if (km > 0) {
                const T rp = one<T>() / colj[kv];
                for (int t = 1 + lane; t <= km; t += 32) colj[kv + t] = rp * colj[kv + t];
                __syncwarp();
                const int w = ju - j;
                const int cnt = w * km;
                for (int idx = lane; idx < cnt; idx += 32) {
                    const int c = j + 1 + idx / km;
                    const int t = 1 + idx % km;
                    T* cc = ab + (size_t)c * ldab;
                    const T u = cc[kv + j - c];
                    cc[kv + j + t - c] = cc[kv + j + t - c] - colj[kv + t] * u;
                }
                __syncwarp();
            }
        } else if (info == 0) {
            info = j + 1;
        }
    }
    return info;
}

// y := B^{-1} y with the band LU (gbtrs 'N'); y in shared or global memory, one warp.
template <class T>
__device__ void warp_band_solve(const T* ab, const int* ipiv, T* y, int n, int kl, int ku, int ldab) {
    const int lane = threadIdx.x & 31;
    const int kv = kl + ku;
    if (kl > 0) {
        for (int j = 0; j < n - 1; ++j) {
            const int lm = min(kl, n - 1 - j);
            const int l = ipiv[j];
            const T bj = y[l];
            const T yj0 = y[j];
            __syncwarp();
            const T* colj = ab + (size_t)j * ldab + kv + 1;
            for (int t = lane; t < lm; t += 32) {
                const int i = j + 1 + t;
                const T v = (i == l) ? yj0 : y[i];
                y[i] = v - colj[t] * bj;
            }
            if (lane == 0) y[j] = bj;
            __syncwarp();
        }
    }
    for (int j = n - 1; j >= 0; --j) {
        T yj = y[j];
        if (is_zero(yj)) {
            __syncwarp();
            continue;
        }
        const T* colj = ab + (size_t)j * ldab;
        yj = yj * colj[kv];                          // the diagonal holds 1 / u_jj
        const int m = min(kv, j);
        for (int t = lane; t < m; t += 32) {
            const int i = j - 1 - t;
            y[i] = y[i] - yj * colj[kv - 1 - t];
        }
        if (lane == 0) y[j] = yj;
        __syncwarp();
    }
}

// y := B^{-T} y (gbtrs 'T', plain transpose): U^T then L^T with the interchanges.
template <class T>
__device__ void warp_band_solve_T(const T* ab, const int* ipiv, T* y, int n, int kl, int ku, int ldab) {
    const int lane = threadIdx.x & 31;
    const int kv = kl + ku;
    for (int j = 0; j < n; ++j) {
        const T* colj = ab + (size_t)j * ldab;
        const int i0 = max(0, j - kv);
        T acc = T(0.0);
        for (int i = i0 + lane; i < j; i += 32) acc = acc + colj[kv + i - j] * y[i];
        acc = warp_sum(acc);
        const T yj = (y[j] - acc) * colj[kv];          // the diagonal holds 1 / u_jj
        __syncwarp();
        if (lane == 0) y[j] = yj;
        __syncwarp();
    }
    if (kl > 0) {
        for (int j = n - 2; j >= 0; --j) {
            const int lm = min(kl, n - 1 - j);
            const T* colj = ab + (size_t)j * ldab + kv + 1;
            T acc = T(0.0);
            for (int t = lane; t < lm; t += 32) acc = acc + colj[t] * y[j + 1 + t];
            acc = warp_sum(acc);
            const T yj = y[j] - acc;
            const int l = ipiv[j];
            const T yl = y[l];
            __syncwarp();
            if (lane == 0) {
                if (l != j) {
                    y[j] = yl;
                    y[l] = yj;
                } else {
                    y[j] = yj;
                }
            }
            __syncwarp();
        }
    }
}

// LU with partial pivoting of a small r x r column-major matrix by lane 0 (getrf semantics).
// Returns 0 or k+1 of the first zero pivot.
template <class T>
__device__ int small_getrf(T* a, int* piv, int r) {
    int info = 0;
    for (int k = 0; k < r; ++k) {
        int p = k;
        double best = abs1(a[k * r + k]);
        for (int i = k + 1; i < r; ++i) {
            double v = abs1(a[k * r + i]);
            if (v > best) { best = v; p = i; }
        }
        piv[k] = p;
        if (is_zero(a[k * r + p])) {
            if (info == 0) info = k + 1;
            continue;
        }
        if (p != k)
            for (int c = 0; c < r; ++c) {
                T t = a[c * r + k];
                a[c * r + k] = a[c * r + p];
                a[c * r + p] = t;
            }
        const T rp = one<T>() / a[k * r + k];
        for (int i = k + 1; i < r; ++i) a[k * r + i] = rp * a[k * r + i];
        for (int c = k + 1; c < r; ++c) {
            const T u = a[c * r + k];
            for (int i = k + 1; i < r; ++i) a[c * r + i] = a[c * r + i] - a[k * r + i] * u;
        }
    }
    // the factored form keeps 1 / u_kk on the diagonal (solves multiply; no division per solve)
    if (info == 0)
        for (int k = 0; k < r; ++k) a[k * r + k] = one<T>() / a[k * r + k];
    return info;
}

// z := S^{-1} z with the small LU (getrs 'N'), lane 0.
template <class T>
__device__ void small_getrs(const T* a, const int* piv, T* z, int r) {
    for (int k = 0; k < r; ++k) {
        const int p = piv[k];
        if (p != k) {
            T t = z[k];
            z[k] = z[p];
            z[p] = t;
        }
    }
    for (int k = 0; k < r; ++k)
        for (int i = k + 1; i < r; ++i) z[i] = z[i] - a[k * r + i] * z[k];
    for (int k = r - 1; k >= 0; --k) {
        z[k] = z[k] * a[k * r + k];
        for (int i = 0; i < k; ++i) z[i] = z[i] - a[k * r + i] * z[k];
    }
}

// z := S^{-1} z with the small LU staged in shared memory (lane 0; r <= kMaxRUnroll): the
// pivots are read at once, the factor from shared memory
constexpr int kMaxRUnroll = 8;
template <class T>
__device__ void small_getrs_staged(const T* a, const int* piv, T* z, int r) {
    int pv[kMaxRUnroll];
#pragma unroll
    for (int k = 0; k < kMaxRUnroll; ++k) pv[k] = k < r ? piv[k] : k;
#pragma unroll
    for (int k = 0; k < kMaxRUnroll; ++k) {
        if (k < r && pv[k] != k) {
            T t = z[k];
            z[k] = z[pv[k]];
            z[pv[k]] = t;
        }
    }
    for (int k = 0; k < r; ++k)
        for (int i = k + 1; i < r; ++i) z[i] = z[i] - a[k * r + i] * z[k];
    for (int k = r - 1; k >= 0; --k) {
        z[k] = z[k] * a[k * r + k];
        for (int i = 0; i < k; ++i) z[i] = z[i] - a[k * r + i] * z[k];
    }
}

// 1-norm of an r x r column-major matrix (NaN propagates as in the reference's norm1).
template <class T>
__device__ double small_norm1(const T* a, int r) {
    double m = 0.0;
    for (int c = 0; c < r; ++c) {
        double s = 0.0;
        for (int i = 0; i < r; ++i) s += absval(a[c * r + i]);
        if (!(s <= m)) m = s;
    }
    return m;
}

// ------------------------------------------------------------------------------------------------
// kernels

// Factor: band LU, W = B^{-1} U, S = I + V^T W, LU of S and its 1-norm condition. Scratch for the
// r x r work lives in the slu/w buffers of the system itself.
template <class T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_factor(BandView<T> v) {
    const int sys = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (sys >= v.batch) return;
    const int lane = threadIdx.x & 31;
    const int n = v.n, r = v.r, ldab = v.ldab;
    T* ab = v.ab + (size_t)sys * n * ldab;
    int* ipiv = v.ipiv + (size_t)sys * n;
    int info = warp_gbtf2(ab, ipiv, n, v.kl, v.ku, ldab, v.pivot);
    if (info == 0) {
        // factored form: 1 / u_jj on the band diagonal, so that every sweep multiplies
        const int kv = v.kl + v.ku;
        for (int j = lane; j < n; j += 32) ab[(size_t)j * ldab + kv] = one<T>() / ab[(size_t)j * ldab + kv];
        __syncwarp();
    }
    double cond = 1.0;
    if (info == 0 && r > 0) {
        T* w = v.w + (size_t)sys * r * n;
        const T* vt = v.vt + (size_t)sys * r * n;
        for (int k = 0; k < r; ++k) {
            T* wk = w + (size_t)k * n;
            for (int i = lane; i < n; i += 32) wk[i] = (i == k) ? one<T>() : T(0.0);
            __syncwarp();
            warp_band_solve(ab, ipiv, wk, n, v.kl, v.ku, ldab);
            __syncwarp();
        }
        T* S = v.slu + (size_t)sys * r * r;
        for (int a = 0; a < r; ++a)
            for (int b = 0; b < r; ++b) {
                const T* va = vt + (size_t)a * n;
                const T* wb = w + (size_t)b * n;
                T acc = T(0.0);
                for (int i = lane; i < n; i += 32) acc = acc + va[i] * wb[i];
                acc = warp_sum(acc);
                if (lane == 0) S[b * r + a] = ((a == b) ? one<T>() : T(0.0)) + acc;
            }
        __syncwarp();
        if (lane == 0) {
            const double nS = small_norm1(S, r);
            int* sp = v.spiv + (size_t)sys * r;
            int sinfo = small_getrf(S, sp, r);
            if (sinfo != 0) {
                info = -1;
            } else {
                // ||S^{-1}||_1 column by column (r solves with unit vectors); r <= 64
                double ninv = 0.0;
                T z[64];
                for (int c = 0; c < r; ++c) {
                    for (int i = 0; i < r; ++i) z[i] = (i == c) ? one<T>() : T(0.0);
                    small_getrs(S, sp, z, r);
                    double s = 0.0;
                    for (int i = 0; i < r; ++i) s += absval(z[i]);
                    if (!(s <= ninv)) ninv = s;
                }
                cond = nS * ninv;
                if (isnan(cond)) info = -2;
            }
        }
        info = __shfl_sync(0xffffffffu, info, 0);
    }
    if (lane == 0) {
        v.info[sys] = info;
        v.cond[sys] = cond;
    }
}

// Transposed Woodbury data: Wt = B^{-T} V (rows of V^T solved), St = I + U^T Wt, LU of St.
template <class T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_prepare_T(BandView<T> v) {
    const int sys = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (sys >= v.batch) return;
    const int lane = threadIdx.x & 31;
    const int n = v.n, r = v.r;
    const T* ab = v.ab + (size_t)sys * n * v.ldab;
    const int* ipiv = v.ipiv + (size_t)sys * n;
    T* wt = v.wt + (size_t)sys * r * n;
    const T* vt = v.vt + (size_t)sys * r * n;
    for (int k = 0; k < r; ++k) {
        T* wk = wt + (size_t)k * n;
        for (int i = lane; i < n; i += 32) wk[i] = vt[(size_t)k * n + i];
        __syncwarp();
        warp_band_solve_T(ab, ipiv, wk, n, v.kl, v.ku, v.ldab);
        __syncwarp();
    }
    if (lane == 0) {
        T* St = v.stlu + (size_t)sys * r * r;
        for (int a = 0; a < r; ++a)
            for (int b = 0; b < r; ++b)
                St[b * r + a] = ((a == b) ? one<T>() : T(0.0)) + wt[(size_t)b * n + a];
        small_getrf(St, v.stpiv + (size_t)sys * r, r);
    }
}

// Woodbury correction y -= W S^{-1} V^T y (one warp; zbuf: r entries of shared memory).
template <class T>
__device__ void warp_woodbury(const T* vt, const T* w, const T* slu, const int* spiv, T* y, T* zbuf,
                              int n, int r) {
    const int lane = threadIdx.x & 31;
    for (int a = 0; a < r; ++a) {
        const T* va = vt + (size_t)a * n;
        T acc = T(0.0);
        for (int i = lane; i < n; i += 32) acc = acc + va[i] * y[i];
        acc = warp_sum(acc);
        if (lane == 0) zbuf[a] = acc;
    }
    __syncwarp();
    if (lane == 0) small_getrs(slu, spiv, zbuf, r);
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
        T acc = y[i];
        for (int k = 0; k < r; ++k) acc = acc - w[(size_t)k * n + i] * zbuf[k];
        y[i] = acc;
    }
    __syncwarp();
}

// ---- staged solve ---------------------------------------------------------------------------
// The sweeps of warp_band_solve wait on two dependent global loads per column (the pivot index and
// the column entries). The staged solve streams the band into shared memory CH columns ahead with
// cp.async (two buffers, hardware wait_group, no spin), and keeps the pivots of the current and the
// next chunk in registers (lane t holds ipiv[chunk + t], broadcast by shuffle).
template <class T>
__device__ __forceinline__ void cp_async_el(T* s, const T* g) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(s));
    if constexpr (sizeof(T) == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(g) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int kChunk = 16;

// forward chunk c: columns j = c CH .. min(c CH + CH, n - 1) - 1, L entries rows kv+1 .. kv+lm
template <class T>
__device__ __forceinline__ void issue_fwd(const T* ab, T* buf, int c, int n, int kl, int kv, int ldab) {
    const int lane = threadIdx.x & 31;
    const int j0 = c * kChunk, j1 = min(j0 + kChunk, n - 1);
    const int cnt = (j1 - j0) * kl;
    for (int e = lane; e < cnt; e += 32) {
        const int jj = e / kl, t = e - jj * kl;
        const int j = j0 + jj;
        if (t < n - 1 - j) cp_async_el(buf + jj * kl + t, ab + (size_t)j * ldab + kv + 1 + t);
    }
    cp_async_commit();
}

// backward chunk c: columns j = n-1 - (c CH + jj), rows max(0, kv - j) .. kv
template <class T>
__device__ __forceinline__ void issue_bwd(const T* ab, T* buf, int c, int n, int kv, int ldab) {
    const int lane = threadIdx.x & 31;
    const int w = kv + 1;
    const int jj1 = min(kChunk, n - c * kChunk);
    const int cnt = jj1 * w;
    for (int e = lane; e < cnt; e += 32) {
        const int jj = e / w, q = e - jj * w;
        const int j = n - 1 - (c * kChunk + jj);
        if (q >= kv - j) cp_async_el(buf + jj * w + q, ab + (size_t)j * ldab + q);
    }
    cp_async_commit();
}

template <class T>
__device__ void warp_band_solve_staged(const T* __restrict__ ab, const int* __restrict__ ipiv, T* y, T* stage,
                                       int n, int kl, int ku, int ldab) {
    const int lane = threadIdx.x & 31;
    const int kv = kl + ku;
    const int sw = max(kl, kv + 1) * kChunk;          // elements per stage buffer
    if (kl > 0 && n > 1) {
        const int nch = (n - 1 + kChunk - 1) / kChunk;
        issue_fwd(ab, stage, 0, n, kl, kv, ldab);
        int ip_cur = lane < kChunk && lane < n - 1 ? ipiv[lane] : 0;
        for (int c = 0; c < nch; ++c) {
            const int nxt = (c + 1) * kChunk + lane;
            int ip_nxt = 0;
            if (c + 1 < nch) {
                issue_fwd(ab, stage + ((c + 1) & 1) * sw, c + 1, n, kl, kv, ldab);
                ip_nxt = lane < kChunk && nxt < n - 1 ? ipiv[nxt] : 0;
                cp_async_wait1();
            } else {
                cp_async_wait0();
            }
            __syncwarp();
            const T* buf = stage + (c & 1) * sw;
            const int j0 = c * kChunk, j1 = min(j0 + kChunk, n - 1);
            for (int j = j0; j < j1; ++j) {
                const int jj = j - j0;
                const int lm = min(kl, n - 1 - j);
                const int l = __shfl_sync(0xffffffffu, ip_cur, jj);
                const T bj = y[l];
                const T yj0 = y[j];
                __syncwarp();
                for (int t = lane; t < lm; t += 32) {
                    const int i = j + 1 + t;
                    const T v = (i == l) ? yj0 : y[i];
                    y[i] = v - buf[jj * kl + t] * bj;
                }
                if (lane == 0) y[j] = bj;
                __syncwarp();
            }
            ip_cur = ip_nxt;
        }
    }
    {
        const int w = kv + 1;
        const int nch = (n + kChunk - 1) / kChunk;
        issue_bwd(ab, stage, 0, n, kv, ldab);
        for (int c = 0; c < nch; ++c) {
            if (c + 1 < nch) {
                issue_bwd(ab, stage + ((c + 1) & 1) * sw, c + 1, n, kv, ldab);
                cp_async_wait1();
            } else {
                cp_async_wait0();
            }
            __syncwarp();
            const T* buf = stage + (c & 1) * sw;
            const int jj1 = min(kChunk, n - c * kChunk);
            for (int jj = 0; jj < jj1; ++jj) {
                const int j = n - 1 - (c * kChunk + jj);
                T yj = y[j];
                if (is_zero(yj)) {
                    __syncwarp();
                    continue;
                }
                const T* col = buf + jj * w;
                yj = yj * col[kv];                   // the diagonal holds 1 / u_jj
                const int m = min(kv, j);
                for (int t = lane; t < m; t += 32) {
                    const int i = j - 1 - t;
                    y[i] = y[i] - yj * col[kv - 1 - t];
                }
                if (lane == 0) y[j] = yj;
                __syncwarp();
            }
        }
    }
}

// Input/output adapters of the solve kernel: plain in-place, mapped (int64 gather/scatter maps)
// and split (complex system with real data: b = re[rows_c] + i re[rows_s]).
enum IoKind { IO_PLAIN = 0, IO_MAPPED = 1, IO_SPLIT = 2, IO_MIXED = 3 };

struct SolveIo {
    const void* rhs;
    void* x;
    const long long* rows;
    const long long* cols;
    const long long* rows_s;
    const long long* cols_s;
    int accumulate = 0;
    void* xT = nullptr;            // IO_MIXED: x also written row-major over the systems, [n][batch]
};

template <class T, int IO>
__device__ inline T io_load(const SolveIo& io, int sys, int n, int i) {
    const size_t k = (size_t)sys * n + i;
    if constexpr (IO == IO_PLAIN) {
        return static_cast<const T*>(io.rhs)[k];
    } else if constexpr (IO == IO_MAPPED) {
        const T* rhs = static_cast<const T*>(io.rhs);
        return rhs[io.rows ? io.rows[k] : (long long)k];
    } else {
        const double* re = static_cast<const double*>(io.rhs);
        return T(zd(re[io.rows[k]], re[io.rows_s[k]]));
    }
}

template <class T, int IO>
__device__ inline void io_store(const SolveIo& io, int sys, int n, int i, T v) {
    const size_t k = (size_t)sys * n + i;
    if constexpr (IO == IO_PLAIN) {
        static_cast<T*>(io.x)[k] = v;
    } else if constexpr (IO == IO_MAPPED) {
        static_cast<T*>(io.x)[io.cols ? io.cols[k] : (long long)k] = v;
    } else {
        double* x = static_cast<double*>(io.x);
        const zd z = *reinterpret_cast<const zd*>(&v);
        x[io.cols[k]] = z.re;
        x[io.cols_s[k]] = z.im;
    }
}

template <class T, int IO>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_solve(BandView<T> v, SolveIo io) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wib = threadIdx.x >> 5;
    const int sys = blockIdx.x * kWarpsPerBlock + wib;
    if (sys >= v.batch) return;
    const int lane = threadIdx.x & 31;
    const int n = v.n, r = v.r;
    const int per = n + 64 + 2 * max(v.kl, v.kl + v.ku + 1) * kChunk;
    T* y = reinterpret_cast<T*>(smem_raw) + (size_t)wib * per;
    T* zbuf = y + n;
    T* stage = zbuf + 64;
    for (int i = lane; i < n; i += 32) y[i] = io_load<T, IO>(io, sys, n, v.perm[i]);
    __syncwarp();
    warp_band_solve_staged(v.ab + (size_t)sys * n * v.ldab, v.ipiv + (size_t)sys * n, y, stage, n, v.kl, v.ku,
                           v.ldab);
    if (r > 0)
        warp_woodbury(v.vt + (size_t)sys * r * n, v.w + (size_t)sys * r * n, v.slu + (size_t)sys * r * r,
                      v.spiv + (size_t)sys * r, y, zbuf, n, r);
    for (int i = lane; i < n; i += 32) io_store<T, IO>(io, sys, n, i, y[i]);
}

template <class T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_solve_T(BandView<T> v, T* b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wib = threadIdx.x >> 5;
    const int sys = blockIdx.x * kWarpsPerBlock + wib;
    if (sys >= v.batch) return;
    const int lane = threadIdx.x & 31;
    const int n = v.n, r = v.r;
    T* y = reinterpret_cast<T*>(smem_raw) + (size_t)wib * (n + 64);
    T* zbuf = y + n;
    T* bs = b + (size_t)sys * n;
    for (int i = lane; i < n; i += 32) y[i] = bs[i];
    __syncwarp();
    warp_band_solve_T(v.ab + (size_t)sys * n * v.ldab, v.ipiv + (size_t)sys * n, y, n, v.kl, v.ku, v.ldab);
    if (r > 0) {
        const T* wt = v.wt + (size_t)sys * r * n;
        if (lane == 0) {
            for (int k = 0; k < r; ++k) zbuf[k] = y[k];
            small_getrs(v.stlu + (size_t)sys * r * r, v.stpiv + (size_t)sys * r, zbuf, r);
        }
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            T acc = y[i];
            for (int k = 0; k < r; ++k) acc = acc - wt[(size_t)k * n + i] * zbuf[k];
            y[i] = acc;
        }
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) bs[v.perm[i]] = y[i];
}


// Mixed precision: FP32 factors (demoted from the FP64 factorization), complex128 right-hand side
// and result. accumulate = 0: x = A32^{-1} b; 1: x += A32^{-1} b (the refinement update in FP64).
struct MixedView {
    int batch, n, r, kl, ku, ldab;
    const zf* ab;
    const int* ipiv;
    const zf* vt;
    const zf* w;
    const zf* slu;
    const int* spiv;
    const int* perm;
};

__global__ void __launch_bounds__(32 * kWarpsPerBlock)
k_solve_mixed(MixedView v, const zd* __restrict__ b, zd* __restrict__ x, int accumulate) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wib = threadIdx.x >> 5;
    const int sys = blockIdx.x * kWarpsPerBlock + wib;
    if (sys >= v.batch) return;
    const int lane = threadIdx.x & 31;
    const int n = v.n, r = v.r;
    const int per = n + 64 + 2 * max(v.kl, v.kl + v.ku + 1) * kChunk;
    zf* y = reinterpret_cast<zf*>(smem_raw) + (size_t)wib * per;
    zf* zbuf = y + n;
    zf* stage = zbuf + 64;
    const zd* bs = b + (size_t)sys * n;
    for (int i = lane; i < n; i += 32) y[i] = to_zf(bs[v.perm[i]]);
    __syncwarp();
    warp_band_solve_staged<zf>(v.ab + (size_t)sys * n * v.ldab, v.ipiv + (size_t)sys * n, y, stage, n,
                               v.kl, v.ku, v.ldab);
    if (r > 0)
        warp_woodbury<zf>(v.vt + (size_t)sys * r * n, v.w + (size_t)sys * r * n, v.slu + (size_t)sys * r * r,
                          v.spiv + (size_t)sys * r, y, zbuf, n, r);
    zd* xs = x + (size_t)sys * n;
    for (int i = lane; i < n; i += 32) {
        const zd d(y[i].re, y[i].im);
        xs[i] = accumulate ? xs[i] + d : d;
    }
}

__global__ void k_demote(const zd* __restrict__ a, zf* __restrict__ b, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = to_zf(a[i]);
}

// Device layout of a batch sharing one CSR pattern: values [batch][nnz] -> band of B and V^T.
// bulk_dest[p] >= 0: band offset (j*ldab + kv + i - j) of bulk entry p, -1 for a border entry.
// Border position i owns the entries bptr[i]..bptr[i+1]-1 of (bp: CSR position, bcol: column), in
// CSR order: V^T row i accumulates them, s_i = max |entry| (1 if the row is zero) goes on the
// diagonal of B and is subtracted from V^T(i, i) (banded.hpp:197-214).
template <class T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
k_layout_shared(BandView<T> v, const T* values, int nnz, const long long* bulk_dest, const int* bptr,
                const int* bp, const int* bcol) {
    const int sys = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (sys >= v.batch) return;
    const int lane = threadIdx.x & 31;
    const int n = v.n, r = v.r, kv = v.kl + v.ku;
    T* ab = v.ab + (size_t)sys * n * v.ldab;
    T* vt = v.vt + (size_t)sys * r * n;
    const T* val = values + (size_t)sys * nnz;
    for (size_t i = lane; i < (size_t)n * v.ldab; i += 32) ab[i] = T(0.0);
    for (size_t i = lane; i < (size_t)r * n; i += 32) vt[i] = T(0.0);
    __syncwarp();
    for (int p = lane; p < nnz; p += 32) {
        const long long d = bulk_dest[p];
        if (d >= 0) ab[d] = ab[d] + val[p];
    }
    for (int i = lane; i < r; i += 32) {
        double s = 0.0;
        T* row = vt + (size_t)i * n;
        for (int q = bptr[i]; q < bptr[i + 1]; ++q) {
            const T a = val[bp[q]];
            s = fmax(s, absval(a));
            row[bcol[q]] = row[bcol[q]] + a;
        }
        if (s == 0.0) s = 1.0;
        ab[(size_t)i * v.ldab + kv] = T(s);
        row[i] = row[i] - T(s);
    }
}

// ================================================================================================
// host side

struct Banded {
    int dtype = 0;                // 0 = float64, 1 = complex128
    int batch = 0, n = 0, r = 0, kl = 0, ku = 0, ldab = 1, pivot = 1;
    size_t esz = 8;
    void* ab = nullptr;
    int* ipiv = nullptr;
    void* vt = nullptr;
    void* w = nullptr;
    void* slu = nullptr;
    int* spiv = nullptr;
    int* perm = nullptr;
    int* info = nullptr;
    double* cond = nullptr;
    void* wt = nullptr;
    void* stlu = nullptr;
    int* stpiv = nullptr;
    bool transposed_ready = false;
    double factor_ms = 0.0;
    double cond_max = 1.0;
    std::vector<int> perm_host;
    // compact bucket-union form (built by compact())
    bool compact_ready = false;
    int cL = 0, cU = 0, cV = 0, cWg = 0;
    int cMaxLk[4] = {0, 0, 0, 0}, cMaxUk[4] = {0, 0, 0, 0};   // largest stream chunk per chunk size 2, 4, 8, 16
    int cMaxLcol = 0, cMaxUcol = 0;                            // most entries of one column (L, U)
    // partitioned solve (kPartSchedule): per system and block of 32 columns, the responses of the
    // block's forward and backward sweeps to unit boundary values (built by build_part)
    bool part_ready = false;
    int p_nbf = 0, p_nbb = 0, p_kwf = 0, p_kwb = 0, p_maxLc = 0, p_maxUc = 0;
    void* p_Rf = nullptr;           // [batch][nbf][32 + kwf][kwf] complex128
    void* p_Rb = nullptr;           // [batch][nbb][32 + kwb][kwb] complex128
    // windowed schedules: the scratch the sweeps spill finished rows to ([cWg][kGroup][n], room
    // for complex128; allocated by cng_banded_set_schedule)
    void* w_scr = nullptr;
    size_t w_cap = 0;               // entries
    int sched = 0;                 // compact solve schedule (index into kSchedules); -1: band kernel
    int cG = 2;                     // systems per warp group of the compact streams (1: shared pair)
    bool shared = false;            // factors shared with a sign-similar partner bucket
    unsigned char* flip_r = nullptr;    // partner = diag(dr) A diag(dc): 1 where dr_i = -1
    unsigned char* flip_c = nullptr;    //                                1 where dc_j = -1
    int* c_offL = nullptr;
    unsigned char* c_Lrow = nullptr;
    unsigned* c_Lmask = nullptr;
    int* c_offU = nullptr;
    unsigned char* c_Udist = nullptr;
    int* c_offV = nullptr;
    int* c_Vcol = nullptr;
    void* c_L = nullptr;
    void* c_U = nullptr;
    void* c_V = nullptr;
    int* c_piv = nullptr;
    zf* c_L32 = nullptr;
    zf* c_U32 = nullptr;
    zf* c_V32 = nullptr;
    // FP32 copies of the factors (mixed-precision solves)
    zf* ab32 = nullptr;
    zf* vt32 = nullptr;
    zf* w32 = nullptr;
    zf* slu32 = nullptr;
    bool fp32_ready = false;
    // shared-pattern refactorization data (create_shared)
    int nnz = 0;
    long long* bulk_dest = nullptr;
    int* bptr = nullptr;
    int* bp = nullptr;
    int* bcol = nullptr;

    ~Banded() {
        for (void* p : {ab, (void*)ipiv, vt, w, slu, (void*)spiv, (void*)perm, (void*)info,
                        (void*)cond, wt, stlu, (void*)stpiv, (void*)bulk_dest, (void*)bptr,
                        (void*)bp, (void*)bcol, (void*)ab32, (void*)vt32, (void*)w32, (void*)slu32,
                        (void*)c_offL, (void*)c_Lrow, (void*)c_Lmask, (void*)c_offU, (void*)c_Udist,
                        (void*)c_offV, (void*)c_Vcol, c_L, c_U, c_V, (void*)c_piv, (void*)c_L32,
                        (void*)c_U32, (void*)c_V32, (void*)flip_r, (void*)flip_c, p_Rf, p_Rb, w_scr})
            dev_free(p);
    }

    template <class T>
    BandView<T> view() const {
        BandView<T> v;
        v.batch = batch; v.n = n; v.r = r; v.kl = kl; v.ku = ku; v.ldab = ldab; v.pivot = pivot;
        v.ab = static_cast<T*>(ab); v.ipiv = ipiv; v.vt = static_cast<T*>(vt);
        v.w = static_cast<T*>(w); v.slu = static_cast<T*>(slu); v.spiv = spiv; v.perm = perm;
        v.info = info; v.cond = cond; v.wt = static_cast<T*>(wt); v.stlu = static_cast<T*>(stlu);
        v.stpiv = stpiv;
        return v;
    }

    size_t solve_smem(size_t elem = 0) const {
        const size_t e = elem ? elem : esz;
        return (size_t)kWarpsPerBlock * (size_t)(n + 64 + 2 * std::max(kl, kl + ku + 1) * kChunk) * e;
    }
};

template <class P>
static void dalloc(P** p, size_t count, size_t esz) {
    *p = static_cast<P*>(dev_alloc(std::max<size_t>(count * esz, 16)));
}

static void alloc_handle(Banded& h) {
    const size_t B = h.batch, n = h.n, r = h.r;
    dalloc(&h.ab, B * n * h.ldab, h.esz);
    dalloc(&h.ipiv, B * n, sizeof(int));
    dalloc(&h.vt, B * r * n, h.esz);
    dalloc(&h.w, B * r * n, h.esz);
    dalloc(&h.slu, B * r * r, h.esz);
    dalloc(&h.spiv, B * r, sizeof(int));
    dalloc(&h.perm, n, sizeof(int));
    dalloc(&h.info, B, sizeof(int));
    dalloc(&h.cond, B, sizeof(double));
}

static std::vector<int> border_perm(int n, const int* border, int r) {
    if (r < 0 || r > n) throw InvalidArgument("border row count out of range");
    if (r > 64) throw InvalidArgument("at most 64 border rows are supported (capacitance size)");
    std::vector<char> is_border(n, 0);
    std::vector<int> perm;
    perm.reserve(n);
    for (int k = 0; k < r; ++k) {
        int i = border[k];
        if (i < 0 || i >= n) throw InvalidArgument("border row out of range");
        if (is_border[i]) throw InvalidArgument("duplicate border row");
        is_border[i] = 1;
        perm.push_back(i);
    }
    for (int i = 0; i < n; ++i)
        if (!is_border[i]) perm.push_back(i);
    return perm;
}

static void check_csr(int n, const int* ip, const int* ix, long long nnz) {
    if (ip[0] != 0 || ip[n] != nnz)
        throw InvalidArgument("inconsistent CSR arrays (indptr[0] = 0, indptr[n] = nnz = "
                              "len(indices) = len(data) required)");
    for (int i = 0; i < n; ++i)
        if (ip[i + 1] < ip[i])
            throw InvalidArgument("CSR: indptr decreases at row " + std::to_string(i));
    for (long long p = 0; p < nnz; ++p)
        if (ix[p] < 0 || ix[p] >= n)
            throw InvalidArgument("CSR: column index " + std::to_string(ix[p]) + " outside [0, " +
                                  std::to_string(n) + ")");
}

template <class T>
static void check_finite(int n, const int* ip, const int* ix, const T* d) {
    for (int i = 0; i < n; ++i)
        for (int p = ip[i]; p < ip[i + 1]; ++p)
            if (!finite_val(d[p]))
                throw InvalidArgument("BorderedBanded: non-finite matrix entry at (" + std::to_string(i) +
                                      ", " + std::to_string(ix[p]) + "): the operator must be finite");
}

static void finish_factor(Banded& h, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1) {
    CNG_CUDA(cudaEventRecord(e1, st));
    CNG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    h.factor_ms = ms;
    std::vector<int> info(h.batch);
    std::vector<double> cond(h.batch);
    CNG_CUDA(cudaMemcpy(info.data(), h.info, sizeof(int) * h.batch, cudaMemcpyDeviceToHost));
    CNG_CUDA(cudaMemcpy(cond.data(), h.cond, sizeof(double) * h.batch, cudaMemcpyDeviceToHost));
    h.cond_max = 1.0;
    for (int k = 0; k < h.batch; ++k) {
        if (info[k] > 0)
            throw RuntimeFailure("BandedBatch: banded part of system " + std::to_string(k) +
                                 " is singular at pivot " + std::to_string(info[k]) +
                                 "; the non-border rows must form an invertible banded operator "
                                 "(check the row/column ordering of the plan)");
        if (info[k] == -1)
            throw RuntimeFailure("BandedBatch: capacitance matrix of system " + std::to_string(k) +
                                 " is singular: the boundary rows are not independent of the banded "
                                 "operator (ill-posed or rank-deficient BCs)");
        if (info[k] == -2)
            throw RuntimeFailure("BandedBatch: capacitance condition number is NaN");
        if (!(cond[k] <= h.cond_max)) h.cond_max = cond[k];
    }
}

static void launch_factor(Banded& h, cudaStream_t st) {
    const int blocks = ceil_div(h.batch, kWarpsPerBlock);
    if (h.dtype == 0) k_factor<double><<<blocks, 32 * kWarpsPerBlock, 0, st>>>(h.view<double>());
    else k_factor<zd><<<blocks, 32 * kWarpsPerBlock, 0, st>>>(h.view<zd>());
    CNG_LAUNCH("k_factor");
}

// General path: one CSR matrix per system (host arrays), layout on the host (border rows first,
// common band of the batch), then the factorization on the device.
template <class T>
static void build_csr(Banded& h, const int* indptr, const int* indices, const T* data,
                      const long long* off, const int* border, cudaStream_t st) {
    const int n = h.n, B = h.batch;
    h.perm_host = border_perm(n, border, h.r);
    std::vector<int> pos(n);
    for (int i = 0; i < n; ++i) pos[h.perm_host[i]] = i;
    // band of the bulk rows over the batch (explicit zeros do not count, banded.hpp:116-133)
    int kl = 0, ku = 0;
    for (int k = 0; k < B; ++k) {
        const int* ip = indptr + (size_t)k * (n + 1);
        const int* ix = indices + off[k];
        const T* d = data + off[k];
        check_csr(n, ip, ix, ip[n]);
        if (k + 1 < B && off[k] + ip[n] > off[k + 1])
            throw InvalidArgument("CSR: matrix " + std::to_string(k) + " has " + std::to_string(ip[n]) +
                                  " entries and overlaps the next matrix's");
        check_finite(n, ip, ix, d);
        for (int o = 0; o < n; ++o) {
            const int i = pos[o];
            if (i < h.r) continue;
            for (int p = ip[o]; p < ip[o + 1]; ++p) {
                if (is_zero(d[p])) continue;
                kl = std::max(kl, i - ix[p]);
                ku = std::max(ku, ix[p] - i);
            }
        }
    }
    h.kl = kl;
    h.ku = ku;
    const long long ldab = 2LL * kl + ku + 1;
    if (ldab > 1 << 20) throw InvalidArgument("banded layout: band too wide");
    h.ldab = static_cast<int>(ldab);
    alloc_handle(h);
    const int kv = kl + ku;
    std::vector<T> ab((size_t)n * h.ldab), vt((size_t)h.r * n);
    // staged in chunks of systems to bound host memory
    const int chunk = std::max(1, (int)std::min<long long>(B, (64LL << 20) / std::max<long long>(1, (long long)n * h.ldab * sizeof(T))));
    std::vector<T> stage_ab((size_t)chunk * n * h.ldab), stage_vt((size_t)chunk * h.r * n);
    for (int k0 = 0; k0 < B; k0 += chunk) {
        const int k1 = std::min(B, k0 + chunk);
        for (int k = k0; k < k1; ++k) {
            T* abk = stage_ab.data() + (size_t)(k - k0) * n * h.ldab;
            T* vtk = stage_vt.data() + (size_t)(k - k0) * h.r * n;
            std::fill(abk, abk + (size_t)n * h.ldab, T(0.0));
            std::fill(vtk, vtk + (size_t)h.r * n, T(0.0));
            const int* ip = indptr + (size_t)k * (n + 1);
            const int* ix = indices + off[k];
            const T* d = data + off[k];
            for (int i = 0; i < n; ++i) {
                const int o = h.perm_host[i];
                if (i < h.r) {
                    double s = 0.0;
                    for (int p = ip[o]; p < ip[o + 1]; ++p) {
                        s = std::max(s, absval(d[p]));
                        vtk[(size_t)i * n + ix[p]] = vtk[(size_t)i * n + ix[p]] + d[p];
                    }
                    if (s == 0.0) s = 1.0;
                    abk[(size_t)i * h.ldab + kv] = T(s);
                    vtk[(size_t)i * n + i] = vtk[(size_t)i * n + i] - T(s);
                } else {
                    for (int p = ip[o]; p < ip[o + 1]; ++p) {
                        if (is_zero(d[p])) continue;
                        const int j = ix[p];
                        T& slot = abk[(size_t)j * h.ldab + kv + i - j];
                        slot = slot + d[p];
                    }
                }
            }
        }
        CNG_CUDA(cudaMemcpyAsync(static_cast<T*>(h.ab) + (size_t)k0 * n * h.ldab, stage_ab.data(),
                                 sizeof(T) * (size_t)(k1 - k0) * n * h.ldab, cudaMemcpyHostToDevice, st));
        if (h.r)
            CNG_CUDA(cudaMemcpyAsync(static_cast<T*>(h.vt) + (size_t)k0 * h.r * n, stage_vt.data(),
                                     sizeof(T) * (size_t)(k1 - k0) * h.r * n, cudaMemcpyHostToDevice, st));
        CNG_CUDA(cudaStreamSynchronize(st));   // the staging buffers are reused
    }
    CNG_CUDA(cudaMemcpyAsync(h.perm, h.perm_host.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
}

// Shared-pattern path: structure analysed once on the host, values assembled on the device.
static void build_shared_structure(Banded& h, const int* indptr, const int* indices, int nnz,
                                   const int* border, cudaStream_t st) {
    const int n = h.n;
    check_csr(n, indptr, indices, nnz);
    h.perm_host = border_perm(n, border, h.r);
    std::vector<int> pos(n);
    for (int i = 0; i < n; ++i) pos[h.perm_host[i]] = i;
    int kl = 0, ku = 0;
    for (int o = 0; o < n; ++o) {
        const int i = pos[o];
        if (i < h.r) continue;
        for (int p = indptr[o]; p < indptr[o + 1]; ++p) {
            kl = std::max(kl, i - indices[p]);
            ku = std::max(ku, indices[p] - i);
        }
    }
    h.kl = kl;
    h.ku = ku;
    h.ldab = 2 * kl + ku + 1;
    h.nnz = nnz;
    const int kv = kl + ku;
    std::vector<long long> dest(std::max(nnz, 1), -1);
    std::vector<int> bptr(h.r + 1, 0), bp, bcol;
    for (int i = 0; i < n; ++i) {
        const int o = h.perm_host[i];
        for (int p = indptr[o]; p < indptr[o + 1]; ++p) {
            const int j = indices[p];
            if (i < h.r) {
                bp.push_back(p);
                bcol.push_back(j);
            } else {
                dest[p] = (long long)j * h.ldab + kv + i - j;
            }
        }
        if (i < h.r) bptr[i + 1] = static_cast<int>(bp.size());
    }
    // duplicate (row, column) entries would land twice in one band slot: refused
    {
        std::vector<long long> d2;
        for (long long d : dest) if (d >= 0) d2.push_back(d);
        std::sort(d2.begin(), d2.end());
        if (std::adjacent_find(d2.begin(), d2.end()) != d2.end())
            throw InvalidArgument("shared CSR pattern has duplicate entries (sum them first)");
    }
    alloc_handle(h);     // after every host check: invalid input is refused before device work
    dalloc(&h.bulk_dest, dest.size(), sizeof(long long));
    dalloc(&h.bptr, bptr.size(), sizeof(int));
    dalloc(&h.bp, std::max<size_t>(bp.size(), 1), sizeof(int));
    dalloc(&h.bcol, std::max<size_t>(bcol.size(), 1), sizeof(int));
    CNG_CUDA(cudaMemcpyAsync(h.bulk_dest, dest.data(), sizeof(long long) * dest.size(), cudaMemcpyHostToDevice, st));
    CNG_CUDA(cudaMemcpyAsync(h.bptr, bptr.data(), sizeof(int) * bptr.size(), cudaMemcpyHostToDevice, st));
    if (!bp.empty()) {
        CNG_CUDA(cudaMemcpyAsync(h.bp, bp.data(), sizeof(int) * bp.size(), cudaMemcpyHostToDevice, st));
        CNG_CUDA(cudaMemcpyAsync(h.bcol, bcol.data(), sizeof(int) * bcol.size(), cudaMemcpyHostToDevice, st));
    }
    CNG_CUDA(cudaMemcpyAsync(h.perm, h.perm_host.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    CNG_CUDA(cudaStreamSynchronize(st));     // host vectors go out of scope
}

static void launch_layout_shared(Banded& h, const void* values, cudaStream_t st) {
    const int blocks = ceil_div(h.batch, kWarpsPerBlock);
    if (h.dtype == 0)
        k_layout_shared<double><<<blocks, 32 * kWarpsPerBlock, 0, st>>>(
            h.view<double>(), static_cast<const double*>(values), h.nnz, h.bulk_dest, h.bptr, h.bp, h.bcol);
    else
        k_layout_shared<zd><<<blocks, 32 * kWarpsPerBlock, 0, st>>>(
            h.view<zd>(), static_cast<const zd*>(values), h.nnz, h.bulk_dest, h.bptr, h.bp, h.bcol);
    CNG_LAUNCH("k_layout_shared");
}

static void check_smem(const Banded& h) {
    if (h.solve_smem() > kMaxSolveSmem)
        throw InvalidArgument("BandedBatch: n = " + std::to_string(h.n) + " with band kl = " +
                              std::to_string(h.kl) + ", ku = " + std::to_string(h.ku) +
                              " is too large for the shared-memory solve");
}

template <class T, int IO>
static void launch_solve_t(const Banded& h, const SolveIo& io, cudaStream_t st) {
    ensure_smem_attr((const void*)k_solve<T, IO>, (int)kMaxSolveSmem);
    const int blocks = ceil_div(h.batch, kWarpsPerBlock);
    k_solve<T, IO><<<blocks, 32 * kWarpsPerBlock, h.solve_smem(), st>>>(h.view<T>(), io);
    CNG_LAUNCH("k_solve");
}

static bool launch_solve_compact(const Banded& h, int io_kind, const SolveIo& io, cudaStream_t st);

static void launch_solve(const Banded& h, int io_kind, const SolveIo& io, cudaStream_t st) {
    if (h.compact_ready && h.sched >= 0 && launch_solve_compact(h, io_kind, io, st)) return;
    if (h.dtype == 0) {
        if (io_kind == IO_PLAIN) launch_solve_t<double, IO_PLAIN>(h, io, st);
        else if (io_kind == IO_MAPPED) launch_solve_t<double, IO_MAPPED>(h, io, st);
        else throw InvalidArgument("solve_split needs complex (complex128) factors");
    } else {
        if (io_kind == IO_PLAIN) launch_solve_t<zd, IO_PLAIN>(h, io, st);
        else if (io_kind == IO_MAPPED) launch_solve_t<zd, IO_MAPPED>(h, io, st);
        else launch_solve_t<zd, IO_SPLIT>(h, io, st);
    }
}

static void demote_compact(Banded& h, cudaStream_t st);

// FP32 band-kernel solve (one warp per system) of the mixed form: x (+)= A^{-1} b, complex128 data
static void launch_mixed_dense(const Banded& h, const void* b, void* x, int accumulate, cudaStream_t st) {
    ensure_smem_attr((const void*)k_solve_mixed, (int)kMaxSolveSmem);
    MixedView v{h.batch, h.n, h.r, h.kl, h.ku, h.ldab, h.ab32, h.ipiv, h.vt32, h.w32, h.slu32, h.spiv, h.perm};
    const size_t smem = h.solve_smem(sizeof(zf));
    k_solve_mixed<<<ceil_div(h.batch, kWarpsPerBlock), 32 * kWarpsPerBlock, smem, st>>>(
        v, static_cast<const zd*>(b), static_cast<zd*>(x), accumulate);
    CNG_LAUNCH("k_solve_mixed");
}

static void make_fp32(Banded& h, cudaStream_t st) {
    if (h.dtype != 1) throw InvalidArgument("FP32 factors need complex128 factors (complex bucket)");
    const size_t B = h.batch, n = h.n, r = h.r;
    if (!h.ab32) dalloc(&h.ab32, B * n * h.ldab, sizeof(zf));
    if (!h.vt32) dalloc(&h.vt32, B * r * n, sizeof(zf));
    if (!h.w32) dalloc(&h.w32, B * r * n, sizeof(zf));
    if (!h.slu32) dalloc(&h.slu32, B * r * r, sizeof(zf));
    auto dem = [&](const void* a, zf* b, long long cnt) {
        if (cnt <= 0) return;
        k_demote<<<(int)std::min<long long>((cnt + 255) / 256, 152LL * 32), 256, 0, st>>>(
            static_cast<const zd*>(a), b, cnt);
        CNG_LAUNCH("k_demote");
    };
    dem(h.ab, h.ab32, (long long)(B * n * h.ldab));
    dem(h.vt, h.vt32, (long long)(B * r * n));
    dem(h.w, h.w32, (long long)(B * r * n));
    dem(h.slu, h.slu32, (long long)(B * r * r));
    if (h.compact_ready) demote_compact(h, st);
    CNG_CUDA(cudaStreamSynchronize(st));
    h.fp32_ready = true;
}

static void prepare_transpose(Banded& h, cudaStream_t st) {
    if (h.transposed_ready) return;
    if (h.r > 0) {
        if (!h.wt) dalloc(&h.wt, (size_t)h.batch * h.r * h.n, h.esz);
        if (!h.stlu) dalloc(&h.stlu, (size_t)h.batch * h.r * h.r, h.esz);
        if (!h.stpiv) dalloc(&h.stpiv, (size_t)h.batch * h.r, sizeof(int));
        const int blocks = ceil_div(h.batch, kWarpsPerBlock);
        if (h.dtype == 0) k_prepare_T<double><<<blocks, 32 * kWarpsPerBlock, 0, st>>>(h.view<double>());
        else k_prepare_T<zd><<<blocks, 32 * kWarpsPerBlock, 0, st>>>(h.view<zd>());
        CNG_LAUNCH("k_prepare_T");
        CNG_CUDA(cudaStreamSynchronize(st));
    }
    h.transposed_ready = true;
}

template <class T>
static void launch_solve_T_t(const Banded& h, void* b, cudaStream_t st) {
    ensure_smem_attr((const void*)k_solve_T<T>, (int)kMaxSolveSmem);
    const int blocks = ceil_div(h.batch, kWarpsPerBlock);
    k_solve_T<T><<<blocks, 32 * kWarpsPerBlock, (size_t)kWarpsPerBlock * (h.n + 64) * sizeof(T), st>>>(
        h.view<T>(), static_cast<T*>(b));
    CNG_LAUNCH("k_solve_T");
}

}  // namespace cng

// ================================================================================================
// C-ABI

using namespace cng;

static Banded* as_banded(cng_banded* h) {
    if (!h) throw InvalidArgument("null BandedBatch handle");
    return reinterpret_cast<Banded*>(h);
}
static const Banded* as_banded(const cng_banded* h) {
    if (!h) throw InvalidArgument("null BandedBatch handle");
    return reinterpret_cast<const Banded*>(h);
}

// ------------------------------------------------------------------------------------------------
// Static staging for cng_banded_solve_host_static: a fixed 8 MiB device array (1 Mi complex64 or
// 512 Ki complex128 entries), no allocation at run time. Nothing in it needs to start at zero (a
// solve overwrites the bytes it uses). Every call on a device uses the same array, one at a time.
namespace cng {
constexpr size_t kStaticSolveBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_static_solve[kStaticSolveBytes];

// The array's device address, looked up once per device (the device current at the call).
static void* static_solve_scratch() {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static void* ptr[kMaxDevices] = {};
    int dev = 0;
    CNG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw InvalidArgument("device index above 63");
    std::lock_guard<std::mutex> lock(mu);
    if (!ptr[dev]) {
        void* p = nullptr;
        CNG_CUDA(cudaGetSymbolAddress(&p, g_static_solve));
        ptr[dev] = p;
    }
    return ptr[dev];
}

// Calls on one device take turns on the array: each holds the device's lock from its copy in to
// the end of its copy out, so calls from several host threads do not overwrite each other's data.
static std::mutex& static_solve_turn() {
    constexpr int kMaxDevices = 64;
    static std::mutex mu[kMaxDevices];
    int dev = 0;
    CNG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw InvalidArgument("device index above 63");
    return mu[dev];
}
}  // namespace cng

extern "C" {

int cng_banded_create_csr(int dtype, int batch, int n, const int32_t* indptr, const int32_t* indices,
                          const void* data, const int64_t* nnz_offsets, const int32_t* border, int r,
                          int pivot, void* stream, cng_banded** out) {
    CNG_TRY({
        if (!out) throw InvalidArgument("null output handle");
        *out = nullptr;
        if (dtype != 0 && dtype != 1) throw InvalidArgument("dtype must be 0 (float64) or 1 (complex128)");
        if (batch < 1) throw InvalidArgument("BandedBatch: no matrix given");
        if (n < 1) throw InvalidArgument("BandedBatch: n must be >= 1");
        if (!indptr || !indices || !data || !nnz_offsets || (r > 0 && !border))
            throw InvalidArgument("null CSR array");
        auto h = std::make_unique<Banded>();
        h->dtype = dtype; h->batch = batch; h->n = n; h->r = r; h->pivot = pivot ? 1 : 0;
        h->esz = dtype ? sizeof(zd) : sizeof(double);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        // the host checks of build_csr (pattern, border rows, finite entries) run before any
        // device call, so invalid input is refused the same way with or without a device
        if (dtype == 0)
            build_csr<double>(*h, indptr, indices, static_cast<const double*>(data),
                              reinterpret_cast<const long long*>(nnz_offsets), border, st);
        else
            build_csr<zd>(*h, indptr, indices, static_cast<const zd*>(data),
                          reinterpret_cast<const long long*>(nnz_offsets), border, st);
        check_smem(*h);
        EventPair ev;
        CNG_CUDA(cudaEventRecord(ev.e0, st));
        launch_factor(*h, st);
        finish_factor(*h, st, ev.e0, ev.e1);
        *out = reinterpret_cast<cng_banded*>(h.release());
    })
}

int cng_banded_create_shared(int dtype, int batch, int n, const int32_t* indptr, const int32_t* indices,
                             int nnz, const void* values, const int32_t* border, int r, int pivot,
                             void* stream, cng_banded** out) {
    CNG_TRY({
        if (!out) throw InvalidArgument("null output handle");
        *out = nullptr;
        if (dtype != 0 && dtype != 1) throw InvalidArgument("dtype must be 0 (float64) or 1 (complex128)");
        if (batch < 1) throw InvalidArgument("BandedBatch: no matrix given");
        if (n < 1 || nnz < 0) throw InvalidArgument("BandedBatch: n must be >= 1");
        if (!indptr || (nnz > 0 && !indices) || !values || (r > 0 && !border))
            throw InvalidArgument("null array");
        auto h = std::make_unique<Banded>();
        h->dtype = dtype; h->batch = batch; h->n = n; h->r = r; h->pivot = pivot ? 1 : 0;
        h->esz = dtype ? sizeof(zd) : sizeof(double);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        build_shared_structure(*h, indptr, indices, nnz, border, st);
        check_smem(*h);
        EventPair ev;
        CNG_CUDA(cudaEventRecord(ev.e0, st));
        launch_layout_shared(*h, values, st);
        launch_factor(*h, st);
        finish_factor(*h, st, ev.e0, ev.e1);
        *out = reinterpret_cast<cng_banded*>(h.release());
    })
}

int cng_banded_destroy(cng_banded* h) {
    CNG_TRY({ delete reinterpret_cast<Banded*>(h); })
}

int cng_banded_info(const cng_banded* hh, int32_t* dims, double* stats) {
    CNG_TRY({
        const Banded* h = as_banded(hh);
        if (dims) {
            dims[0] = h->batch; dims[1] = h->n; dims[2] = h->r; dims[3] = h->kl;
            dims[4] = h->ku; dims[5] = h->ldab; dims[6] = h->dtype; dims[7] = h->pivot;
        }
        if (stats) {
            stats[0] = h->factor_ms;
            stats[1] = h->cond_max;
        }
    })
}

int cng_banded_capacitance_cond(const cng_banded* hh, double* cond_host) {
    CNG_TRY({
        const Banded* h = as_banded(hh);
        if (!cond_host) throw InvalidArgument("null output");
        CNG_CUDA(cudaMemcpy(cond_host, h->cond, sizeof(double) * h->batch, cudaMemcpyDeviceToHost));
    })
}

int cng_banded_solve(const cng_banded* hh, void* b, void* stream) {
    CNG_TRY({
        const Banded* h = as_banded(hh);
        if (!b) throw InvalidArgument("BandedBatch.solve: null device pointer");
        SolveIo io{b, b, nullptr, nullptr, nullptr, nullptr};
        launch_solve(*h, IO_PLAIN, io, static_cast<cudaStream_t>(stream));
    })
}

int cng_banded_solve_mapped(const cng_banded* hh, const void* rhs, const int64_t* rows, void* x,
                            const int64_t* cols, void* stream) {
    CNG_TRY({
        const Banded* h = as_banded(hh);
        if (!rhs || !x) throw InvalidArgument("BandedBatch.solve_mapped_ptr: null device pointer");
        // in place with one map for both is a solve in place (every kernel reads a system's whole
        // right-hand side before it writes any of its solution, and the systems' entries are
        // disjoint); with two maps, systems would read entries that others already wrote
        if (rhs == x && rows != cols)
            throw InvalidArgument("BandedBatch.solve_mapped_ptr: rhs and x alias with different maps "
                                  "(pass a separate x, or the same map for rows and cols)");
        SolveIo io{rhs, x, reinterpret_cast<const long long*>(rows), reinterpret_cast<const long long*>(cols),
                   nullptr, nullptr};
        launch_solve(*h, IO_MAPPED, io, static_cast<cudaStream_t>(stream));
    })
}

int cng_banded_solve_split(const cng_banded* hh, const double* re, const int64_t* rows_c,
                           const int64_t* rows_s, double* x, const int64_t* cols_c,
                           const int64_t* cols_s, void* stream) {
    CNG_TRY({
        const Banded* h = as_banded(hh);
        if (!re || !x || !rows_c || !rows_s || !cols_c || !cols_s)
            throw InvalidArgument("BandedBatch.solve_split_ptr: null device pointer");
        if (static_cast<const void*>(re) == static_cast<const void*>(x))
            throw InvalidArgument("BandedBatch.solve_split_ptr: re and x must not alias");
        SolveIo io{re, x, reinterpret_cast<const long long*>(rows_c), reinterpret_cast<const long long*>(cols_c),
                   reinterpret_cast<const long long*>(rows_s), reinterpret_cast<const long long*>(cols_s)};
        launch_solve(*h, IO_SPLIT, io, static_cast<cudaStream_t>(stream));
    })
}

int cng_banded_prepare_transpose(cng_banded* hh, void* stream) {
    CNG_TRY({ prepare_transpose(*as_banded(hh), static_cast<cudaStream_t>(stream)); })
}

int cng_banded_solve_transpose(const cng_banded* hh, void* b, void* stream) {
    CNG_TRY({
        const Banded* h = as_banded(hh);
        if (!b) throw InvalidArgument("BandedBatch.solve_transpose_ptr: null device pointer");
        if (!h->transposed_ready)
            throw InvalidArgument("BandedBatch.solve_transpose_ptr: call prepare_transpose() first "
                                  "(it allocates; never inside a graph capture)");
        if (h->dtype == 0) launch_solve_T_t<double>(*h, b, static_cast<cudaStream_t>(stream));
        else launch_solve_T_t<zd>(*h, b, static_cast<cudaStream_t>(stream));
    })
}

int cng_banded_solve_host(cng_banded* hh, const void* b_host, void* x_host, int transpose) {
    CNG_TRY({
        Banded* h = as_banded(hh);
        if (!b_host || !x_host) throw InvalidArgument("BorderedBandedBatch.solve: null host pointer");
        const size_t bytes = h->esz * (size_t)h->batch * h->n;
        void* d = nullptr;
        cudaStream_t st = nullptr;
        CNG_CUDA(cudaMalloc(&d, bytes));
        try {
            CNG_CUDA(cudaMemcpyAsync(d, b_host, bytes, cudaMemcpyHostToDevice, st));
            if (transpose) {
                prepare_transpose(*h, st);
                if (h->dtype == 0) launch_solve_T_t<double>(*h, d, st);
                else launch_solve_T_t<zd>(*h, d, st);
            } else {
                SolveIo io{d, d, nullptr, nullptr, nullptr, nullptr};
                launch_solve(*h, IO_PLAIN, io, st);
            }
            CNG_CUDA(cudaMemcpyAsync(x_host, d, bytes, cudaMemcpyDeviceToHost, st));
            CNG_CUDA(cudaStreamSynchronize(st));
        } catch (...) {
            cudaFree(d);
            throw;
        }
        CNG_CUDA(cudaFree(d));
    })
}

// Host-buffer solve without any device allocation. The staging buffer is one file-scope device
// array shared by every call on a device, looked up once per device (cudaGetSymbolAddress).
int cng_banded_solve_host_static(cng_banded* hh, const void* b_host, void* x_host, int transpose) {
    CNG_TRY({
        Banded* h = as_banded(hh);
        if (!b_host || !x_host) throw InvalidArgument("solve_host_static: null host pointer");
        const size_t bytes = h->esz * (size_t)h->batch * h->n;
        if (bytes > kStaticSolveBytes)
            throw InvalidArgument("solve_host_static: the right-hand sides take " + std::to_string(bytes) +
                                  " bytes, above the static staging buffer of " +
                                  std::to_string(kStaticSolveBytes) + " bytes (use cng_banded_solve_host)");
        if (transpose && !h->transposed_ready)
            throw InvalidArgument("solve_host_static: call cng_banded_prepare_transpose first (it allocates)");
        std::lock_guard<std::mutex> turn(static_solve_turn());
        void* d = static_solve_scratch();
        cudaStream_t st = nullptr;
        CNG_CUDA(cudaMemcpyAsync(d, b_host, bytes, cudaMemcpyHostToDevice, st));
        if (transpose) {
            if (h->dtype == 0) launch_solve_T_t<double>(*h, d, st);
            else launch_solve_T_t<zd>(*h, d, st);
        } else {
            SolveIo io{d, d, nullptr, nullptr, nullptr, nullptr};
            launch_solve(*h, IO_PLAIN, io, st);
        }
        CNG_CUDA(cudaMemcpyAsync(x_host, d, bytes, cudaMemcpyDeviceToHost, st));
        CNG_CUDA(cudaStreamSynchronize(st));
    })
}

int cng_banded_make_fp32(cng_banded* hh, void* stream) {
    CNG_TRY({ make_fp32(*as_banded(hh), static_cast<cudaStream_t>(stream)); })
}

int cng_banded_solve_fp32(const cng_banded* hh, const void* b, void* x, int accumulate, void* stream) {
    CNG_TRY({
        const Banded* h = as_banded(hh);
        if (!h->fp32_ready) throw InvalidArgument("call cng_banded_make_fp32 first (it allocates)");
        if (!b || !x) throw InvalidArgument("null device pointer");
        if (b == x) throw InvalidArgument("b and x must not alias");
        if (h->compact_ready && h->sched >= 0) {
            SolveIo io{b, x, nullptr, nullptr, nullptr, nullptr, accumulate};
            launch_solve_compact(*h, IO_MIXED, io, static_cast<cudaStream_t>(stream));
            return CNG_OK;
        }
        launch_mixed_dense(*h, b, x, accumulate, static_cast<cudaStream_t>(stream));
    })
}

int cng_banded_refactor_shared(cng_banded* hh, const void* values, void* stream) {
    CNG_TRY({
        Banded* h = as_banded(hh);
        if (!h->bulk_dest) throw InvalidArgument("refactor_shared: handle was not created from a shared pattern");
        if (!values) throw InvalidArgument("null values");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        EventPair ev;
        CNG_CUDA(cudaEventRecord(ev.e0, st));
        launch_layout_shared(*h, values, st);
        launch_factor(*h, st);
        h->transposed_ready = false;
        finish_factor(*h, st, ev.e0, ev.e1);
        if (h->fp32_ready) make_fp32(*h, st);
    })
}

}  // extern "C"

// ================================================================================================
// Compact bucket-union solve.
//
// All systems of a bucket share one sparsity pattern, so the union over the bucket of the nonzero
// slots of their LU factors (pivoting differs per system) is a fixed pattern: about 40% of the L
// band and 20% of the U band for the channel. The compact solve keeps only those slots, packed for
// kGroup systems per warp that sweep in lockstep (the pattern, hence the control flow, is shared):
//   L stream  [wg][e][G]  e = forward entries, columns ascending (offL)
//   U stream  [wg][e][G]  per column j, descending: 1/u_jj, then the U entries (offU in sweep order)
//   pivots    [wg][j][G]
//   V^T       [wg][e][G]  the union nonzeros of the border rows (offV, Vcol)
//   W         [sys][r][n] dense (as before)
// with wg = warp group of kGroup consecutive systems (the last one padded with identity systems).
// The band index lists live in shared memory; the streams are staged chunk by chunk with cp.async.
namespace cng {

constexpr int kGroup = 2;               // systems per warp, 16 lanes each (measured against 1, 4 and 8:
                                        // fastest on the channel and RB, FP64 and FP32)
constexpr int kLanesPer = 32 / kGroup;
constexpr int kCChunk = 8;              // columns per staged chunk (the default schedule)

// Schedules of the compact solve: columns per staged chunk of the factor streams and the depth of
// the cp.async ring (chunks in flight + 1). Deeper rings keep more of the stream in flight per warp
// (the sweep waits on memory otherwise) at the cost of shared memory, hence of resident warps; the
// autotuner (conatus_gb300.autotune) times them on the factors at hand. Schedule 0 is the default.
// Schedules 8-10 run one system per warp with the lanes split over entries and components (the
// latency variant for small batches, k_solve_split_multi).
// Schedule 11 (split = 2) is the partitioned solve of small batches (k_solve_part: one block of
// warps per system, blocks of 32 columns swept at once; FP64 only).
// Schedules 12-15 (split = 3) are the windowed compact solve (k_solve_window_multi: the two-systems
// sweeps with a window of each vector in shared memory and the rest in a global scratch, for more
// resident warps per SM; the same bits as schedule 0); 16-18 the same with 8 lanes per system
// (four systems, two warp groups of the streams per warp: fewer instructions per system).
struct CompactSchedule { int chunk, stages, split, lanes = 16; };
constexpr int kNumSchedules = 19;
constexpr int kPartSchedule = 11;
constexpr int kWindowFlag = 3;
constexpr CompactSchedule kSchedules[kNumSchedules] = {{8, 2, 0}, {8, 3, 0}, {4, 3, 0}, {16, 2, 0},
                                                       {16, 3, 0}, {4, 4, 0}, {2, 4, 0}, {16, 4, 0},
                                                       {8, 2, 1}, {16, 2, 1}, {4, 3, 1}, {8, 2, 2},
                                                       {8, 2, 3}, {4, 3, 3}, {16, 2, 3}, {8, 3, 3},
                                                       {8, 2, 3, 8}, {4, 3, 3, 8}, {8, 3, 3, 8}};
constexpr int kChunkSizes[4] = {2, 4, 8, 16};
__host__ __device__ constexpr int chunk_index(int ch) { return ch == 2 ? 0 : (ch == 4 ? 1 : (ch == 8 ? 2 : 3)); }

struct CompactIdx {
    int n, r, kl, kv, nL, nU, nV, wgroups, batch;
    int gs;                             // systems per warp group in the streams: kGroup, or 1 for a
                                        // shared pair (both halves of the warp read one system's factors)
    int wg0;                            // first warp group solved (wgroups: one past the last)
    int maxLc, maxUc;                   // largest chunk of the L / U streams (entries)
    int maxLcol, maxUcol;               // most entries of one column of the L / U streams
    int wmask;                          // windowed schedules: window slots - 1 (a power of two)
    void* scratch;                      // windowed schedules: [warp group][kGroup][n] TF
    const int* offL;                    // n + 1
    const unsigned char* Lrow;          // nL: t (row kv + 1 + t of the column)
    const unsigned* Lmask;              // n: bit t set if row t is in the union
    const int* offU;                    // n + 1, sweep order s = n - 1 - j, entries incl. diagonal
    const unsigned char* Udist;         // per U stream entry: distance d >= 1 above the diagonal (0 = diagonal)
    const int* offV;                    // r + 1
    const int* Vcol;                    // nV
};

template <class TF>
struct CompactData {
    const TF* L;
    const TF* U;
    const int* piv;
    const TF* V;
    const TF* W;        // [sys][r][n]
    const TF* slu;      // [sys][r][r] (1/u_kk on the diagonal)
    const int* spiv;    // [sys][r]
    const int* perm;    // n
    // shared pair (gs = 1): the partner's matrix is diag(dr) A diag(dc); flip_r[i] = 1 where dr_i =
    // -1 (row index of the matrix), flip_c[j] = 1 where dc_j = -1
    const unsigned char* flip_r = nullptr;
    const unsigned char* flip_c = nullptr;
};

template <class T>
__device__ __forceinline__ void cp_async_bytes(void* s, const void* g, int bytes) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(s));
    if (bytes == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(g) : "memory");
    else if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(g) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(g) : "memory");
}

// copy cnt elements of T from global to shared with cp.async (one warp), commit as one group
template <class T>
__device__ __forceinline__ void warp_stage(T* dst, const T* src, int cnt) {
    const int lane = threadIdx.x & 31;
    for (int e = lane; e < cnt; e += 32) cp_async_bytes<T>(dst + e, src + e, (int)sizeof(T));
}
// the same by `stride` lanes of a warp, this thread being lane l0 of them
template <class T>
__device__ __forceinline__ void lanes_stage(T* dst, const T* src, int cnt, int l0, int stride) {
    for (int e = l0; e < cnt; e += stride) cp_async_bytes<T>(dst + e, src + e, (int)sizeof(T));
}

// The solve: TF = factor type, IO as k_solve (IO_MIXED: TF = zf, data complex128 with accumulate).
// Shared pair (ix.gs = 1): warp group wg is system wg of the handle; lanes 0-15 solve it for io,
// lanes 16-31 solve the partner system wg (io2, matrix diag(dr) A diag(dc)) with the same factors:
// y = A^{-1} (dr b), x = dc y, which is bit for bit the partner's own factorization's solve (the
// pivot search compares magnitudes, and every operation commutes with exact sign flips).
template <class TF, class TD, int IO, int CH = kCChunk, int ST = 2>
__device__ __forceinline__ void solve_compact_body(const CompactIdx& ix, const CompactData<TF>& cd,
                                                   const SolveIo& io0, const SolveIo& io2, int block) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int g = lane / kLanesPer, lg = lane % kLanesPer;
    const int wg = ix.wg0 + block * nw + wib;
    const int gs = ix.gs;
    const bool pair = gs == 1;
    const bool partner = pair && g == 1;
    const int gsel = pair ? 0 : g;              // slot of this half in the interleaved streams
    const int sys = pair ? wg : wg * kGroup + g;
    const SolveIo& io = partner ? io2 : io0;
    const bool live = sys < ix.batch && (!partner || io2.rhs != nullptr);
    const bool wlive = wg < ix.wgroups;
    const int n = ix.n, r = ix.r;
    // shared memory: index lists, then y[G][n + 64], then the staging buffers
    int* s_offL = reinterpret_cast<int*>(sm);
    int* s_offU = s_offL + (n + 1);
    unsigned* s_Lmask = reinterpret_cast<unsigned*>(s_offU + (n + 1));
    unsigned char* s_Lrow = reinterpret_cast<unsigned char*>(s_Lmask + n);
    unsigned char* s_Udist = s_Lrow + ix.nL;
    size_t off = (size_t)(n + 1) * 8 + (size_t)n * 4 + ix.nL + ix.nU;
    off = (off + 15) & ~(size_t)15;
    const size_t per_warp = (size_t)kGroup * (n + 64) + ST * (size_t)(ix.maxLc + ix.maxUc) * gs +
                            (ST * (size_t)CH * gs * sizeof(int) + sizeof(TF) - 1) / sizeof(TF);
    TF* y0 = reinterpret_cast<TF*>(sm + off) + (size_t)wib * per_warp;
    TF* y = y0 + (size_t)g * (n + 64);
    TF* zb = y + n;
    TF* Lb = y0 + (size_t)kGroup * (n + 64);
    TF* Ub = Lb + ST * (size_t)ix.maxLc * gs;
    int* Pb = reinterpret_cast<int*>(Ub + ST * (size_t)ix.maxUc * gs);
    for (int i = threadIdx.x; i <= n; i += blockDim.x) {
        s_offL[i] = ix.offL[i];
        s_offU[i] = ix.offU[i];
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_Lmask[i] = ix.Lmask[i];
    for (int i = threadIdx.x; i < ix.nL; i += blockDim.x) s_Lrow[i] = ix.Lrow[i];
    for (int i = threadIdx.x; i < ix.nU; i += blockDim.x) s_Udist[i] = ix.Udist[i];
    __syncthreads();
    if (!wlive) return;
    // gather the right-hand side (permuted rows first); four rows per lane in flight (the loads of
    // one row wait on the permutation, not on the previous row)
    constexpr int kU = 4;
    for (int i0 = lg; i0 < n; i0 += kU * kLanesPer) {
        int pr[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) pr[u] = (live && i0 + u * kLanesPer < n) ? cd.perm[i0 + u * kLanesPer] : -1;
        TF v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            v[u] = TF(0.0);
            if (pr[u] >= 0) {
                if constexpr (IO == IO_MIXED) {
                    v[u] = to_zf(static_cast<const zd*>(io.rhs)[(size_t)sys * n + pr[u]]);
                } else {
                    v[u] = io_load<TF, IO>(io, sys, n, pr[u]);
                }
                if (partner && cd.flip_r[pr[u]]) v[u] = -v[u];
            }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u)
            if (i0 + u * kLanesPer < n) y[i0 + u * kLanesPer] = v[u];
    }
    __syncwarp();
    const TF* Lg = cd.L + (size_t)wg * ix.nL * gs;
    const TF* Ug = cd.U + (size_t)wg * (ix.nU) * gs;
    const int* Pg = cd.piv + (size_t)wg * n * gs;
    // ---------------- forward: L with the row interchanges
    // ST-deep ring: chunk c sits in buffer c % ST; chunks c + 1 .. c + ST - 1 are in flight while
    // chunk c is swept (an empty commit group keeps the count of pending groups uniform)
    if (ix.kl > 0 && n > 1) {
        const int nch = (n - 1 + CH - 1) / CH;
        auto issue = [&](int c) {
            if (c < nch) {
                const int buf = c % ST;
                const int j0 = c * CH, j1 = min(j0 + CH, n - 1);
                warp_stage(Lb + (size_t)buf * ix.maxLc * gs, Lg + (size_t)s_offL[j0] * gs,
                           (s_offL[j1] - s_offL[j0]) * gs);
                warp_stage(Pb + (size_t)buf * CH * gs, Pg + (size_t)j0 * gs, (j1 - j0) * gs);
            }
            cp_async_commit();
        };
        for (int c = 0; c < ST - 1; ++c) issue(c);
        for (int c = 0; c < nch; ++c) {
            issue(c + ST - 1);
            cp_async_wait<ST - 1>();
            __syncwarp();
            const TF* Lc = Lb + (size_t)(c % ST) * ix.maxLc * gs;
            const int* Pc = Pb + (size_t)(c % ST) * CH * gs;
            const int j0 = c * CH, j1 = min(j0 + CH, n - 1);
            const int base = s_offL[j0];
            int e1 = base;
#pragma unroll
            for (int jj = 0; jj < CH; ++jj) {
                const int j = j0 + jj;
                if (j >= j1) break;
                const int l = Pc[jj * gs + gsel];
                const TF bj = y[l];
                const TF yj0 = y[j];
                const int e0 = e1;
                e1 = s_offL[j + 1];
                __syncwarp();
                for (int e = e0 + lg; e < e1; e += kLanesPer) {
                    const int i = j + 1 + s_Lrow[e];
                    const TF v = (i == l) ? yj0 : y[i];
                    y[i] = cfms(v, Lc[(e - base) * gs + gsel], bj);
                }
                if (lg == 0) {
                    y[j] = bj;
                    if (l != j && !((s_Lmask[j] >> (l - j - 1)) & 1u)) y[l] = yj0;
                }
                __syncwarp();
            }
        }
    }
    // ---------------- backward: U (diagonal holds -1/u_jj)
    {
        const int nch = (n + CH - 1) / CH;
        auto issue = [&](int c) {
            if (c < nch) {
                const int s0 = c * CH, s1 = min(s0 + CH, n);
                warp_stage(Ub + (size_t)(c % ST) * ix.maxUc * gs, Ug + (size_t)s_offU[s0] * gs,
                           (s_offU[s1] - s_offU[s0]) * gs);
            }
            cp_async_commit();
        };
        for (int c = 0; c < ST - 1; ++c) issue(c);
        for (int c = 0; c < nch; ++c) {
            issue(c + ST - 1);
            cp_async_wait<ST - 1>();
            __syncwarp();
            const TF* Uc = Ub + (size_t)(c % ST) * ix.maxUc * gs;
            const int s0 = c * CH, s1 = min(s0 + CH, n);
            const int base = s_offU[s0];
            int e1 = base;
#pragma unroll
            for (int ss = 0; ss < CH; ++ss) {
                const int s = s0 + ss;
                if (s >= s1) break;
                const int j = n - 1 - s;
                const int e0 = e1;
                e1 = s_offU[s + 1];
                const TF yj = y[j];                       // entries hold u_ij / u_jj
                __syncwarp();
                // the column's first entry is the diagonal, held as -1/u_jj: it takes a lane of the
                // same pass (y_j = 0 - (-1/u_jj) y_j) instead of a pass of its own
                for (int e = e0 + lg; e < e1; e += kLanesPer) {
                    const int i = j - s_Udist[e];
                    y[i] = cfms(e == e0 ? TF(0.0) : y[i], Uc[(e - base) * gs + gsel], yj);
                }
                __syncwarp();
            }
        }
    }
    // ---------------- Woodbury: z = S^{-1} V^T y, y -= W z
    if (r > 0) {
        // the small LU of S staged beside z in shared memory (one round trip for all its entries),
        // when it fits in the 64 slots after the system's vector
        const bool staged = r + r * r <= 64 && r <= kMaxRUnroll;
        TF* sl = zb + r;
        if (staged && live)
            for (int q = lg; q < r * r; q += kLanesPer) sl[q] = cd.slu[(size_t)sys * r * r + q];
        const TF* Vg = cd.V + (size_t)wg * ix.nV * gs;
        for (int a = 0; a < r; ++a) {
            TF acc = TF(0.0);
            const int ea = ix.offV[a], eb = ix.offV[a + 1];
            for (int e0 = ea + lg; e0 < eb; e0 += kU * kLanesPer) {
                int c[kU];
                TF v[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int e = e0 + u * kLanesPer;
                    c[u] = e < eb ? ix.Vcol[e] : -1;
                    v[u] = e < eb ? Vg[(size_t)e * gs + gsel] : TF(0.0);
                }
#pragma unroll
                for (int u = 0; u < kU; ++u)
                    if (c[u] >= 0) acc = cfma(acc, v[u], y[c[u]]);
            }
            for (int m = kLanesPer / 2; m > 0; m >>= 1) acc = acc + shfl_xor(acc, m);
            if (lg == 0) zb[a] = acc;
        }
        __syncwarp();
        if (lg == 0 && live) {
            if (staged) small_getrs_staged(sl, cd.spiv + (size_t)sys * r, zb, r);
            else small_getrs(cd.slu + (size_t)sys * r * r, cd.spiv + (size_t)sys * r, zb, r);
        }
        __syncwarp();
        if (live) {
            const TF* Ws = cd.W + (size_t)sys * r * n;
            if (r <= kMaxRUnroll) {
                // the r entries of W for a row loaded together, then the r updates
                for (int i = lg; i < n; i += kLanesPer) {
                    TF w[kMaxRUnroll];
#pragma unroll
                    for (int k = 0; k < kMaxRUnroll; ++k)
                        if (k < r) w[k] = Ws[(size_t)k * n + i];
                    TF acc = y[i];
#pragma unroll
                    for (int k = 0; k < kMaxRUnroll; ++k)
                        if (k < r) acc = cfms(acc, w[k], zb[k]);
                    y[i] = acc;
                }
            } else {
                for (int i = lg; i < n; i += kLanesPer) {
                    TF acc = y[i];
                    for (int k = 0; k < r; ++k) acc = cfms(acc, Ws[(size_t)k * n + i], zb[k]);
                    y[i] = acc;
                }
            }
        }
        __syncwarp();
    }
    if (!live) return;
    if (partner)                                 // x = dc y (each lane flips the entries it stores)
        for (int i = lg; i < n; i += kLanesPer)
            if (cd.flip_c[i]) y[i] = -y[i];
    if constexpr (IO == IO_MIXED) {
        zd* xs = static_cast<zd*>(io.x) + (size_t)sys * n;
        zd* xt = static_cast<zd*>(io.xT);
        const size_t nb = (size_t)ix.batch;
        if (io.accumulate) {
            for (int i0 = lg; i0 < n; i0 += kU * kLanesPer) {
                zd o[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u)
                    if (i0 + u * kLanesPer < n) o[u] = xs[i0 + u * kLanesPer];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int i = i0 + u * kLanesPer;
                    if (i < n) {
                        const zd v = o[u] + zd(y[i].re, y[i].im);
                        xs[i] = v;
                        if (xt) xt[(size_t)i * nb + sys] = v;
                    }
                }
            }
        } else {
            for (int i = lg; i < n; i += kLanesPer) {
                const zd v(y[i].re, y[i].im);
                xs[i] = v;
                if (xt) xt[(size_t)i * nb + sys] = v;
            }
        }
    } else {
        for (int i = lg; i < n; i += kLanesPer) io_store<TF, IO>(io, sys, n, i, y[i]);
    }
}

template <class TF, class TD, int IO>
__global__ void __launch_bounds__(256)
k_solve_compact(CompactIdx ix, CompactData<TF> cd, SolveIo io) {
    const SolveIo none{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    solve_compact_body<TF, TD, IO>(ix, cd, io, none, blockIdx.x);
}

// One launch for several buckets (the systems of a whole step): blocks block_start[b] ..
// block_start[b+1]-1 solve bucket b, so small buckets run beside the large ones.
constexpr int kMaxMulti = 8;
template <class TF>
struct MultiSolve {
    int nb;
    int block_start[kMaxMulti + 1];
    CompactIdx ix[kMaxMulti];
    CompactData<TF> cd[kMaxMulti];
    SolveIo io[kMaxMulti];
    SolveIo io2[kMaxMulti];         // the partner bucket of a shared pair (rhs NULL: none)
};

template <class TF, class TD, int IO, int CH, int ST>
__global__ void __launch_bounds__(256)
k_solve_compact_multi(MultiSolve<TF> ms) {
    int b = 0;
    while (b + 1 < ms.nb && (int)blockIdx.x >= ms.block_start[b + 1]) ++b;
    solve_compact_body<TF, TD, IO, CH, ST>(ms.ix[b], ms.cd[b], ms.io[b], ms.io2[b], blockIdx.x - ms.block_start[b]);
}

// ---- windowed compact solve: the sweeps of solve_compact_body with a window of each vector -------
// In the compact solve a system's vector y (n entries) takes most of a warp's shared memory, which
// bounds the warps resident per SM, and the sweeps are latency-bound chains: more resident warps
// is more throughput. A column touches rows j .. j + kl (forward) or j - kv .. j (backward) only,
// so a ring of WS >= CH + kv + 1 rows (a power of two, ix.wmask = WS - 1) holds every row a chunk of
// CH columns needs. The rows the next chunk brings in are loaded into registers one chunk ahead
// (forward: the permuted right-hand side; backward: the forward result); the rows a chunk finishes
// go to a per-handle scratch in global memory ([warp group][kGroup][n], ix.scratch: the forward
// result, then the solution before the border correction), which the Woodbury pass and the output
// read back. The operations and their order are those of the compact solve: the same bits.
template <class TF, class TD, int IO, int CH, int ST, int LP>
__device__ __forceinline__ void solve_window_body(const CompactIdx& ix, const CompactData<TF>& cd,
                                                  const SolveIo& io0, const SolveIo& io2, int block) {
    extern __shared__ __align__(16) unsigned char sm[];
    // LP lanes per system: 16 (a warp sweeps one warp group of the streams: two systems, or a shared
    // pair), or 8 (two warp groups, four systems: a column's entries fill more of each FP64
    // instruction's lanes; each half of the warp stages its own group's streams)
    constexpr int NS = 32 / LP, NH = NS / kGroup, HL = 32 / NH;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int gq = lane / LP, lg = lane % LP;
    const int half = gq / kGroup, g = gq % kGroup, hl = lane % HL;
    const int wg0w = ix.wg0 + (block * nw + wib) * NH;
    const int wg = wg0w + half;
    const bool hlive = wg < ix.wgroups;          // this half's warp group is solved by this launch
    const int wgc = hlive ? wg : wg0w;           // the streams a half without a group reads (unused)
    const int gs = ix.gs;
    const bool pair = gs == 1;
    const bool partner = pair && g == 1;
    const int gsel = pair ? 0 : g;
    const int sys = pair ? wg : wg * kGroup + g;
    const SolveIo& io = partner ? io2 : io0;
    const bool live = hlive && sys < ix.batch && (!partner || io2.rhs != nullptr);
    const bool wlive = wg0w < ix.wgroups;
    const int n = ix.n, r = ix.r, M = ix.wmask, WS = ix.wmask + 1;
    // shared memory: index lists, then per warp the NS windows of WS rows, the staging rings of the
    // factor streams (one per warp group, at least kGroup x 64 entries each: z and S of every system
    // take them over after the sweeps), and the pivots' rings
    int* s_offL = reinterpret_cast<int*>(sm);
    int* s_offU = s_offL + (n + 1);
    unsigned* s_Lmask = reinterpret_cast<unsigned*>(s_offU + (n + 1));
    unsigned char* s_Lrow = reinterpret_cast<unsigned char*>(s_Lmask + n);
    unsigned char* s_Udist = s_Lrow + ix.nL;
    size_t off = (size_t)(n + 1) * 8 + (size_t)n * 4 + ix.nL + ix.nU;
    off = (off + 15) & ~(size_t)15;
    const size_t ring = max(ST * (size_t)(ix.maxLc + ix.maxUc) * gs, (size_t)kGroup * 64);
    // each system's window 64 (16 lanes) or 32 (8 lanes) bytes after the previous one (PAD
    // elements): the systems touch the same rows in lockstep, and windows a power of two apart
    // would put those rows in the same banks
    constexpr int PAD = (LP == 16 ? 64 : 32) / sizeof(TF);
    const size_t pivw = (ST * (size_t)CH * gs * sizeof(int) + sizeof(TF) - 1) / sizeof(TF);
    const size_t wins = (size_t)NS * WS + (NS - 1) * PAD;
    const size_t per_warp = wins + NH * ring + NH * pivw;
    TF* y0 = reinterpret_cast<TF*>(sm + off) + (size_t)wib * per_warp;
    TF* win = y0 + (size_t)gq * (WS + PAD);
    TF* Lb = y0 + wins + (size_t)half * ring;
    TF* Ub = Lb + ST * (size_t)ix.maxLc * gs;
    TF* zb = y0 + wins + (size_t)gq * 64;
    int* Pb = reinterpret_cast<int*>(y0 + wins + NH * ring + (size_t)half * pivw);
    for (int i = threadIdx.x; i <= n; i += blockDim.x) {
        s_offL[i] = ix.offL[i];
        s_offU[i] = ix.offU[i];
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_Lmask[i] = ix.Lmask[i];
    for (int i = threadIdx.x; i < ix.nL; i += blockDim.x) s_Lrow[i] = ix.Lrow[i];
    for (int i = threadIdx.x; i < ix.nU; i += blockDim.x) s_Udist[i] = ix.Udist[i];
    __syncthreads();
    if (!wlive) return;
    TF* scr = static_cast<TF*>(ix.scratch) + ((size_t)wgc * kGroup + g) * n;
    // the scratch of a half without a group is neither read nor written
    auto sget = [&](int i) -> TF { return hlive ? scr[i] : TF(0.0); };
    auto sput = [&](int i, TF v) {
        if (hlive) scr[i] = v;
    };

    // row i (solver order) of this half's right-hand side
    auto rhs_row = [&](int i) -> TF {
        TF v = TF(0.0);
        if (live) {
            const int p = cd.perm[i];
            if constexpr (IO == IO_MIXED) {
                v = to_zf(static_cast<const zd*>(io.rhs)[(size_t)sys * n + p]);
            } else {
                v = io_load<TF, IO>(io, sys, n, p);
            }
            if (partner && cd.flip_r[p]) v = -v;
        }
        return v;
    };
    const TF* Lg = cd.L + (size_t)wgc * ix.nL * gs;
    const TF* Ug = cd.U + (size_t)wgc * (ix.nU) * gs;
    const int* Pg = cd.piv + (size_t)wgc * n * gs;
    constexpr int PF = (CH + LP - 1) / LP;        // rows a chunk brings in, per lane
    // ---------------- forward: L with the row interchanges (rows [0, hi) have entered the window)
    if (ix.kl > 0 && n > 1) {
        const int nch = (n - 1 + CH - 1) / CH;
        int hi = min(n, min(CH, n - 1) + ix.kl);
        for (int i = lg; i < hi; i += LP) win[i & M] = rhs_row(i);
        auto issue = [&](int c) {
            if (c < nch) {
                const int buf = c % ST;
                const int j0 = c * CH, j1 = min(j0 + CH, n - 1);
                lanes_stage(Lb + (size_t)buf * ix.maxLc * gs, Lg + (size_t)s_offL[j0] * gs,
                            (s_offL[j1] - s_offL[j0]) * gs, hl, HL);
                lanes_stage(Pb + (size_t)buf * CH * gs, Pg + (size_t)j0 * gs, (j1 - j0) * gs, hl, HL);
            }
            cp_async_commit();
        };
        for (int c = 0; c < ST - 1; ++c) issue(c);
        for (int c = 0; c < nch; ++c) {
            issue(c + ST - 1);
            // the rows chunk c + 1 brings in (at most CH), loaded while c is swept
            const int hin = (c + 1 < nch) ? min(n, min((c + 2) * CH, n - 1) + ix.kl) : hi;
            TF pf[PF];
#pragma unroll
            for (int u = 0; u < PF; ++u) pf[u] = hi + lg + u * LP < hin ? rhs_row(hi + lg + u * LP) : TF(0.0);
            cp_async_wait<ST - 1>();
            __syncwarp();
            const TF* Lc = Lb + (size_t)(c % ST) * ix.maxLc * gs;
            const int* Pc = Pb + (size_t)(c % ST) * CH * gs;
            const int j0 = c * CH, j1 = min(j0 + CH, n - 1);
            const int base = s_offL[j0];
            int e1 = base;
#pragma unroll
            for (int jj = 0; jj < CH; ++jj) {
                const int j = j0 + jj;
                if (j >= j1) break;
                const int l = Pc[jj * gs + gsel];
                const TF bj = win[l & M];
                const TF yj0 = win[j & M];
                const int e0 = e1;
                e1 = s_offL[j + 1];
                __syncwarp();
                for (int e = e0 + lg; e < e1; e += LP) {
                    const int i = j + 1 + s_Lrow[e];
                    const TF v = (i == l) ? yj0 : win[i & M];
                    win[i & M] = cfms(v, Lc[(e - base) * gs + gsel], bj);
                }
                if (lg == 0) {
                    win[j & M] = bj;
                    if (l != j && !((s_Lmask[j] >> (l - j - 1)) & 1u)) win[l & M] = yj0;
                }
                __syncwarp();
            }
            // rows j0 .. j1 - 1 are final: out to the scratch, then chunk c + 1's rows in (rows
            // j1 .. hin - 1 span at most CH + kl < WS slots)
            for (int i = j0 + lg; i < j1; i += LP) sput(i, win[i & M]);
            __syncwarp();
#pragma unroll
            for (int u = 0; u < PF; ++u)
                if (hi + lg + u * LP < hin) win[(hi + lg + u * LP) & M] = pf[u];
            hi = hin;
        }
        __syncwarp();
        if (lg == 0) sput(n - 1, win[(n - 1) & M]);      // the last row has no column of its own
    } else {
        for (int i = lg; i < n; i += LP) sput(i, rhs_row(i));
    }
    __syncwarp();
    // ---------------- backward: U (diagonal holds -1/u_jj); rows [lo, n) have entered the window
    {
        const int nch = (n + CH - 1) / CH;
        int lo = max(0, n - min(CH, n) - ix.kv);
        for (int i = lo + lg; i < n; i += LP) win[i & M] = sget(i);
        auto issue = [&](int c) {
            if (c < nch) {
                const int s0 = c * CH, s1 = min(s0 + CH, n);
                lanes_stage(Ub + (size_t)(c % ST) * ix.maxUc * gs, Ug + (size_t)s_offU[s0] * gs,
                            (s_offU[s1] - s_offU[s0]) * gs, hl, HL);
            }
            cp_async_commit();
        };
        for (int c = 0; c < ST - 1; ++c) issue(c);
        for (int c = 0; c < nch; ++c) {
            issue(c + ST - 1);
            const int lon = (c + 1 < nch) ? max(0, n - min((c + 2) * CH, n) - ix.kv) : lo;
            TF pf[PF];
#pragma unroll
            for (int u = 0; u < PF; ++u) pf[u] = lon + lg + u * LP < lo ? sget(lon + lg + u * LP) : TF(0.0);
            cp_async_wait<ST - 1>();
            __syncwarp();
            const TF* Uc = Ub + (size_t)(c % ST) * ix.maxUc * gs;
            const int s0 = c * CH, s1 = min(s0 + CH, n);
            const int base = s_offU[s0];
            int e1 = base;
#pragma unroll
            for (int ss = 0; ss < CH; ++ss) {
                const int s = s0 + ss;
                if (s >= s1) break;
                const int j = n - 1 - s;
                const int e0 = e1;
                e1 = s_offU[s + 1];
                const TF yj = win[j & M];
                __syncwarp();
                for (int e = e0 + lg; e < e1; e += LP) {
                    const int i = j - s_Udist[e];
                    win[i & M] = cfms(e == e0 ? TF(0.0) : win[i & M], Uc[(e - base) * gs + gsel], yj);
                }
                __syncwarp();
            }
            // rows n - s1 .. n - s0 - 1 are final (before the border correction): out to the
            // scratch over their forward values (read when they entered), then chunk c + 1's rows
            for (int i = n - s1 + lg; i < n - s0; i += LP) sput(i, win[i & M]);
            __syncwarp();
#pragma unroll
            for (int u = 0; u < PF; ++u)
                if (lon + lg + u * LP < lo) win[(lon + lg + u * LP) & M] = pf[u];
            lo = lon;
        }
    }
    cp_async_wait<0>();                          // the ring is free for z and S
    __syncwarp();
    // ---------------- Woodbury: z = S^{-1} V^T y, x = y - W z (y from the scratch)
    constexpr int kU = 2;
    if (r > 0) {
        const bool staged = r + r * r <= 64 && r <= kMaxRUnroll;
        TF* sl = zb + r;
        if (staged && live)
            for (int q = lg; q < r * r; q += LP) sl[q] = cd.slu[(size_t)sys * r * r + q];
        const TF* Vg = cd.V + (size_t)wgc * ix.nV * gs;
        for (int a = 0; a < r; ++a) {
            TF acc = TF(0.0);
            const int ea = ix.offV[a], eb = ix.offV[a + 1];
            if constexpr (LP == kLanesPer) {
                for (int e0 = ea + lg; e0 < eb; e0 += kU * kLanesPer) {
                    int c[kU];
                    TF v[kU];
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        const int e = e0 + u * kLanesPer;
                        c[u] = e < eb ? ix.Vcol[e] : -1;
                        v[u] = e < eb ? Vg[(size_t)e * gs + gsel] : TF(0.0);
                    }
                    TF yc[kU];
#pragma unroll
                    for (int u = 0; u < kU; ++u) yc[u] = c[u] >= 0 ? sget(c[u]) : TF(0.0);
#pragma unroll
                    for (int u = 0; u < kU; ++u)
                        if (c[u] >= 0) acc = cfma(acc, v[u], yc[u]);
                }
            } else {
                // each lane sums the entries of two of the 16-lane solve's lanes (lg and lg + 8) and
                // adds the two sums as that solve's first reduction level does: the same bits
                TF a0 = TF(0.0), a1 = TF(0.0);
                for (int e0 = ea + lg; e0 < eb; e0 += kLanesPer) {
                    const int e1 = e0 + LP;
                    const int c0 = ix.Vcol[e0], c1 = e1 < eb ? ix.Vcol[e1] : -1;
                    const TF v0 = Vg[(size_t)e0 * gs + gsel];
                    const TF v1 = c1 >= 0 ? Vg[(size_t)e1 * gs + gsel] : TF(0.0);
                    const TF y0v = sget(c0), y1v = c1 >= 0 ? sget(c1) : TF(0.0);
                    a0 = cfma(a0, v0, y0v);
                    if (c1 >= 0) a1 = cfma(a1, v1, y1v);
                }
                acc = a0 + a1;
            }
            for (int m = LP / 2; m > 0; m >>= 1) acc = acc + shfl_xor(acc, m);
            if (lg == 0) zb[a] = acc;
        }
        __syncwarp();
        if (lg == 0 && live) {
            if (staged) small_getrs_staged(sl, cd.spiv + (size_t)sys * r, zb, r);
            else small_getrs(cd.slu + (size_t)sys * r * r, cd.spiv + (size_t)sys * r, zb, r);
        }
        __syncwarp();
    }
    if (!live) return;
    const TF* Ws = cd.W + (size_t)sys * r * n;
    // the solution's row i: y_i - sum_k W_ki z_k (the compact solve's order), x = dc y for a partner
    auto fin = [&](int i) -> TF {
        TF acc = scr[i];
        if (r > 0) {
            if (r <= kMaxRUnroll) {
                TF w[kMaxRUnroll];
#pragma unroll
                for (int k = 0; k < kMaxRUnroll; ++k)
                    if (k < r) w[k] = Ws[(size_t)k * n + i];
#pragma unroll
                for (int k = 0; k < kMaxRUnroll; ++k)
                    if (k < r) acc = cfms(acc, w[k], zb[k]);
            } else {
                for (int k = 0; k < r; ++k) acc = cfms(acc, Ws[(size_t)k * n + i], zb[k]);
            }
        }
        if (partner && cd.flip_c[i]) acc = -acc;
        return acc;
    };
    if constexpr (IO == IO_MIXED) {
        zd* xs = static_cast<zd*>(io.x) + (size_t)sys * n;
        zd* xt = static_cast<zd*>(io.xT);
        const size_t nb = (size_t)ix.batch;
        for (int i = lg; i < n; i += LP) {
            const TF f = fin(i);
            const zd v = io.accumulate ? xs[i] + zd(f.re, f.im) : zd(f.re, f.im);
            xs[i] = v;
            if (xt) xt[(size_t)i * nb + sys] = v;
        }
    } else {
        for (int i = lg; i < n; i += LP) io_store<TF, IO>(io, sys, n, i, fin(i));
    }
}

// warps per block of the windowed solve: FP32 16 (the index lists shared by more warps; measured on
// the channel's FP32 solve 2.36 ms against 2.47 with 8), FP64 8 (the register budget of 8-warp
// blocks keeps it at 48 registers: 3.05 ms against 3.20 with 16)
template <class TF>
constexpr int window_max_warps() { return sizeof(TF) == 8 ? 16 : 8; }
template <class TF, class TD, int IO, int CH, int ST, int LP>
__global__ void __launch_bounds__(32 * window_max_warps<TF>())
k_solve_window_multi(MultiSolve<TF> ms) {
    int b = 0;
    while (b + 1 < ms.nb && (int)blockIdx.x >= ms.block_start[b + 1]) ++b;
    solve_window_body<TF, TD, IO, CH, ST, LP>(ms.ix[b], ms.cd[b], ms.io[b], ms.io2[b], blockIdx.x - ms.block_start[b]);
}

// ---- one system per warp, lanes split over (entry, real/imaginary part) -------------------------
// The latency variant for small batches: a column's updates take two fused multiply-adds per lane
// (one component each) where the two-systems-per-warp sweep takes four, so the chain from column
// to column is half as long; throughput per system is the same. It reads the same compact streams
// (system sys is slot sys % 2 of warp group sys / 2) and stages the pair's chunk.
template <class TF> struct CompT;
template <> struct CompT<zd> { using T = double; };
template <> struct CompT<zf> { using T = float; };
__device__ __forceinline__ double fm(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fm(float a, float b, float c) { return fmaf(a, b, c); }
template <class TF>
__device__ __forceinline__ typename CompT<TF>::T comp(const TF& v, int c) { return c ? v.im : v.re; }
// component c of v - a b, in the order of cfms (the two-systems sweep's arithmetic): with the lane's
// operands of b picked once per column, B0 = b.re (c = 0) or b.im (c = 1) and B1 = b.im or -b.re,
// it is fma(a.im, B1, fma(-a.re, B0, v)) -- the products are exact sign flips of cfms's, so the
// roundings are the same
template <class TF>
struct CompB {
    typename CompT<TF>::T b0, b1;
};
template <class TF>
__device__ __forceinline__ CompB<TF> comp_b(const TF& b, int c) {
    return c ? CompB<TF>{b.im, -b.re} : CompB<TF>{b.re, b.im};
}
template <class TF>
__device__ __forceinline__ typename CompT<TF>::T cfms_comp(typename CompT<TF>::T vc, const TF& a, const CompB<TF>& b) {
    return fm(a.im, b.b1, fm(-a.re, b.b0, vc));
}

// The sweeps of the split-lane solve (one system per warp; lane = entry slot es, component c).
template <class TF>
struct SplitSweep {
    TF* y;
    const int* s_offL;
    const int* s_offU;
    const unsigned* s_Lmask;
    const unsigned char* s_Lrow;
    const unsigned char* s_Udist;
    TF* Lb;
    TF* Ub;
    int* Pb;
    const TF* Lg;
    const TF* Ug;
    const int* Pg;
    int n, maxLc, maxUc, gs, es, c, lane;
    // a block of the partitioned solve (PART sweeps): columns [c0, c1), y holds rows base ..
    int c0 = 0, c1 = 0, base = 0;
};

// One pass of a column's entries (slots es, es + 16, ...): NP > 0 unrolls NP predicated passes
// (every column holds at most 16 NP entries), NP = 0 loops over any count. The same updates in the
// same order either way.
template <int NP, class F>
__device__ __forceinline__ void column_passes(int e0, int e1, int es, F&& f) {
    if constexpr (NP > 0) {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const int e = e0 + es + 16 * p;
            if (e < e1) f(e);
        }
    } else {
        for (int e = e0 + es; e < e1; e += 16) f(e);
    }
}

// forward: L with the row interchanges (PART: the columns [c0, c1) of a block, on the rows held
// from w.base; else every column)
template <class TF, int CH, int ST, int NP, bool PART = false>
__device__ __forceinline__ void split_forward(const SplitSweep<TF>& w) {
    using T = typename CompT<TF>::T;
    TF* y = w.y;
    const int n = w.n, gs = w.gs, c = w.c;
    const int cb = PART ? w.c0 : 0, ce = PART ? w.c1 : n - 1;
    const int yb = PART ? w.base : 0;
    const int nch = (ce - cb + CH - 1) / CH;
    auto issue = [&](int ch) {
        if (ch < nch) {
            const int buf = ch % ST;
            const int j0 = cb + ch * CH, j1 = min(j0 + CH, ce);
            warp_stage(w.Lb + (size_t)buf * w.maxLc * 2, w.Lg + (size_t)w.s_offL[j0] * 2,
                       (w.s_offL[j1] - w.s_offL[j0]) * 2);
            warp_stage(w.Pb + (size_t)buf * CH * 2, w.Pg + (size_t)j0 * 2, (j1 - j0) * 2);
        }
        cp_async_commit();
    };
    for (int ch = 0; ch < ST - 1; ++ch) issue(ch);
    for (int ch = 0; ch < nch; ++ch) {
        issue(ch + ST - 1);
        cp_async_wait<ST - 1>();
        __syncwarp();
        const TF* Lc = w.Lb + (size_t)(ch % ST) * w.maxLc * 2;
        const int* Pc = w.Pb + (size_t)(ch % ST) * CH * 2;
        const int j0 = cb + ch * CH, j1 = min(j0 + CH, ce);
        const int base = w.s_offL[j0];
        int e1 = base;
#pragma unroll
        for (int jj = 0; jj < CH; ++jj) {
            const int j = j0 + jj;
            if (j >= j1) break;
            const int l = Pc[jj * 2 + gs];
            const TF bj = y[l - yb];
            const TF yj0 = y[j - yb];
            const int e0 = e1;
            e1 = w.s_offL[j + 1];
            __syncwarp();
            const CompB<TF> bq = comp_b(bj, c);
            const T yj0c = comp(yj0, c);
            column_passes<NP>(e0, e1, w.es, [&](int e) {
                const int i = j + 1 + w.s_Lrow[e];
                T* yi = reinterpret_cast<T*>(&y[i - yb]) + c;
                const T vc = (i == l) ? yj0c : *yi;
                *yi = cfms_comp<TF>(vc, Lc[(e - base) * 2 + gs], bq);
            });
            if (w.lane == 0) {
                y[j - yb] = bj;
                if (l != j && !((w.s_Lmask[j] >> (l - j - 1)) & 1u)) y[l - yb] = yj0;
            }
            __syncwarp();
        }
    }
}

// backward: U (each column's first entry is its diagonal, held as -1/u_jj); PART as split_forward
template <class TF, int CH, int ST, int NP, bool PART = false>
__device__ __forceinline__ void split_backward(const SplitSweep<TF>& w) {
    using T = typename CompT<TF>::T;
    TF* y = w.y;
    const int n = w.n, gs = w.gs, c = w.c;
    const int sb = PART ? n - w.c1 : 0, se = PART ? n - w.c0 : n;     // sweep index s = n - 1 - j
    const int yb = PART ? w.base : 0;
    const int nch = (se - sb + CH - 1) / CH;
    auto issue = [&](int ch) {
        if (ch < nch) {
            const int s0 = sb + ch * CH, s1 = min(s0 + CH, se);
            warp_stage(w.Ub + (size_t)(ch % ST) * w.maxUc * 2, w.Ug + (size_t)w.s_offU[s0] * 2,
                       (w.s_offU[s1] - w.s_offU[s0]) * 2);
        }
        cp_async_commit();
    };
    for (int ch = 0; ch < ST - 1; ++ch) issue(ch);
    for (int ch = 0; ch < nch; ++ch) {
        issue(ch + ST - 1);
        cp_async_wait<ST - 1>();
        __syncwarp();
        const TF* Uc = w.Ub + (size_t)(ch % ST) * w.maxUc * 2;
        const int s0 = sb + ch * CH, s1 = min(s0 + CH, se);
        const int base = w.s_offU[s0];
        int e1 = base;
#pragma unroll
        for (int ss = 0; ss < CH; ++ss) {
            const int s = s0 + ss;
            if (s >= s1) break;
            const int j = n - 1 - s;
            const int e0 = e1;
            e1 = w.s_offU[s + 1];
            const TF yj = y[j - yb];
            __syncwarp();
            const CompB<TF> bq = comp_b(yj, c);
            column_passes<NP>(e0, e1, w.es, [&](int e) {
                const int i = j - w.s_Udist[e];
                T* yi = reinterpret_cast<T*>(&y[i - yb]) + c;
                const T vc = e == e0 ? T(0) : *yi;
                *yi = cfms_comp<TF>(vc, Uc[(e - base) * 2 + gs], bq);
            });
            __syncwarp();
        }
    }
}

template <class TF, class TD, int IO, int CH, int ST>
__device__ __forceinline__ void solve_split_body(const CompactIdx& ix, const CompactData<TF>& cd,
                                                 const SolveIo& io, int block) {
    using T = typename CompT<TF>::T;
    extern __shared__ __align__(16) unsigned char sm[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // systems ix.wg0 .. ix.wgroups - 1 (one per warp; launch_split_t sets the range in systems)
    const int sys = ix.wg0 + block * nw + wib;
    const int gs = sys & 1, wgs = sys >> 1;
    const int es = lane >> 1, c = lane & 1;           // entry slot, component
    const bool live = sys < ix.wgroups;
    const int n = ix.n, r = ix.r;
    int* s_offL = reinterpret_cast<int*>(sm);
    int* s_offU = s_offL + (n + 1);
    unsigned* s_Lmask = reinterpret_cast<unsigned*>(s_offU + (n + 1));
    unsigned char* s_Lrow = reinterpret_cast<unsigned char*>(s_Lmask + n);
    unsigned char* s_Udist = s_Lrow + ix.nL;
    size_t off = (size_t)(n + 1) * 8 + (size_t)n * 4 + ix.nL + ix.nU;
    off = (off + 15) & ~(size_t)15;
    const size_t per_warp = (size_t)(n + 64) + ST * (size_t)(ix.maxLc + ix.maxUc) * 2 +
                            (ST * (size_t)CH * 2 * sizeof(int) + sizeof(TF) - 1) / sizeof(TF);
    TF* y = reinterpret_cast<TF*>(sm + off) + (size_t)wib * per_warp;
    TF* zb = y + n;
    TF* Lb = y + (n + 64);
    TF* Ub = Lb + ST * (size_t)ix.maxLc * 2;
    int* Pb = reinterpret_cast<int*>(Ub + ST * (size_t)ix.maxUc * 2);
    for (int i = threadIdx.x; i <= n; i += blockDim.x) {
        s_offL[i] = ix.offL[i];
        s_offU[i] = ix.offU[i];
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_Lmask[i] = ix.Lmask[i];
    for (int i = threadIdx.x; i < ix.nL; i += blockDim.x) s_Lrow[i] = ix.Lrow[i];
    for (int i = threadIdx.x; i < ix.nU; i += blockDim.x) s_Udist[i] = ix.Udist[i];
    __syncthreads();
    if (!live) return;                               // one system per warp: the whole warp leaves
    constexpr int kU = 4;
    for (int i0 = lane; i0 < n; i0 += kU * 32) {
        int pr[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) pr[u] = i0 + u * 32 < n ? cd.perm[i0 + u * 32] : -1;
        TF v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            v[u] = TF(0.0);
            if (pr[u] >= 0) {
                if constexpr (IO == IO_MIXED) v[u] = to_zf(static_cast<const zd*>(io.rhs)[(size_t)sys * n + pr[u]]);
                else v[u] = io_load<TF, IO>(io, sys, n, pr[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u)
            if (i0 + u * 32 < n) y[i0 + u * 32] = v[u];
    }
    __syncwarp();
    const TF* Lg = cd.L + (size_t)wgs * ix.nL * 2;
    const TF* Ug = cd.U + (size_t)wgs * ix.nU * 2;
    const int* Pg = cd.piv + (size_t)wgs * n * 2;
    const SplitSweep<TF> sw{y, s_offL, s_offU, s_Lmask, s_Lrow, s_Udist, Lb, Ub, Pb, Lg, Ug, Pg,
                            n, ix.maxLc, ix.maxUc, gs, es, c, lane};
    // the column passes unrolled and predicated where every column fits 16 or 32 entry slots
    if (ix.kl > 0 && n > 1) {
        if (ix.maxLcol <= 16) split_forward<TF, CH, ST, 1>(sw);
        else if (ix.maxLcol <= 32) split_forward<TF, CH, ST, 2>(sw);
        else split_forward<TF, CH, ST, 0>(sw);
    }
    if (ix.maxUcol <= 16) split_backward<TF, CH, ST, 1>(sw);
    else if (ix.maxUcol <= 32) split_backward<TF, CH, ST, 2>(sw);
    else split_backward<TF, CH, ST, 0>(sw);
    if (r > 0) {
        const bool staged = r + r * r <= 64 && r <= kMaxRUnroll;
        TF* sl = zb + r;
        if (staged)
            for (int q = lane; q < r * r; q += 32) sl[q] = cd.slu[(size_t)sys * r * r + q];
        const TF* Vg = cd.V + (size_t)wgs * ix.nV * 2;
        for (int a = 0; a < r; ++a) {
            // kU entries per lane in flight (their column ids and values loaded together), in the
            // order of one entry per lane and pass
            TF acc = TF(0.0);
            const int ea = ix.offV[a], eb = ix.offV[a + 1];
            for (int e0 = ea + lane; e0 < eb; e0 += kU * 32) {
                int cix[kU];
                TF v[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int e = e0 + u * 32;
                    cix[u] = e < eb ? ix.Vcol[e] : -1;
                    v[u] = e < eb ? Vg[(size_t)e * 2 + gs] : TF(0.0);
                }
#pragma unroll
                for (int u = 0; u < kU; ++u)
                    if (cix[u] >= 0) acc = cfma(acc, v[u], y[cix[u]]);
            }
            for (int m = 16; m > 0; m >>= 1) acc = acc + shfl_xor(acc, m);
            if (lane == 0) zb[a] = acc;
        }
        __syncwarp();
        if (lane == 0) {
            if (staged) small_getrs_staged(sl, cd.spiv + (size_t)sys * r, zb, r);
            else small_getrs(cd.slu + (size_t)sys * r * r, cd.spiv + (size_t)sys * r, zb, r);
        }
        __syncwarp();
        const TF* Ws = cd.W + (size_t)sys * r * n;
        if (r <= kMaxRUnroll) {
            // the r entries of W for a row loaded together, then the r updates in order
            for (int i = lane; i < n; i += 32) {
                TF w[kMaxRUnroll];
#pragma unroll
                for (int k = 0; k < kMaxRUnroll; ++k)
                    if (k < r) w[k] = Ws[(size_t)k * n + i];
                TF acc = y[i];
#pragma unroll
                for (int k = 0; k < kMaxRUnroll; ++k)
                    if (k < r) acc = cfms(acc, w[k], zb[k]);
                y[i] = acc;
            }
        } else {
            for (int i = lane; i < n; i += 32) {
                TF acc = y[i];
                for (int k = 0; k < r; ++k) acc = cfms(acc, Ws[(size_t)k * n + i], zb[k]);
                y[i] = acc;
            }
        }
        __syncwarp();
    }
    if constexpr (IO == IO_MIXED) {
        zd* xs = static_cast<zd*>(io.x) + (size_t)sys * n;
        zd* xt = static_cast<zd*>(io.xT);
        for (int i = lane; i < n; i += 32) {
            const zd v = io.accumulate ? xs[i] + zd(y[i].re, y[i].im) : zd(y[i].re, y[i].im);
            xs[i] = v;
            if (xt) xt[(size_t)i * ix.batch + sys] = v;
        }
    } else {
        for (int i = lane; i < n; i += 32) io_store<TF, IO>(io, sys, n, i, y[i]);
    }
}

template <class TF, class TD, int IO, int CH, int ST>
__global__ void __launch_bounds__(256)
k_solve_split_multi(MultiSolve<TF> ms) {
    int b = 0;
    while (b + 1 < ms.nb && (int)blockIdx.x >= ms.block_start[b + 1]) ++b;
    solve_split_body<TF, TD, IO, CH, ST>(ms.ix[b], ms.cd[b], ms.io[b], blockIdx.x - ms.block_start[b]);
}

// ------------------------------------------------------------------------------------------------
// Partitioned solve (small batches, FP64): the latency of one warp's column chain bounds the sweeps
// of a small batch (one warp per system, the SMs mostly idle). The columns of a system are split in
// blocks of kPartM; block k's forward sweep maps the values on its first kwf rows (the window the
// previous blocks leave) and the right-hand side on its other rows linearly to its final rows and
// to the window it leaves the next block, so
//     out_k = sweep_k(b) + R_k delta_k,   delta_{k+1} = (window part of out_k) - b on those rows,
// where sweep_k(b) is the block's sweep of the right-hand side alone (all blocks at once, one warp
// each), R_k the block's responses to unit window values (built once per factorization by the same
// sweep), and the kwf-vectors delta_k the only sequential part. The backward sweep is split the same
// way, from the last block up, with windows of kwb = kl + ku rows (the reach of a U column). The
// same operations as the sequential sweeps, grouped otherwise: the results agree to rounding. This
// is the partitioned ("SPIKE") solve of banded systems (Polizzi and Sameh, 2006) applied to the
// sweeps of the factored system.
constexpr int kPartM = 32;              // columns per block
constexpr int kPartCH = 8, kPartST = 2; // staging of the blocks' factor streams
constexpr int kPartMaxWarps = 32;       // blocks per system: n <= 1024

struct PartArgs {
    CompactIdx ix;
    CompactData<zd> cd;
    SolveIo io;
    const zd* Rf;                       // [batch][nbf][32 + kwf][kwf]
    const zd* Rb;                       // [batch][nbb][32 + kwb][kwb]
    int nbf, nbb, kwf, kwb, maxLc, maxUc;
};

// shared memory of one warp's block sweep: its block buffer and the staging ring
__host__ __device__ inline size_t part_warp_elems(int maxLc, int maxUc) {
    return 64 + (size_t)kPartST * (maxLc + maxUc) * 2 + ((size_t)kPartST * kPartCH * 2 * sizeof(int) + 15) / 16;
}
__host__ __device__ inline size_t part_index_bytes(int n, int nL, int nU) {
    return (((size_t)(n + 1) * 8 + (size_t)n * 4 + nL + nU) + 15) & ~(size_t)15;
}

// load the stream index lists of a bucket into shared memory (every thread of the block)
__device__ __forceinline__ void part_load_index(const CompactIdx& ix, unsigned char* sm, int** offL, int** offU,
                                                unsigned** Lmask, unsigned char** Lrow, unsigned char** Udist) {
    const int n = ix.n;
    *offL = reinterpret_cast<int*>(sm);
    *offU = *offL + (n + 1);
    *Lmask = reinterpret_cast<unsigned*>(*offU + (n + 1));
    *Lrow = reinterpret_cast<unsigned char*>(*Lmask + n);
    *Udist = *Lrow + ix.nL;
    for (int i = threadIdx.x; i <= n; i += blockDim.x) {
        (*offL)[i] = ix.offL[i];
        (*offU)[i] = ix.offU[i];
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) (*Lmask)[i] = ix.Lmask[i];
    for (int i = threadIdx.x; i < ix.nL; i += blockDim.x) (*Lrow)[i] = ix.Lrow[i];
    for (int i = threadIdx.x; i < ix.nU; i += blockDim.x) (*Udist)[i] = ix.Udist[i];
}

template <int NPF, int NPB>
__device__ __forceinline__ void part_sweep(const SplitSweep<zd>& w, bool forward) {
    if (forward) split_forward<zd, kPartCH, kPartST, NPF, true>(w);
    else split_backward<zd, kPartCH, kPartST, NPB, true>(w);
}

// The responses: one warp per (system, direction, block, unit position u). Forward: the unit at the
// block's window row u (row c0 + u); backward: at row c1 - kwb + u (the rows the blocks below
// update), the last block's (never used: nothing lies below it) written as zeros.
template <int NPF, int NPB>
__global__ void __launch_bounds__(256) k_part_build(PartArgs pa, zd* Rf, zd* Rb) {
    extern __shared__ __align__(16) unsigned char sm[];
    const CompactIdx& ix = pa.ix;
    int *s_offL, *s_offU;
    unsigned* s_Lmask;
    unsigned char *s_Lrow, *s_Udist;
    part_load_index(ix, sm, &s_offL, &s_offU, &s_Lmask, &s_Lrow, &s_Udist);
    __syncthreads();
    const int n = ix.n, lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const long long per_sys = (long long)pa.nbf * pa.kwf + (long long)pa.nbb * pa.kwb;
    const long long task = (long long)blockIdx.x * nw + wib;
    if (task >= per_sys * ix.batch) return;
    const int sys = (int)(task / per_sys);
    long long rem = task - (long long)sys * per_sys;
    const bool fwd = rem < (long long)pa.nbf * pa.kwf;
    if (!fwd) rem -= (long long)pa.nbf * pa.kwf;
    const int kw = fwd ? pa.kwf : pa.kwb;
    const int k = (int)(rem / kw), u = (int)(rem - (long long)k * kw);
    const int c0 = k * kPartM;
    const int c1 = fwd ? min(c0 + kPartM, n - 1) : min(c0 + kPartM, n);
    const int len = kPartM + kw;
    zd* buf = reinterpret_cast<zd*>(sm + part_index_bytes(n, ix.nL, ix.nU)) +
              (size_t)wib * part_warp_elems(pa.maxLc, pa.maxUc);
    for (int i = lane; i < 64; i += 32) buf[i] = zd(0.0, 0.0);
    __syncwarp();
    const bool last_b = !fwd && k == pa.nbb - 1;
    if (!last_b) {
        if (lane == 0) buf[fwd ? u : kPartM + u] = zd(1.0, 0.0);
        __syncwarp();
        const int gs = sys & 1, wgs = sys >> 1;
        SplitSweep<zd> w{buf, s_offL, s_offU, s_Lmask, s_Lrow, s_Udist, buf + 64,
                         buf + 64 + (size_t)kPartST * pa.maxLc * 2,
                         reinterpret_cast<int*>(buf + 64 + (size_t)kPartST * (pa.maxLc + pa.maxUc) * 2),
                         pa.cd.L + (size_t)wgs * ix.nL * 2, pa.cd.U + (size_t)wgs * ix.nU * 2,
                         pa.cd.piv + (size_t)wgs * n * 2, n, pa.maxLc, pa.maxUc, gs, lane >> 1, lane & 1, lane};
        w.c0 = c0;
        w.c1 = c1;
        w.base = fwd ? c0 : c0 - pa.kwb;
        if (c1 > c0) part_sweep<NPF, NPB>(w, fwd);
    }
    zd* R = fwd ? Rf + (((size_t)sys * pa.nbf + k) * len) * kw : Rb + (((size_t)sys * pa.nbb + k) * len) * kw;
    for (int i = lane; i < len; i += 32) R[(size_t)i * kw + u] = buf[i];
}

// complex c = a b (component by component, for the responses' sums)
__device__ __forceinline__ zd part_cmac(zd acc, zd a, zd b) {
    return zd(fma(-a.im, b.im, fma(a.re, b.re, acc.re)), fma(a.im, b.re, fma(a.re, b.im, acc.im)));
}

// The solve: one block per system, one warp per column block.
struct MultiPart {
    int nb;
    int block_start[kMaxMulti + 1];
    PartArgs a[kMaxMulti];
};

template <int NPF, int NPB>
__global__ void __launch_bounds__(32 * kPartMaxWarps) k_solve_part(const __grid_constant__ MultiPart mp) {
    extern __shared__ __align__(16) unsigned char sm[];
    int b = 0;
    while (b + 1 < mp.nb && (int)blockIdx.x >= mp.block_start[b + 1]) ++b;
    const PartArgs& pa = mp.a[b];
    const CompactIdx& ix = pa.ix;
    const CompactData<zd>& cd = pa.cd;
    const int sys = blockIdx.x - mp.block_start[b];
    const int n = ix.n, r = ix.r, lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int kwf = pa.kwf, kwb = pa.kwb, nbf = pa.nbf, nbb = pa.nbb;
    int *s_offL, *s_offU;
    unsigned* s_Lmask;
    unsigned char *s_Lrow, *s_Udist;
    part_load_index(ix, sm, &s_offL, &s_offU, &s_Lmask, &s_Lrow, &s_Udist);
    zd* y = reinterpret_cast<zd*>(sm + part_index_bytes(n, ix.nL, ix.nU));      // n (+ 64: z, S)
    zd* df = y + n + 64;                                                       // (nbf + 1) x kwf
    zd* db = df + (size_t)(nbf + 1) * kwf;                                     // (nbb + 1) x kwb
    zd* wk = db + (size_t)(nbb + 1) * kwb;
    zd* buf = wk + (size_t)wib * part_warp_elems(pa.maxLc, pa.maxUc);
    // the right-hand side, rows in solver order
    for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = io_load<zd, IO_MAPPED>(pa.io, sys, n, cd.perm[i]);
    for (int i = threadIdx.x; i < (nbf + 1) * kwf; i += blockDim.x) df[i] = zd(0.0, 0.0);
    for (int i = threadIdx.x; i < (nbb + 1) * kwb; i += blockDim.x) db[i] = zd(0.0, 0.0);
    __syncthreads();
    const int gs = sys & 1, wgs = sys >> 1;
    SplitSweep<zd> w{buf, s_offL, s_offU, s_Lmask, s_Lrow, s_Udist, buf + 64,
                     buf + 64 + (size_t)kPartST * pa.maxLc * 2,
                     reinterpret_cast<int*>(buf + 64 + (size_t)kPartST * (pa.maxLc + pa.maxUc) * 2),
                     cd.L + (size_t)wgs * ix.nL * 2, cd.U + (size_t)wgs * ix.nU * 2, cd.piv + (size_t)wgs * n * 2,
                     n, pa.maxLc, pa.maxUc, gs, lane >> 1, lane & 1, lane};
    const int lenf = kPartM + kwf, lenb = kPartM + kwb;
    // ---- forward: every block's sweep of the right-hand side (rows c0 .. c1 + kwf)
    const int kf = wib, c0f = kf * kPartM, c1f = min(c0f + kPartM, n - 1);
    if (kf < nbf) {
        for (int i = lane; i < 64; i += 32) buf[i] = (i < lenf && c0f + i < n) ? y[c0f + i] : zd(0.0, 0.0);
        __syncwarp();
        w.c0 = c0f;
        w.c1 = c1f;
        w.base = c0f;
        if (c1f > c0f) part_sweep<NPF, NPB>(w, true);
    }
    __syncthreads();
    // the windows, block after block (one warp; lanes over window row and component)
    if (wib == 0) {
        const int t = lane >> 1, cc = lane & 1;
        for (int k = 0; k + 1 < nbf; ++k) {
            const int c1 = (k + 1) * kPartM;
            const zd* bk = wk + (size_t)k * part_warp_elems(pa.maxLc, pa.maxUc);
            if (t < kwf && c1 + t < n) {
                const zd* Rk = pa.Rf + (((size_t)sys * nbf + k) * lenf + kPartM + t) * kwf;
                const zd* dk = df + (size_t)k * kwf;
                zd acc = bk[kPartM + t] - y[c1 + t];
                for (int v = 0; v < kwf; ++v) acc = part_cmac(acc, Rk[v], dk[v]);
                if (cc == 0) df[(size_t)(k + 1) * kwf + t] = acc;
            }
            __syncwarp();
        }
    }
    __syncthreads();
    // final rows of the forward sweep: out = sweep(b) + R delta
    if (kf < nbf) {
        const int rows = (kf == nbf - 1) ? n - c0f : kPartM;
        const zd* dk = df + (size_t)kf * kwf;
        const zd* Rk = pa.Rf + ((size_t)sys * nbf + kf) * lenf * kwf;
        for (int i = lane; i < rows; i += 32) {
            zd acc = buf[i];
            for (int v = 0; v < kwf; ++v) acc = part_cmac(acc, Rk[(size_t)i * kwf + v], dk[v]);
            y[c0f + i] = acc;
        }
    }
    __syncthreads();
    // ---- backward: every block's sweep of the forward result (rows c0 - kwb .. c1)
    const int kb = wib, c0b = kb * kPartM, c1b = min(c0b + kPartM, n);
    if (kb < nbb) {
        for (int i = lane; i < 64; i += 32) {
            const int g = c0b - kwb + i;
            buf[i] = (i < lenb && g >= 0 && g < c1b) ? y[g] : zd(0.0, 0.0);
        }
        __syncwarp();
        w.c0 = c0b;
        w.c1 = c1b;
        w.base = c0b - kwb;
        part_sweep<NPF, NPB>(w, false);
    }
    __syncthreads();
    // the windows from the last block up (warps 0 and 1: lanes over window row and component; every
    // warp takes part in the block barrier of each step)
    for (int k = nbb - 1; k >= 1; --k) {
        const int t = 16 * wib + (lane >> 1), cc = lane & 1;
        const int c0 = k * kPartM;
        if (wib < 2 && t < kwb && c0 - kwb + t >= 0) {
            const zd* bk = wk + (size_t)k * part_warp_elems(pa.maxLc, pa.maxUc);
            const zd* Rk = pa.Rb + (((size_t)sys * nbb + k) * lenb + t) * kwb;
            const zd* dk = db + (size_t)k * kwb;
            zd acc = bk[t] - y[c0 - kwb + t];
            for (int v = 0; v < kwb; ++v) acc = part_cmac(acc, Rk[v], dk[v]);
            if (cc == 0) db[(size_t)(k - 1) * kwb + t] = acc;
        }
        __syncthreads();
    }
    if (kb < nbb) {
        const int rows = c1b - c0b;
        const zd* dk = db + (size_t)kb * kwb;
        const zd* Rk = pa.Rb + ((size_t)sys * nbb + kb) * lenb * kwb;
        for (int i = lane; i < rows; i += 32) {
            zd acc = buf[kwb + i];
            for (int v = 0; v < kwb; ++v) acc = part_cmac(acc, Rk[(size_t)(kwb + i) * kwb + v], dk[v]);
            y[c0b + i] = acc;
        }
    }
    __syncthreads();
    // ---- Woodbury: z = S^{-1} V^T y (warp a % nw takes border row a), y -= W z
    zd* zb = y + n;
    if (r > 0) {
        const zd* Vg = cd.V + (size_t)wgs * ix.nV * 2;
        for (int a = wib; a < r; a += nw) {
            zd acc(0.0, 0.0);
            for (int e = ix.offV[a] + lane; e < ix.offV[a + 1]; e += 32)
                acc = cfma(acc, Vg[(size_t)e * 2 + gs], y[ix.Vcol[e]]);
            for (int m = 16; m > 0; m >>= 1) acc = acc + shfl_xor(acc, m);
            if (lane == 0) zb[a] = acc;
        }
        __syncthreads();
        if (threadIdx.x == 0) small_getrs(cd.slu + (size_t)sys * r * r, cd.spiv + (size_t)sys * r, zb, r);
        __syncthreads();
        const zd* Ws = cd.W + (size_t)sys * r * n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            zd acc = y[i];
            for (int k = 0; k < r; ++k) acc = cfms(acc, Ws[(size_t)k * n + i], zb[k]);
            y[i] = acc;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) io_store<zd, IO_MAPPED>(pa.io, sys, n, i, y[i]);
}

}  // namespace cng

namespace cng {

template <class T>
__global__ void k_union_mask(const T* __restrict__ a, long long stride, int batch, long long count,
                             unsigned char* __restrict__ mask) {
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < count;
         q += (long long)gridDim.x * blockDim.x) {
        unsigned char any = 0;
        for (int k = 0; k < batch && !any; ++k)
            if (!is_zero(a[(size_t)k * stride + q])) any = 1;
        mask[q] = any;
    }
}

// one warp per system: band LU, pivots and V^T into the interleaved compact streams
template <class T>
__global__ void k_pack_compact(BandView<T> v, CompactIdx ix, T* __restrict__ L, T* __restrict__ U,
                               T* __restrict__ V, int* __restrict__ piv, int total_sys) {
    const int sys = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (sys >= total_sys) return;
    const int lane = threadIdx.x & 31;
    const int kGroup = ix.gs;                   // systems per warp group of the streams
    const int wg = sys / kGroup, g = sys % kGroup;
    const bool live = sys < v.batch;
    const int n = v.n, kv = v.kl + v.ku;
    const T* ab = v.ab + (size_t)(live ? sys : 0) * n * v.ldab;
    T* Lw = L + (size_t)wg * ix.nL * kGroup;
    T* Uw = U + (size_t)wg * ix.nU * kGroup;
    for (int j = lane; j < n - 1; j += 32)
        for (int e = ix.offL[j]; e < ix.offL[j + 1]; ++e)
            Lw[(size_t)e * kGroup + g] = live ? ab[(size_t)j * v.ldab + kv + 1 + ix.Lrow[e]] : T(0.0);
    for (int s = lane; s < n; s += 32) {
        const int j = n - 1 - s;
        const T dinv = live ? ab[(size_t)j * v.ldab + kv] : T(0.0);     // 1 / u_jj
        for (int e = ix.offU[s]; e < ix.offU[s + 1]; ++e) {
            const int d = ix.Udist[e];
            // the diagonal entry holds -1 / u_jj (the sweep applies it as y_j = 0 - (-1/u_jj) y_j);
            // the others are pre-scaled: u_ij / u_jj
            Uw[(size_t)e * kGroup + g] = !live ? T(0.0) : (d == 0 ? -dinv : ab[(size_t)j * v.ldab + kv - d] * dinv);
        }
    }
    int* Pw = piv + (size_t)wg * n * kGroup;
    for (int j = lane; j < n; j += 32) Pw[(size_t)j * kGroup + g] = live ? v.ipiv[(size_t)sys * n + j] : j;
    if (v.r > 0) {
        T* Vw = V + (size_t)wg * ix.nV * kGroup;
        const T* vt = v.vt + (size_t)(live ? sys : 0) * v.r * n;
        for (int a = 0; a < v.r; ++a)
            for (int e = ix.offV[a] + lane; e < ix.offV[a + 1]; e += 32)
                Vw[(size_t)e * kGroup + g] = live ? vt[(size_t)a * n + ix.Vcol[e]] : T(0.0);
    }
}

__global__ void k_demote_n(const zd* __restrict__ a, zf* __restrict__ b, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = to_zf(a[i]);
}

// FP32 copies of the compact factor streams (the FP32 form's solves read these).
static void demote_compact(Banded& h, cudaStream_t st) {
    const size_t G = h.cG, W = h.cWg;
    if (!h.c_L32) {
        dalloc(&h.c_L32, W * std::max(h.cL, 1) * G, sizeof(zf));
        dalloc(&h.c_U32, W * std::max(h.cU, 1) * G, sizeof(zf));
        dalloc(&h.c_V32, W * std::max(h.cV, 1) * G, sizeof(zf));
    }
    auto dem = [&](const void* a, zf* b, long long c) {
        k_demote_n<<<(int)std::min<long long>((c + 255) / 256, 152LL * 32), 256, 0, st>>>(static_cast<const zd*>(a), b, c);
        CNG_LAUNCH("k_demote_n");
    };
    dem(h.c_L, h.c_L32, (long long)(W * std::max(h.cL, 1) * G));
    dem(h.c_U, h.c_U32, (long long)(W * std::max(h.cU, 1) * G));
    dem(h.c_V, h.c_V32, (long long)(W * std::max(h.cV, 1) * G));
}

// rows of the windowed sweeps' ring: a power of two >= chunk + kl + ku + 1 (every row a chunk of
// columns touches, with the next chunk's rows)
static int window_slots(const Banded& h, int chunk) {
    int p = 1;
    while (p < chunk + h.kl + h.ku + 1) p <<= 1;
    return p;
}

static CompactIdx compact_idx(const Banded& h, int chunk = kCChunk) {
    CompactIdx ix;
    ix.n = h.n; ix.r = h.r; ix.kl = h.kl; ix.kv = h.kl + h.ku; ix.nL = h.cL; ix.nU = h.cU; ix.nV = h.cV;
    ix.wgroups = h.cWg; ix.batch = h.batch; ix.gs = h.cG; ix.wg0 = 0;
    ix.maxLc = h.cMaxLk[chunk_index(chunk)];
    ix.maxUc = h.cMaxUk[chunk_index(chunk)];
    ix.maxLcol = h.cMaxLcol;
    ix.maxUcol = h.cMaxUcol;
    ix.offL = h.c_offL; ix.Lrow = h.c_Lrow; ix.Lmask = h.c_Lmask; ix.offU = h.c_offU; ix.Udist = h.c_Udist;
    ix.offV = h.c_offV; ix.Vcol = h.c_Vcol;
    ix.wmask = window_slots(h, chunk) - 1;
    ix.scratch = h.w_scr;
    return ix;
}

static void compact(Banded& h, cudaStream_t st) {
    if (h.dtype != 1) throw InvalidArgument("the compact solve is built for complex128 buckets");
    const int n = h.n, kv = h.kl + h.ku, r = h.r;
    if (kv > 255 || h.kl > 31) throw InvalidArgument("compact solve: band too wide (kl <= 31, kl + ku <= 255)");
    // 1. union masks over the batch
    std::vector<unsigned char> mab((size_t)n * h.ldab), mvt((size_t)std::max(1, r) * n);
    unsigned char* dm = nullptr;
    dalloc(&dm, std::max(mab.size(), mvt.size()), 1);
    try {
        const long long cnt = (long long)n * h.ldab;
        k_union_mask<zd><<<ceil_div(cnt, 256), 256, 0, st>>>(static_cast<const zd*>(h.ab), cnt, h.batch, cnt, dm);
        CNG_LAUNCH("k_union_mask");
        CNG_CUDA(cudaMemcpyAsync(mab.data(), dm, mab.size(), cudaMemcpyDeviceToHost, st));
        if (r > 0) {
            const long long c2 = (long long)r * n;
            CNG_CUDA(cudaStreamSynchronize(st));
            k_union_mask<zd><<<ceil_div(c2, 256), 256, 0, st>>>(static_cast<const zd*>(h.vt), c2, h.batch, c2, dm);
            CNG_LAUNCH("k_union_mask");
            CNG_CUDA(cudaMemcpyAsync(mvt.data(), dm, (size_t)r * n, cudaMemcpyDeviceToHost, st));
        }
        CNG_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        cudaFree(dm);
        throw;
    }
    cudaFree(dm);
    // 2. index lists
    std::vector<int> offL(n + 1, 0), offU(n + 1, 0), offV(r + 1, 0), Vcol;
    std::vector<unsigned char> Lrow, Udist;
    std::vector<unsigned> Lmask(n, 0u);
    for (int j = 0; j < n; ++j) {
        if (j < n - 1) {
            const int lm = std::min(h.kl, n - 1 - j);
            for (int t = 0; t < lm; ++t)
                if (mab[(size_t)j * h.ldab + kv + 1 + t]) {
                    Lrow.push_back((unsigned char)t);
                    Lmask[j] |= 1u << t;
                }
        }
        offL[j + 1] = (int)Lrow.size();
    }
    for (int s2 = 0; s2 < n; ++s2) {
        const int j = n - 1 - s2;
        Udist.push_back(0);                                  // 1 / u_jj
        for (int d = 1; d <= std::min(kv, j); ++d)
            if (mab[(size_t)j * h.ldab + kv - d]) Udist.push_back((unsigned char)d);
        offU[s2 + 1] = (int)Udist.size();
    }
    for (int a = 0; a < r; ++a) {
        for (int i = 0; i < n; ++i)
            if (mvt[(size_t)a * n + i]) Vcol.push_back(i);
        offV[a + 1] = (int)Vcol.size();
    }
    for (int k = 0; k < 4; ++k) {
        const int ch = kChunkSizes[k];
        int ml = 1, mu = 1;
        for (int j0 = 0; j0 < n - 1; j0 += ch) ml = std::max(ml, offL[std::min(j0 + ch, n - 1)] - offL[j0]);
        for (int s0 = 0; s0 < n; s0 += ch) mu = std::max(mu, offU[std::min(s0 + ch, n)] - offU[s0]);
        h.cMaxLk[k] = ml;
        h.cMaxUk[k] = mu;
    }
    h.cMaxLcol = h.cMaxUcol = 0;
    for (int j = 0; j + 1 < n; ++j) h.cMaxLcol = std::max(h.cMaxLcol, offL[j + 1] - offL[j]);
    for (int s2 = 0; s2 < n; ++s2) h.cMaxUcol = std::max(h.cMaxUcol, offU[s2 + 1] - offU[s2]);
    // the partitioned solve stages each block's streams in chunks of kPartCH columns from the
    // block's first column (forward) or from its last (backward): the largest such chunk
    h.p_maxLc = h.p_maxUc = 1;
    for (int c0 = 0; c0 < n - 1; c0 += kPartM) {
        const int c1 = std::min(c0 + kPartM, n - 1);
        for (int j0 = c0; j0 < c1; j0 += kPartCH)
            h.p_maxLc = std::max(h.p_maxLc, offL[std::min(j0 + kPartCH, c1)] - offL[j0]);
    }
    for (int c0 = 0; c0 < n; c0 += kPartM) {
        const int c1 = std::min(c0 + kPartM, n), sb = n - c1, se = n - c0;
        for (int s0 = sb; s0 < se; s0 += kPartCH)
            h.p_maxUc = std::max(h.p_maxUc, offU[std::min(s0 + kPartCH, se)] - offU[s0]);
    }
    // responses of an earlier factor set are stale
    dev_free(h.p_Rf);
    dev_free(h.p_Rb);
    h.p_Rf = h.p_Rb = nullptr;
    h.part_ready = false;
    h.cL = (int)Lrow.size();
    h.cU = (int)Udist.size();
    h.cV = (int)Vcol.size();
    h.cG = h.shared ? 1 : kGroup;
    h.cWg = (h.batch + h.cG - 1) / h.cG;
    auto up = [&](auto** d, const auto& v) {
        using E = std::remove_reference_t<decltype(v[0])>;
        dalloc(d, std::max<size_t>(v.size(), 1), sizeof(E));
        if (!v.empty()) CNG_CUDA(cudaMemcpyAsync(*d, v.data(), sizeof(E) * v.size(), cudaMemcpyHostToDevice, st));
    };
    if (!h.c_offL) {
        up(&h.c_offL, offL); up(&h.c_Lrow, Lrow); up(&h.c_Lmask, Lmask); up(&h.c_offU, offU);
        up(&h.c_Udist, Udist); up(&h.c_offV, offV); up(&h.c_Vcol, Vcol);
        const size_t G = h.cG, W = h.cWg;
        dalloc(&h.c_L, W * std::max(h.cL, 1) * G, sizeof(zd));
        dalloc(&h.c_U, W * std::max(h.cU, 1) * G, sizeof(zd));
        dalloc(&h.c_V, W * std::max(h.cV, 1) * G, sizeof(zd));
        dalloc(&h.c_piv, W * n * G, sizeof(int));
    } else {
        // refactorization: the pattern of the new factors must fit the stored union
        throw InvalidArgument("compact(): already built; refactor into a new handle");
    }
    CNG_CUDA(cudaStreamSynchronize(st));
    // 3. pack
    const int total = h.cWg * h.cG;
    k_pack_compact<zd><<<ceil_div(total, 4), 128, 0, st>>>(h.view<zd>(), compact_idx(h), static_cast<zd*>(h.c_L),
                                                           static_cast<zd*>(h.c_U), static_cast<zd*>(h.c_V), h.c_piv, total);
    CNG_LAUNCH("k_pack_compact");
    if (h.fp32_ready) demote_compact(h, st);
    CNG_CUDA(cudaStreamSynchronize(st));
    h.compact_ready = true;
}

template <class TF>
static size_t compact_smem(const Banded& h, int nwarps, int sched = 0) {
    const CompactSchedule sc = kSchedules[sched];
    const int k = chunk_index(sc.chunk);
    size_t off = (size_t)(h.n + 1) * 8 + (size_t)h.n * 4 + h.cL + h.cU;
    off = (off + 15) & ~(size_t)15;
    const size_t ring = (size_t)sc.stages * (size_t)(h.cMaxLk[k] + h.cMaxUk[k]) * h.cG;
    const size_t pivots = ((size_t)sc.stages * sc.chunk * h.cG * sizeof(int) + sizeof(TF) - 1) / sizeof(TF);
    // the windowed schedules: a window of each vector, z and S in the ring after the sweeps; with
    // 8 lanes per system four windows and two warp groups' rings
    if (sc.split == kWindowFlag) {
        const size_t ns = 32 / sc.lanes, nh = ns / kGroup, pad = (sc.lanes == 16 ? 64 : 32) / sizeof(TF);
        return off + sizeof(TF) * nwarps *
                         (ns * window_slots(h, sc.chunk) + (ns - 1) * pad +
                          nh * (std::max(ring, (size_t)kGroup * 64) + pivots));
    }
    const size_t per_warp = (size_t)kGroup * (h.n + 64) + ring + pivots;
    return off + sizeof(TF) * per_warp * nwarps;
}

// entries of the windowed schedules' scratch for handle h
static size_t window_scratch_entries(const Banded& h) { return (size_t)h.cWg * kGroup * h.n; }

template <class TF, class TD, int IO>
static void launch_compact(const Banded& h, const CompactData<TF>& cd, const SolveIo& io, cudaStream_t st) {
    ensure_smem_attr((const void*)k_solve_compact<TF, TD, IO>, 220 * 1024);
    int nw = 8;
    while (nw > 1 && compact_smem<TF>(h, nw) > 220 * 1024) --nw;
    nw = std::min(nw, std::max(1, ceil_div(h.cWg, sm_count())));
    const size_t smem = compact_smem<TF>(h, nw);
    if (smem > 220 * 1024) throw InvalidArgument("compact solve: system too large for shared memory");
    k_solve_compact<TF, TD, IO><<<ceil_div(h.cWg, nw), 32 * nw, smem, st>>>(compact_idx(h), cd, io);
    CNG_LAUNCH("k_solve_compact");
}

static bool launch_solve_compact(const Banded& h, int io_kind, const SolveIo& io, cudaStream_t st) {
    if (h.dtype != 1) return false;
    if (io_kind == IO_MIXED) {
        if (!h.fp32_ready) throw InvalidArgument("call cng_banded_make_fp32 first");
        CompactData<zf> cd{h.c_L32, h.c_U32, h.c_piv, h.c_V32, h.w32, h.slu32, h.spiv, h.perm};
        launch_compact<zf, zd, IO_MIXED>(h, cd, io, st);
        return true;
    }
    CompactData<zd> cd{static_cast<const zd*>(h.c_L), static_cast<const zd*>(h.c_U), h.c_piv,
                       static_cast<const zd*>(h.c_V), static_cast<const zd*>(h.w), static_cast<const zd*>(h.slu),
                       h.spiv, h.perm};
    if (io_kind == IO_PLAIN) launch_compact<zd, zd, IO_PLAIN>(h, cd, io, st);
    else if (io_kind == IO_MAPPED) launch_compact<zd, zd, IO_MAPPED>(h, cd, io, st);
    else launch_compact<zd, zd, IO_SPLIT>(h, cd, io, st);
    return true;
}

}  // namespace cng

namespace cng {

// ---- the partitioned solve: arguments, responses, launch
static PartArgs part_args(const Banded& h, const SolveIo& io) {
    PartArgs pa{};
    pa.ix = compact_idx(h, kPartCH);
    pa.cd = CompactData<zd>{static_cast<const zd*>(h.c_L), static_cast<const zd*>(h.c_U), h.c_piv,
                            static_cast<const zd*>(h.c_V), static_cast<const zd*>(h.w),
                            static_cast<const zd*>(h.slu), h.spiv, h.perm, h.flip_r, h.flip_c};
    pa.io = io;
    pa.Rf = static_cast<const zd*>(h.p_Rf);
    pa.Rb = static_cast<const zd*>(h.p_Rb);
    pa.nbf = h.p_nbf;
    pa.nbb = h.p_nbb;
    pa.kwf = h.p_kwf;
    pa.kwb = h.p_kwb;
    pa.maxLc = h.p_maxLc;
    pa.maxUc = h.p_maxUc;
    return pa;
}

// unrolled column passes: 1 or 2 where every column fits 16 or 32 entry slots, 0 (a loop) else
static int part_passes(int maxcol) { return maxcol <= 16 ? 1 : (maxcol <= 32 ? 2 : 0); }

template <class F>
static void part_dispatch(int npf, int npb, F&& f) {
    auto b = [&](auto pf) {
        if (npb == 1) f(pf, std::integral_constant<int, 1>{});
        else if (npb == 2) f(pf, std::integral_constant<int, 2>{});
        else f(pf, std::integral_constant<int, 0>{});
    };
    if (npf == 1) b(std::integral_constant<int, 1>{});
    else if (npf == 2) b(std::integral_constant<int, 2>{});
    else b(std::integral_constant<int, 0>{});
}

// The responses of every block of every system (once per factor set; the legacy stream, waited
// for). Refused where the partitioned solve does not apply or would hold too much memory: shared
// pairs, kl > 16, kl + ku > 32, n > 1024, or more than 256 MB of responses (it is meant for the
// small batches whose sweeps one warp per system leaves latency-bound).
static void build_part(Banded& h) {
    if (h.part_ready) return;
    if (!h.compact_ready || h.dtype != 1) throw InvalidArgument("the partitioned solve needs a compact complex128 handle");
    if (h.shared) throw InvalidArgument("the partitioned solve does not solve shared pairs: a compact two-system schedule");
    const int n = h.n, kwf = h.kl, kwb = h.kl + h.ku;
    if (kwf < 1 || kwf > 16 || kwb > kPartM)
        throw InvalidArgument("partitioned solve: band outside kl <= 16, kl + ku <= 32");
    const int nbf = ceil_div(n - 1, kPartM), nbb = ceil_div(n, kPartM);
    if (n < 2 || std::max(nbf, nbb) > kPartMaxWarps) throw InvalidArgument("partitioned solve: 2 <= n <= 1024");
    const size_t ef = (size_t)h.batch * nbf * (kPartM + kwf) * kwf, eb = (size_t)h.batch * nbb * (kPartM + kwb) * kwb;
    if ((ef + eb) * sizeof(zd) > ((size_t)256 << 20))
        throw InvalidArgument("partitioned solve: a small-batch schedule (its responses would exceed 256 MB)");
    const int nw = 8;
    const size_t smem = part_index_bytes(n, h.cL, h.cU) + (size_t)nw * part_warp_elems(h.p_maxLc, h.p_maxUc) * sizeof(zd);
    if (smem > 220 * 1024) throw InvalidArgument("partitioned solve: streams too large for shared memory");
    dalloc(&h.p_Rf, ef, sizeof(zd));
    dalloc(&h.p_Rb, eb, sizeof(zd));
    h.p_nbf = nbf;
    h.p_nbb = nbb;
    h.p_kwf = kwf;
    h.p_kwb = kwb;
    const PartArgs pa = part_args(h, SolveIo{});
    const long long tasks = (long long)h.batch * ((long long)nbf * kwf + (long long)nbb * kwb);
    part_dispatch(part_passes(h.cMaxLcol), part_passes(h.cMaxUcol), [&](auto pf, auto pb) {
        constexpr int PF = decltype(pf)::value, PB = decltype(pb)::value;
        ensure_smem_attr((const void*)k_part_build<PF, PB>, 220 * 1024);
        k_part_build<PF, PB><<<ceil_div(tasks, nw), 32 * nw, smem, nullptr>>>(pa, static_cast<zd*>(h.p_Rf),
                                                                            static_cast<zd*>(h.p_Rb));
        CNG_LAUNCH("k_part_build");
    });
    CNG_CUDA(cudaStreamSynchronize(nullptr));
    h.part_ready = true;
}

static void launch_part(const std::vector<const Banded*>& hs, const std::vector<SolveIo>& ios,
                        const std::vector<SolveIo>& ios2, const std::vector<int>& rng, cudaStream_t st) {
    MultiPart mp{};
    mp.nb = (int)hs.size();
    int nw = 2, npf = 1, npb = 1, blocks = 0;
    size_t smem = 0;
    for (size_t i = 0; i < hs.size(); ++i) {
        const Banded& h = *hs[i];
        if (!h.part_ready) throw InvalidArgument("the partitioned solve's responses are not built (cng_banded_set_schedule)");
        if (rng[2 * i + 1] >= 0) throw InvalidArgument("the partitioned solve solves whole batches (no system range)");
        if (ios2[i].rhs) throw InvalidArgument("the partitioned solve does not solve shared pairs");
        nw = std::max(nw, std::max(h.p_nbf, h.p_nbb));
        const int pf = part_passes(h.cMaxLcol), pb = part_passes(h.cMaxUcol);
        npf = (pf == 0 || npf == 0) ? 0 : std::max(npf, pf);
        npb = (pb == 0 || npb == 0) ? 0 : std::max(npb, pb);
    }
    for (size_t i = 0; i < hs.size(); ++i) {
        const Banded& h = *hs[i];
        mp.block_start[i] = blocks;
        mp.a[i] = part_args(h, ios[i]);
        blocks += h.batch;
        const size_t vec = (size_t)h.n + 64 + (size_t)(h.p_nbf + 1) * h.p_kwf + (size_t)(h.p_nbb + 1) * h.p_kwb;
        smem = std::max(smem, part_index_bytes(h.n, h.cL, h.cU) +
                                  (vec + (size_t)nw * part_warp_elems(h.p_maxLc, h.p_maxUc)) * sizeof(zd));
    }
    mp.block_start[mp.nb] = blocks;
    if (smem > 220 * 1024) throw InvalidArgument("partitioned solve: streams too large for shared memory");
    part_dispatch(npf, npb, [&](auto pf, auto pb) {
        constexpr int PF = decltype(pf)::value, PB = decltype(pb)::value;
        ensure_smem_attr((const void*)k_solve_part<PF, PB>, 220 * 1024);
        k_solve_part<PF, PB><<<blocks, 32 * nw, smem, st>>>(mp);
        CNG_LAUNCH("k_solve_part");
    });
}

// warp groups [first, end) of handle h that solve systems [s0, s1) (s1 < 0: all)
static void group_range(const Banded& h, int s0, int s1, int& first, int& end) {
    if (s1 < 0) { first = 0; end = h.cWg; return; }
    first = s0 / h.cG;
    end = std::min(h.cWg, (s1 + h.cG - 1) / h.cG);
}

template <class TF, class TD, int IO, int CH, int ST, bool WIN = false, int LP = kLanesPer>
static void launch_multi_t(const std::vector<const Banded*>& hs, const std::vector<CompactData<TF>>& cds,
                           const std::vector<SolveIo>& ios, const std::vector<SolveIo>& ios2,
                           const std::vector<int>& rng, int sched, cudaStream_t st) {
    // the two-systems sweeps, over whole vectors or (WIN) windows of them, LP lanes per system
    // (8: a warp sweeps two warp groups)
    constexpr int NH = 32 / LP / kGroup;
    auto kern = [] {
        if constexpr (WIN) return k_solve_window_multi<TF, TD, IO, CH, ST, LP>;
        else return k_solve_compact_multi<TF, TD, IO, CH, ST>;
    }();
    if (WIN)
        for (const Banded* h : hs)
            if (!h->w_scr || h->w_cap < window_scratch_entries(*h))
                throw InvalidArgument("windowed solve: the scratch is not allocated (cng_banded_set_schedule "
                                      "after cng_banded_compact)");
    ensure_smem_attr((const void*)kern, 220 * 1024);
    // one warp count for all blocks: the one that keeps the most warps resident per SM (blocks per
    // SM are bounded by their shared memory: eight warps in one block can lose to seven in two),
    // and no more than it takes to give every SM a block (a small batch spreads over the SMs: each
    // SM's FP64 pipe and shared memory serve fewer sweeps)
    auto smem_of = [&](int w) {
        size_t m = 0;
        for (const Banded* h : hs) m = std::max(m, compact_smem<TF>(*h, w, sched));
        return m;
    };
    std::vector<int> first(hs.size()), end(hs.size());
    int total = 0;                                   // warps
    for (size_t i = 0; i < hs.size(); ++i) {
        group_range(*hs[i], rng[2 * i], rng[2 * i + 1], first[i], end[i]);
        total += ceil_div(end[i] - first[i], NH);
    }
    int nw = 1, resident = 0;
    for (int w = 1; w <= (WIN ? window_max_warps<TF>() : 8); ++w) {
        const size_t m = smem_of(w);
        if (m > 220 * 1024) break;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * w, m) != cudaSuccess)
            per_sm = 1;
        if (per_sm * w >= resident) { resident = per_sm * w; nw = w; }
    }
    nw = std::min(nw, std::max(1, ceil_div(total, sm_count())));
    size_t smem = 0;
    for (const Banded* h : hs) smem = std::max(smem, compact_smem<TF>(*h, nw, sched));
    if (smem > 220 * 1024) throw InvalidArgument("compact solve: system too large for shared memory");
    MultiSolve<TF> ms{};
    ms.nb = (int)hs.size();
    // largest buckets first: their long tails start earliest
    std::vector<int> order(hs.size());
    for (size_t i = 0; i < hs.size(); ++i) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return end[a] - first[a] > end[b] - first[b]; });
    int blocks = 0;
    for (int k = 0; k < ms.nb; ++k) {
        const int i = order[k];
        ms.block_start[k] = blocks;
        ms.ix[k] = compact_idx(*hs[i], CH);
        ms.ix[k].wg0 = first[i];
        ms.ix[k].wgroups = end[i];
        ms.cd[k] = cds[i];
        ms.io[k] = ios[i];
        ms.io2[k] = ios2[i];
        blocks += ceil_div(ceil_div(end[i] - first[i], NH), nw);
    }
    ms.block_start[ms.nb] = blocks;
    kern<<<blocks, 32 * nw, smem, st>>>(ms);
    CNG_LAUNCH(WIN ? "k_solve_window_multi" : "k_solve_compact_multi");
}

template <class TF>
static size_t split_smem(const Banded& h, int nwarps, int sched) {
    const CompactSchedule sc = kSchedules[sched];
    const int k = chunk_index(sc.chunk);
    size_t off = (size_t)(h.n + 1) * 8 + (size_t)h.n * 4 + h.cL + h.cU;
    off = (off + 15) & ~(size_t)15;
    const size_t per_warp = (size_t)(h.n + 64) + (size_t)sc.stages * (size_t)(h.cMaxLk[k] + h.cMaxUk[k]) * 2 +
                            ((size_t)sc.stages * sc.chunk * 2 * sizeof(int) + sizeof(TF) - 1) / sizeof(TF);
    return off + sizeof(TF) * per_warp * nwarps;
}

template <class TF, class TD, int IO, int CH, int ST>
static void launch_split_t(const std::vector<const Banded*>& hs, const std::vector<CompactData<TF>>& cds,
                           const std::vector<SolveIo>& ios, const std::vector<SolveIo>&,
                           const std::vector<int>& rng, int sched, cudaStream_t st) {
    for (const Banded* h : hs)
        if (h->cG != kGroup)
            throw InvalidArgument("the split-lane schedules do not solve shared pairs: a compact two-system schedule");
    ensure_smem_attr((const void*)k_solve_split_multi<TF, TD, IO, CH, ST>, 220 * 1024);
    // warps per block as launch_multi_t: the most resident warps per SM, and a block for every SM
    // when the batch is small
    auto smem_of = [&](int w) {
        size_t m = 0;
        for (const Banded* h : hs) m = std::max(m, split_smem<TF>(*h, w, sched));
        return m;
    };
    std::vector<int> first(hs.size()), end(hs.size());
    int total = 0;
    for (size_t i = 0; i < hs.size(); ++i) {
        first[i] = rng[2 * i + 1] < 0 ? 0 : rng[2 * i];
        end[i] = rng[2 * i + 1] < 0 ? hs[i]->batch : rng[2 * i + 1];
        total += end[i] - first[i];
    }
    int nw = 1, resident = 0;
    for (int w = 1; w <= 8; ++w) {
        const size_t m = smem_of(w);
        if (m > 220 * 1024) break;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_split_multi<TF, TD, IO, CH, ST>, 32 * w,
                                                          m) != cudaSuccess)
            per_sm = 1;
        if (per_sm * w >= resident) { resident = per_sm * w; nw = w; }
    }
    nw = std::min(nw, std::max(1, ceil_div(total, sm_count())));
    const size_t smem = smem_of(nw);
    if (smem > 220 * 1024) throw InvalidArgument("compact solve: system too large for shared memory");
    MultiSolve<TF> ms{};
    ms.nb = (int)hs.size();
    std::vector<int> order(hs.size());
    for (size_t i = 0; i < hs.size(); ++i) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return end[a] - first[a] > end[b] - first[b]; });
    int blocks = 0;
    for (int k = 0; k < ms.nb; ++k) {
        const int i = order[k];
        ms.block_start[k] = blocks;
        ms.ix[k] = compact_idx(*hs[i], CH);
        ms.ix[k].wg0 = first[i];              // in systems: one system per warp
        ms.ix[k].wgroups = end[i];
        ms.cd[k] = cds[i];
        ms.io[k] = ios[i];
        blocks += ceil_div(end[i] - first[i], nw);
    }
    ms.block_start[ms.nb] = blocks;
    k_solve_split_multi<TF, TD, IO, CH, ST><<<blocks, 32 * nw, smem, st>>>(ms);
    CNG_LAUNCH("k_solve_split_multi");
}

// the schedule of the handles (the autotuner sets one for all the buckets of a step; the default
// when they differ)
template <class TF, class TD, int IO>
static void launch_multi(const std::vector<const Banded*>& hs, const std::vector<CompactData<TF>>& cds,
                         const std::vector<SolveIo>& ios, const std::vector<SolveIo>& ios2, const std::vector<int>& rng,
                         cudaStream_t st) {
    int sched = hs[0]->sched;
    for (const Banded* h : hs)
        if (h->sched != sched) sched = 0;
    if (sched < 0 || sched >= kNumSchedules) sched = 0;
    switch (sched) {
        case 1: launch_multi_t<TF, TD, IO, 8, 3>(hs, cds, ios, ios2, rng, sched, st); break;
        case 2: launch_multi_t<TF, TD, IO, 4, 3>(hs, cds, ios, ios2, rng, sched, st); break;
        case 3: launch_multi_t<TF, TD, IO, 16, 2>(hs, cds, ios, ios2, rng, sched, st); break;
        case 4: launch_multi_t<TF, TD, IO, 16, 3>(hs, cds, ios, ios2, rng, sched, st); break;
        case 5: launch_multi_t<TF, TD, IO, 4, 4>(hs, cds, ios, ios2, rng, sched, st); break;
        case 6: launch_multi_t<TF, TD, IO, 2, 4>(hs, cds, ios, ios2, rng, sched, st); break;
        case 7: launch_multi_t<TF, TD, IO, 16, 4>(hs, cds, ios, ios2, rng, sched, st); break;
        case 8: launch_split_t<TF, TD, IO, 8, 2>(hs, cds, ios, ios2, rng, sched, st); break;
        case 9: launch_split_t<TF, TD, IO, 16, 2>(hs, cds, ios, ios2, rng, sched, st); break;
        case 10: launch_split_t<TF, TD, IO, 4, 3>(hs, cds, ios, ios2, rng, sched, st); break;
        case kPartSchedule:
            if constexpr (std::is_same<TF, zd>::value) launch_part(hs, ios, ios2, rng, st);
            else throw InvalidArgument("the partitioned solve is FP64 only: another schedule for the FP32 form");
            break;
        case 12: launch_multi_t<TF, TD, IO, 8, 2, true>(hs, cds, ios, ios2, rng, sched, st); break;
        case 13: launch_multi_t<TF, TD, IO, 4, 3, true>(hs, cds, ios, ios2, rng, sched, st); break;
        case 14: launch_multi_t<TF, TD, IO, 16, 2, true>(hs, cds, ios, ios2, rng, sched, st); break;
        case 15: launch_multi_t<TF, TD, IO, 8, 3, true>(hs, cds, ios, ios2, rng, sched, st); break;
        case 16: launch_multi_t<TF, TD, IO, 8, 2, true, 8>(hs, cds, ios, ios2, rng, sched, st); break;
        case 17: launch_multi_t<TF, TD, IO, 4, 3, true, 8>(hs, cds, ios, ios2, rng, sched, st); break;
        case 18: launch_multi_t<TF, TD, IO, 8, 3, true, 8>(hs, cds, ios, ios2, rng, sched, st); break;
        default: launch_multi_t<TF, TD, IO, 8, 2>(hs, cds, ios, ios2, rng, sched, st); break;
    }
}

}  // namespace cng

extern "C" {

int cng_banded_solve_batch2(int nh, cng_banded* const* hh, const void* const* b, void* const* x,
                            const void* const* b2, void* const* x2, void* const* xt, void* const* xt2,
                            const int32_t* range, int fp32, int accumulate, void* stream) {
    CNG_TRY({
        if (nh < 1 || nh > kMaxMulti) throw InvalidArgument("1 to 8 handles per batched solve");
        if (!hh || !b || !x) throw InvalidArgument("null argument");
        if ((xt || xt2) && !fp32) throw InvalidArgument("the row-major copy of x is written by the FP32 solve only");
        std::vector<const Banded*> hs;
        std::vector<SolveIo> ios, ios2;
        std::vector<int> rng(2 * nh, -1);
        bool any_pair = false, any_range = false;
        for (int k = 0; k < nh; ++k) {
            const Banded* h = reinterpret_cast<const Banded*>(hh[k]);
            if (!h || !h->compact_ready || h->dtype != 1)
                throw InvalidArgument("batched solve needs complex128 handles in compact form");
            if (range && !(range[2 * k] == 0 && range[2 * k + 1] == h->batch)) {
                const int s0 = range[2 * k], s1 = range[2 * k + 1];
                if (s0 < 0 || s1 <= s0 || s1 > h->batch || s0 % h->cG || (s1 % h->cG && s1 != h->batch))
                    throw InvalidArgument("system range: 0 <= s0 < s1 <= batch, on warp-group boundaries");
                rng[2 * k] = s0;
                rng[2 * k + 1] = s1;
                any_range = true;
            }
            if (fp32 && !h->fp32_ready) throw InvalidArgument("call cng_banded_make_fp32 first");
            if (!b[k] || !x[k] || b[k] == x[k]) throw InvalidArgument("b and x: device pointers, not aliased");
            const void* pb = b2 ? b2[k] : nullptr;
            void* px = x2 ? x2[k] : nullptr;
            if ((pb == nullptr) != (px == nullptr))
                throw InvalidArgument("a partner right-hand side needs its solution and the converse");
            if (pb) {
                if (!h->shared) throw InvalidArgument("a partner solve needs a handle shared with cng_banded_share");
                if (pb == px || px == x[k] || pb == x[k] || px == b[k])
                    throw InvalidArgument("partner b and x: device pointers, not aliased with each other or b, x");
                any_pair = true;
            }
            if (xt && xt[k] && (xt[k] == x[k] || xt[k] == b[k])) throw InvalidArgument("xt aliases b or x");
            hs.push_back(h);
            SolveIo io{b[k], x[k], nullptr, nullptr, nullptr, nullptr, accumulate};
            io.xT = xt ? xt[k] : nullptr;
            ios.push_back(io);
            SolveIo io2{pb, px, nullptr, nullptr, nullptr, nullptr, accumulate};
            io2.xT = (pb && xt2) ? xt2[k] : nullptr;
            ios2.push_back(io2);
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        bool dense = true;
        for (const Banded* h : hs) dense = dense && h->sched < 0;
        if (dense) {              // the band kernel, one launch per bucket
            if (any_pair) throw InvalidArgument("the band kernel does not solve shared pairs: a compact schedule");
            if (any_range) throw InvalidArgument("the band kernel solves whole batches (no system range)");
            if (xt) throw InvalidArgument("the transposed copy of x: compact schedules only");
            for (size_t k = 0; k < hs.size(); ++k) {
                if (fp32) launch_mixed_dense(*hs[k], b[k], x[k], accumulate, st);
                else launch_solve(*hs[k], IO_MAPPED, ios[k], st);
            }
            return CNG_OK;
        }
        if (fp32) {
            std::vector<CompactData<zf>> cds;
            for (const Banded* h : hs)
                cds.push_back(CompactData<zf>{h->c_L32, h->c_U32, h->c_piv, h->c_V32, h->w32, h->slu32, h->spiv, h->perm,
                                              h->flip_r, h->flip_c});
            launch_multi<zf, zd, IO_MIXED>(hs, cds, ios, ios2, rng, st);
        } else {
            std::vector<CompactData<zd>> cds;
            for (const Banded* h : hs)
                cds.push_back(CompactData<zd>{static_cast<const zd*>(h->c_L), static_cast<const zd*>(h->c_U), h->c_piv,
                                              static_cast<const zd*>(h->c_V), static_cast<const zd*>(h->w),
                                              static_cast<const zd*>(h->slu), h->spiv, h->perm, h->flip_r, h->flip_c});
            launch_multi<zd, zd, IO_MAPPED>(hs, cds, ios, ios2, rng, st);
        }
    })
}

int cng_banded_solve_batch(int nh, cng_banded* const* hh, const void* const* b, void* const* x, int fp32,
                           int accumulate, void* stream) {
    return cng_banded_solve_batch2(nh, hh, b, x, nullptr, nullptr, nullptr, nullptr, nullptr, fp32, accumulate, stream);
}

int cng_banded_solve_batch_xt(int nh, cng_banded* const* hh, const void* const* b, void* const* x,
                              void* const* xt, int accumulate, void* stream) {
    if (!xt) {
        cng::set_error("null argument");
        return cng::CNG_EINVAL;
    }
    return cng_banded_solve_batch2(nh, hh, b, x, nullptr, nullptr, xt, nullptr, nullptr, 1, accumulate, stream);
}

int cng_banded_share(cng_banded* hh, const int8_t* dr, const int8_t* dc, void* stream) {
    CNG_TRY({
        cng::Banded* h = reinterpret_cast<cng::Banded*>(hh);
        if (!h || !dr || !dc) throw InvalidArgument("null argument");
        if (h->dtype != 1) throw InvalidArgument("shared factors: complex128 handles");
        if (h->compact_ready) throw InvalidArgument("cng_banded_share must come before cng_banded_compact");
        const int n = h->n;
        std::vector<unsigned char> fr(n), fc(n);
        for (int i = 0; i < n; ++i) {
            if ((dr[i] != 1 && dr[i] != -1) || (dc[i] != 1 && dc[i] != -1))
                throw InvalidArgument("sign vectors hold +1 or -1");
            fr[i] = dr[i] < 0;
            fc[i] = dc[i] < 0;
        }
        // the band part of the partner is the sign flip of this one only if every border row keeps
        // the sign of its s e_i (dr_i dc_i = +1 at the border positions)
        for (int k = 0; k < h->r; ++k)
            if (dr[h->perm_host[k]] * dc[k] != 1)
                throw InvalidArgument("shared factors: a border row changes the sign of its diagonal");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (!h->flip_r) {
            dalloc(&h->flip_r, n, 1);
            dalloc(&h->flip_c, n, 1);
        }
        CNG_CUDA(cudaMemcpyAsync(h->flip_r, fr.data(), n, cudaMemcpyHostToDevice, st));
        CNG_CUDA(cudaMemcpyAsync(h->flip_c, fc.data(), n, cudaMemcpyHostToDevice, st));
        CNG_CUDA(cudaStreamSynchronize(st));
        h->shared = true;
    })
}

int cng_banded_compact(cng_banded* hh, void* stream) {
    CNG_TRY({ cng::compact(*reinterpret_cast<cng::Banded*>(hh), static_cast<cudaStream_t>(stream)); })
}

int cng_banded_schedules(int32_t* count, int32_t* chunk, int32_t* stages, int32_t* split) {
    CNG_TRY({
        if (!count) throw InvalidArgument("null argument");
        *count = kNumSchedules;
        for (int k = 0; k < kNumSchedules; ++k) {
            if (chunk) chunk[k] = kSchedules[k].chunk;
            if (stages) stages[k] = kSchedules[k].stages;
            if (split) split[k] = kSchedules[k].split;
        }
    })
}

int cng_banded_set_schedule(cng_banded* hh, int sched) {
    CNG_TRY({
        cng::Banded* h = reinterpret_cast<cng::Banded*>(hh);
        if (!h) throw InvalidArgument("null handle");
        if (sched < -1 || sched >= kNumSchedules) throw InvalidArgument("schedule out of range");
        if (sched >= 0 && !h->compact_ready) throw InvalidArgument("compact schedules need cng_banded_compact first");
        if (sched == cng::kPartSchedule) {
            cng::build_part(*h);                   // the responses (refused where it does not apply)
        } else if (h->part_ready) {                // another schedule: the responses are not kept
            dev_free(h->p_Rf);
            dev_free(h->p_Rb);
            h->p_Rf = h->p_Rb = nullptr;
            h->part_ready = false;
        }
        if (sched >= 0 && cng::kSchedules[sched].split == cng::kWindowFlag) {
            const size_t need = cng::window_scratch_entries(*h);     // the windowed sweeps' scratch
            if (h->w_cap < need) {
                dev_free(h->w_scr);
                h->w_scr = nullptr;
                h->w_cap = 0;
                dalloc(&h->w_scr, need, sizeof(zd));
                h->w_cap = need;
            }
        } else if (h->w_scr) {                     // another schedule: the scratch is not kept
            dev_free(h->w_scr);
            h->w_scr = nullptr;
            h->w_cap = 0;
        }
        h->sched = sched;
    })
}

}  // extern "C"
