// Pseudospectral explicit right-hand side F(X) on the mode layout, and the transform kernels.
//
// F is the reference's polynomial form (python/conatus/timestep/fused.py:524-537):
// out_o = sum_m c_m prod_j f_j over the 3/2-dealiased grid, f_j = derivatives of state components,
// then projected back (truncation) and converted to each equation's C^(lambda) rows
// (system.py:910-931). Pipeline for Fourier (x[, z]) x Chebyshev (y):
//
//   unpack   state (mode layout) -> factor spectra S[f][jx][jz][n]: complex-view amplitudes scaled
//            to FFT coefficients (1, 1/2, 1/4 for 0, 1, 2 nonzero Fourier indices), Fourier
//            derivatives (i k)^o, Chebyshev derivative by the backward recurrence (as a suffix scan)
//   cheb_bwd Chebyshev N -> My Gauss points along y (DCT-III by Makhoul's length-My FFT)
//   fft_z    complex inverse FFT along z (compact fftfreq spectrum -> Mz points)     [2 directions]
//   irfft_x  Hermitian half spectrum -> Mx real points along x (two columns per complex FFT)
//   products out_o(x, z, y)
//   rfft_x, fft_z (forward, truncation = dealias projection), cheb_fwd (DCT-II, My -> N)
//   pack     rows: 2^d_act * C^(lambda) conversion of the output coefficients + constant part F(0)
//
// The Chebyshev grid My is any even size >= the reference's floor(3N/2): Gauss quadrature on My
// points is exact for the degree of the dealiased products, so the projected coefficients are the
// reference's (to rounding) and My can be FFT-friendly (193 -> 200 for N = 129).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "conatus_gb300.h"
#include "fft.cuh"

namespace cng {

static constexpr int kFftThreads = 256;
static constexpr size_t kFftSmemMax = 200 * 1024;

// Division by a divisor uniform over the kernel (sizes of the staging loops): q = e / d through
// a multiply-high with m = ceil(2^32 / d), exact for e d < 2^32 (e, d below 2^16 here); the runtime
// integer division it replaces was the largest item of the FP32 transforms' integer work.
struct FastDiv {
    unsigned d, m;
    __device__ __forceinline__ explicit FastDiv(int d_) : d((unsigned)d_), m(d_ <= 1 ? 0u : 0xFFFFFFFFu / (unsigned)d_ + 1u) {}
    __device__ __forceinline__ int div(int e) const { return d <= 1 ? e : (int)__umulhi((unsigned)e, m); }
};

FftPlan make_plan(int L) {
    FftPlan p;
    p.L = L;
    p.nstages = 0;
    int r = L;
    const int order[] = {8, 4, 2, 3, 5};
    for (int rad : order) {
        while (r % rad == 0) {
            if (p.nstages >= 12) throw InvalidArgument("FFT length has too many factors");
            p.radix[p.nstages++] = rad;
            r /= rad;
        }
    }
    if (r != 1 || L < 1)
        throw InvalidArgument("FFT length " + std::to_string(L) + " must be 2^a 3^b 5^c");
    return p;
}

// ---- twiddle tables (host double precision, uploaded once per length and precision) ----------
// kind 0: exp(-2 pi i q / L), q < L (FFT twiddles); kind 1: exp(-i pi k / (2L)), k < L (the
// Makhoul post-twiddles of the Chebyshev transforms); kind 2: (-1)^k / 2 exp(+i pi k / (2L)) (the
// backward pre-twiddles with the sign of a_k = (-1)^k c_k and the factor 1/2 folded in: exact
// scalings, so the product is the one of the separate steps). Angles reduced in long double.
template <class R>
struct TwiddleCache {
    std::mutex mu;
    std::vector<std::pair<long long, c2<R>*>> tables;
    const c2<R>* get(int L, int kind = 0) {
        std::lock_guard<std::mutex> lock(mu);
        const long long key = (long long)L * 4 + kind;
        for (auto& t : tables)
            if (t.first == key) return t.second;
        std::vector<c2<R>> h(L);
        const long double pi = 3.14159265358979323846264338327950288L;
        for (int q = 0; q < L; ++q) {
            const long double ang = kind == 0 ? -2.0L * pi * q / L : -pi * q / (2.0L * L);
            h[q].x = static_cast<R>(cosl(ang));
            h[q].y = static_cast<R>(sinl(ang));
            if (kind == 2) {
                const R sc = (q & 1) ? R(-0.5) : R(0.5);
                h[q].x = sc * h[q].x;
                h[q].y = -sc * h[q].y;
            }
        }
        c2<R>* d = nullptr;
        CNG_CUDA(cudaMalloc(&d, sizeof(c2<R>) * L));
        CNG_CUDA(cudaMemcpy(d, h.data(), sizeof(c2<R>) * L, cudaMemcpyHostToDevice));
        tables.push_back({key, d});
        return d;
    }
};
template <class R>
TwiddleCache<R>& twiddles() {
    static TwiddleCache<R> c;
    return c;
}

// ------------------------------------------------------------------------------------------------
// Chebyshev transforms of contiguous complex columns (Makhoul; conventions of the reference's
// reference/transforms.py:117-121,158-164: Gauss nodes t_j = -cos(pi (j + 1/2) / M)).

// Arguments of one Chebyshev transform launch (a grouped launch holds one set per problem).
template <class R>
struct ChebArgs {
    const c2<R>* in;
    c2<R>* out;
    long long ncols;
    int N;
    FftPlan plan;
    int B;
    const c2<R>* tw;
    const c2<R>* tq;
};

// backward: c[0..N) -> f[0..M): f_j = sum_n c_n T_n(t_j). Block `bid` takes columns bid B ...
template <class R>
__device__ __forceinline__ void cheb_bwd_body(unsigned bid, const c2<R>* __restrict__ in, c2<R>* __restrict__ out,
                                              long long ncols, int N, const FftPlan& plan, int B,
                                              const c2<R>* __restrict__ tw_g, const c2<R>* __restrict__ tq_g) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int M = plan.L;
    c2<R>* tw = reinterpret_cast<c2<R>*>(sm);
    c2<R>* tq = tw + M;
    c2<R>* b0 = tq + M;
    c2<R>* b1 = b0 + (size_t)B * M;
    c2<R>* a = b1 + (size_t)B * M;     // staging of the coefficients (B x (M + 1))
    const int tid = threadIdx.x, nt = blockDim.x;
    const FastDiv dM(M), dM1(M + 1);
    for (int q = tid; q < M; q += nt) {
        tw[q] = tw_g[q];
        tq[q] = tq_g[q];
    }
    const long long col0 = (long long)bid * B;
    for (int e = tid; e < B * (M + 1); e += nt) {
        const int t = dM1.div(e), k = e - t * (M + 1);
        const long long col = col0 + t;
        c2<R> v = mk<R>(0, 0);
        if (col < ncols && k < N) v = in[col * N + k];     // c_k (the sign of a_k is in tq)
        a[e] = v;
    }
    __syncthreads();
    // Z_k = 1/2 e^{i pi k / (2M)} (a_k - i a_{M-k}) = tq_k (c_k - i c_{M-k}) with a_k = (-1)^k c_k
    // (M even) and tq_k = (-1)^k / 2 e^{i pi k / (2M)}; Z_0 = a_0 = c_0
    for (int e = tid; e < B * M; e += nt) {
        const int t = dM.div(e), k = e - t * M;
        const c2<R>* at = a + (size_t)t * (M + 1);
        c2<R> z;
        if (k == 0) {
            z = at[0];
        } else {
            c2<R> u = at[k], w = at[M - k];
            c2<R> d = mk<R>(u.x + w.y, u.y - w.x);     // c_k - i c_{M-k}
            z = mul<R>(tq[k], d);
        }
        b0[e] = z;
    }
    __syncthreads();
    c2<R>* r = smem_fft_fast<R>(b0, b1, plan, B, tw, +1, M);
    // f_{2j} = z_j, f_{2j+1} = z_{M-1-j}
    for (int e = tid; e < B * M; e += nt) {
        const int t = dM.div(e), j = e - t * M;
        const long long col = col0 + t;
        if (col >= ncols) continue;
        const int src = (j & 1) ? (M - 1 - (j >> 1)) : (j >> 1);
        out[col * M + j] = r[(size_t)t * M + src];
    }
}

template <class R>
__global__ void k_cheb_bwd(const c2<R>* __restrict__ in, c2<R>* __restrict__ out, long long ncols, int N,
                           FftPlan plan, int B, const c2<R>* __restrict__ tw_g,
                           const c2<R>* __restrict__ tq_g) {
    cheb_bwd_body<R>(blockIdx.x, in, out, ncols, N, plan, B, tw_g, tq_g);
}

template <class R>
__global__ void k_cheb_bwd_grp(const __grid_constant__ Grp<ChebArgs<R>> g) {
    const int k = g.find(blockIdx.x);
    const ChebArgs<R>& a = g.a[k];
    cheb_bwd_body<R>(blockIdx.x - g.start[k], a.in, a.out, a.ncols, a.N, a.plan, a.B, a.tw, a.tq);
}

// forward: f[0..M) -> c[0..N): c_k = (2/M) sum_j f_j T_k(t_j), halved at k = 0 (DCT-II / M).
template <class R>
__device__ __forceinline__ void cheb_fwd_body(unsigned bid, const c2<R>* __restrict__ in, c2<R>* __restrict__ out,
                                              long long ncols, int N, const FftPlan& plan, int B,
                                              const c2<R>* __restrict__ tw_g, const c2<R>* __restrict__ tq_g) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int M = plan.L;
    c2<R>* tw = reinterpret_cast<c2<R>*>(sm);
    c2<R>* tq = tw + M;
    c2<R>* b0 = tq + M;
    c2<R>* b1 = b0 + (size_t)B * M;
    const int tid = threadIdx.x, nt = blockDim.x;
    const FastDiv dM(M), dN(N);
    for (int q = tid; q < M; q += nt) {
        tw[q] = tw_g[q];
        tq[q] = tq_g[q];
    }
    const long long col0 = (long long)bid * B;
    // v_j = f_{2j}, v_{M-1-j} = f_{2j+1}
    for (int e = tid; e < B * M; e += nt) {
        const int t = dM.div(e), i = e - t * M;
        const long long col = col0 + t;
        c2<R> v = mk<R>(0, 0);
        if (col < ncols) v = in[col * M + i];
        const int dst = (i & 1) ? (M - 1 - (i >> 1)) : (i >> 1);
        b0[(size_t)t * M + dst] = v;
    }
    __syncthreads();
    c2<R>* Z = smem_fft_fast<R>(b0, b1, plan, B, tw, -1, M);
    const R invM = R(1) / R(M), invMh = invM * R(0.5);
    for (int e = tid; e < B * N; e += nt) {
        const int t = dN.div(e), k = e - t * N;
        const long long col = col0 + t;
        if (col >= ncols) continue;
        const c2<R>* Zt = Z + (size_t)t * M;
        c2<R> zk = Zt[k], zm = conjg<R>(Zt[k == 0 ? 0 : M - k]);
        const c2<R> w = tq[k];                         // e^{-i pi k / (2M)}
        R re = mul<R>(w, add<R>(zk, zm)).x;
        R im = mul<R>(w, sub<R>(zk, zm)).y;
        const R sg = k == 0 ? invMh : ((k & 1) ? -invM : invM);
        out[col * N + k] = mk<R>(re * sg, im * sg);
    }
}

template <class R>
__global__ void k_cheb_fwd(const c2<R>* __restrict__ in, c2<R>* __restrict__ out, long long ncols, int N,
                           FftPlan plan, int B, const c2<R>* __restrict__ tw_g,
                           const c2<R>* __restrict__ tq_g) {
    cheb_fwd_body<R>(blockIdx.x, in, out, ncols, N, plan, B, tw_g, tq_g);
}

template <class R>
__global__ void k_cheb_fwd_grp(const __grid_constant__ Grp<ChebArgs<R>> g) {
    const int k = g.find(blockIdx.x);
    const ChebArgs<R>& a = g.a[k];
    cheb_fwd_body<R>(blockIdx.x - g.start[k], a.in, a.out, a.ncols, a.N, a.plan, a.B, a.tw, a.tq);
}

// ------------------------------------------------------------------------------------------------
// Derivative expansion fused into the load of a backward transform (fields that differ only by a
// derivative along the transform's axis share the transforms before it): output group og of the
// batch reads input group src[og] and multiplies each value by (i k_j)^ord[og], k_j the wavenumber
// of its index j along the axis, from a table [order - 1][nidx] rounded to R on the host. Outer row
// o = (c nout + og) per + r reads row (c nin + src[og]) per + r.
template <class R>
struct Expand {
    int nout = 0;                 // 0: no expansion (row o reads row o)
    int nin = 0, per = 1, nidx = 0;
    const int* src = nullptr;
    const int* ord = nullptr;
    const c2<R>* tab = nullptr;
};

// the source row of outer row o and its factor table (nullptr: no derivative)
template <class R>
__device__ __forceinline__ long long expand_row(const Expand<R>& ex, long long o, const c2<R>** wt) {
    *wt = nullptr;
    if (ex.nout == 0) return o;
    const long long g = o / ex.per;
    const long long r = o - g * ex.per;
    const long long c = g / ex.nout;
    const int og = (int)(g - c * ex.nout);
    const int od = ex.ord[og];
    if (od > 0) *wt = ex.tab + (size_t)(od - 1) * ex.nidx;
    return (c * ex.nin + ex.src[og]) * ex.per + r;
}

// w v with w = (i k)^o (the product of the separate expansion pass)
template <class R>
__device__ __forceinline__ c2<R> ikmul(c2<R> w, c2<R> v) {
    return mk<R>(w.x * v.x - w.y * v.y, w.x * v.y + w.y * v.x);
}

// ------------------------------------------------------------------------------------------------
// complex FFT along a strided axis: data [outer][len][inner]. Backward: compact spectrum of Nc
// entries (fftfreq order, Nyquist entry Nc/2 ignored) -> L grid points, unnormalized inverse.
// Forward: L points -> compact Nc (|k| < Nc/2, Nyquist set to 0), scaled 1/L.
// Arguments of one strided-axis transform launch (complex or real; a grouped launch holds one set
// per problem).
template <class R>
struct AxisArgs {
    const void* in;
    void* out;
    long long outer;
    int inner, ncompact;       // ncompact: Nc (complex transform) or K (real transform)
    FftPlan plan;
    int B, forward;
    const c2<R>* tw;
    Expand<R> ex;
};

template <class R>
__device__ __forceinline__ void fft_axis_body(unsigned bid, const c2<R>* __restrict__ in, c2<R>* __restrict__ out,
                                              long long outer, int inner, int Nc, const FftPlan& plan, int B,
                                              int forward, const c2<R>* __restrict__ tw_g, const Expand<R>& ex) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int L = plan.L, LS = L + 1;        // padded rows: the column-wise staging is conflict-free
    c2<R>* tw = reinterpret_cast<c2<R>*>(sm);
    c2<R>* b0 = tw + L;
    c2<R>* b1 = b0 + (size_t)B * LS;
    const int tid = threadIdx.x, nt = blockDim.x;
    const FastDiv dB(B);
    for (int q = tid; q < L; q += nt) tw[q] = tw_g[q];
    const int chunks = (inner + B - 1) / B;
    const long long o = bid / chunks;
    const int i0 = (bid - o * chunks) * B;
    const int K = Nc / 2;
    const int lin = forward ? L : Nc;
    const int lout = forward ? Nc : L;
    const c2<R>* wt;
    const c2<R>* src = in + (forward ? o : expand_row<R>(ex, o, &wt)) * (long long)lin * inner;
    c2<R>* dst = out + o * (long long)lout * inner;
    if (!forward) {
        for (int e = tid; e < B * LS; e += nt) b0[e] = mk<R>(0, 0);
        __syncthreads();
        for (int e = tid; e < B * Nc; e += nt) {
            const int k = dB.div(e), t = e - k * B;
            if (i0 + t >= inner || k == K) continue;
            const int slot = k < K ? k : L - (Nc - k);
            const c2<R> v = src[(long long)k * inner + i0 + t];
            b0[(size_t)t * LS + slot] = wt ? ikmul<R>(wt[k], v) : v;
        }
    } else {
        for (int e = tid; e < B * L; e += nt) {
            const int k = dB.div(e), t = e - k * B;
            b0[(size_t)t * LS + k] = (i0 + t < inner) ? src[(long long)k * inner + i0 + t] : mk<R>(0, 0);
        }
    }
    __syncthreads();
    c2<R>* r = smem_fft_fast<R>(b0, b1, plan, B, tw, forward ? -1 : +1, LS);
    if (!forward) {
        for (int e = tid; e < B * L; e += nt) {
            const int k = dB.div(e), t = e - k * B;
            if (i0 + t < inner) dst[(long long)k * inner + i0 + t] = r[(size_t)t * LS + k];
        }
    } else {
        const R invL = R(1) / R(L);
        for (int e = tid; e < B * Nc; e += nt) {
            const int k = dB.div(e), t = e - k * B;
            if (i0 + t >= inner) continue;
            c2<R> v = mk<R>(0, 0);
            if (k != K) v = scl<R>(invL, r[(size_t)t * LS + (k < K ? k : L - (Nc - k))]);
            dst[(long long)k * inner + i0 + t] = v;
        }
    }
}

template <class R>
__global__ void k_fft_axis(const c2<R>* __restrict__ in, c2<R>* __restrict__ out, long long outer, int inner,
                           int Nc, FftPlan plan, int B, int forward, const c2<R>* __restrict__ tw_g, Expand<R> ex) {
    fft_axis_body<R>(blockIdx.x, in, out, outer, inner, Nc, plan, B, forward, tw_g, ex);
}

template <class R>
__global__ void k_fft_axis_grp(const __grid_constant__ Grp<AxisArgs<R>> g) {
    const int k = g.find(blockIdx.x);
    const AxisArgs<R>& a = g.a[k];
    fft_axis_body<R>(blockIdx.x - g.start[k], static_cast<const c2<R>*>(a.in), static_cast<c2<R>*>(a.out), a.outer,
                     a.inner, a.ncompact, a.plan, a.B, a.forward, a.tw, a.ex);
}

// Real FFT along the outer axis of [outer][len][inner]: two adjacent inner columns per complex FFT
// (an odd last column is paired with zero). Backward (c2r): half spectrum [outer][K][inner] complex (modes 0..K-1,
// Hermitian continuation, zero padding) -> [outer][L][inner] real, unnormalized. Forward (r2c):
// real -> modes 0..K-1, scaled 1/L.
template <class R>
__device__ __forceinline__ void rfft_axis_body(unsigned bid, const void* __restrict__ in_, void* __restrict__ out_,
                                               long long outer, int inner, int K, const FftPlan& plan, int B,
                                               int forward, const c2<R>* __restrict__ tw_g, const Expand<R>& ex) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int L = plan.L, LS = L + 1;
    c2<R>* tw = reinterpret_cast<c2<R>*>(sm);
    c2<R>* b0 = tw + L;
    c2<R>* b1 = b0 + (size_t)B * LS;
    const int tid = threadIdx.x, nt = blockDim.x;
    const FastDiv dB(B);
    for (int q = tid; q < L; q += nt) tw[q] = tw_g[q];
    const int pairs = (inner + 1) / 2;             // an odd last column is paired with zero
    const int chunks = (pairs + B - 1) / B;
    const long long o = bid / chunks;
    const int p0 = (bid - o * chunks) * B;     // first pair
    if (!forward) {
        const c2<R>* wt;
        const c2<R>* src = static_cast<const c2<R>*>(in_) + expand_row<R>(ex, o, &wt) * (long long)K * inner;
        R* dst = static_cast<R*>(out_) + o * (long long)L * inner;
        for (int e = tid; e < B * LS; e += nt) b0[e] = mk<R>(0, 0);
        __syncthreads();
        // Z_k = A_k + i B_k, Z_{L-k} = conj(A_k) + i conj(B_k)
        for (int e = tid; e < B * K; e += nt) {
            const int k = dB.div(e), t = e - k * B;
            const int p = p0 + t;
            if (p >= pairs) continue;
            c2<R> A = src[(long long)k * inner + 2 * p];
            c2<R> Bv = 2 * p + 1 < inner ? src[(long long)k * inner + 2 * p + 1] : mk<R>(0, 0);
            if (wt) {
                const c2<R> w = wt[k];
                A = ikmul<R>(w, A);
                Bv = ikmul<R>(w, Bv);
            }
            if (k == 0) {
                b0[(size_t)t * LS] = mk<R>(A.x - Bv.y, A.y + Bv.x);
            } else {
                b0[(size_t)t * LS + k] = mk<R>(A.x - Bv.y, A.y + Bv.x);
                b0[(size_t)t * LS + L - k] = mk<R>(A.x + Bv.y, -A.y + Bv.x);
            }
        }
        __syncthreads();
        c2<R>* r = smem_fft_fast<R>(b0, b1, plan, B, tw, +1, LS);
        for (int e = tid; e < B * L; e += nt) {
            const int j = dB.div(e), t = e - j * B;
            const int p = p0 + t;
            if (p >= pairs) continue;
            c2<R> z = r[(size_t)t * LS + j];
            R* d = dst + (long long)j * inner + 2 * p;
            d[0] = z.x;
            if (2 * p + 1 < inner) d[1] = z.y;
        }
    } else {
        const R* src = static_cast<const R*>(in_) + o * (long long)L * inner;
        c2<R>* dst = static_cast<c2<R>*>(out_) + o * (long long)K * inner;
        for (int e = tid; e < B * L; e += nt) {
            const int j = dB.div(e), t = e - j * B;
            const int p = p0 + t;
            c2<R> z = mk<R>(0, 0);
            if (p < pairs) {
                const R* s = src + (long long)j * inner + 2 * p;
                z = mk<R>(s[0], 2 * p + 1 < inner ? s[1] : R(0));
            }
            b0[(size_t)t * LS + j] = z;
        }
        __syncthreads();
        c2<R>* Z = smem_fft_fast<R>(b0, b1, plan, B, tw, -1, LS);
        const R h = R(0.5) / R(L);
        for (int e = tid; e < B * K; e += nt) {
            const int k = dB.div(e), t = e - k * B;
            const int p = p0 + t;
            if (p >= pairs) continue;
            c2<R> zk = Z[(size_t)t * LS + k];
            c2<R> zm = conjg<R>(Z[(size_t)t * LS + (k == 0 ? 0 : L - k)]);
            c2<R> A = scl<R>(h, add<R>(zk, zm));
            c2<R> d = sub<R>(zk, zm);                      // B = d / (2i)
            c2<R> Bv = mk<R>(h * d.y, -h * d.x);
            dst[(long long)k * inner + 2 * p] = A;
            if (2 * p + 1 < inner) dst[(long long)k * inner + 2 * p + 1] = Bv;
        }
    }
}

template <class R>
__global__ void k_rfft_axis(const void* __restrict__ in_, void* __restrict__ out_, long long outer, int inner,
                            int K, FftPlan plan, int B, int forward, const c2<R>* __restrict__ tw_g,
                            Expand<R> ex) {
    rfft_axis_body<R>(blockIdx.x, in_, out_, outer, inner, K, plan, B, forward, tw_g, ex);
}

template <class R>
__global__ void k_rfft_axis_grp(const __grid_constant__ Grp<AxisArgs<R>> g) {
    const int k = g.find(blockIdx.x);
    const AxisArgs<R>& a = g.a[k];
    rfft_axis_body<R>(blockIdx.x - g.start[k], a.in, a.out, a.outer, a.inner, a.ncompact, a.plan, a.B, a.forward,
                      a.tw, a.ex);
}

// ------------------------------------------------------------------------------------------------
// F pipeline: descriptors on the device

struct RhsDev {
    int ndir, Kx, Nzc, Ny, nfactors, noutputs, nbuckets;
    int ncase;                 // cases stacked in the work arrays (field index case nf + f)
    // Fields that differ only by x / z derivatives share their transforms along y (and, for x,
    // along z): the (i k)^o factors are diagonal in the Fourier indices, so they commute with the
    // transforms of the other directions and are applied between the stages.
    // Both forms share whenever there is a Fourier direction: the derivative factor (i k)^o is
    // constant along the transforms it is moved across, so each line's relative rounding error is
    // the same as with the derivative applied first (the FP32 form's error against the FP64 form:
    // 5.2e-7 -> 5.5e-7 after 50 channel steps, its F 2.77 -> 2.43 ms).
    int share;                 // 1: shared transforms with expansions; 0: one transform per factor
    int ngy, ngz;              // distinct (var, comp, oy) and (var, comp, oy, oz); nfactors if 0
    const int* yg_rep;         // ngy: a factor of each y-group (its column positions and oy)
    const int* zg_y;           // ngz: the y-group of each z-group
    const int* zg_oz;          // ngz: oz of each z-group
    const int* f_z;            // nfactors: the z-group of each factor
    double lx, lz, ly;
    const int* factors;        // nfactors x 5: var, comp, ox, oy, oz
    const int* out_lam;        // noutputs: lambda (0: no conversion)
    const int* out_mono_ptr;   // noutputs + 1
    const double* mono_coef;   // per monomial
    const int* mono_fac;       // per monomial: 4 factor ids (-1 pad)
    const double* conv;        // per lambda 1..: (Ny x Ny) dense, conv + (lam - 1) Ny Ny
    const int* conv_bw;        // per lambda: upper bandwidth of the conversion
    const int* conv_step;      // per lambda: 2 when it couples one parity only (odd offsets zero), else 1
};

struct BucketDev {
    int nsys, n, dact, sign, real;
    long long offset;          // complex elements into the state / rows
    const int* modes;          // nsys x 2
    const int* colpos;         // nfactors x Ny
    const int* rowmap;         // n x 2: output index (-1: none), Chebyshev index
    const int* case_of;        // nsys: case of each system (nullptr: case 0)
};

// Spectral slot of mode (jx, jz, sign) along the compact z axis.
__device__ __forceinline__ int zslot(int jz, int sign, int Nzc) {
    return (jz == 0 || sign > 0) ? jz : Nzc - jz;
}

// one warp per system: state -> factor spectra (with derivatives), complex<R> output
// der[n] = sum_{k > n, k - n odd} 2 k c[k] for n < N (der[N-1] = 0): with v_k = 2 k c[k], der[n] is
// the suffix sum from k = n + 1 over entries of parity (n + 1) % 2. Each lane sums a contiguous
// chunk of k from the top down (one running sum per parity), the chunk totals are combined by a
// suffix scan over the lanes, and each lane then writes der[k - 1] for the k of its chunk.
template <class R>
__device__ __forceinline__ void cheb_der_warp(const c2<R>* __restrict__ c, c2<R>* __restrict__ der, int N,
                                              int lane) {
    const int C = (N + 31) >> 5;
    const int k0 = lane * C, k1 = min(k0 + C, N);
    // chunk totals per parity (of k)
    R tx[2] = {R(0), R(0)}, ty[2] = {R(0), R(0)};
    for (int k = k1 - 1; k >= k0; --k) {
        if (k == 0) continue;
        const R w = R(2 * k);
        tx[k & 1] = tx[k & 1] + w * c[k].x;
        ty[k & 1] = ty[k & 1] + w * c[k].y;
    }
    // exclusive suffix scan over lanes: sums of the chunks above this lane
    R sx[2] = {tx[0], tx[1]}, sy[2] = {ty[0], ty[1]};
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const R ux = shfl_down_r(sx[p], off), uy = shfl_down_r(sy[p], off);
            if (lane + off < 32) { sx[p] = sx[p] + ux; sy[p] = sy[p] + uy; }
        }
    }
    R ax[2], ay[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) { ax[p] = sx[p] - tx[p]; ay[p] = sy[p] - ty[p]; }
    if (lane == 0 && N >= 1) der[N - 1] = mk<R>(R(0), R(0));
    for (int k = k1 - 1; k >= k0; --k) {
        if (k == 0) continue;
        const R w = R(2 * k);
        ax[k & 1] = ax[k & 1] + w * c[k].x;
        ay[k & 1] = ay[k & 1] + w * c[k].y;
        der[k - 1] = mk<R>(ax[k & 1], ay[k & 1]);
    }
}

// Arguments of the per-bucket stages (unpack, pack; a grouped launch holds one set per bucket).
template <class R>
struct BucketArgs {
    RhsDev d;
    BucketDev b;
    const void* in;
    void* out;
    int split = 1;          // warps per system (unpack: over the y-groups; pack: over the rows)
};

template <class R>
__device__ __forceinline__ void unpack_body(unsigned bid, const RhsDev& d, const BucketDev& b,
                                            const double2* __restrict__ state, c2<R>* __restrict__ S,
                                            int split) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    const int q = bid * nw + wib;
    const int m = q / split, part = q - m * split;      // system, and its y-groups part, part + split, ...
    if (m >= b.nsys) return;
    const int Ny = d.Ny;
    // the system's state, rounded once to the transform precision R
    c2<R>* x = reinterpret_cast<c2<R>*>(sm) + (size_t)wib * (b.n + 2 * Ny);
    c2<R>* col = x + b.n;
    c2<R>* der = col + Ny;
    const double2* src = state + b.offset + (long long)m * b.n;
#pragma unroll 4
    for (int i = lane; i < b.n; i += 32) {             // unrolled: the loads of 4 rows in flight
        const double2 v = src[i];
        x[i] = mk<R>(R(v.x), R(v.y));
    }
    __syncwarp();
    const int jx = b.modes[2 * m], jz = b.modes[2 * m + 1];
    const double kx = 6.283185307179586476925286766559 * jx / d.lx;
    const double kz = b.sign * 6.283185307179586476925286766559 * jz / d.lz;
    const double w = b.dact == 0 ? 1.0 : (b.dact == 1 ? 0.5 : 0.25);
    const int slot = zslot(jz, b.sign, d.Nzc);
    const int cbase = (b.case_of ? b.case_of[m] : 0) * d.ngy;
    for (int gy = part; gy < d.ngy; gy += split) {
        const int f = d.yg_rep[gy];
        const int* fd = d.factors + 5 * f;
        const int oy = fd[3];
        const int ox = d.share ? 0 : fd[2], oz = d.share ? 0 : fd[4];   // shared: applied later
        const int* cp = b.colpos + (size_t)f * Ny;
#pragma unroll 4
        for (int nn = lane; nn < Ny; nn += 32) {
            const int pos = cp[nn];
            col[nn] = pos >= 0 ? x[pos] : mk<R>(R(0), R(0));
        }
        __syncwarp();
        // Chebyshev derivative oy times: out[n] = sum_{k > n, k - n odd} 2 k c[k], out[0] /= 2,
        // x 2/L (in the transform precision R: the derivative is part of F), as a suffix sum per
        // parity across the warp
        for (int rep = 0; rep < oy; ++rep) {
            cheb_der_warp<R>(col, der, Ny, lane);
            __syncwarp();
            const R sc = R(2.0 / d.ly);
            for (int nn = lane; nn < Ny; nn += 32) {
                c2<R> v = der[nn];
                if (nn == 0) { v.x = v.x / 2; v.y = v.y / 2; }
                col[nn] = mk<R>(v.x * sc, v.y * sc);
            }
            __syncwarp();
        }
        // Fourier derivatives and the amplitude scale: w (i kx)^ox (i kz)^oz
        double fr = w, fi = 0.0;
        for (int q = 0; q < ox; ++q) { double t = fr; fr = -fi * kx; fi = t * kx; }
        for (int q = 0; q < oz; ++q) { double t = fr; fr = -fi * kz; fi = t * kz; }
        c2<R>* dst;
        c2<R>* dstc = nullptr;
        const long long fc = cbase + gy;
        if (d.ndir == 2) {
            dst = S + ((fc * d.Kx + jx) * d.Nzc + slot) * Ny;
            if (jx == 0 && jz > 0) dstc = S + ((fc * d.Kx) * d.Nzc + (d.Nzc - jz)) * Ny;
        } else if (d.ndir == 1) {
            dst = S + (fc * d.Kx + jx) * Ny;
        } else {
            dst = S + fc * Ny;
        }
        // the scale w (i kx)^ox (i kz)^oz in the transform precision R (a product: no cancellation)
        const R frR = R(fr), fiR = R(fi);
        for (int nn = lane; nn < Ny; nn += 32) {
            const c2<R> c = col[nn];
            const R cr = c.x, ci = c.y;
            const R vr = frR * cr - fiR * ci;
            const R vi = b.real ? R(0) : frR * ci + fiR * cr;
            dst[nn] = mk<R>(vr, vi);
            if (dstc) dstc[nn] = mk<R>(vr, -vi);
        }
        __syncwarp();
    }
}

// every bucket of one or more evaluators in one launch (launch_unpack)
template <class R>
__global__ void k_unpack_grp(const __grid_constant__ Grp<BucketArgs<R>> g) {
    const int k = g.find(blockIdx.x);
    const BucketArgs<R>& a = g.a[k];
    unpack_body<R>(blockIdx.x - g.start[k], a.d, a.b, static_cast<const double2*>(a.in), static_cast<c2<R>*>(a.out),
                   a.split);
}

// products on the grid: out_o = sum_m c_m prod_j G_j. The monomial tables are staged in shared
// memory; a thread takes V consecutive points (one 16-byte load per factor field: V = 4 in FP32,
// 2 in FP64), which needs P % V == 0 (else V = 1).
constexpr int kMaxMono = 64;
template <class R> struct Vec;
template <> struct Vec<float> { using t4 = float4; };
template <> struct Vec<double> { using t4 = double2; };

template <class R, int V>
__device__ __forceinline__ void load_v(const R* p, R* v) {
    if constexpr (V == 1) {
        v[0] = __ldg(p);
    } else if constexpr (sizeof(R) == 4) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(p));
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
        const double2 q = __ldg(reinterpret_cast<const double2*>(p));
        v[0] = q.x; v[1] = q.y;
    }
}

template <class R, int V>
__device__ __forceinline__ void store_v(R* p, const R* v) {
    if constexpr (V == 1) {
        p[0] = v[0];
    } else if constexpr (sizeof(R) == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
        *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    }
}

// Arguments of one products launch (a grouped launch holds one set per problem).
template <class R>
struct ProductArgs {
    RhsDev d;
    const R* G;
    R* O;
    long long P;
};

template <class R, int V>
__device__ __forceinline__ void products_body(unsigned bid, unsigned nblk, const RhsDev& d, const R* __restrict__ G,
                                              R* __restrict__ O, long long P) {
    __shared__ int s_ptr[17];
    __shared__ R s_coef[kMaxMono];
    __shared__ int s_kind[kMaxMono];         // 1: coefficient +1, -1: coefficient -1, 0: other
    __shared__ int s_fac[4 * kMaxMono];
    const int no = d.noutputs;
    for (int q = threadIdx.x; q <= no; q += blockDim.x) s_ptr[q] = d.out_mono_ptr[q];
    __syncthreads();
    const int nm = s_ptr[no];
    for (int q = threadIdx.x; q < nm; q += blockDim.x) {
        s_coef[q] = R(d.mono_coef[q]);
        s_kind[q] = d.mono_coef[q] == 1.0 ? 1 : (d.mono_coef[q] == -1.0 ? -1 : 0);
    }
    for (int q = threadIdx.x; q < 4 * nm; q += blockDim.x) s_fac[q] = d.mono_fac[q];
    __syncthreads();
    const long long total = P * d.ncase;
    for (long long t0 = ((long long)bid * blockDim.x + threadIdx.x) * V; t0 < total;
         t0 += (long long)nblk * blockDim.x * V) {
        const long long c = t0 / P, p = t0 - c * P;
        const R* Gc = G + c * d.nfactors * P + p;
        R* Oc = O + c * no * P + p;
        for (int o = 0; o < no; ++o) {
            R acc[V];
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v] = R(0);
            for (int mi = s_ptr[o]; mi < s_ptr[o + 1]; ++mi) {
                // c G_a (G_b G_c G_d): the product of the later factors, then one fused
                // multiply-add with the first factor times c (c = +-1: the sign goes into the
                // fused multiply-add; the kind of c is read, not compared, per point)
                const R cf = s_coef[mi];
                const int kind = s_kind[mi];
                R pr[V];
                bool have = false;
#pragma unroll
                for (int q = 1; q < 4; ++q) {
                    const int f = s_fac[4 * mi + q];
                    if (f >= 0) {
                        R g[V];
                        load_v<R, V>(Gc + (long long)f * P, g);
                        if (have) {
#pragma unroll
                            for (int v = 0; v < V; ++v) pr[v] = pr[v] * g[v];
                        } else {
#pragma unroll
                            for (int v = 0; v < V; ++v) pr[v] = g[v];
                        }
                        have = true;
                    }
                }
                const int f0 = s_fac[4 * mi];
                R a[V];
                if (f0 >= 0) {
                    load_v<R, V>(Gc + (long long)f0 * P, a);
                    if (kind == 0) {
#pragma unroll
                        for (int v = 0; v < V; ++v) a[v] = cf * a[v];
                    }
                } else {
#pragma unroll
                    for (int v = 0; v < V; ++v) a[v] = cf;
                }
                if (have && f0 >= 0 && kind < 0) {
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v] = fmar(-a[v], pr[v], acc[v]);
                } else if (have) {
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v] = fmar(a[v], pr[v], acc[v]);
                } else if (f0 >= 0 && kind < 0) {
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v] = acc[v] - a[v];
                } else {
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v] = acc[v] + a[v];
                }
            }
            store_v<R, V>(Oc + (long long)o * P, acc);
        }
    }
}

template <class R, int V>
__global__ void k_products(RhsDev d, const R* __restrict__ G, R* __restrict__ O, long long P) {
    products_body<R, V>(blockIdx.x, gridDim.x, d, G, O, P);
}

template <class R, int V>
__global__ void k_products_grp(const __grid_constant__ Grp<ProductArgs<R>> g) {
    const int k = g.find(blockIdx.x);
    const ProductArgs<R>& a = g.a[k];
    products_body<R, V>(blockIdx.x - g.start[k], g.start[k + 1] - g.start[k], a.d, a.G, a.O, a.P);
}

// one warp per system: output spectra -> rows (C^(lambda) conversion, 2^d_act, real buckets real)
template <class R>
__device__ __forceinline__ void pack_body(unsigned bid, const RhsDev& d, const BucketDev& b,
                                          const c2<R>* __restrict__ H, double2* __restrict__ rows, int split) {
    // the system's output spectra are staged in shared memory (coalesced), then gathered by row
    // (split warps per system: each stages the spectra and takes every split-th run of 32 rows)
    extern __shared__ __align__(16) unsigned char sm[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    const int q = bid * nw + wib;
    const int m = q / split, part = q - m * split;
    if (m >= b.nsys) return;
    const int Ny = d.Ny;
    const int jx = b.modes[2 * m], jz = b.modes[2 * m + 1];
    const int slot = zslot(jz, b.sign, d.Nzc);
    const double sc = (double)(1 << b.dact);
    double2* dst = rows + b.offset + (long long)m * b.n;
    const long long obase = (long long)(b.case_of ? b.case_of[m] : 0) * d.noutputs;
    double2* hs = reinterpret_cast<double2*>(sm) + (size_t)wib * d.noutputs * Ny;   // widened once
    for (int o = 0; o < d.noutputs; ++o) {
        const long long oc = obase + o;
        const c2<R>* h;
        if (d.ndir == 2) h = H + ((oc * d.Kx + jx) * d.Nzc + slot) * Ny;
        else if (d.ndir == 1) h = H + (oc * d.Kx + jx) * Ny;
        else h = H + oc * Ny;
#pragma unroll 4
        for (int nn = lane; nn < Ny; nn += 32) {
            const c2<R> v = h[nn];
            hs[o * Ny + nn] = make_double2((double)v.x, (double)v.y);
        }
    }
    __syncwarp();
#pragma unroll 2
    for (int i = 32 * part + lane; i < b.n; i += 32 * split) {
        const int o = b.rowmap[2 * i], nn = b.rowmap[2 * i + 1];
        double2 v = make_double2(0.0, 0.0);
        if (o >= 0) {
            const double2* h = hs + o * Ny;
            const int lam = d.out_lam[o];
            if (lam <= 0) {
                v = h[nn];
            } else {
                // the C^(lambda) conversion, accumulated in FP64 (its alternating sums cancel);
                // conversions that couple one parity only step over the other (its zeros)
                const double* cv = d.conv + (size_t)(lam - 1) * Ny * Ny + (size_t)nn * Ny;
                const int hi = min(Ny - 1, nn + d.conv_bw[lam - 1]);
                const int step = d.conv_step[lam - 1];
                double ar = 0.0, ai = 0.0;
                for (int k = nn; k <= hi; k += step) {
                    ar += cv[k] * h[k].x;
                    ai += cv[k] * h[k].y;
                }
                v = make_double2(ar, ai);
            }
            v.x *= sc;
            v.y *= sc;
            if (b.real) v.y = 0.0;
        }
        dst[i] = v;
    }
}

// every bucket of one or more evaluators in one launch (launch_pack)
template <class R>
__global__ void k_pack_grp(const __grid_constant__ Grp<BucketArgs<R>> g) {
    const int k = g.find(blockIdx.x);
    const BucketArgs<R>& a = g.a[k];
    pack_body<R>(blockIdx.x - g.start[k], a.d, a.b, static_cast<const c2<R>*>(a.in), static_cast<double2*>(a.out),
                 a.split);
}

// constant part of F: rows[idx] += value
__device__ __forceinline__ void add_sparse_body(unsigned bid, unsigned nblk, double2* rows, const long long* idx,
                                                const double2* val, long long n) {
    for (long long q = (long long)bid * blockDim.x + threadIdx.x; q < n; q += (long long)nblk * blockDim.x) {
        double2 r = rows[idx[q]];
        rows[idx[q]] = make_double2(r.x + val[q].x, r.y + val[q].y);
    }
}

__global__ void k_add_sparse(double2* rows, const long long* idx, const double2* val, long long n) {
    add_sparse_body(blockIdx.x, gridDim.x, rows, idx, val, n);
}

struct SparseArgs {
    double2* rows;
    const long long* idx;
    const double2* val;
    long long n;
};

__global__ void k_add_sparse_grp(const __grid_constant__ Grp<SparseArgs> g) {
    const int k = g.find(blockIdx.x);
    const SparseArgs& a = g.a[k];
    add_sparse_body(blockIdx.x - g.start[k], g.start[k + 1] - g.start[k], a.rows, a.idx, a.val, a.n);
}

template <class R>
__global__ void k_realpart(const c2<R>* __restrict__ in, R* __restrict__ out, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = in[i].x;
}
template <class R>
__global__ void k_complexify(const R* __restrict__ in, c2<R>* __restrict__ out, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = mk<R>(in[i], R(0));
}
template <class R>
void realpart_kernel_launch(const c2<R>* in, R* out, long long n, cudaStream_t st) {
    k_realpart<R><<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, st>>>(in, out, n);
    CNG_LAUNCH("k_realpart");
}
template <class R>
void complexify_kernel_launch(const R* in, void* out, long long n, cudaStream_t st) {
    k_complexify<R><<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, st>>>(in, static_cast<c2<R>*>(out), n);
    CNG_LAUNCH("k_complexify");
}

// ------------------------------------------------------------------------------------------------
// host: transform launchers

template <class R>
static void set_smem_attr(const void* fn) { ensure_smem_attr(fn, (int)kFftSmemMax); }

// Sequences per block of the shared-memory transforms: at most 8 in FP32 and 4 in FP64 (measured
// on the channel's F: fewer sequences per block, more blocks per SM; 16 was 6 % slower in FP32 and
// 12 % in FP64, where the FP64 pipe is the bound and occupancy hides its latency).
constexpr int kMaxSeq32 = 8, kMaxSeq64 = 4;
template <class R>
static int pick_B(int L, int extra_per_col, int maxB) {
    const size_t per = sizeof(c2<R>) * (size_t)(2 * L + extra_per_col);
    int B = (int)std::max<size_t>(1, (kFftSmemMax - sizeof(c2<R>) * 2 * (size_t)L) / per);
    return std::max(1, std::min(B, maxB));
}

// A transform launch's arguments with its dynamic shared memory and block count.
template <class A>
struct Planned {
    A a;
    size_t smem = 0;
    unsigned blocks = 0;
};

template <class R>
static Planned<ChebArgs<R>> plan_cheb(const c2<R>* in, c2<R>* out, long long ncols, int N, int M, bool forward,
                                      int maxseq) {
    if (M % 2) throw InvalidArgument("Chebyshev grid size must be even");
    Planned<ChebArgs<R>> p;
    const int B = pick_B<R>(M, forward ? 0 : M + 1, maxseq > 0 ? maxseq : (sizeof(R) == 4 ? kMaxSeq32 : kMaxSeq64));
    p.a = ChebArgs<R>{in, out, ncols, N, make_plan(M), B, twiddles<R>().get(M, 0),
                      twiddles<R>().get(M, forward ? 1 : 2)};
    p.smem = sizeof(c2<R>) * ((size_t)2 * M + (size_t)B * (2 * M + (forward ? 0 : M + 1)));
    p.blocks = (unsigned)((ncols + B - 1) / B);
    return p;
}

// complex (real = false) or real (real = true) transform along the strided axis
template <class R>
static Planned<AxisArgs<R>> plan_axis(bool real, const void* in, void* out, long long outer, int inner, int ncompact,
                                      int L, bool forward, int maxseq, const Expand<R>& ex) {
    Planned<AxisArgs<R>> p;
    const int B = pick_B<R>(L + 1, 0, maxseq > 0 ? maxseq : (sizeof(R) == 4 ? kMaxSeq32 : kMaxSeq64));
    p.a = AxisArgs<R>{in, out, outer, inner, ncompact, make_plan(L), B, forward ? 1 : 0, twiddles<R>().get(L, 0), ex};
    p.smem = sizeof(c2<R>) * ((size_t)L + (size_t)B * 2 * (L + 1));
    const long long cols = real ? (inner + 1) / 2 : inner;
    p.blocks = (unsigned)(outer * ((cols + B - 1) / B));
    return p;
}

template <class R>
void launch_cheb(const c2<R>* in, c2<R>* out, long long ncols, int N, int M, bool forward, cudaStream_t st,
                 int maxseq = 0, int threads = 0) {
    if (threads <= 0) threads = kFftThreads;
    if (ncols <= 0) return;
    if (N == 1 && M == 1) {        // no Chebyshev direction: the single coefficient is the value
        CNG_CUDA(cudaMemcpyAsync(out, in, sizeof(c2<R>) * (size_t)ncols, cudaMemcpyDeviceToDevice, st));
        return;
    }
    set_smem_attr<R>((const void*)k_cheb_bwd<R>);
    set_smem_attr<R>((const void*)k_cheb_fwd<R>);
    const auto p = plan_cheb<R>(in, out, ncols, N, M, forward, maxseq);
    const ChebArgs<R>& a = p.a;
    if (forward) k_cheb_fwd<R><<<p.blocks, threads, p.smem, st>>>(a.in, a.out, a.ncols, a.N, a.plan, a.B, a.tw, a.tq);
    else k_cheb_bwd<R><<<p.blocks, threads, p.smem, st>>>(a.in, a.out, a.ncols, a.N, a.plan, a.B, a.tw, a.tq);
    CNG_LAUNCH("k_cheb");
}

template <class R>
void launch_fft_axis(const c2<R>* in, c2<R>* out, long long outer, int inner, int Nc, int L, bool forward,
                     cudaStream_t st, int maxseq = 0, int threads = 0, Expand<R> ex = Expand<R>{}) {
    if (threads <= 0) threads = kFftThreads;
    if (outer <= 0 || inner <= 0) return;
    set_smem_attr<R>((const void*)k_fft_axis<R>);
    const auto p = plan_axis<R>(false, in, out, outer, inner, Nc, L, forward, maxseq, ex);
    k_fft_axis<R><<<p.blocks, threads, p.smem, st>>>(in, out, outer, inner, Nc, p.a.plan, p.a.B, p.a.forward,
                                                      p.a.tw, ex);
    CNG_LAUNCH("k_fft_axis");
}

template <class R>
void launch_rfft_axis(const void* in, void* out, long long outer, int inner, int K, int L, bool forward,
                      cudaStream_t st, int maxseq = 0, int threads = 0, Expand<R> ex = Expand<R>{}) {
    if (threads <= 0) threads = kFftThreads;
    if (outer <= 0 || inner <= 0) return;
    set_smem_attr<R>((const void*)k_rfft_axis<R>);
    const auto p = plan_axis<R>(true, in, out, outer, inner, K, L, forward, maxseq, ex);
    k_rfft_axis<R><<<p.blocks, threads, p.smem, st>>>(in, out, outer, inner, K, p.a.plan, p.a.B, p.a.forward,
                                                       p.a.tw, ex);
    CNG_LAUNCH("k_rfft_axis");
}

// Grouped launches of planned stages: one launch per kMaxGrp argument sets, dynamic shared memory
// the largest of the group's.
template <class A, class Kernel>
static void launch_planned(const std::vector<Planned<A>>& ps, Kernel kernel, int threads, cudaStream_t st,
                           const char* what) {
    std::vector<A> args;
    std::vector<unsigned> blocks;
    size_t smem = 0;
    for (const auto& p : ps) {
        args.push_back(p.a);
        blocks.push_back(p.blocks);
        if (p.blocks) smem = std::max(smem, p.smem);
    }
    launch_groups(args, blocks, [&](const Grp<A>& g, unsigned total) {
        kernel<<<total, threads, smem, st>>>(g);
        CNG_LAUNCH(what);
    });
}

// ------------------------------------------------------------------------------------------------
// the F pipeline object

template <class P>
static P* upload(const P* h, size_t n) {
    P* d = static_cast<P*>(dev_alloc(std::max<size_t>(sizeof(P) * n, 16)));
    if (n) {
        const cudaError_t e = cudaMemcpy(d, h, sizeof(P) * n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            dev_free(d);
            cuda_check(e, "cudaMemcpy (upload)");
        }
    }
    return d;
}

struct Rhs {
    int precision = 0;         // 0 = FP64 transforms and products, 1 = FP32
    int ndir = 0, nx = 0, nz = 0, mx = 1, mz = 1, ny = 1, my = 1;
    int Kx = 1, Nzc = 1;
    double lx = 1, lz = 1, ly = 2;
    int nfactors = 0, noutputs = 0;
    int ncase = 1;             // cases stacked along the field index
    int maxseq = 0;            // sequences per block of the transforms (0: the per-precision default)
    int threads = 0;           // threads per block of the transforms (0: 256)
    RhsDev dev{};
    std::vector<BucketDev> buckets;
    std::vector<void*> owned;
    long long nb0 = 0;
    long long* b0_idx = nullptr;
    double2* b0_val = nullptr;
    // work buffers
    void* S = nullptr;     // factor spectra after unpack / output spectra before pack
    void* W1 = nullptr;
    void* W2 = nullptr;
    size_t S_bytes = 0, W_bytes = 0;
    // shared transforms: (i k)^o tables along z (Nzc slots) and x (Kx modes), ox per factor
    void* ktab_z = nullptr;
    void* ktab_x = nullptr;
    int* f_ox = nullptr;

    ~Rhs() {
        for (void* p : owned) dev_free(p);
    }
    template <class P> P* keep(P* p) { owned.push_back((void*)p); return p; }

    long long spec_cols(int nfields) const {      // Chebyshev columns of the spectral arrays
        return (long long)nfields * (ndir >= 1 ? Kx : 1) * (ndir == 2 ? Nzc : 1);
    }
    long long grid_points() const { return (long long)(ndir >= 1 ? mx : 1) * (ndir == 2 ? mz : 1) * my; }

    template <class R>
    void run(const double2* state, double2* rows, cudaStream_t st);
};

// The per-bucket stages of one or more evaluators, every bucket in one grouped launch (one warp per
// system; buckets of different lengths run side by side instead of one after the other).
constexpr int kBucketWarps = 4;

// warps per system of unpack and pack: one where the systems fill the SMs, else up to `most` (a
// small problem's few systems: RB 256x64 has 129, Burgers one)
static int bucket_split(Rhs* const* hs, int n, int most) {
    long long systems = 0;
    for (int i = 0; i < n; ++i)
        for (const auto& b : hs[i]->buckets) systems += b.nsys;
    return systems < 2LL * sm_count() * kBucketWarps ? most : 1;
}

template <class R>
static void launch_unpack(Rhs* const* hs, int n, const double2* state, cudaStream_t st) {
    std::vector<BucketArgs<R>> args;
    std::vector<unsigned> blocks;
    size_t smem = 0;
    int ngy = 1;
    for (int i = 0; i < n; ++i) ngy = std::max(ngy, hs[i]->dev.ngy);
    const int split = bucket_split(hs, n, std::min(ngy, 8));
    for (int i = 0; i < n; ++i)
        for (const auto& b : hs[i]->buckets) {
            args.push_back(BucketArgs<R>{hs[i]->dev, b, state, hs[i]->S, split});
            blocks.push_back((unsigned)ceil_div(b.nsys * split, kBucketWarps));
            if (b.nsys) smem = std::max(smem, (size_t)kBucketWarps * (b.n + 2 * hs[i]->ny) * sizeof(c2<R>));
        }
    ensure_smem_attr((const void*)k_unpack_grp<R>, 200 * 1024);
    launch_groups(args, blocks, [&](const Grp<BucketArgs<R>>& g, unsigned total) {
        k_unpack_grp<R><<<total, 32 * kBucketWarps, smem, st>>>(g);
        CNG_LAUNCH("k_unpack_grp");
    });
}

template <class R>
static void launch_pack(Rhs* const* hs, int n, double2* rows, cudaStream_t st) {
    std::vector<BucketArgs<R>> args;
    std::vector<unsigned> blocks;
    size_t smem = 0;
    const int split = bucket_split(hs, n, 4);
    for (int i = 0; i < n; ++i)
        for (const auto& b : hs[i]->buckets) {
            args.push_back(BucketArgs<R>{hs[i]->dev, b, hs[i]->S, rows, split});
            blocks.push_back((unsigned)ceil_div(b.nsys * split, kBucketWarps));
            if (b.nsys) smem = std::max(smem, (size_t)kBucketWarps * hs[i]->noutputs * hs[i]->ny * sizeof(double2));
        }
    ensure_smem_attr((const void*)k_pack_grp<R>, 200 * 1024);
    launch_groups(args, blocks, [&](const Grp<BucketArgs<R>>& g, unsigned total) {
        k_pack_grp<R><<<total, 32 * kBucketWarps, smem, st>>>(g);
        CNG_LAUNCH("k_pack_grp");
    });
}

template <class R>
void Rhs::run(const double2* state, double2* rows, cudaStream_t st) {
    using C = c2<R>;
    const int nf = nfactors * ncase, no = noutputs * ncase;     // fields of every case
    C* Sp = static_cast<C*>(S);
    Rhs* self = this;
    // 1. unpack (one warp per system, every bucket in one launch)
    launch_unpack<R>(&self, 1, state, st);
    // 2. Chebyshev backward along y of the y-groups: S [cols][ny] -> W1 [cols][my]
    C* A = static_cast<C*>(W1);
    C* Bf = static_cast<C*>(W2);
    const int ngy = dev.ngy * ncase, ngz = dev.ngz * ncase;
    launch_cheb<R>(Sp, A, spec_cols(ngy), ny, my, false, st, maxseq, threads);
    C* cur = A;
    C* other = Bf;
    // 3. z: the z-groups ((i kz)^oz of their y-group), then the z backward transform
    //    [ngz Kx][Nzc][my] -> [ngz Kx][mz][my]
    if (ndir == 2) {
        Expand<R> ez{};
        if (dev.share) {
            ez.nout = dev.ngz; ez.nin = dev.ngy; ez.per = Kx; ez.nidx = Nzc;
            ez.src = dev.zg_y; ez.ord = dev.zg_oz; ez.tab = static_cast<const C*>(ktab_z);
        }
        launch_fft_axis<R>(cur, other, (long long)ngz * Kx, my, Nzc, mz, false, st, maxseq, threads, ez);
        std::swap(cur, other);
    }
    // 4. x: the factors ((i kx)^ox of their z-group), then the x backward (c2r) transform
    //    [nf][Kx][inner] -> [nf][mx][inner] real
    const long long inner = (long long)(ndir == 2 ? mz : 1) * my;
    R* G = reinterpret_cast<R*>(cur);
    if (ndir >= 1) {
        Expand<R> exx{};
        if (dev.share) {
            exx.nout = nfactors; exx.nin = dev.ngz; exx.per = 1; exx.nidx = Kx;
            exx.src = dev.f_z; exx.ord = f_ox; exx.tab = static_cast<const C*>(ktab_x);
        }
        launch_rfft_axis<R>(cur, other, nf, (int)inner, Kx, mx, false, st, maxseq, threads, exx);
        G = reinterpret_cast<R*>(other);
        std::swap(cur, other);
    } else {
        // no Fourier direction: the grid values are complex with zero imaginary part; compact them
        // to reals in place of the c2r step (real buckets only, so the imaginary part is zero)
        G = reinterpret_cast<R*>(cur);
    }
    // 5. products: G [nf][P] -> O [no][P] (real)
    const long long P = grid_points();
    R* O = reinterpret_cast<R*>(other);
    if (ndir == 0) {
        // complex grid values -> real: O_tmp holds reals of the factors
        R* Gr = reinterpret_cast<R*>(S);
        const long long n = (long long)nf * P;
        realpart_kernel_launch<R>(reinterpret_cast<const C*>(G), Gr, n, st);
        G = Gr;
    }
    {
        const int threads = 256;
        constexpr int V = sizeof(R) == 4 ? 4 : 2;
        if (P % V == 0) {
            const long long blocks = std::min<long long>((P * ncase / V + threads - 1) / threads, 152LL * 16);
            k_products<R, V><<<(unsigned)blocks, threads, 0, st>>>(dev, G, O, P);
        } else {
            const long long blocks = std::min<long long>((P * ncase + threads - 1) / threads, 152LL * 16);
            k_products<R, 1><<<(unsigned)blocks, threads, 0, st>>>(dev, G, O, P);
        }
        CNG_LAUNCH("k_products");
    }
    std::swap(cur, other);           // cur = O
    // 6. x forward (r2c): [no][mx][inner] -> [no][Kx][inner]
    if (ndir >= 1) {
        launch_rfft_axis<R>(cur, other, no, (int)inner, Kx, mx, true, st, maxseq, threads);
        std::swap(cur, other);
    } else {
        complexify_kernel_launch<R>(reinterpret_cast<const R*>(cur), other, (long long)no * P, st);
        std::swap(cur, other);
    }
    // 7. z forward: [no Kx][mz][my] -> [no Kx][Nzc][my]
    if (ndir == 2) {
        launch_fft_axis<R>(cur, other, (long long)no * Kx, my, Nzc, mz, true, st, maxseq, threads);
        std::swap(cur, other);
    }
    // 8. Chebyshev forward: [cols][my] -> S [cols][ny]
    launch_cheb<R>(cur, Sp, spec_cols(no), ny, my, true, st, maxseq, threads);
    // 9. pack rows (every bucket in one launch) and add the constant part
    launch_pack<R>(&self, 1, rows, st);
    if (nb0) {
        k_add_sparse<<<ceil_div(nb0, 256), 256, 0, st>>>(rows, b0_idx, b0_val, nb0);
        CNG_LAUNCH("k_add_sparse");
    }
}

// F of several problems (templates and sizes may differ; one precision, the same Fourier
// directions) with one launch per stage: each stage's grouped kernel runs every problem's
// arguments over its own block range. The problems read one state and write one set of rows
// (their bucket offsets place them in it). The arithmetic of each problem is that of Rhs::run.
template <class R>
void run_group(Rhs* const* hs, int n, const double2* state, double2* rows, cudaStream_t st) {
    using C = c2<R>;
    const int threads = hs[0]->threads > 0 ? hs[0]->threads : kFftThreads;
    const int ndir = hs[0]->ndir;
    for (int i = 0; i < n; ++i) {
        if (hs[i]->ndir != ndir || hs[i]->precision != hs[0]->precision)
            throw InvalidArgument("grouped F: every problem needs the same precision and Fourier directions");
        if ((hs[i]->threads > 0 ? hs[i]->threads : kFftThreads) != threads)
            throw InvalidArgument("grouped F: every problem needs the same transform block size");
    }
    if (ndir < 1) throw InvalidArgument("grouped F: at least one Fourier direction");
    // 1. unpack
    launch_unpack<R>(hs, n, state, st);
    // the stages' buffers per problem, as Rhs::run rotates them
    std::vector<C*> cur(n), other(n);
    std::vector<Planned<ChebArgs<R>>> cheb;
    for (int i = 0; i < n; ++i) {
        const Rhs& h = *hs[i];
        cur[i] = static_cast<C*>(h.W1);
        other[i] = static_cast<C*>(h.W2);
        const long long cols = h.spec_cols(h.dev.ngy * h.ncase);
        if (h.ny == 1 && h.my == 1) throw InvalidArgument("grouped F: a Chebyshev direction is needed");
        cheb.push_back(plan_cheb<R>(static_cast<const C*>(h.S), cur[i], cols, h.ny, h.my, false, h.maxseq));
    }
    set_smem_attr<R>((const void*)k_cheb_bwd_grp<R>);
    launch_planned(cheb, k_cheb_bwd_grp<R>, threads, st, "k_cheb_bwd_grp");
    if (ndir == 2) {
        std::vector<Planned<AxisArgs<R>>> z;
        for (int i = 0; i < n; ++i) {
            const Rhs& h = *hs[i];
            Expand<R> ez{};
            if (h.dev.share) {
                ez.nout = h.dev.ngz; ez.nin = h.dev.ngy; ez.per = h.Kx; ez.nidx = h.Nzc;
                ez.src = h.dev.zg_y; ez.ord = h.dev.zg_oz; ez.tab = static_cast<const C*>(h.ktab_z);
            }
            z.push_back(plan_axis<R>(false, cur[i], other[i], (long long)h.dev.ngz * h.ncase * h.Kx, h.my, h.Nzc,
                                     h.mz, false, h.maxseq, ez));
            std::swap(cur[i], other[i]);
        }
        set_smem_attr<R>((const void*)k_fft_axis_grp<R>);
        launch_planned(z, k_fft_axis_grp<R>, threads, st, "k_fft_axis_grp");
    }
    // x backward (c2r) with the x expansions
    std::vector<Planned<AxisArgs<R>>> xb;
    std::vector<R*> G(n);
    for (int i = 0; i < n; ++i) {
        const Rhs& h = *hs[i];
        const long long inner = (long long)(ndir == 2 ? h.mz : 1) * h.my;
        Expand<R> exx{};
        if (h.dev.share) {
            exx.nout = h.nfactors; exx.nin = h.dev.ngz; exx.per = 1; exx.nidx = h.Kx;
            exx.src = h.dev.f_z; exx.ord = h.f_ox; exx.tab = static_cast<const C*>(h.ktab_x);
        }
        xb.push_back(plan_axis<R>(true, cur[i], other[i], (long long)h.nfactors * h.ncase, (int)inner, h.Kx, h.mx,
                                  false, h.maxseq, exx));
        G[i] = reinterpret_cast<R*>(other[i]);
        std::swap(cur[i], other[i]);
    }
    set_smem_attr<R>((const void*)k_rfft_axis_grp<R>);
    launch_planned(xb, k_rfft_axis_grp<R>, threads, st, "k_rfft_axis_grp(backward)");
    // products
    {
        constexpr int VV = sizeof(R) == 4 ? 4 : 2;
        bool vec = true;
        for (int i = 0; i < n; ++i) vec = vec && hs[i]->grid_points() % VV == 0;
        std::vector<ProductArgs<R>> args;
        std::vector<unsigned> blocks;
        for (int i = 0; i < n; ++i) {
            const Rhs& h = *hs[i];
            const long long P = h.grid_points();
            args.push_back(ProductArgs<R>{h.dev, G[i], reinterpret_cast<R*>(other[i]), P});
            const long long per = vec ? P * h.ncase / VV : P * h.ncase;
            blocks.push_back((unsigned)std::min<long long>((per + 255) / 256, 152LL * 16));
            std::swap(cur[i], other[i]);       // cur = the products
        }
        launch_groups(args, blocks, [&](const Grp<ProductArgs<R>>& g, unsigned total) {
            if (vec) k_products_grp<R, VV><<<total, 256, 0, st>>>(g);
            else k_products_grp<R, 1><<<total, 256, 0, st>>>(g);
            CNG_LAUNCH("k_products_grp");
        });
    }
    // x forward (r2c)
    std::vector<Planned<AxisArgs<R>>> xf;
    for (int i = 0; i < n; ++i) {
        const Rhs& h = *hs[i];
        const long long inner = (long long)(ndir == 2 ? h.mz : 1) * h.my;
        xf.push_back(plan_axis<R>(true, cur[i], other[i], (long long)h.noutputs * h.ncase, (int)inner, h.Kx, h.mx,
                                  true, h.maxseq, Expand<R>{}));
        std::swap(cur[i], other[i]);
    }
    launch_planned(xf, k_rfft_axis_grp<R>, threads, st, "k_rfft_axis_grp(forward)");
    if (ndir == 2) {
        std::vector<Planned<AxisArgs<R>>> z;
        for (int i = 0; i < n; ++i) {
            const Rhs& h = *hs[i];
            z.push_back(plan_axis<R>(false, cur[i], other[i], (long long)h.noutputs * h.ncase * h.Kx, h.my, h.Nzc,
                                     h.mz, true, h.maxseq, Expand<R>{}));
            std::swap(cur[i], other[i]);
        }
        launch_planned(z, k_fft_axis_grp<R>, threads, st, "k_fft_axis_grp(forward)");
    }
    // Chebyshev forward into S
    cheb.clear();
    for (int i = 0; i < n; ++i) {
        const Rhs& h = *hs[i];
        cheb.push_back(plan_cheb<R>(cur[i], static_cast<C*>(h.S), h.spec_cols(h.noutputs * h.ncase), h.ny, h.my,
                                    true, h.maxseq));
    }
    set_smem_attr<R>((const void*)k_cheb_fwd_grp<R>);
    launch_planned(cheb, k_cheb_fwd_grp<R>, threads, st, "k_cheb_fwd_grp");
    // pack and the constant parts
    {
        launch_pack<R>(hs, n, rows, st);
        std::vector<SparseArgs> sp;
        std::vector<unsigned> sb;
        for (int i = 0; i < n; ++i) {
            sp.push_back(SparseArgs{rows, hs[i]->b0_idx, hs[i]->b0_val, hs[i]->nb0});
            sb.push_back((unsigned)ceil_div(hs[i]->nb0, 256));
        }
        launch_groups(sp, sb, [&](const Grp<SparseArgs>& g, unsigned total) {
            k_add_sparse_grp<<<total, 256, 0, st>>>(g);
            CNG_LAUNCH("k_add_sparse_grp");
        });
    }
}

}  // namespace cng

// ================================================================================================
// C-ABI

using namespace cng;

static Rhs* build_rhs(const cng_rhs_desc* D) {
    if (!D) throw InvalidArgument("null descriptor");
    auto h = std::make_unique<Rhs>();
    h->precision = D->precision;
    if (D->precision != 0 && D->precision != 1) throw InvalidArgument("precision must be 0 (FP64) or 1 (FP32)");
    h->ndir = D->ndir;
    if (D->ndir < 0 || D->ndir > 2) throw InvalidArgument("0, 1 or 2 Fourier directions");
    h->nx = D->nx; h->nz = D->nz; h->mx = D->mx; h->mz = D->mz; h->ny = D->ny; h->my = D->my;
    h->lx = D->lx; h->lz = D->lz; h->ly = D->ly;
    if (!(h->ny == 1 && h->my == 1) && (h->ny < 1 || h->my < h->ny || h->my % 2))
        throw InvalidArgument("Chebyshev grid my must be even and >= ny (ny = my = 1: no Chebyshev direction)");
    if (h->ndir >= 1) {
        if (h->nx % 2 || h->mx < h->nx) throw InvalidArgument("Fourier sizes: nx even, mx >= nx");
        h->Kx = h->nx / 2;
        make_plan(h->mx);
    }
    if (h->ndir == 2) {
        if (h->nz % 2 || h->mz < h->nz) throw InvalidArgument("Fourier sizes: nz even, mz >= nz");
        h->Nzc = h->nz;
        make_plan(h->mz);
    }
    make_plan(h->my);
    h->nfactors = D->nfactors;
    h->noutputs = D->noutputs;
    if (h->nfactors < 1 || h->nfactors > 16) throw InvalidArgument("1 to 16 factors");
    if (h->noutputs < 1) throw InvalidArgument("at least one output");
    RhsDev& dv = h->dev;
    dv.ndir = h->ndir; dv.Kx = h->Kx; dv.Nzc = h->Nzc; dv.Ny = h->ny;
    dv.nfactors = h->nfactors; dv.noutputs = h->noutputs; dv.nbuckets = D->nbuckets;
    h->ncase = D->ncase > 0 ? D->ncase : 1;
    dv.ncase = h->ncase;
    dv.lx = h->lx; dv.lz = h->lz; dv.ly = h->ly;
    dv.factors = h->keep(upload(D->factors, (size_t)5 * h->nfactors));
    {   // transform groups: distinct (var, comp, oy) and (var, comp, oy, oz), first occurrence order
        std::vector<int> yrep, zy, zoz, fz(h->nfactors);
        std::vector<std::array<int, 3>> ykeys;
        std::vector<std::array<int, 4>> zkeys;
        for (int f = 0; f < h->nfactors; ++f) {
            const int* fd = D->factors + 5 * f;
            if (h->ndir < 2 && fd[4] != 0) throw InvalidArgument("z derivative without a z direction");
            if (h->ndir < 1 && fd[2] != 0) throw InvalidArgument("x derivative without an x direction");
            const std::array<int, 3> yk{fd[0], fd[1], fd[3]};
            int gy = (int)(std::find(ykeys.begin(), ykeys.end(), yk) - ykeys.begin());
            if (gy == (int)ykeys.size()) { ykeys.push_back(yk); yrep.push_back(f); }
            const std::array<int, 4> zk{fd[0], fd[1], fd[3], fd[4]};
            int gz = (int)(std::find(zkeys.begin(), zkeys.end(), zk) - zkeys.begin());
            if (gz == (int)zkeys.size()) { zkeys.push_back(zk); zy.push_back(gy); zoz.push_back(fd[4]); }
            fz[f] = gz;
        }
        if (h->ndir == 0 && (int)ykeys.size() != h->nfactors) throw InvalidArgument("repeated factor");
        dv.share = h->ndir >= 1 ? 1 : 0;
        if (!dv.share) {                    // one transform per factor
            ykeys.assign(h->nfactors, {0, 0, 0});
            zkeys.assign(h->nfactors, {0, 0, 0, 0});
            yrep.resize(h->nfactors);
            zy.resize(h->nfactors);
            zoz.assign(h->nfactors, 0);
            for (int f = 0; f < h->nfactors; ++f) yrep[f] = zy[f] = fz[f] = f;
        }
        dv.ngy = (int)ykeys.size();
        dv.ngz = (int)zkeys.size();
        dv.yg_rep = h->keep(upload(yrep.data(), yrep.size()));
        dv.zg_y = h->keep(upload(zy.data(), zy.size()));
        dv.zg_oz = h->keep(upload(zoz.data(), zoz.size()));
        dv.f_z = h->keep(upload(fz.data(), fz.size()));
        if (dv.share) {
            // (i k)^o per index along z (compact fftfreq slots) and x (modes 0..Kx-1), o = 1..max,
            // in the transform precision: fr + i fi by o quarter turns of k in double, then rounded
            std::vector<int> ox(h->nfactors);
            int maxz = 0, maxx = 0;
            for (int f = 0; f < h->nfactors; ++f) { ox[f] = D->factors[5 * f + 2]; maxx = std::max(maxx, ox[f]); }
            for (int o : zoz) maxz = std::max(maxz, o);
            auto table = [&](int nidx, int maxo, bool zaxis) -> void* {
                std::vector<double> re((size_t)std::max(1, maxo) * nidx), im(re.size());
                for (int o = 1; o <= maxo; ++o)
                    for (int j = 0; j < nidx; ++j) {
                        const int jj = zaxis ? (j < nidx / 2 ? j : j - nidx) : j;
                        const double k = 6.283185307179586476925286766559 * jj / (zaxis ? h->lz : h->lx);
                        double fr = 1.0, fi = 0.0;
                        for (int q = 0; q < o; ++q) { const double t = fr; fr = -fi * k; fi = t * k; }
                        re[(size_t)(o - 1) * nidx + j] = fr;
                        im[(size_t)(o - 1) * nidx + j] = fi;
                    }
                if (h->precision) {
                    std::vector<float2> t(re.size());
                    for (size_t i = 0; i < re.size(); ++i) t[i] = make_float2((float)re[i], (float)im[i]);
                    return h->keep(upload(t.data(), t.size()));
                }
                std::vector<double2> t(re.size());
                for (size_t i = 0; i < re.size(); ++i) t[i] = make_double2(re[i], im[i]);
                return h->keep(upload(t.data(), t.size()));
            };
            if (h->ndir == 2) h->ktab_z = table(h->Nzc, maxz, true);
            h->ktab_x = table(h->Kx, maxx, false);
            h->f_ox = h->keep(upload(ox.data(), ox.size()));
        }
    }
    dv.out_lam = h->keep(upload(D->out_lam, (size_t)h->noutputs));
    dv.out_mono_ptr = h->keep(upload(D->out_mono_ptr, (size_t)h->noutputs + 1));
    const int nmono = D->out_mono_ptr[h->noutputs];
    if (nmono > kMaxMono || h->noutputs > 16) throw InvalidArgument("at most 64 monomials and 16 outputs");
    for (int mi = 0; mi < 4 * nmono; ++mi)
        if (D->mono_factors[mi] >= h->nfactors) throw InvalidArgument("monomial factor id out of range");
    dv.mono_coef = h->keep(upload(D->mono_coef, (size_t)nmono));
    dv.mono_fac = h->keep(upload(D->mono_factors, (size_t)4 * nmono));
    int maxlam = 0;
    for (int o = 0; o < h->noutputs; ++o) maxlam = std::max(maxlam, D->out_lam[o]);
    if (maxlam > D->nlam) throw InvalidArgument("output lambda without a conversion matrix");
    std::vector<int> bw(std::max(1, D->nlam), 0), cstep(std::max(1, D->nlam), 2);
    for (int l = 0; l < D->nlam; ++l) {
        const double* cv = D->conv + (size_t)l * h->ny * h->ny;
        for (int i = 0; i < h->ny; ++i)
            for (int k = 0; k < h->ny; ++k)
                if (cv[(size_t)i * h->ny + k] != 0.0) {
                    if (k < i) throw InvalidArgument("conversion matrices must be upper triangular");
                    bw[l] = std::max(bw[l], k - i);
                    if ((k - i) & 1) cstep[l] = 1;
                }
    }
    dv.conv = h->keep(upload(D->conv, (size_t)std::max(1, D->nlam) * h->ny * h->ny * (D->nlam ? 1 : 0)));
    dv.conv_bw = h->keep(upload(bw.data(), bw.size()));
    dv.conv_step = h->keep(upload(cstep.data(), cstep.size()));
    for (int bi = 0; bi < D->nbuckets; ++bi) {
        const int* bd = D->buckets + 5 * bi;
        BucketDev b{};
        b.nsys = bd[0]; b.n = bd[1]; b.dact = bd[2]; b.sign = bd[3]; b.real = bd[4];
        b.offset = D->bucket_offset[bi];
        // shared memory of unpack and pack (four warps per block): the system's vector and two
        // columns, and the FP64 output spectra
        if ((size_t)4 * (b.n + 2 * h->ny) * sizeof(double2) > 200 * 1024 ||
            (size_t)4 * h->noutputs * h->ny * sizeof(double2) > 200 * 1024)
            throw InvalidArgument("system too long for the shared-memory unpack/pack");
        for (int m = 0; m < b.nsys; ++m) {
            const int jx = D->modes[bi][2 * m], jz = D->modes[bi][2 * m + 1];
            if (jx < 0 || (h->ndir >= 1 && jx >= h->Kx) || jz < 0 || (h->ndir == 2 && jz >= h->Nzc / 2))
                throw InvalidArgument("mode index out of range");
        }
        for (int q = 0; q < h->nfactors * h->ny; ++q)
            if (D->colpos[bi][q] >= b.n) throw InvalidArgument("column position out of range");
        for (int i = 0; i < b.n; ++i)
            if (D->rowmap[bi][2 * i] >= h->noutputs || D->rowmap[bi][2 * i + 1] >= h->ny)
                throw InvalidArgument("row map out of range");
        b.modes = h->keep(upload(D->modes[bi], (size_t)2 * b.nsys));
        b.colpos = h->keep(upload(D->colpos[bi], (size_t)h->nfactors * h->ny));
        b.rowmap = h->keep(upload(D->rowmap[bi], (size_t)2 * b.n));
        b.case_of = nullptr;
        if (h->ncase > 1) {
            if (!D->case_of || !D->case_of[bi]) throw InvalidArgument("stacked cases: a case index per system");
            for (int m = 0; m < b.nsys; ++m)
                if (D->case_of[bi][m] < 0 || D->case_of[bi][m] >= h->ncase) throw InvalidArgument("case index out of range");
            b.case_of = h->keep(upload(D->case_of[bi], (size_t)b.nsys));
        }
        h->buckets.push_back(b);
    }
    h->nb0 = D->nb0;
    if (h->nb0) {
        h->b0_idx = h->keep(upload(reinterpret_cast<const long long*>(D->b0_index), (size_t)h->nb0));
        h->b0_val = h->keep(upload(reinterpret_cast<const double2*>(D->b0_value), (size_t)h->nb0));
    }
    // work buffers
    const size_t cs = h->precision ? sizeof(float2) : sizeof(double2);
    const size_t rs = cs / 2;
    const int nfo = std::max(h->nfactors, h->noutputs) * h->ncase;
    const long long Kx = h->ndir >= 1 ? h->Kx : 1, Nzc = h->ndir == 2 ? h->Nzc : 1;
    const long long mx = h->ndir >= 1 ? h->mx : 1, mz = h->ndir == 2 ? h->mz : 1;
    const long long P = h->grid_points();
    h->S_bytes = std::max<size_t>(cs * nfo * Kx * Nzc * h->ny, rs * (size_t)h->nfactors * h->ncase * P);
    size_t w = 0;
    w = std::max<size_t>(w, cs * nfo * Kx * Nzc * h->my);
    w = std::max<size_t>(w, cs * nfo * Kx * mz * h->my);
    w = std::max<size_t>(w, rs * nfo * mx * mz * h->my);
    w = std::max<size_t>(w, cs * nfo * P);
    h->W_bytes = w;
    h->S = h->keep(dev_alloc(h->S_bytes));
    h->W1 = h->keep(dev_alloc(w));
    h->W2 = h->keep(dev_alloc(w));
    // the Nyquist and padding slots of the spectra are never written: zero them once
    CNG_CUDA(cudaMemset(h->S, 0, h->S_bytes));
    CNG_CUDA(cudaMemset(h->W1, 0, w));
    CNG_CUDA(cudaMemset(h->W2, 0, w));
    // on the device current at creation (the handle's device)
    ensure_smem_attr((const void*)k_unpack_grp<double>, 200 * 1024);
    ensure_smem_attr((const void*)k_unpack_grp<float>, 200 * 1024);
    ensure_smem_attr((const void*)k_pack_grp<double>, 200 * 1024);
    ensure_smem_attr((const void*)k_pack_grp<float>, 200 * 1024);
    return h.release();
}

extern "C" {

int cng_rhs_create(const cng_rhs_desc* desc, cng_rhs** out) {
    CNG_TRY({
        if (!out) throw InvalidArgument("null output handle");
        *out = nullptr;
        *out = reinterpret_cast<cng_rhs*>(build_rhs(desc));
    })
}

int cng_twiddle_table(int length, int precision, const void** table) {
    CNG_TRY({
        if (!table) throw InvalidArgument("null output");
        make_plan(length);
        *table = precision ? static_cast<const void*>(twiddles<float>().get(length, 0))
                           : static_cast<const void*>(twiddles<double>().get(length, 0));
    })
}

int cng_rhs_destroy(cng_rhs* h) {
    CNG_TRY({ delete reinterpret_cast<Rhs*>(h); })
}

int cng_rhs_evaluate(cng_rhs* hh, const void* state, void* rows, void* stream) {
    CNG_TRY({
        Rhs* h = reinterpret_cast<Rhs*>(hh);
        if (!h) throw InvalidArgument("null RHS handle");
        if (!state || !rows) throw InvalidArgument("null device pointer");
        if (state == rows) throw InvalidArgument("state and rows must not alias");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (h->precision == 0) h->run<double>(static_cast<const double2*>(state), static_cast<double2*>(rows), st);
        else h->run<float>(static_cast<const double2*>(state), static_cast<double2*>(rows), st);
    })
}

int cng_rhs_evaluate_group(int n, cng_rhs* const* hh, const void* state, void* rows, void* stream) {
    CNG_TRY({
        if (n <= 0 || !hh) throw InvalidArgument("grouped F: no handles");
        if (!state || !rows) throw InvalidArgument("null device pointer");
        if (state == rows) throw InvalidArgument("state and rows must not alias");
        std::vector<Rhs*> hs(n);
        for (int i = 0; i < n; ++i) {
            hs[i] = reinterpret_cast<Rhs*>(hh[i]);
            if (!hs[i]) throw InvalidArgument("null RHS handle");
            for (int j = 0; j < i; ++j)
                if (hs[j] == hs[i]) throw InvalidArgument("grouped F: a handle appears twice (shared work buffers)");
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const double2* s = static_cast<const double2*>(state);
        double2* r = static_cast<double2*>(rows);
        if (hs[0]->precision == 0) run_group<double>(hs.data(), n, s, r, st);
        else run_group<float>(hs.data(), n, s, r, st);
    })
}

int cng_rhs_set_tuning(cng_rhs* hh, int maxseq, int threads) {
    CNG_TRY({
        Rhs* h = reinterpret_cast<Rhs*>(hh);
        if (!h) throw InvalidArgument("null handle");
        if (maxseq < 0 || maxseq > 32) throw InvalidArgument("sequences per block: 0 (default) to 32");
        if (threads != 0 && (threads < 64 || threads > 512 || threads % 32))
            throw InvalidArgument("threads per block: 0 (default) or a multiple of 32 in 64..512");
        h->maxseq = maxseq;
        h->threads = threads;
    })
}

int cng_rhs_workspace_bytes(const cng_rhs* hh, uint64_t* bytes) {
    CNG_TRY({
        const Rhs* h = reinterpret_cast<const Rhs*>(hh);
        if (!h || !bytes) throw InvalidArgument("null argument");
        *bytes = h->S_bytes + 2 * h->W_bytes;
    })
}

// Standalone transforms on caller-owned device memory (complex128 columns / axes).
int cng_cheb_transform(int forward, const void* in, void* out, int64_t ncols, int n, int m, void* stream) {
    CNG_TRY({
        if (!in || !out) throw InvalidArgument("null device pointer");
        if (n < 1 || m < n) throw InvalidArgument("need 1 <= n <= m");
        launch_cheb<double>(static_cast<const double2*>(in), static_cast<double2*>(out), ncols, n, m,
                            forward != 0, static_cast<cudaStream_t>(stream));
    })
}

int cng_fft_axis(int forward, const void* in, void* out, int64_t outer, int inner, int ncompact, int length,
                 void* stream) {
    CNG_TRY({
        if (!in || !out) throw InvalidArgument("null device pointer");
        if (ncompact % 2 || ncompact > length) throw InvalidArgument("compact size must be even and <= length");
        launch_fft_axis<double>(static_cast<const double2*>(in), static_cast<double2*>(out), outer, inner,
                                ncompact, length, forward != 0, static_cast<cudaStream_t>(stream));
    })
}

int cng_rfft_axis(int forward, const void* in, void* out, int64_t outer, int inner, int nmodes, int length,
                  void* stream) {
    CNG_TRY({
        if (!in || !out) throw InvalidArgument("null device pointer");
        if (nmodes < 1 || 2 * (nmodes - 1) >= length) throw InvalidArgument("need 2 (nmodes - 1) < length");
        launch_rfft_axis<double>(in, out, outer, inner, nmodes, length, forward != 0,
                                 static_cast<cudaStream_t>(stream));
    })
}

}  // extern "C"
