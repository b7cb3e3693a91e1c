// Shared-memory batched FFT core (complex, mixed radix 2/3/4/5/8, Stockham autosort) used by the
// Fourier and Chebyshev transform kernels of the spectral pipeline.
//
// One CTA transforms B sequences of length L held in shared memory (two ping-pong buffers of
// B*L complex values). Stage s with radix R and stride Ns (product of the earlier radices) maps
// a -> b by   v_t = a[j + t L/R] * w^(t (j % Ns) L/(Ns R)),   v = DFT_R(v),
//             b[(j / Ns) Ns R + j % Ns + t Ns] = v_t,          j < L/R,
// which leaves the result in natural order after the last stage (Stockham autosort). Twiddles
// w^q = exp(sign 2 pi i q / L) come from a table computed on the host in double precision.
#pragma once

#include <cuda_runtime.h>

namespace cng {

template <class R> struct c2t;
template <> struct c2t<double> { using type = double2; };
template <> struct c2t<float> { using type = float2; };

template <class R> using c2 = typename c2t<R>::type;

template <class R> __device__ __forceinline__ c2<R> mk(R x, R y) { c2<R> v; v.x = x; v.y = y; return v; }
template <class R> __device__ __forceinline__ c2<R> add(c2<R> a, c2<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <class R> __device__ __forceinline__ c2<R> sub(c2<R> a, c2<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <class R> __device__ __forceinline__ c2<R> mul(c2<R> a, c2<R> b) {
    return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class R> __device__ __forceinline__ c2<R> scl(R s, c2<R> a) { return mk<R>(s * a.x, s * a.y); }
template <class R> __device__ __forceinline__ c2<R> conjg(c2<R> a) { return mk<R>(a.x, -a.y); }
// fused multiply-add in the transform precision
__device__ __forceinline__ double fmar(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmar(float a, float b, float c) { return fmaf(a, b, c); }

// multiply by S i (S = -1 forward, +1 inverse)
template <class R, int S> __device__ __forceinline__ c2<R> muli(c2<R> a) {
    return S > 0 ? mk<R>(-a.y, a.x) : mk<R>(a.y, -a.x);
}

// Stage plan: radices of L (product = L), at most 12 stages.
struct FftPlan {
    int L;
    int nstages;
    int radix[12];
};

// Exact small DFTs of size R with sign S (-1 forward, +1 inverse), in place on v[0..R). A product
// that feeds a sum and a difference is fused into both (two fused multiply-adds instead of a
// multiply and two adds); the sign is a compile-time constant, so no arithmetic goes into it.
template <class R>
__device__ __forceinline__ void dft2(c2<R>* v) {
    c2<R> a = v[0], b = v[1];
    v[0] = add<R>(a, b);
    v[1] = sub<R>(a, b);
}

template <class R, int S>
__device__ __forceinline__ void dft4(c2<R>* v) {
    c2<R> a0 = add<R>(v[0], v[2]), a1 = sub<R>(v[0], v[2]);
    c2<R> b0 = add<R>(v[1], v[3]), b1 = muli<R, S>(sub<R>(v[1], v[3]));
    v[0] = add<R>(a0, b0);
    v[2] = sub<R>(a0, b0);
    v[1] = add<R>(a1, b1);
    v[3] = sub<R>(a1, b1);
}

template <class R, int S>
__device__ __forceinline__ void dft3(c2<R>* v) {
    const R s = R(S) * R(0.86602540378443864676372317075294);   // sqrt(3)/2
    const c2<R> t1 = add<R>(v[1], v[2]);
    const c2<R> t2 = sub<R>(v[1], v[2]);
    const c2<R> m1 = mk<R>(fmar(R(-0.5), t1.x, v[0].x), fmar(R(-0.5), t1.y, v[0].y));
    v[0] = add<R>(v[0], t1);
    // m1 +- i s t2, i s t2 = (-s t2.y, s t2.x)
    v[1] = mk<R>(fmar(-s, t2.y, m1.x), fmar(s, t2.x, m1.y));
    v[2] = mk<R>(fmar(s, t2.y, m1.x), fmar(-s, t2.x, m1.y));
}

template <class R, int S>
__device__ __forceinline__ void dft5(c2<R>* v) {
    const R c1 = R(0.30901699437494742410229341718282);    // cos(2 pi/5)
    const R c2v = R(-0.80901699437494742410229341718282);  // cos(4 pi/5)
    const R s1 = R(S) * R(0.95105651629515357211643933337938);   // sin(2 pi/5)
    const R s2 = R(S) * R(0.58778525229247312916870595463907);   // sin(4 pi/5)
    const c2<R> t1 = add<R>(v[1], v[4]), t2 = add<R>(v[2], v[3]);
    const c2<R> t3 = sub<R>(v[1], v[4]), t4 = sub<R>(v[2], v[3]);
    const c2<R> a1 = mk<R>(fmar(c2v, t2.x, fmar(c1, t1.x, v[0].x)), fmar(c2v, t2.y, fmar(c1, t1.y, v[0].y)));
    const c2<R> a2 = mk<R>(fmar(c1, t2.x, fmar(c2v, t1.x, v[0].x)), fmar(c1, t2.y, fmar(c2v, t1.y, v[0].y)));
    // b1 = i (s1 t3 + s2 t4), b2 = i (s2 t3 - s1 t4)
    const c2<R> u1 = mk<R>(fmar(s1, t3.x, s2 * t4.x), fmar(s1, t3.y, s2 * t4.y));
    const c2<R> u2 = mk<R>(fmar(s2, t3.x, -(s1 * t4.x)), fmar(s2, t3.y, -(s1 * t4.y)));
    const c2<R> b1 = mk<R>(-u1.y, u1.x), b2 = mk<R>(-u2.y, u2.x);
    v[0] = add<R>(v[0], add<R>(t1, t2));
    v[1] = add<R>(a1, b1);
    v[4] = sub<R>(a1, b1);
    v[2] = add<R>(a2, b2);
    v[3] = sub<R>(a2, b2);
}

template <class R, int S>
__device__ __forceinline__ void dft8(c2<R>* v) {
    // two radix-4 DFTs on even/odd entries, then the radix-2 combination with w8^k
    c2<R> e[4] = {v[0], v[2], v[4], v[6]};
    c2<R> o[4] = {v[1], v[3], v[5], v[7]};
    dft4<R, S>(e);
    dft4<R, S>(o);
    const R h = R(0.70710678118654752440084436210485);
    // w8^1 o1 = h (o1.x - S o1.y, o1.y + S o1.x); w8^2 = S i; w8^3 o3 = h (-(o3.x + S o3.y), S o3.x - o3.y)
    const R p1x = S > 0 ? o[1].x - o[1].y : o[1].x + o[1].y;
    const R p1y = S > 0 ? o[1].y + o[1].x : o[1].y - o[1].x;
    const R q3x = S > 0 ? o[3].x + o[3].y : o[3].x - o[3].y;      // w8^3 o3 .x = -h q3x
    const R q3y = S > 0 ? o[3].x - o[3].y : o[3].x + o[3].y;      // w8^3 o3 .y = S' h q3y
    const R h3y = S > 0 ? h : -h;
    const c2<R> o2 = muli<R, S>(o[2]);
    v[0] = add<R>(e[0], o[0]);
    v[4] = sub<R>(e[0], o[0]);
    v[1] = mk<R>(fmar(h, p1x, e[1].x), fmar(h, p1y, e[1].y));
    v[5] = mk<R>(fmar(-h, p1x, e[1].x), fmar(-h, p1y, e[1].y));
    v[2] = add<R>(e[2], o2);
    v[6] = sub<R>(e[2], o2);
    v[3] = mk<R>(fmar(-h, q3x, e[3].x), fmar(h3y, q3y, e[3].y));
    v[7] = mk<R>(fmar(h, q3x, e[3].x), fmar(-h3y, q3y, e[3].y));
}

template <class R, int S, int RAD>
__device__ __forceinline__ void dft(c2<R>* v) {
    if constexpr (RAD == 2) dft2<R>(v);
    else if constexpr (RAD == 3) dft3<R, S>(v);
    else if constexpr (RAD == 4) dft4<R, S>(v);
    else if constexpr (RAD == 5) dft5<R, S>(v);
    else dft8<R, S>(v);
}

template <class R, int S, int RAD>
__device__ __forceinline__ void stage(const c2<R>* __restrict__ a, c2<R>* __restrict__ b, int L, int LS, int Ns,
                                      int B, const c2<R>* tw, int tid, int nthreads) {
    const int Lr = L / RAD;
    const int tstep = L / (Ns * RAD);
    for (int idx = tid; idx < B * Lr; idx += nthreads) {
        const int bt = idx / Lr;
        const int j = idx - bt * Lr;
        const c2<R>* ab = a + bt * LS;
        c2<R>* bb = b + bt * LS;
        const int k = j % Ns;
        c2<R> v[RAD];
#pragma unroll
        for (int t = 0; t < RAD; ++t) v[t] = ab[j + t * Lr];
#pragma unroll
        for (int t = 1; t < RAD; ++t) {
            int q = (t * k * tstep) % L;
            c2<R> w = tw[q];
            if (S > 0) w.y = -w.y;
            v[t] = mul<R>(v[t], w);
        }
        dft<R, S, RAD>(v);
        const int d = (j / Ns) * Ns * RAD + k;
#pragma unroll
        for (int t = 0; t < RAD; ++t) bb[d + t * Ns] = v[t];
    }
}

// Transform B sequences in buf0 (length L each, row stride LS >= L: rows padded against bank
// conflicts); result in buf0 or buf1 (returned). tw: L twiddles exp(-2 pi i q / L) in shared memory.
// Caller synchronizes before the call.
template <class R, int S>
__device__ c2<R>* smem_fft(c2<R>* buf0, c2<R>* buf1, const FftPlan& p, int B, const c2<R>* tw, int LS) {
    const int tid = threadIdx.x, nt = blockDim.x;
    c2<R>* a = buf0;
    c2<R>* b = buf1;
    int Ns = 1;
    for (int s = 0; s < p.nstages; ++s) {
        const int rad = p.radix[s];
        switch (rad) {
            case 2: stage<R, S, 2>(a, b, p.L, LS, Ns, B, tw, tid, nt); break;
            case 3: stage<R, S, 3>(a, b, p.L, LS, Ns, B, tw, tid, nt); break;
            case 4: stage<R, S, 4>(a, b, p.L, LS, Ns, B, tw, tid, nt); break;
            case 5: stage<R, S, 5>(a, b, p.L, LS, Ns, B, tw, tid, nt); break;
            default: stage<R, S, 8>(a, b, p.L, LS, Ns, B, tw, tid, nt); break;
        }
        __syncthreads();
        Ns *= rad;
        c2<R>* t = a;
        a = b;
        b = t;
    }
    return a;
}

// ---- compile-time plans: the same Stockham stages with L, Ns and the radix known at compile time.
// A thread takes one butterfly position j and a group g of the B sequences: the twiddles and the
// index arithmetic of j are computed once and reused for the sequences g, g + G, ... (G = number
// of groups), which keeps the integer work per butterfly low (the FP32 transforms were bound by it).
template <class R, int S, int L, int Ns, int RAD>
__device__ __forceinline__ void stage_ct(const c2<R>* __restrict__ a, c2<R>* __restrict__ b, int B,
                                         const c2<R>* tw, int LS) {
    constexpr int Lr = L / RAD;
    constexpr int tstep = L / (Ns * RAD);
    const int nt = blockDim.x;
    if constexpr (Ns == 1 || (Ns < 32 && sizeof(R) == 8)) {
        // early stages (short runs of Ns consecutive outputs): the sequence index fastest across
        // the threads, so the stride-RAD writes of neighbouring threads fall in rows LS apart (LS
        // odd: other banks) instead of Ns RAD elements apart in one row (a few banks for all).
        // Measured on the channel's F: the first stage in both precisions (FP32 2.40 -> 2.20 ms),
        // the twiddled early stages in FP64 only (FP64 15.29 -> 14.94 ms; FP32 lost 0.07 ms: its
        // twiddles are then loaded per butterfly instead of once per thread)
        if ((B & (B - 1)) == 0) {
            const int sh = __ffs(B) - 1;
            for (int q = threadIdx.x; q < Lr * B; q += nt) {
                const int bt = q & (B - 1), j = q >> sh;
                const int k = j % Ns;
                const c2<R>* ab = a + bt * LS + j;
                c2<R>* bb = b + bt * LS + (j / Ns) * Ns * RAD + k;
                c2<R> v[RAD];
#pragma unroll
                for (int t = 0; t < RAD; ++t) v[t] = ab[t * Lr];
                if (Ns > 1) {
#pragma unroll
                    for (int t = 1; t < RAD; ++t) {
                        c2<R> w = tw[t * k * tstep];
                        if (S > 0) w.y = -w.y;
                        v[t] = mul<R>(v[t], w);
                    }
                }
                dft<R, S, RAD>(v);
#pragma unroll
                for (int t = 0; t < RAD; ++t) bb[t * Ns] = v[t];
            }
            return;
        }
    }
    const int G = nt >= Lr ? nt / Lr : 1;
    for (int q = threadIdx.x; q < Lr * G; q += nt) {
        const int j = q % Lr, g = q / Lr;
        const int k = j % Ns;
        const int d = (j / Ns) * Ns * RAD + k;
        c2<R> w[RAD];
        if (Ns > 1) {
#pragma unroll
            for (int t = 1; t < RAD; ++t) {
                w[t] = tw[t * k * tstep];
                if (S > 0) w[t].y = -w[t].y;
            }
        }
        for (int bt = g; bt < B; bt += G) {
            const c2<R>* ab = a + bt * LS + j;
            c2<R>* bb = b + bt * LS + d;
            c2<R> v[RAD];
#pragma unroll
            for (int t = 0; t < RAD; ++t) v[t] = ab[t * Lr];
            if (Ns > 1) {
#pragma unroll
                for (int t = 1; t < RAD; ++t) v[t] = mul<R>(v[t], w[t]);
            }
            dft<R, S, RAD>(v);
#pragma unroll
            for (int t = 0; t < RAD; ++t) bb[t * Ns] = v[t];
        }
    }
}

template <class R, int S, int L, int Ns, int RAD, int... REST>
__device__ __forceinline__ c2<R>* run_ct(c2<R>* a, c2<R>* b, int B, const c2<R>* tw, int LS) {
    stage_ct<R, S, L, Ns, RAD>(a, b, B, tw, LS);
    __syncthreads();
    if constexpr (sizeof...(REST) == 0) {
        return b;
    } else {
        return run_ct<R, S, L, Ns * RAD, REST...>(b, a, B, tw, LS);
    }
}

// Lengths of the benchmark configurations get compile-time plans; others take the runtime plan.
template <class R, int S>
__device__ c2<R>* smem_fft_signed(c2<R>* b0, c2<R>* b1, const FftPlan& p, int B, const c2<R>* tw, int LS) {
    switch (p.L) {
        case 12: return run_ct<R, S, 12, 1, 4, 3>(b0, b1, B, tw, LS);
        case 24: return run_ct<R, S, 24, 1, 8, 3>(b0, b1, B, tw, LS);
        case 30: return run_ct<R, S, 30, 1, 2, 3, 5>(b0, b1, B, tw, LS);
        case 32: return run_ct<R, S, 32, 1, 8, 4>(b0, b1, B, tw, LS);
        case 48: return run_ct<R, S, 48, 1, 4, 4, 3>(b0, b1, B, tw, LS);
        case 64: return run_ct<R, S, 64, 1, 8, 8>(b0, b1, B, tw, LS);
        case 72: return run_ct<R, S, 72, 1, 8, 3, 3>(b0, b1, B, tw, LS);
        case 96: return run_ct<R, S, 96, 1, 8, 4, 3>(b0, b1, B, tw, LS);
        case 128: return run_ct<R, S, 128, 1, 8, 4, 4>(b0, b1, B, tw, LS);
        case 144: return run_ct<R, S, 144, 1, 4, 4, 3, 3>(b0, b1, B, tw, LS);
        case 192: return run_ct<R, S, 192, 1, 8, 8, 3>(b0, b1, B, tw, LS);
        case 200: return run_ct<R, S, 200, 1, 8, 5, 5>(b0, b1, B, tw, LS);
        case 256: return run_ct<R, S, 256, 1, 8, 8, 4>(b0, b1, B, tw, LS);
        case 288: return run_ct<R, S, 288, 1, 8, 4, 3, 3>(b0, b1, B, tw, LS);
        case 384: return run_ct<R, S, 384, 1, 8, 4, 4, 3>(b0, b1, B, tw, LS);
        default: return smem_fft<R, S>(b0, b1, p, B, tw, LS);
    }
}

// sign -1: forward (exp(-2 pi i ...)), +1: inverse
template <class R>
__device__ __forceinline__ c2<R>* smem_fft_fast(c2<R>* b0, c2<R>* b1, const FftPlan& p, int B, const c2<R>* tw,
                                                int sign, int LS) {
    return sign > 0 ? smem_fft_signed<R, 1>(b0, b1, p, B, tw, LS) : smem_fft_signed<R, -1>(b0, b1, p, B, tw, LS);
}

}  // namespace cng
