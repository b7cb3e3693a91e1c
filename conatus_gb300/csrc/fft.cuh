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
// multiply by sign*i
template <class R> __device__ __forceinline__ c2<R> muli(c2<R> a, int sign) {
    return sign > 0 ? mk<R>(-a.y, a.x) : mk<R>(a.y, -a.x);
}

// Stage plan: radices of L (product = L), at most 12 stages.
struct FftPlan {
    int L;
    int nstages;
    int radix[12];
};

// Exact small DFTs of size R (sign = -1 forward, +1 inverse), in place on v[0..R).
template <class R>
__device__ __forceinline__ void dft2(c2<R>* v) {
    c2<R> a = v[0], b = v[1];
    v[0] = add<R>(a, b);
    v[1] = sub<R>(a, b);
}

template <class R>
__device__ __forceinline__ void dft4(c2<R>* v, int sign) {
    c2<R> a0 = add<R>(v[0], v[2]), a1 = sub<R>(v[0], v[2]);
    c2<R> b0 = add<R>(v[1], v[3]), b1 = muli<R>(sub<R>(v[1], v[3]), sign);
    v[0] = add<R>(a0, b0);
    v[2] = sub<R>(a0, b0);
    v[1] = add<R>(a1, b1);
    v[3] = sub<R>(a1, b1);
}

template <class R>
__device__ __forceinline__ void dft3(c2<R>* v, int sign) {
    const R c = R(-0.5);
    const R s = R(sign) * R(0.86602540378443864676372317075294);   // sqrt(3)/2
    c2<R> t1 = add<R>(v[1], v[2]);
    c2<R> t2 = sub<R>(v[1], v[2]);
    c2<R> m1 = add<R>(v[0], scl<R>(c, t1));
    c2<R> m2 = mk<R>(-s * t2.y, s * t2.x);
    v[0] = add<R>(v[0], t1);
    v[1] = add<R>(m1, m2);
    v[2] = sub<R>(m1, m2);
}

template <class R>
__device__ __forceinline__ void dft5(c2<R>* v, int sign) {
    const R c1 = R(0.30901699437494742410229341718282);    // cos(2 pi/5)
    const R c2v = R(-0.80901699437494742410229341718282);  // cos(4 pi/5)
    const R s1 = R(sign) * R(0.95105651629515357211643933337938);   // sin(2 pi/5)
    const R s2 = R(sign) * R(0.58778525229247312916870595463907);   // sin(4 pi/5)
    c2<R> t1 = add<R>(v[1], v[4]), t2 = add<R>(v[2], v[3]);
    c2<R> t3 = sub<R>(v[1], v[4]), t4 = sub<R>(v[2], v[3]);
    c2<R> a1 = add<R>(v[0], add<R>(scl<R>(c1, t1), scl<R>(c2v, t2)));
    c2<R> a2 = add<R>(v[0], add<R>(scl<R>(c2v, t1), scl<R>(c1, t2)));
    // b1 = i (s1 t3 + s2 t4), b2 = i (s2 t3 - s1 t4)
    c2<R> u1 = add<R>(scl<R>(s1, t3), scl<R>(s2, t4));
    c2<R> u2 = sub<R>(scl<R>(s2, t3), scl<R>(s1, t4));
    c2<R> b1 = mk<R>(-u1.y, u1.x), b2 = mk<R>(-u2.y, u2.x);
    v[0] = add<R>(v[0], add<R>(t1, t2));
    v[1] = add<R>(a1, b1);
    v[4] = sub<R>(a1, b1);
    v[2] = add<R>(a2, b2);
    v[3] = sub<R>(a2, b2);
}

template <class R>
__device__ __forceinline__ void dft8(c2<R>* v, int sign) {
    // two radix-4 DFTs on even/odd entries, then the radix-2 combination with w8^k
    c2<R> e[4] = {v[0], v[2], v[4], v[6]};
    c2<R> o[4] = {v[1], v[3], v[5], v[7]};
    dft4<R>(e, sign);
    dft4<R>(o, sign);
    const R h = R(0.70710678118654752440084436210485);
    // w8^1 = (h, sign h), w8^2 = sign i, w8^3 = (-h, sign h)
    c2<R> o1 = mk<R>(h * (o[1].x - R(sign) * o[1].y), h * (o[1].y + R(sign) * o[1].x));
    c2<R> o2 = muli<R>(o[2], sign);
    c2<R> o3 = mk<R>(-h * (o[3].x + R(sign) * o[3].y), h * (R(sign) * o[3].x - o[3].y));
    v[0] = add<R>(e[0], o[0]);
    v[4] = sub<R>(e[0], o[0]);
    v[1] = add<R>(e[1], o1);
    v[5] = sub<R>(e[1], o1);
    v[2] = add<R>(e[2], o2);
    v[6] = sub<R>(e[2], o2);
    v[3] = add<R>(e[3], o3);
    v[7] = sub<R>(e[3], o3);
}

template <class R, int RAD>
__device__ __forceinline__ void stage(const c2<R>* __restrict__ a, c2<R>* __restrict__ b, int L, int LS, int Ns,
                                      int B, const c2<R>* tw, int sign, int tid, int nthreads) {
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
            if (sign > 0) w.y = -w.y;
            v[t] = mul<R>(v[t], w);
        }
        if constexpr (RAD == 2) dft2<R>(v);
        else if constexpr (RAD == 3) dft3<R>(v, sign);
        else if constexpr (RAD == 4) dft4<R>(v, sign);
        else if constexpr (RAD == 5) dft5<R>(v, sign);
        else dft8<R>(v, sign);
        const int d = (j / Ns) * Ns * RAD + k;
#pragma unroll
        for (int t = 0; t < RAD; ++t) bb[d + t * Ns] = v[t];
    }
}

// Transform B sequences in buf0 (length L each, row stride LS >= L: rows padded against bank
// conflicts); result in buf0 or buf1 (returned). tw: L twiddles exp(-2 pi i q / L) in shared memory.
// Caller synchronizes before the call.
template <class R>
__device__ c2<R>* smem_fft(c2<R>* buf0, c2<R>* buf1, const FftPlan& p, int B, const c2<R>* tw,
                           int sign, int LS) {
    const int tid = threadIdx.x, nt = blockDim.x;
    c2<R>* a = buf0;
    c2<R>* b = buf1;
    int Ns = 1;
    for (int s = 0; s < p.nstages; ++s) {
        const int rad = p.radix[s];
        switch (rad) {
            case 2: stage<R, 2>(a, b, p.L, LS, Ns, B, tw, sign, tid, nt); break;
            case 3: stage<R, 3>(a, b, p.L, LS, Ns, B, tw, sign, tid, nt); break;
            case 4: stage<R, 4>(a, b, p.L, LS, Ns, B, tw, sign, tid, nt); break;
            case 5: stage<R, 5>(a, b, p.L, LS, Ns, B, tw, sign, tid, nt); break;
            default: stage<R, 8>(a, b, p.L, LS, Ns, B, tw, sign, tid, nt); break;
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
template <class R, int L, int Ns, int RAD>
__device__ __forceinline__ void stage_ct(const c2<R>* __restrict__ a, c2<R>* __restrict__ b, int B,
                                         const c2<R>* tw, int sign, int LS) {
    constexpr int Lr = L / RAD;
    constexpr int tstep = L / (Ns * RAD);
    const int nt = blockDim.x;
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
                if (sign > 0) w[t].y = -w[t].y;
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
            if constexpr (RAD == 2) dft2<R>(v);
            else if constexpr (RAD == 3) dft3<R>(v, sign);
            else if constexpr (RAD == 4) dft4<R>(v, sign);
            else if constexpr (RAD == 5) dft5<R>(v, sign);
            else dft8<R>(v, sign);
#pragma unroll
            for (int t = 0; t < RAD; ++t) bb[t * Ns] = v[t];
        }
    }
}

template <class R, int L, int Ns, int RAD, int... REST>
__device__ __forceinline__ c2<R>* run_ct(c2<R>* a, c2<R>* b, int B, const c2<R>* tw, int sign, int LS) {
    stage_ct<R, L, Ns, RAD>(a, b, B, tw, sign, LS);
    __syncthreads();
    if constexpr (sizeof...(REST) == 0) {
        return b;
    } else {
        return run_ct<R, L, Ns * RAD, REST...>(b, a, B, tw, sign, LS);
    }
}

// Lengths of the benchmark configurations get compile-time plans; others take the runtime plan.
template <class R>
__device__ c2<R>* smem_fft_fast(c2<R>* b0, c2<R>* b1, const FftPlan& p, int B, const c2<R>* tw, int sign,
                                int LS) {
    switch (p.L) {
        case 12: return run_ct<R, 12, 1, 4, 3>(b0, b1, B, tw, sign, LS);
        case 24: return run_ct<R, 24, 1, 8, 3>(b0, b1, B, tw, sign, LS);
        case 30: return run_ct<R, 30, 1, 2, 3, 5>(b0, b1, B, tw, sign, LS);
        case 32: return run_ct<R, 32, 1, 8, 4>(b0, b1, B, tw, sign, LS);
        case 48: return run_ct<R, 48, 1, 4, 4, 3>(b0, b1, B, tw, sign, LS);
        case 64: return run_ct<R, 64, 1, 8, 8>(b0, b1, B, tw, sign, LS);
        case 72: return run_ct<R, 72, 1, 8, 3, 3>(b0, b1, B, tw, sign, LS);
        case 96: return run_ct<R, 96, 1, 8, 4, 3>(b0, b1, B, tw, sign, LS);
        case 128: return run_ct<R, 128, 1, 8, 4, 4>(b0, b1, B, tw, sign, LS);
        case 144: return run_ct<R, 144, 1, 4, 4, 3, 3>(b0, b1, B, tw, sign, LS);
        case 192: return run_ct<R, 192, 1, 8, 8, 3>(b0, b1, B, tw, sign, LS);
        case 200: return run_ct<R, 200, 1, 8, 5, 5>(b0, b1, B, tw, sign, LS);
        case 256: return run_ct<R, 256, 1, 8, 8, 4>(b0, b1, B, tw, sign, LS);
        case 288: return run_ct<R, 288, 1, 8, 4, 3, 3>(b0, b1, B, tw, sign, LS);
        case 384: return run_ct<R, 384, 1, 8, 4, 4, 3>(b0, b1, B, tw, sign, LS);
        default: return smem_fft<R>(b0, b1, p, B, tw, sign, LS);
    }
}

}  // namespace cng
