// Ensembles of one-dimensional periodic IMEX problems (Kuramoto-Sivashinsky and the like), every
// member advanced by one fused kernel per step: one CTA per member, members of different sizes and
// periods in the same launch.
//
// A member with N RealFourier coefficients holds K = N/2 complex mode amplitudes C_k (the reference's
// complexified (cos, -sin) pairs, C_0 real). Its step is the reference's SBDF step
// (python/conatus/timestep/integrator.py:361-373) with diagonal implicit systems (each Fourier mode
// is a 1 x 1 system a M(k) + b L(k)):
//   F   = the polynomial form of the right-hand side (fused.py:524-537) on the 3/2-dealiased grid:
//         factors (i k)^o u_hat, inverse real FFT (two factors per complex FFT), products, forward
//         real FFT, truncation; rows 2 F_hat_k (1 for the mean mode)
//   rhs = sum_j c_j F_j - d_j M C_j (lincomb.py:146-162), C_new = rhs / (a0/dt M(k) + L(k))
// The history ring (M C and F of the last q steps) stays in device memory. FFTs and products in R
// (double, or float for the mixed form); state, history and the solve in double.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "conatus_gb300.h"
#include "fft.cuh"

namespace cng {

FftPlan make_plan(int L);

struct EnsArgs {
    int nmem, nfactors, nmono, q, head;
    const int* N;
    const int* M;
    const long long* off;
    const double* len;
    const int* plan_idx;
    FftPlan plans[4];
    const void* tw[4];
    int factor_order[4];
    double mono_coef[4];
    int mono_fac[16];
    double mre[5], mim[5], lre[5], lim[5];     // M(k), L(k) for k > 0: sum_t c_t k^t
    double m0re, m0im, l0re, l0im;             // the mean mode
    double c[4], d[4];                         // SBDF weights of F_j and M C_j (j = 0: newest)
    double a0dt;
    double2* X;
    double2* MXh[4];
    double2* Fh[4];
};

template <class R>
__global__ void __launch_bounds__(128) k_fourier_ensemble_step(EnsArgs a) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int m = blockIdx.x;
    if (m >= a.nmem) return;
    const int N = a.N[m], M = a.M[m], K = N / 2;
    const int pi = a.plan_idx[m];
    const FftPlan& plan = a.plans[pi];
    const c2<R>* twg = static_cast<const c2<R>*>(a.tw[pi]);
    c2<R>* tw = reinterpret_cast<c2<R>*>(sm);
    c2<R>* b0 = tw + M;
    c2<R>* b1 = b0 + M;
    R* grid = reinterpret_cast<R*>(b1 + M);             // nfactors x M real
    double2* Rk = reinterpret_cast<double2*>(grid + (size_t)((a.nfactors * M + 3) & ~3));
    const int tid = threadIdx.x, nt = blockDim.x;
    const double kscale = 6.283185307179586476925286766559 / a.len[m];
    const double2* C = a.X + a.off[m];
    for (int q = tid; q < M; q += nt) tw[q] = twg[q];
    // factor grids, two per complex inverse FFT
    for (int f0 = 0; f0 < a.nfactors; f0 += 2) {
        const int f1 = f0 + 1 < a.nfactors ? f0 + 1 : -1;
        for (int q = tid; q < M; q += nt) b0[q] = mk<R>(0, 0);
        __syncthreads();
        for (int k = tid; k < K; k += nt) {
            const double2 c = C[k];
            const double w = k == 0 ? 1.0 : 0.5;             // FFT coefficient of the amplitude
            const double kk = k * kscale;
            double ar[2] = {0, 0}, ai[2] = {0, 0};
            for (int s = 0; s < 2; ++s) {
                const int f = s == 0 ? f0 : f1;
                if (f < 0) continue;
                double re = w * c.x, im = k == 0 ? 0.0 : w * c.y;
                for (int o = 0; o < a.factor_order[f]; ++o) {   // times i k
                    const double t = re;
                    re = -im * kk;
                    im = t * kk;
                }
                ar[s] = re;
                ai[s] = im;
            }
            // Z_k = A_k + i B_k, Z_{M-k} = conj(A_k) + i conj(B_k)
            b0[k] = mk<R>(R(ar[0] - ai[1]), R(ai[0] + ar[1]));
            if (k > 0) b0[M - k] = mk<R>(R(ar[0] + ai[1]), R(-ai[0] + ar[1]));
        }
        __syncthreads();
        c2<R>* z = smem_fft_fast<R>(b0, b1, plan, 1, tw, +1, M);
        for (int j = tid; j < M; j += nt) {
            grid[(size_t)f0 * M + j] = z[j].x;
            if (f1 >= 0) grid[(size_t)f1 * M + j] = z[j].y;
        }
        __syncthreads();
    }
    // products (one output), then the forward real FFT
    for (int j = tid; j < M; j += nt) {
        R acc = R(0);
        for (int mi = 0; mi < a.nmono; ++mi) {
            R t = R(a.mono_coef[mi]);
            for (int q = 0; q < 4; ++q) {
                const int f = a.mono_fac[4 * mi + q];
                if (f >= 0) t = t * grid[(size_t)f * M + j];
            }
            acc = acc + t;
        }
        b0[j] = mk<R>(acc, R(0));
    }
    __syncthreads();
    c2<R>* Z = smem_fft_fast<R>(b0, b1, plan, 1, tw, -1, M);
    const double invM = 1.0 / M;
    for (int k = tid; k < K; k += nt) {
        const double s = (k == 0 ? 1.0 : 2.0) * invM;
        double2 r = make_double2(s * (double)Z[k].x, k == 0 ? 0.0 : s * (double)Z[k].y);
        Rk[k] = r;
    }
    __syncthreads();
    // SBDF right-hand side and the diagonal solve
    double2* X = a.X + a.off[m];
    double2* Fn = a.Fh[0] + a.off[m];
    double2* MXn = a.MXh[0] + a.off[m];
    for (int k = tid; k < K; k += nt) {
        const double kk = k * kscale;
        double mre, mim, lre, lim;
        if (k == 0) {
            mre = a.m0re; mim = a.m0im; lre = a.l0re; lim = a.l0im;
        } else {
            mre = mim = lre = lim = 0.0;
            double p = 1.0;
            for (int t = 0; t < 5; ++t) {
                mre += a.mre[t] * p; mim += a.mim[t] * p;
                lre += a.lre[t] * p; lim += a.lim[t] * p;
                p *= kk;
            }
        }
        const double2 c = X[k];
        const double2 mx = make_double2(mre * c.x - mim * c.y, mre * c.y + mim * c.x);
        const double2 fk = Rk[k];
        Fn[k] = fk;
        MXn[k] = mx;
        double rr = 0.0, ri = 0.0;
        for (int j = 0; j < a.q; ++j) {
            const double2 F = j == 0 ? fk : (a.Fh[j] + a.off[m])[k];
            const double2 MX = j == 0 ? mx : (a.MXh[j] + a.off[m])[k];
            rr += a.c[j] * F.x - a.d[j] * MX.x;
            ri += a.c[j] * F.y - a.d[j] * MX.y;
        }
        // (a0/dt M + L) x = rhs
        const double dr = a.a0dt * mre + lre, di = a.a0dt * mim + lim;
        const double den = dr * dr + di * di;
        double xr = (rr * dr + ri * di) / den, xi = (ri * dr - rr * di) / den;
        if (k == 0) xi = 0.0;
        X[k] = make_double2(xr, xi);
    }
}

}  // namespace cng

using namespace cng;

extern "C" {

int cng_fourier_ensemble_step(const cng_fourier_ensemble_desc* D, void* X, void* const* MXh, void* const* Fh,
                              int q, const double* c, const double* d, double a0dt, void* stream) {
    CNG_TRY({
        if (!D || !X || !MXh || !Fh || !c || !d) throw InvalidArgument("null argument");
        if (q < 1 || q > 4) throw InvalidArgument("SBDF order 1..4");
        if (D->nmem < 1) return CNG_OK;
        if (D->nfactors < 1 || D->nfactors > 4 || D->nmono < 1 || D->nmono > 4)
            throw InvalidArgument("1 to 4 factors and monomials");
        EnsArgs a{};
        a.nmem = D->nmem;
        a.nfactors = D->nfactors;
        a.nmono = D->nmono;
        a.q = q;
        a.N = D->size_dev;
        a.M = D->grid_dev;
        a.off = reinterpret_cast<const long long*>(D->offset_dev);
        a.len = D->length_dev;
        a.plan_idx = D->plan_dev;
        if (D->nplans < 1 || D->nplans > 4) throw InvalidArgument("1 to 4 distinct grid sizes");
        int maxM = 0;
        for (int p = 0; p < D->nplans; ++p) {
            a.plans[p] = make_plan(D->plan_sizes[p]);
            a.tw[p] = D->precision ? D->twiddles32[p] : D->twiddles64[p];
            maxM = std::max(maxM, D->plan_sizes[p]);
        }
        for (int f = 0; f < a.nfactors; ++f) a.factor_order[f] = D->factor_order[f];
        for (int mi = 0; mi < a.nmono; ++mi) {
            a.mono_coef[mi] = D->mono_coef[mi];
            for (int qq = 0; qq < 4; ++qq) {
                a.mono_fac[4 * mi + qq] = D->mono_factors[4 * mi + qq];
                if (a.mono_fac[4 * mi + qq] >= a.nfactors) throw InvalidArgument("monomial factor out of range");
            }
        }
        for (int t = 0; t < 5; ++t) {
            a.mre[t] = D->m_poly[2 * t]; a.mim[t] = D->m_poly[2 * t + 1];
            a.lre[t] = D->l_poly[2 * t]; a.lim[t] = D->l_poly[2 * t + 1];
        }
        a.m0re = D->m_mean[0]; a.m0im = D->m_mean[1]; a.l0re = D->l_mean[0]; a.l0im = D->l_mean[1];
        for (int j = 0; j < q; ++j) {
            a.c[j] = c[j];
            a.d[j] = d[j];
            a.MXh[j] = static_cast<double2*>(MXh[j]);
            a.Fh[j] = static_cast<double2*>(Fh[j]);
            if (!a.MXh[j] || !a.Fh[j]) throw InvalidArgument("null history buffer");
        }
        a.a0dt = a0dt;
        a.X = static_cast<double2*>(X);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const size_t cs = D->precision ? sizeof(float2) : sizeof(double2);
        const size_t rs = cs / 2;
        const size_t smem = cs * 3 * (size_t)maxM + rs * ((size_t)(a.nfactors * maxM + 3) & ~(size_t)3) +
                            sizeof(double2) * (size_t)maxM + 64;
        if (D->precision) {
            ensure_smem_attr((const void*)k_fourier_ensemble_step<float>, 200 * 1024);
            k_fourier_ensemble_step<float><<<a.nmem, 128, smem, st>>>(a);
        } else {
            ensure_smem_attr((const void*)k_fourier_ensemble_step<double>, 200 * 1024);
            k_fourier_ensemble_step<double><<<a.nmem, 128, smem, st>>>(a);
        }
        CNG_LAUNCH("k_fourier_ensemble_step");
    })
}

}  // extern "C"
