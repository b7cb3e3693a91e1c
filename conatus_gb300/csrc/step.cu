// Pieces of the IMEX step on the mode layout: M X per bucket and the SBDF right-hand side.
#include <cuda_runtime.h>

#include "common.cuh"
#include "conatus_gb300.h"

namespace cng {

// one warp per (system, row chunk): y[m][i] = sum_p M[i, p] x[m][col p]
__global__ void k_csr_matvec(int nsys, int n, const int* __restrict__ ip, const int* __restrict__ ix,
                             const double2* __restrict__ val, int per_sys, const double2* __restrict__ x,
                             double2* __restrict__ y) {
    const long long total = (long long)nsys * n;
    const int nnz = ip[n];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long m = t / n;
        const int i = (int)(t - m * n);
        const double2* xm = x + m * n;
        const double2* v = val + (per_sys ? m * nnz : 0);
        double ar = 0.0, ai = 0.0;
        for (int p = ip[i]; p < ip[i + 1]; ++p) {
            const double2 a = v[p], b = xm[ix[p]];
            ar += a.x * b.x - a.y * b.y;
            ai += a.x * b.y + a.y * b.x;
        }
        y[t] = make_double2(ar, ai);
    }
}

// y = M x with real M values (M of the tau systems is real: conversions between Chebyshev and
// ultraspherical bases). A warp takes one row i for 32 systems (lane = system): uniform trip
// counts across the warp, the row's entries as broadcast loads, x gathered per lane.
__device__ __forceinline__ void csr_matvec_real_body(unsigned bid, unsigned nblk, int nsys, int n,
                                                     const int* __restrict__ ip, const int* __restrict__ ix,
                                                     const double* __restrict__ val, const double2* __restrict__ x,
                                                     double2* __restrict__ y) {
    // one thread per (system, row), rows fastest: a warp reads a contiguous stretch of one
    // system's vector (the band around its rows) and writes 32 consecutive rows; the row pattern
    // and values, shared by every system, stay in L1
    const unsigned total = (unsigned)nsys * (unsigned)n;
    const unsigned stride = nblk * blockDim.x;
    for (unsigned t = bid * blockDim.x + threadIdx.x; t < total; t += stride) {
        const unsigned m = t / (unsigned)n;
        const int i = (int)(t - m * (unsigned)n);
        const double2* xm = x + (size_t)m * n;
        double ar[2] = {0.0, 0.0}, ai[2] = {0.0, 0.0};
        int q = 0;
        for (int p = ip[i]; p < ip[i + 1]; ++p, q ^= 1) {
            const double a = val[p];
            const double2 b = xm[ix[p]];
            ar[q] = fma(a, b.x, ar[q]);
            ai[q] = fma(a, b.y, ai[q]);
        }
        y[t] = make_double2(ar[0] + ar[1], ai[0] + ai[1]);
    }
}

__global__ void k_csr_matvec_real(int nsys, int n, const int* __restrict__ ip, const int* __restrict__ ix,
                                  const double* __restrict__ val, const double2* __restrict__ x,
                                  double2* __restrict__ y) {
    csr_matvec_real_body(blockIdx.x, gridDim.x, nsys, n, ip, ix, val, x, y);
}

__global__ void k_csr_matvec_real_grp(const __grid_constant__ Grp<cng_matvec_part> g) {
    const int k = g.find(blockIdx.x);
    const cng_matvec_part& a = g.a[k];
    csr_matvec_real_body(blockIdx.x - g.start[k], g.start[k + 1] - g.start[k], a.nsys, a.n, a.indptr, a.indices,
                         a.values, static_cast<const double2*>(a.x), static_cast<double2*>(a.y));
}

struct SbdfArgs {
    int q;
    double c[4], d[4];
    const double* F[4];
    const double* MX[4];
};

// rhs = sum_j (c_j F_j - d_j MX_j) on real and imaginary parts, explicit roundings in the order of
// the reference's sbdf_rhs (a = 0; a = a + (c F - d MX)).
__global__ void k_sbdf_rhs(SbdfArgs a, double* __restrict__ rhs, long long count) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < count;
         t += (long long)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int j = 0; j < a.q; ++j)
            acc = __dadd_rn(acc, __dsub_rn(__dmul_rn(a.c[j], a.F[j][t]), __dmul_rn(a.d[j], a.MX[j][t])));
        rhs[t] = acc;
    }
}

constexpr int kMaxTerms = 12;
struct LincombArgs {
    int nterms;
    double coef[kMaxTerms];
    int neg[kMaxTerms];
    const double* v[kMaxTerms];
};

// out = base + sum_k (+/-) coef_k v_k on real and imaginary parts, applied in order with explicit
// roundings (acc = acc +/- coef_k * v_k), base = 0 when absent: the right-hand side of an IMEX
// Runge-Kutta stage (lincomb.py:73-95) and of a CN-family step (integrator.py:581-594).
__global__ void k_lincomb(LincombArgs a, const double* __restrict__ base, double* __restrict__ out,
                          long long count) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < count;
         t += (long long)gridDim.x * blockDim.x) {
        double acc = base ? base[t] : 0.0;
        for (int k = 0; k < a.nterms; ++k) {
            const double p = __dmul_rn(a.coef[k], a.v[k][t]);
            acc = a.neg[k] ? __dsub_rn(acc, p) : __dadd_rn(acc, p);
        }
        out[t] = acc;
    }
}

// The same combination with fused multiply-adds (two FP64 operations per history level instead of
// four): the FP32 form's right-hand side, which is not held to the reference's order of roundings.
__global__ void k_sbdf_rhs_fused(SbdfArgs a, double* __restrict__ rhs, long long count) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < count;
         t += (long long)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int j = 0; j < a.q; ++j) {
            acc = fma(a.c[j], a.F[j][t], acc);
            acc = fma(-a.d[j], a.MX[j][t], acc);
        }
        rhs[t] = acc;
    }
}

// Finite-state check: if any of the count doubles of x is a NaN or an infinity (exponent bits all
// ones), flag[0] = min(flag[0], iteration). One vote per warp, one atomic per warp that saw one.
__global__ void k_check_finite(const unsigned long long* __restrict__ x, long long count, long long iteration,
                               unsigned long long* __restrict__ flag) {
    bool bad = false;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < count;
         t += (long long)gridDim.x * blockDim.x)
        bad |= (x[t] & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
    const unsigned any = __ballot_sync(0xffffffffu, bad);
    if (any && (threadIdx.x & 31) == 0) atomicMin(flag, (unsigned long long)iteration);
}

// r = b - (a M + c sum_t mono[m][t] L_t) x per system, FP64 (the refinement residual). M values
// shared by the bucket (nnz), L_t coefficient rows (nmono x nnz), mono (nsys x nmono).
__global__ void k_poly_residual(int nsys, int n, const int* __restrict__ ip, const int* __restrict__ ix,
                                const double2* __restrict__ mval, const double2* __restrict__ lcoef,
                                const double* __restrict__ mono, int nmono, double a, double c,
                                const double2* __restrict__ x, const double2* __restrict__ b,
                                double2* __restrict__ r) {
    const long long total = (long long)nsys * n;
    const int nnz = ip[n];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long m = t / n;
        const int i = (int)(t - m * n);
        const double2* xm = x + m * n;
        const double* mv = mono + m * nmono;
        double ar = 0.0, ai = 0.0;
        for (int p = ip[i]; p < ip[i + 1]; ++p) {
            double vr = a * mval[p].x, vi = a * mval[p].y;
            for (int q = 0; q < nmono; ++q) {
                const double2 l = lcoef[(long long)q * nnz + p];
                vr += c * mv[q] * l.x;
                vi += c * mv[q] * l.y;
            }
            const double2 xv = xm[ix[p]];
            ar += vr * xv.x - vi * xv.y;
            ai += vr * xv.y + vi * xv.x;
        }
        const double2 bv = b[t];
        r[t] = make_double2(bv.x - ar, bv.y - ai);
    }
}

// r = b - (a M + c sum_t mono[m][t] L_t) x, FP64, with the operator stored as one real-coefficient
// entry list per row: entry e of row i has column col[e], real value val[e] and a code
// code[e] = 2 t + imag (t = monomial index, -1 for M: code -2 / -1; imag: the entry is i val).
// Every coefficient of M and of each L_t is purely real or purely imaginary (derivatives
// contribute (i k)^p). Within a row the entries of one term (M, or one L_t) are summed first with
// their real values (two FP64 multiply-adds per entry), and each term's sum is then scaled by a or
// c mono[m][t] (two more per term): FP64 is the bound of this kernel, and the per-entry scaling
// would cost a third and fourth multiply per entry. Entries of a term need not be contiguous (a
// term split in several runs is scaled once per run).
// Thread mapping: a warp takes one row i for 32 systems (lane = system), so every lane of a warp
// runs the same entry list (uniform trip counts: the border rows have up to n entries, the others
// a dozen) and the entry data is one broadcast load per warp; x is gathered per lane.
constexpr int kMergedTerm = 63;          // an entry list shared by several terms: scale per (row, system)

// Systems s0 .. s0 + cnt - 1 of a bucket of ld systems (rowscale and xT are [n][ld]).
template <bool CONE>
__device__ __forceinline__ void split_residual_body(unsigned bid, unsigned nblk, int cnt, int s0, int ld, int n,
                                                    const int* __restrict__ ptr, const int* __restrict__ col,
                                                    const double* __restrict__ val,
                                                    const signed char* __restrict__ code,
                                                    const double* __restrict__ mono, int nmono, double a, double c,
                                                    const double* __restrict__ rowscale,
                                                    const double2* __restrict__ x, const double2* __restrict__ xT,
                                                    const double2* __restrict__ b, double2* __restrict__ r) {
    const int nsys = ld;
    const unsigned sysw = ((unsigned)cnt + 31u) >> 5;              // warps of 32 systems per row
    const unsigned nwarps = sysw * (unsigned)n;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned wstride = (nblk * blockDim.x) >> 5;
    for (unsigned w = (bid * blockDim.x + threadIdx.x) >> 5; w < nwarps; w += wstride) {
        const int i = (int)(w / sysw);
        const unsigned ml = (w - (unsigned)i * sysw) * 32u + lane;
        if (ml >= (unsigned)cnt) continue;
        const unsigned m = ml + (unsigned)s0;
        const long long t = (long long)m * n + i;
        const double2* xm = x + (long long)m * n;
        const double* mv = mono + (long long)m * nmono;
        const double2 bv = b[t];                            // in flight during the row's entries
        double ar = 0.0, ai = 0.0;
        const int e0 = ptr[i], e1 = ptr[i + 1];
        // one pass over the row's entries (no data-dependent inner loop, so the loads of the next
        // entries issue ahead); a term's group sum joins ar, ai when the term changes, as in the
        // group-by-group order
        auto scale = [&](int tt) {
            // c = 1: no multiply; a merged list: its scale per (row, system) (NaN without the table)
            return tt == kMergedTerm ? (rowscale ? rowscale[(size_t)i * nsys + m] : __longlong_as_double(0x7ff8000000000000LL))
                                     : (tt < 0 ? a : (CONE ? mv[tt] : c * mv[tt]));
        };
        int tt = e0 < e1 ? code[e0] >> 1 : 0;
        double gr = 0.0, gi = 0.0;
#pragma unroll 4
        for (int e = e0; e < e1; ++e) {
            const int cd = code[e];
            if ((cd >> 1) != tt) {
                const double sc = scale(tt);
                ar = fma(sc, gr, ar);
                ai = fma(sc, gi, ai);
                gr = gi = 0.0;
                tt = cd >> 1;
            }
            const double v = val[e];
            // x row-major over the systems when given: the warp's 32 systems read one line
            const double2 xv = xT ? xT[(size_t)col[e] * nsys + m] : xm[col[e]];
            const bool im = cd & 1;                          // i v x
            gr = fma(im ? -v : v, im ? xv.y : xv.x, gr);
            gi = fma(v, im ? xv.x : xv.y, gi);
        }
        if (e0 < e1) {
            const double sc = scale(tt);
            ar = fma(sc, gr, ar);
            ai = fma(sc, gi, ai);
        }
        r[t] = make_double2(bv.x - ar, bv.y - ai);
    }
}

template <bool CONE>
__global__ void k_split_residual(int cnt, int s0, int ld, int n, const int* __restrict__ ptr,
                                 const int* __restrict__ col,
                                 const double* __restrict__ val, const signed char* __restrict__ code,
                                 const double* __restrict__ mono, int nmono, double a, double c,
                                 const double* __restrict__ rowscale, const double2* __restrict__ x,
                                 const double2* __restrict__ xT, const double2* __restrict__ b,
                                 double2* __restrict__ r) {
    split_residual_body<CONE>(blockIdx.x, gridDim.x, cnt, s0, ld, n, ptr, col, val, code, mono, nmono, a, c,
                              rowscale, x, xT, b, r);
}

template <bool CONE>
__global__ void k_split_residual_grp(const __grid_constant__ Grp<cng_residual_part> g, double a, double c) {
    const int k = g.find(blockIdx.x);
    const cng_residual_part& p = g.a[k];
    split_residual_body<CONE>(blockIdx.x - g.start[k], g.start[k + 1] - g.start[k], p.s1 - p.s0, p.s0, p.nsys, p.n,
                              p.ptr, p.col, p.val, reinterpret_cast<const signed char*>(p.code), p.mono, p.nmono, a, c,
                              p.rowscale, static_cast<const double2*>(p.x), static_cast<const double2*>(p.xT),
                              static_cast<const double2*>(p.b), static_cast<double2*>(p.r));
}

}  // namespace cng

using namespace cng;

extern "C" {

int cng_csr_matvec(int nsys, int n, const int32_t* indptr, const int32_t* indices, const void* values,
                   int values_per_system, const void* x, void* y, void* stream) {
    CNG_TRY({
        if (!indptr || !indices || !values || !x || !y) throw InvalidArgument("null device pointer");
        if (x == y) throw InvalidArgument("x and y must not alias");
        if (nsys <= 0 || n <= 0) return CNG_OK;
        const long long total = (long long)nsys * n;
        const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 32);
        k_csr_matvec<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
            nsys, n, indptr, indices, static_cast<const double2*>(values), values_per_system,
            static_cast<const double2*>(x), static_cast<double2*>(y));
        CNG_LAUNCH("k_csr_matvec");
    })
}

int cng_csr_matvec_real(int nsys, int n, const int32_t* indptr, const int32_t* indices, const double* values,
                        const void* x, void* y, void* stream) {
    CNG_TRY({
        if (!indptr || !indices || !values || !x || !y) throw InvalidArgument("null device pointer");
        if (x == y) throw InvalidArgument("x and y must not alias");
        if (nsys <= 0 || n <= 0) return CNG_OK;
        const long long threads = (long long)nsys * n;
        if (threads >= (1LL << 32) - (1LL << 24)) throw InvalidArgument("csr_matvec_real: batch too large");
        const int blocks = (int)std::min<long long>((threads + 255) / 256, 152LL * 64);
        k_csr_matvec_real<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
            nsys, n, indptr, indices, values, static_cast<const double2*>(x), static_cast<double2*>(y));
        CNG_LAUNCH("k_csr_matvec_real");
    })
}

int cng_csr_matvec_real_group(int nparts, const cng_matvec_part* parts, void* stream) {
    CNG_TRY({
        if (nparts < 0 || (nparts > 0 && !parts)) throw InvalidArgument("null argument");
        std::vector<cng_matvec_part> args;
        std::vector<unsigned> blocks;
        for (int k = 0; k < nparts; ++k) {
            const cng_matvec_part& p = parts[k];
            if (!p.indptr || !p.indices || !p.values || !p.x || !p.y) throw InvalidArgument("null device pointer");
            if (p.x == p.y) throw InvalidArgument("x and y must not alias");
            if (p.nsys < 0 || p.n < 0) throw InvalidArgument("csr_matvec_real: negative size");
            const long long threads = (long long)p.nsys * p.n;
            if (threads >= (1LL << 32) - (1LL << 24)) throw InvalidArgument("csr_matvec_real: batch too large");
            args.push_back(p);
            blocks.push_back((unsigned)std::min<long long>((threads + 255) / 256, 152LL * 64));
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        launch_groups(args, blocks, [&](const Grp<cng_matvec_part>& g, unsigned total) {
            k_csr_matvec_real_grp<<<total, 256, 0, st>>>(g);
            CNG_LAUNCH("k_csr_matvec_real_grp");
        });
    })
}

int cng_split_residual_group(int nparts, const cng_residual_part* parts, double a, double c, void* stream) {
    CNG_TRY({
        if (nparts < 0 || (nparts > 0 && !parts)) throw InvalidArgument("null argument");
        std::vector<cng_residual_part> args;
        std::vector<unsigned> blocks;
        for (int k = 0; k < nparts; ++k) {
            const cng_residual_part& p = parts[k];
            if (!p.ptr || !p.col || !p.val || !p.code || (p.nmono > 0 && !p.mono) || !p.x || !p.b || !p.r)
                throw InvalidArgument("null device pointer");
            if (p.r == p.x || p.r == p.b) throw InvalidArgument("r must not alias x or b");
            if (p.s0 < 0 || p.s1 > p.nsys || p.s0 > p.s1 || p.n < 0)
                throw InvalidArgument("split_residual: system range outside the batch");
            const long long w = (long long)((p.s1 - p.s0 + 31) / 32) * p.n;
            if (w >= (1LL << 31)) throw InvalidArgument("split_residual: batch too large");
            args.push_back(p);
            blocks.push_back((unsigned)std::min<long long>((w * 32 + 255) / 256, 152LL * 64));
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        launch_groups(args, blocks, [&](const Grp<cng_residual_part>& g, unsigned total) {
            if (c == 1.0) k_split_residual_grp<true><<<total, 256, 0, st>>>(g, a, c);
            else k_split_residual_grp<false><<<total, 256, 0, st>>>(g, a, c);
            CNG_LAUNCH("k_split_residual_grp");
        });
    })
}

int cng_poly_residual(int nsys, int n, const int32_t* indptr, const int32_t* indices, const void* mval,
                      const void* lcoef, const double* mono, int nmono, double a, double c, const void* x,
                      const void* b, void* r, void* stream) {
    CNG_TRY({
        if (!indptr || !indices || !mval || (nmono > 0 && (!lcoef || !mono)) || !x || !b || !r)
            throw InvalidArgument("null device pointer");
        if (r == x || r == b) throw InvalidArgument("r must not alias x or b");
        if (nsys <= 0 || n <= 0) return CNG_OK;
        const long long total = (long long)nsys * n;
        const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 32);
        k_poly_residual<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
            nsys, n, indptr, indices, static_cast<const double2*>(mval), static_cast<const double2*>(lcoef),
            mono, nmono, a, c, static_cast<const double2*>(x), static_cast<const double2*>(b),
            static_cast<double2*>(r));
        CNG_LAUNCH("k_poly_residual");
    })
}

int cng_split_residual_range(int nsys, int s0, int s1, int n, const int32_t* ptr, const int32_t* col,
                             const double* val, const int8_t* code, const double* mono, int nmono, double a,
                             double c, const double* rowscale, const void* x, const void* xT, const void* b,
                             void* r, void* stream) {
    CNG_TRY({
        if (!ptr || !col || !val || !code || (nmono > 0 && !mono) || !x || !b || !r)
            throw InvalidArgument("null device pointer");
        if (r == x || r == b) throw InvalidArgument("r must not alias x or b");
        if (s0 < 0 || s1 > nsys || s0 > s1) throw InvalidArgument("split_residual: system range outside the batch");
        const int cnt = s1 - s0;
        if (cnt <= 0 || n <= 0) return CNG_OK;
        auto* sc = reinterpret_cast<const signed char*>(code);
        if ((long long)((cnt + 31) / 32) * n >= (1LL << 31)) throw InvalidArgument("split_residual: batch too large");
        const long long threads = (long long)((cnt + 31) / 32) * n * 32;
        const int blk = (int)std::min<long long>((threads + 255) / 256, 152LL * 64);
        if (c == 1.0)
            k_split_residual<true><<<blk, 256, 0, static_cast<cudaStream_t>(stream)>>>(
                cnt, s0, nsys, n, ptr, col, val, sc, mono, nmono, a, c, rowscale, static_cast<const double2*>(x),
                static_cast<const double2*>(xT), static_cast<const double2*>(b), static_cast<double2*>(r));
        else
            k_split_residual<false><<<blk, 256, 0, static_cast<cudaStream_t>(stream)>>>(
                cnt, s0, nsys, n, ptr, col, val, sc, mono, nmono, a, c, rowscale, static_cast<const double2*>(x),
                static_cast<const double2*>(xT), static_cast<const double2*>(b), static_cast<double2*>(r));
        CNG_LAUNCH("k_split_residual");
    })
}

int cng_split_residual(int nsys, int n, const int32_t* ptr, const int32_t* col, const double* val,
                       const int8_t* code, const double* mono, int nmono, double a, double c,
                       const double* rowscale, const void* x, const void* xT, const void* b, void* r,
                       void* stream) {
    return cng_split_residual_range(nsys, 0, nsys, n, ptr, col, val, code, mono, nmono, a, c, rowscale, x, xT, b,
                                    r, stream);
}

int cng_lincomb(int64_t count, const void* base, int nterms, const double* coef, const int32_t* negate,
                const void* const* vecs, void* out, void* stream) {
    CNG_TRY({
        if (nterms < 0 || nterms > kMaxTerms) throw InvalidArgument("lincomb: 0 to 12 terms");
        if (!out || (nterms > 0 && (!coef || !negate || !vecs))) throw InvalidArgument("null argument");
        if (count <= 0) return CNG_OK;
        LincombArgs a{};
        a.nterms = nterms;
        for (int k = 0; k < nterms; ++k) {
            a.coef[k] = coef[k];
            a.neg[k] = negate[k] ? 1 : 0;
            a.v[k] = static_cast<const double*>(vecs[k]);
            if (!a.v[k]) throw InvalidArgument("lincomb: null vector");
        }
        const long long n = 2 * count;      // complex entries -> doubles
        const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 32);
        k_lincomb<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, static_cast<const double*>(base),
                                                                          static_cast<double*>(out), n);
        CNG_LAUNCH("k_lincomb");
    })
}

int cng_check_finite(const void* x, int64_t count, int64_t iteration, int64_t* flag, void* stream) {
    CNG_TRY({
        if (!x || !flag) throw InvalidArgument("null argument");
        if (count < 0 || iteration < 0) throw InvalidArgument("check_finite: negative count or iteration");
        if (count == 0) return CNG_OK;
        const long long n = 2 * count;      // complex entries -> doubles
        const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 8);
        k_check_finite<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const unsigned long long*>(x), n, iteration, reinterpret_cast<unsigned long long*>(flag));
        CNG_LAUNCH("k_check_finite");
    })
}

int cng_sbdf_rhs(int q, const double* c, const double* d, const void* const* F, const void* const* MX,
                 void* rhs, int64_t count, void* stream) {
    return cng_sbdf_rhs_fused(q, c, d, F, MX, rhs, count, 0, stream);
}

int cng_sbdf_rhs_fused(int q, const double* c, const double* d, const void* const* F, const void* const* MX,
                       void* rhs, int64_t count, int fused, void* stream) {
    CNG_TRY({
        if (q < 1 || q > 4) throw InvalidArgument("SBDF order must be 1..4");
        if (!c || !d || !F || !MX || !rhs) throw InvalidArgument("null argument");
        SbdfArgs a{};
        a.q = q;
        for (int j = 0; j < q; ++j) {
            a.c[j] = c[j];
            a.d[j] = d[j];
            a.F[j] = static_cast<const double*>(F[j]);
            a.MX[j] = static_cast<const double*>(MX[j]);
            if (!a.F[j] || !a.MX[j]) throw InvalidArgument("null history vector");
        }
        const long long n = 2 * count;      // complex entries -> doubles
        const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 32);
        if (fused)
            k_sbdf_rhs_fused<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, static_cast<double*>(rhs), n);
        else
            k_sbdf_rhs<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, static_cast<double*>(rhs), n);
        CNG_LAUNCH("k_sbdf_rhs");
    })
}

}  // extern "C"
