// Oracle (test infrastructure only): a C-ABI around the reference's own header-only bordered
// banded solver (core/include/conatus/banded.hpp and parallel.hpp, compiled unmodified from the
// reference tree by oracle/Makefile into oracle/_ref/).
//
// The reference declares Fortran LAPACK symbols (core/include/conatus/lapack.hpp:6-25). They are
// defined here and forwarded to SciPy's cython_lapack function pointers, which the Python side
// (oracle/ref.py) reads from scipy.linalg.cython_lapack.__pyx_capi__ and passes in once. Those
// entry points do not take the hidden Fortran string-length argument, so it is dropped here.
#include <complex>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "conatus/banded.hpp"
#include "conatus/parallel.hpp"

using cplx = std::complex<double>;

namespace {
using gbtrf_d = void (*)(const int*, const int*, const int*, const int*, double*, const int*, int*, int*);
using gbtrs_d = void (*)(const char*, const int*, const int*, const int*, const int*, const double*,
                         const int*, const int*, double*, const int*, int*);
using gbtrf_z = void (*)(const int*, const int*, const int*, const int*, cplx*, const int*, int*, int*);
using gbtrs_z = void (*)(const char*, const int*, const int*, const int*, const int*, const cplx*,
                         const int*, const int*, cplx*, const int*, int*);
using getrf_d = void (*)(const int*, const int*, double*, const int*, int*, int*);
using getrs_d = void (*)(const char*, const int*, const int*, const double*, const int*, const int*,
                         double*, const int*, int*);
using getrf_z = void (*)(const int*, const int*, cplx*, const int*, int*, int*);
using getrs_z = void (*)(const char*, const int*, const int*, const cplx*, const int*, const int*,
                         cplx*, const int*, int*);
gbtrf_d p_dgbtrf;
gbtrs_d p_dgbtrs;
gbtrf_z p_zgbtrf;
gbtrs_z p_zgbtrs;
getrf_d p_dgetrf;
getrs_d p_dgetrs;
getrf_z p_zgetrf;
getrs_z p_zgetrs;
thread_local std::string g_err;

template <class T>
struct Batch {
    std::vector<std::unique_ptr<conatus::BorderedBanded<T>>> sys;
};
}  // namespace

extern "C" {
void dgbtrf_(const int* m, const int* n, const int* kl, const int* ku, double* ab, const int* ldab,
             int* ipiv, int* info) { p_dgbtrf(m, n, kl, ku, ab, ldab, ipiv, info); }
void dgbtrs_(const char* t, const int* n, const int* kl, const int* ku, const int* nrhs,
             const double* ab, const int* ldab, const int* ipiv, double* b, const int* ldb,
             int* info, std::size_t) { p_dgbtrs(t, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb, info); }
void zgbtrf_(const int* m, const int* n, const int* kl, const int* ku, cplx* ab, const int* ldab,
             int* ipiv, int* info) { p_zgbtrf(m, n, kl, ku, ab, ldab, ipiv, info); }
void zgbtrs_(const char* t, const int* n, const int* kl, const int* ku, const int* nrhs,
             const cplx* ab, const int* ldab, const int* ipiv, cplx* b, const int* ldb, int* info,
             std::size_t) { p_zgbtrs(t, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb, info); }
void dgetrf_(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info) {
    p_dgetrf(m, n, a, lda, ipiv, info);
}
void dgetrs_(const char* t, const int* n, const int* nrhs, const double* a, const int* lda,
             const int* ipiv, double* b, const int* ldb, int* info, std::size_t) {
    p_dgetrs(t, n, nrhs, a, lda, ipiv, b, ldb, info);
}
void zgetrf_(const int* m, const int* n, cplx* a, const int* lda, int* ipiv, int* info) {
    p_zgetrf(m, n, a, lda, ipiv, info);
}
void zgetrs_(const char* t, const int* n, const int* nrhs, const cplx* a, const int* lda,
             const int* ipiv, cplx* b, const int* ldb, int* info, std::size_t) {
    p_zgetrs(t, n, nrhs, a, lda, ipiv, b, ldb, info);
}

// order: dgbtrf dgbtrs zgbtrf zgbtrs dgetrf dgetrs zgetrf zgetrs
void ref_set_lapack(void** p) {
    p_dgbtrf = (gbtrf_d)p[0];
    p_dgbtrs = (gbtrs_d)p[1];
    p_zgbtrf = (gbtrf_z)p[2];
    p_zgbtrs = (gbtrs_z)p[3];
    p_dgetrf = (getrf_d)p[4];
    p_dgetrs = (getrs_d)p[5];
    p_zgetrf = (getrf_z)p[6];
    p_zgetrs = (getrs_z)p[7];
}

const char* ref_last_error() { return g_err.c_str(); }

// One batch of systems (complex if is_complex): matrix k is CSR (n, indptr + k*(n+1) offsets
// into one concatenated array). Returns a handle or NULL (message in ref_last_error()).
void* ref_batch_create(int is_complex, int batch, int n, const int* indptr, const int* indices,
                       const void* data, const long long* nnz_off, const int* border, int r) {
    try {
        std::vector<int> bd(border, border + r);
        auto build = [&](auto tag) -> void* {
            using T = decltype(tag);
            auto* B = new Batch<T>();
            const T* d = static_cast<const T*>(data);
            for (int k = 0; k < batch; ++k) {
                conatus::Csr<T> A;
                A.n = n;
                const int* ip = indptr + static_cast<std::size_t>(k) * (n + 1);
                A.indptr.assign(ip, ip + n + 1);
                long long o = nnz_off[k];
                A.indices.assign(indices + o, indices + o + A.indptr[n]);
                A.data.assign(d + o, d + o + A.indptr[n]);
                B->sys.push_back(std::make_unique<conatus::BorderedBanded<T>>(A, bd, false));
            }
            return B;
        };
        return is_complex ? build(cplx{}) : build(double{});
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

int ref_batch_info(int is_complex, void* h, int k, int* n_kl_ku_r, double* cond) {
    auto get = [&](auto* B) {
        auto& s = *B->sys[k];
        n_kl_ku_r[0] = s.n();
        n_kl_ku_r[1] = s.kl();
        n_kl_ku_r[2] = s.ku();
        n_kl_ku_r[3] = s.rank();
        *cond = s.capacitance_cond();
        return 0;
    };
    return is_complex ? get(static_cast<Batch<cplx>*>(h)) : get(static_cast<Batch<double>*>(h));
}

// b: (batch, n) contiguous, solved in place; transpose: A^T x = b; threads: parallel_for chunks.
int ref_batch_solve(int is_complex, void* h, void* b, int transpose, int threads) {
    try {
        auto run = [&](auto* B, auto* x) {
            const std::size_t n = B->sys.empty() ? 0 : B->sys[0]->n();
            if (transpose)
                for (auto& s : B->sys) s->prepare_transpose();
            conatus::parallel_for(B->sys.size(), threads, [&](std::size_t k) {
                if (transpose) B->sys[k]->solve_transpose(x + k * n, 1);
                else B->sys[k]->solve(x + k * n, 1);
            });
        };
        if (is_complex) run(static_cast<Batch<cplx>*>(h), static_cast<cplx*>(b));
        else run(static_cast<Batch<double>*>(h), static_cast<double*>(b));
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

void ref_batch_destroy(int is_complex, void* h) {
    if (is_complex) delete static_cast<Batch<cplx>*>(h);
    else delete static_cast<Batch<double>*>(h);
}
}
