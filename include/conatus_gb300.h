/* conatus_gb300: C-ABI of the GB300-native IMEX hot path (sm_103a).
 *
 * Every function returns 0 on success or a nonzero status (1 invalid argument, 2 numerical or
 * runtime failure such as a singular system, 3 CUDA error, 4 out of memory); the message of the
 * last failure on the calling thread is cng_last_error(). Device pointers are caller-owned unless
 * a handle owns them; `stream` is a cudaStream_t (NULL = the legacy default stream). Nothing here
 * falls back to the CPU.
 *
 * Each entry point names the reference interface it replaces (path:line inside the reference
 * project, conatus v0.5.0).
 */
#ifndef CONATUS_GB300_H
#define CONATUS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- library ------------------------------------------------------------------------------- */

/* Message of the last failure on this thread ("" if none). */
const char* cng_last_error(void);
/* Library version string. */
const char* cng_version(void);
/* 1 if a CUDA device is usable (replaces cuda.available(), core/bindings/module.cpp:445). */
int cng_cuda_available(void);
/* Name of device `dev` into buf (replaces cuda.device_name(), core/bindings/module.cpp:446). */
int cng_device_name(int dev, char* buf, int buflen);
/* Free and total device memory in bytes (admission by footprint; the reference's memory planner
 * python/conatus/runtime/memory.py predicts the same quantity). */
int cng_mem_info(uint64_t* free_bytes, uint64_t* total_bytes);
/* Device memory held by the library's handles: live bytes and allocations so far; cached bytes and
 * reuses are 0 (freed memory goes back to the driver at once, there is no pool). Not counted: the
 * fixed 8 MiB staging array of cng_banded_solve_host_static, resident on every device that loaded
 * the library. Replaces cuda.pool_stats (core/bindings/module.cpp:450-453). Any argument may be
 * NULL. */
int cng_pool_stats(uint64_t* live_bytes, uint64_t* cached_bytes, uint64_t* n_alloc, uint64_t* n_reuse);
/* Nothing is cached, so nothing to return to the driver: 0. Replaces cuda.pool_trim
 * (core/bindings/module.cpp:454). */
int cng_pool_trim(void);

/* ---- batched bordered-banded factor and solves --------------------------------------------- */

typedef struct cng_banded cng_banded;

/* Factor a batch of square CSR matrices of equal size n (dtype 0 = float64, 1 = complex128).
 * indptr: batch*(n+1) int32 (matrix k at k*(n+1)); indices/data: concatenated, matrix k starts at
 * nnz_offsets[k]; border: the r border rows (boundary/tau rows, moved first); pivot: partial
 * pivoting inside the band. Host arrays. Synchronizes `stream`; a singular band or capacitance
 * returns 2 with "singular" in the message.
 * Replaces cuda.BandedBatch{D,Z}.__init__ (core/bindings/module.cpp:284-295,
 * core/src/cuda/banded.cu:1138-1237) and _core.BorderedBandedBatch{D,Z}.__init__
 * (core/bindings/module.cpp:163-169). */
int cng_banded_create_csr(int dtype, int batch, int n, const int32_t* indptr, const int32_t* indices,
                          const void* data, const int64_t* nnz_offsets, const int32_t* border, int r,
                          int pivot, void* stream, cng_banded** out);

/* Factor a batch sharing one CSR pattern (host indptr/indices, nnz entries) whose values live on
 * the device, values[k*nnz + p] for system k. The layout is assembled on the device. Same errors as
 * cng_banded_create_csr. The reference builds each matrix on the host
 * (python/conatus/timestep/system.py:729-755) and passes it to the constructor above. */
int cng_banded_create_shared(int dtype, int batch, int n, const int32_t* indptr, const int32_t* indices,
                             int nnz, const void* values, const int32_t* border, int r, int pivot,
                             void* stream, cng_banded** out);

/* Refactor a shared-pattern handle with new device values (a new a M + b L of the same pattern).
 * The reference keeps one factorization per (a, b) key (python/conatus/timestep/system.py:58-82). */
int cng_banded_refactor_shared(cng_banded* h, const void* values, void* stream);

int cng_banded_destroy(cng_banded* h);

/* dims[8] = {batch, n, r, kl, ku, ldab, dtype, pivot}; stats[2] = {factor_ms,
 * capacitance_cond_max}. Replaces the properties of cuda.BandedBatch (module.cpp:427-434). */
int cng_banded_info(const cng_banded* h, int32_t* dims, double* stats);
/* Per-system 1-norm condition of the capacitance matrix (host array of batch doubles). */
int cng_banded_capacitance_cond(const cng_banded* h, double* cond_host);

/* Solve in place on caller-owned device memory b (C-contiguous (batch, n)), launched on stream;
 * capturable in a CUDA graph. Replaces cuda.BandedBatch.solve_ptr (module.cpp:400-409). */
int cng_banded_solve(const cng_banded* h, void* b, void* stream);

/* b_m[i] = rhs[rows[m*n + i]], x[cols[m*n + i]] = x_m[i]; rows/cols int64 device arrays, NULL =
 * contiguous. rhs == x is a solve in place and needs one map for both (rows == cols, or both
 * NULL); rhs == x with two maps is refused (status 1). Replaces cuda.BandedBatch.solve_mapped_ptr
 * (module.cpp:300-311; in place with one map as python/conatus/runtime/cuda.py:218-230 allows). */
int cng_banded_solve_mapped(const cng_banded* h, const void* rhs, const int64_t* rows, void* x,
                            const int64_t* cols, void* stream);

/* Complex factors, real data: b = re[rows_c] + i re[rows_s], x[cols_c] = Re, x[cols_s] = Im.
 * Replaces cuda.BandedBatch.solve_split_ptr (module.cpp:312-323). */
int cng_banded_solve_split(const cng_banded* h, const double* re, const int64_t* rows_c,
                           const int64_t* rows_s, double* x, const int64_t* cols_c,
                           const int64_t* cols_s, void* stream);

/* Build the transposed Woodbury data (allocates and synchronizes: call before a graph capture).
 * Replaces cuda.BandedBatch.prepare_transpose (module.cpp:416-419). */
int cng_banded_prepare_transpose(cng_banded* h, void* stream);
/* A^T x = b in place (plain transpose, no conjugation). Replaces
 * cuda.BandedBatch.solve_transpose_ptr (module.cpp:420-426). */
int cng_banded_solve_transpose(const cng_banded* h, void* b, void* stream);

/* Build the compact bucket-union form of the factors (complex128 handles): the union over the
 * batch of the nonzero slots of the LU factors and of V^T, packed for lockstep solves of 2 systems
 * per warp; later solves (all variants, FP64 and FP32) use it. Allocates and synchronizes. The
 * reference's GPU path drops the zeros of the factors per system instead (level-scheduled streams,
 * core/src/cuda/banded.cu:824-1121). */
int cng_banded_compact(cng_banded* h, void* stream);

/* One launch solving nh (<= 8) compact complex128 handles: x[k] = A_k^{-1} b[k] (fp32: with the FP32
 * factors, accumulate: x += ...). The buckets of a whole step in one launch, large ones first,
 * so that the latency of small buckets hides behind the large ones. */
int cng_banded_solve_batch(int nh, cng_banded* const* h, const void* const* b, void* const* x, int fp32,
                           int accumulate, void* stream);

/* cng_banded_solve_batch with the FP32 factors that also writes x row-major over the systems,
 * xt[k] = [n][batch] complex128 (NULL: not written), for the refinement residual's coalesced reads
 * (cng_split_residual's xT). */
int cng_banded_solve_batch_xt(int nh, cng_banded* const* h, const void* const* b, void* const* x,
                              void* const* xt, int accumulate, void* stream);

/* Shared factors of sign-similar buckets. With two RealFourier directions the (kx, +kz) and
 * (kx, -kz) systems of a group often differ only by signs: B = diag(dr) A diag(dc), dr and dc of
 * +1/-1 (host int8 arrays of n, in the matrix's own row and column order), the same for every
 * system of the batch. Then B x = b is y = A^{-1} (dr b), x = dc y with A's factors, bit for bit the
 * solve with B's own factorization (the pivot search compares magnitudes; sign flips are exact).
 * Marks handle h (A's batch) as shared: its compact streams (cng_banded_compact, which must come
 * after this call) hold one system per warp group, the partner's systems take the other half of
 * each warp. A border row k must keep the sign of its diagonal s e_k: dr[border[k]] dc[k] = +1,
 * else status 1. The caller checks the relation on the values (every entry of B equal to + or - the
 * entry of A, signs factoring as dr_i dc_j); this call takes it as given. Replaces the reference's
 * SharedFactor (python/conatus/timestep/shared_factors.py:1-40, found by sign_similarity,
 * shared_factors.py:104-138, and solved in timestep/device.py:396-485). */
int cng_banded_share(cng_banded* h, const int8_t* dr, const int8_t* dc, void* stream);

/* The general batched solve: cng_banded_solve_batch, plus for a shared handle k (cng_banded_share)
 * the partner's right-hand side b2[k] and solution x2[k] (NULL entries, or NULL arrays: no partner),
 * solved in the same sweep over the factor streams; fp32 = 1 may also write x row-major over the
 * systems into xt[k] and xt2[k] (the refinement residual's coalesced copy; NULL: not written).
 * range (NULL: every system): systems [range[2k], range[2k+1]) of handle k only (pointers still
 * address the whole batch), on warp-group boundaries (even for unshared handles), so that two
 * launches on two streams can each take a part of one large bucket. The band kernel (schedule -1)
 * and the split-lane schedules solve neither partners nor ranges (status 1). */
int cng_banded_solve_batch2(int nh, cng_banded* const* h, const void* const* b, void* const* x,
                            const void* const* b2, void* const* x2, void* const* xt, void* const* xt2,
                            const int32_t* range, int fp32, int accumulate, void* stream);

/* Schedules of the compact solve (the batched-solve kernel of the step): count, and per schedule
 * the columns per staged chunk of the factor streams, the depth of the staging ring and whether it
 * runs one system per warp with the lanes split over entries and real/imaginary parts (split = 1:
 * the latency variant for small batches; split = 2: the partitioned solve of small FP64 batches,
 * one block of warps per system sweeping its blocks of 32 columns at once; split = 3: the windowed
 * sweeps of two or four systems per warp, a window of each vector in shared memory and the rest in
 * a scratch, the same bits as schedule 0; else two systems per warp). Any output may be NULL. No
 * reference counterpart: the reference picks its solve kernel (level-scheduled streams or the band
 * kernel) by constructor flags (python/conatus/runtime/cuda.py:140-152); here the choice is timed
 * (conatus_gb300.autotune). */
int cng_banded_schedules(int32_t* count, int32_t* chunk, int32_t* stages, int32_t* split);
/* Schedule of a handle: 0 .. count-1 a compact schedule (needs cng_banded_compact), -1 the band
 * kernel (one warp per system, no compact streams). cng_banded_solve_batch uses the handles'
 * common schedule (schedule 0 when they differ; the band kernel per bucket when all are -1).
 * Setting the partitioned schedule builds its responses to unit window values (allocates, runs on
 * the legacy default stream and waits for it) and refuses (status 1) shared pairs, kl > 16,
 * kl + ku > 32, n > 1024 and responses above 256 MB; its solves refuse the FP32 factors and
 * system ranges. Its residuals run up to about 15x the sequential sweeps' (the blocks' separate
 * responses cancel). Setting another schedule frees the responses. Setting a windowed schedule
 * allocates its scratch (16 bytes x 2 x n per warp group of systems; freed when another schedule
 * is set): two solves of the same systems of h must then not run at the same time. */
int cng_banded_set_schedule(cng_banded* h, int sched);

/* Mixed precision: keep FP32 (complex64) copies of the FP64 factors (allocates; refreshed by
 * refactor_shared). No reference counterpart: the FP32 + FP64-refinement form of the solve. */
int cng_banded_make_fp32(cng_banded* h, void* stream);
/* x = A^{-1} b with the FP32 factors, b and x complex128 (accumulate != 0: x += A^{-1} b). One
 * refinement step is solve, residual in FP64 (cng_poly_residual), solve with accumulate. */
int cng_banded_solve_fp32(const cng_banded* h, const void* b, void* x, int accumulate, void* stream);

/* Host buffers: x = A^{-1} b (or A^{-T} b) with the copies inside the call, (batch, n) C-order.
 * The copies and kernels run on the legacy default stream and the call returns when x is on the
 * host; work the caller queued on non-blocking streams (a refactorization, a transpose preparation)
 * is not ordered before it: synchronize those streams first. Replaces
 * _core.BorderedBandedBatch{D,Z}.solve (core/bindings/module.cpp:184-206). */
int cng_banded_solve_host(cng_banded* h, const void* b_host, void* x_host, int transpose);

/* As cng_banded_solve_host, but allocates no device memory: the right-hand sides are staged in a
 * fixed 8 MiB device array built into the library (batch * n * element size must be at most
 * 8388608 bytes, else status 1, invalid argument; transpose needs cng_banded_prepare_transpose
 * first).
 * No counterpart in the reference. For callers that must not allocate: cng_banded_solve_host
 * allocates and frees a staging buffer on every call, and freeing device memory waits for the
 * whole device, which stalls every other stream (other runs in flight in a serving loop); a
 * caller under a planned device-memory budget must not grow its footprint either. The first call
 * on a device looks up the array's address. Every call on a device shares the one array, so
 * calls on one device take turns (a per-device lock, held from the copy in to the copy out). Like
 * cng_banded_solve_host it runs on the legacy default stream: synchronize the caller's own
 * non-blocking streams first. */
int cng_banded_solve_host_static(cng_banded* h, const void* b_host, void* x_host, int transpose);

/* ---- pseudospectral explicit right-hand side F(X) ------------------------------------------ */

typedef struct cng_rhs cng_rhs;

/* Description of F in polynomial form on the mode layout (host arrays, copied at creation).
 * Directions: ndir Fourier directions (0, 1 or 2; sizes nx, nz even, grids mx, mz >= 3/2 of them,
 * lengths lx, lz) and one Chebyshev direction (ny coefficients, even grid my >= the reference's
 * floor(3 ny / 2), length ly; without a Chebyshev direction ny = my = 1).
 * factors[5 f]: variable, component, derivative orders (x, y, z); out_lam[o]: conversion level
 * lambda of output o (0 = none); out_mono_ptr[o]..out_mono_ptr[o+1]-1: its monomials with
 * mono_coef[m] and mono_factors[4 m] (factor ids, -1 padded). buckets[5 b]: nsys, n, number of
 * nonzero Fourier indices, sign of the second direction, real flag; bucket_offset[b]: offset of the
 * bucket in the state (complex elements); modes[b][2 m]: (jx, jz) of system m; colpos[b][f ny + k]:
 * solver position of Chebyshev coefficient k of factor f's component (-1: absent);
 * rowmap[b][2 i]: (output, Chebyshev index) of row i (output -1: no explicit term). conv: nlam
 * dense ny x ny conversions T -> C^(lambda), lambda = 1..nlam. b0: constant part, nb0 entries
 * (state index, re, im). precision 0: FP64 transforms and products; 1: FP32. */
typedef struct {
    int32_t precision, ndir, nx, nz, mx, mz, ny, my;
    double lx, lz, ly;
    int32_t nfactors, noutputs;
    const int32_t* factors;
    const int32_t* out_lam;
    const int32_t* out_mono_ptr;
    const double* mono_coef;
    const int32_t* mono_factors;
    int32_t nbuckets;
    const int32_t* buckets;
    const int64_t* bucket_offset;
    const int32_t* const* modes;
    const int32_t* const* colpos;
    const int32_t* const* rowmap;
    int32_t nlam;
    const double* conv;
    int64_t nb0;
    const int64_t* b0_index;
    const double* b0_value;
    /* stacked cases (an ensemble of one template at one resolution): ncase (0 or 1: a single
     * problem) and per bucket the case of each system (nsys int32); the work arrays hold the
     * factors and outputs of every case (field index case * nfactors + f). No counterpart in the
     * reference, which runs ensemble members as separate solves (ensembles/batched.py:442-613). */
    int32_t ncase;
    const int32_t* const* case_of;
} cng_rhs_desc;

/* Build the F evaluator (allocates its work buffers). Replaces the reference's compiled F
 * (FusedRHS, python/conatus/timestep/fused.py:280-343; the GPU 2D pipeline
 * FourierChebyshev2DRHS, python/conatus/timestep/fc2d.py:433-643). */
int cng_rhs_create(const cng_rhs_desc* desc, cng_rhs** out);
int cng_rhs_destroy(cng_rhs* h);
/* rows = F(state) on the mode layout (complex128 device arrays; must not alias). Capturable.
 * Replaces IVPSolver.F (python/conatus/timestep/integrator.py:308-348). */
int cng_rhs_evaluate(cng_rhs* h, const void* state, void* rows, void* stream);
/* F of n problems of different sizes (or templates) in one launch per stage: every handle reads
 * `state` and writes `rows` at its own bucket offsets (set at creation: the problems share one mode
 * layout), with the arithmetic of cng_rhs_evaluate. The handles share one precision, the same
 * Fourier directions (at least one), a Chebyshev direction and one transform block size; each
 * appears once. Capturable. No reference counterpart: the reference advances ensemble members of
 * one discretization together (python/conatus/ensembles/batched.py:442-613), one size per batch. */
int cng_rhs_evaluate_group(int n, cng_rhs* const* h, const void* state, void* rows, void* stream);
/* Launch shape of the evaluator's shared-memory transforms: sequences per block (0: the default, 8
 * in FP32 and 4 in FP64; at most 32) and threads per block (0: 256; else a multiple of 32 in
 * 64..512). Knobs of the autotuner (conatus_gb300.autotune); no reference counterpart. */
int cng_rhs_set_tuning(cng_rhs* h, int maxseq, int threads);
/* Device bytes of the evaluator's work buffers (admission by footprint). */
int cng_rhs_workspace_bytes(const cng_rhs* h, uint64_t* bytes);

/* Chebyshev transforms of ncols contiguous complex128 columns on Gauss-Chebyshev nodes:
 * forward (m grid values -> n coefficients, DCT-II) or backward (n -> m, DCT-III); m even.
 * Replaces cuda.cheb_forward / cheb_backward (core/bindings/module.cpp:228-239,
 * core/src/cuda/transforms.cu:79-143). */
int cng_cheb_transform(int forward, const void* in, void* out, int64_t ncols, int n, int m, void* stream);
/* Complex FFT along the middle axis of [outer][len][inner] complex128: backward maps a compact
 * fftfreq-ordered spectrum of ncompact entries to length points (zero padding, unnormalized);
 * forward maps length points to ncompact coefficients (truncation, 1/length). Replaces
 * cuda.complexfourier_forward / backward (module.cpp:478-489). */
int cng_fft_axis(int forward, const void* in, void* out, int64_t outer, int inner, int ncompact,
                 int length, void* stream);
/* Real FFT along the middle axis: backward maps nmodes Hermitian half-spectrum modes (complex128)
 * to length real points; forward maps length real points to nmodes modes (1/length).
 * Replaces cuda.rfft / irfft and realfourier_forward / backward (module.cpp:456-477). */
int cng_rfft_axis(int forward, const void* in, void* out, int64_t outer, int inner, int nmodes,
                  int length, void* stream);

/* Device table exp(-2 pi i q / length), q < length (complex128, or complex64 when precision = 1),
 * owned by the library (one per length and precision, kept until exit). */
int cng_twiddle_table(int length, int precision, const void** table);

/* ---- ensembles of one-dimensional periodic problems ------------------------------------------ */

/* Members of different sizes and periods advanced by one launch per step (one CTA per member).
 * Per member (device arrays): N (even), grid M (3/2 dealiased, 2^a 3^b 5^c), offset of its N/2
 * complex mode amplitudes in the ensemble state, period, index of its grid size in plan_sizes.
 * The right-hand side is a polynomial in up to 4 factors (i k)^order u of one field; M(k), L(k)
 * are polynomials of degree <= 4 in k (coefficients as re, im pairs) for k > 0, m_mean/l_mean the
 * mean mode. precision 0: FFTs and products in FP64; 1: in FP32 (state, history, solve FP64). */
typedef struct {
    int32_t nmem, precision, nfactors, nmono, nplans;
    const int32_t* size_dev;
    const int32_t* grid_dev;
    const int64_t* offset_dev;
    const double* length_dev;
    const int32_t* plan_dev;
    int32_t plan_sizes[4];
    const void* twiddles64[4];
    const void* twiddles32[4];
    int32_t factor_order[4];
    double mono_coef[4];
    int32_t mono_factors[16];
    double m_poly[10], l_poly[10];
    double m_mean[2], l_mean[2];
} cng_fourier_ensemble_desc;

/* One SBDF-q step of every member: MXh[0], Fh[0] receive M C and F of the current state (the
 * newest history slot), MXh[j], Fh[j] (j < q) hold the older ones; c[j], d[j] the weights of F_j and
 * M C_j (d includes 1/dt), a0dt = a_0/dt. X is advanced in place. The reference advances ensemble
 * members through batched GlobalSystem solves (python/conatus/ensembles/batched.py:442-613, one
 * discretization per ensemble); here the sizes may differ within one launch. */
int cng_fourier_ensemble_step(const cng_fourier_ensemble_desc* desc, void* X, void* const* MXh, void* const* Fh,
                              int q, const double* c, const double* d, double a0dt, void* stream);

/* ---- IMEX step pieces ------------------------------------------------------------------------ */

/* y = M x per system of a bucket sharing one CSR pattern (indptr/indices device int32, n rows):
 * values_per_system = 0 -> one value array shared by every system, else values[m nnz + p].
 * x, y: (nsys, n) complex128. Replaces system.M @ X (python/conatus/timestep/device.py:78-105). */
int cng_csr_matvec(int nsys, int n, const int32_t* indptr, const int32_t* indices, const void* values,
                   int values_per_system, const void* x, void* y, void* stream);

/* r = b - (a M + c L(k_m)) x for every system m of a bucket, FP64: M values mval (nnz, shared),
 * L(k) = sum_t mono[m nmono + t] lcoef[t nnz + p] (wavenumber polynomial), shared CSR pattern.
 * The residual of the mixed-precision refinement (the reference solves in FP64 only). */
int cng_poly_residual(int nsys, int n, const int32_t* indptr, const int32_t* indices, const void* mval,
                      const void* lcoef, const double* mono, int nmono, double a, double c, const void* x,
                      const void* b, void* r, void* stream);

/* The same residual with the operator split per wavenumber monomial into real coefficients:
 * row i has entries ptr[i]..ptr[i+1]-1 with column col[e], real val[e] and code[e] = 2 t + imag
 * (t = monomial index, -1 for M; imag = 1 when the coefficient is i val). t = 63 marks one entry
 * list shared by several terms of the row (proportional coefficients), scaled by rowscale[i nsys +
 * system] (row-major n x nsys, FP64; NULL when no code holds t = 63). xT (may be NULL): x row-major
 * over the systems ([n][nsys], as cng_banded_solve_batch_xt writes it), read instead of x. */
int cng_split_residual(int nsys, int n, const int32_t* ptr, const int32_t* col, const double* val,
                       const int8_t* code, const double* mono, int nmono, double a, double c,
                       const double* rowscale, const void* x, const void* xT, const void* b, void* r,
                       void* stream);

/* cng_split_residual over systems [s0, s1) of the bucket's nsys only (every pointer addresses the
 * whole bucket): the refinement of one part of a bucket while another part is solved on another
 * stream. No reference counterpart. */
int cng_split_residual_range(int nsys, int s0, int s1, int n, const int32_t* ptr, const int32_t* col,
                             const double* val, const int8_t* code, const double* mono, int nmono, double a,
                             double c, const double* rowscale, const void* x, const void* xT, const void* b,
                             void* r, void* stream);

/* y = M x with one real value array shared by every system of the bucket (the mass matrices of the
 * tau systems are real). */
int cng_csr_matvec_real(int nsys, int n, const int32_t* indptr, const int32_t* indices, const double* values,
                        const void* x, void* y, void* stream);

/* Grouped forms: the buckets of several problems of different sizes in one launch, each part with
 * the arithmetic of its single-bucket call (cng_csr_matvec_real, cng_split_residual_range with a
 * common a and c). No reference counterpart (the reference advances one size per batch,
 * python/conatus/ensembles/batched.py:442-613). */
typedef struct cng_matvec_part {
    int32_t nsys, n;
    const int32_t* indptr;
    const int32_t* indices;
    const double* values;
    const void* x;
    void* y;
} cng_matvec_part;
int cng_csr_matvec_real_group(int nparts, const cng_matvec_part* parts, void* stream);

typedef struct cng_residual_part {
    int32_t nsys, s0, s1, n;
    const int32_t* ptr;
    const int32_t* col;
    const double* val;
    const int8_t* code;
    const double* mono;
    int32_t nmono;
    const double* rowscale;
    const void* x;
    const void* xT;
    const void* b;
    void* r;
} cng_residual_part;
int cng_split_residual_group(int nparts, const cng_residual_part* parts, double a, double c, void* stream);

/* out = base + sum_k (negate[k] ? -1 : +1) coef[k] vecs[k] over count complex128 entries, the terms
 * applied in order with explicit roundings (base NULL: start from 0); out may alias base. The
 * right-hand side of an IMEX Runge-Kutta stage, rk_rhs (python/conatus/timestep/lincomb.py:73-95),
 * and of a CN-family step, _cn_rhs (python/conatus/timestep/integrator.py:581-594). At most 12 terms. */
int cng_lincomb(int64_t count, const void* base, int nterms, const double* coef, const int32_t* negate,
                const void* const* vecs, void* out, void* stream);

/* rhs = sum_j (c_j F_j - d_j MX_j), j < q, on count complex128 entries (explicit roundings, no
 * FMA contraction, in the order of the reference's sbdf_rhs, python/conatus/timestep/lincomb.py:146-162). */
int cng_sbdf_rhs(int q, const double* c, const double* d, const void* const* F, const void* const* MX,
                 void* rhs, int64_t count, void* stream);
/* The same with fused = 1: fused multiply-adds, two FP64 operations per history level instead of
 * four (the FP32 form's combination; fused = 0 is cng_sbdf_rhs). No reference counterpart. */
int cng_sbdf_rhs_fused(int q, const double* c, const double* d, const void* const* F, const void* const* MX,
                       void* rhs, int64_t count, int fused, void* stream);

/* Finite-state check of count complex128 entries of x: when one of them holds a NaN or an
 * infinity, flag[0] (device int64, set to INT64_MAX by the caller) becomes min(flag[0], iteration).
 * Asynchronous on `stream`, capturable; the caller reads the flag. Replaces the reference's
 * check_state_finite (python/conatus/timestep/run_checks.py:67-99), the NumericalError check of
 * IVPSolver.run every FINITE_CHECK_EVERY = 100 steps and at the end of a run
 * (run_checks.py:15-20, python/conatus/timestep/integrator.py:764-767,1306-1312). */
int cng_check_finite(const void* x, int64_t count, int64_t iteration, int64_t* flag, void* stream);

/* Measurement: launch an FP64 fused-multiply-add loop (iters rounds of 8 independent chains per
 * thread, blocks_per_sm blocks of 256 threads on every SM) on `stream` and return its flop count in
 * *flops (16 per thread and round); the caller times it with events. sink: one device double (never
 * written for the probe's inputs). The FP64 peak the transforms' roofline is measured against. No
 * reference counterpart. */
int cng_dfma_probe(int64_t iters, int blocks_per_sm, void* sink, double* flops, void* stream);

/* ---- CUDA graphs of whole steps ------------------------------------------------------------- */

typedef struct cng_graph cng_graph;

/* Begin capturing the work launched on `stream` (thread-local capture mode). */
int cng_graph_begin(void* stream);
/* End the capture and instantiate it. Replaces the reference's CuPy graph capture of a step
 * (IVPSolver.run_graph / _capture_graph, python/conatus/timestep/integrator.py:781-920). */
int cng_graph_end(void* stream, cng_graph** out);
int cng_graph_launch(cng_graph* g, void* stream);
int cng_graph_destroy(cng_graph* g);

#ifdef __cplusplus
}
#endif

#endif /* CONATUS_GB300_H */
