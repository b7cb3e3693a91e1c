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
 * contiguous. rhs and x must not alias. Replaces cuda.BandedBatch.solve_mapped_ptr
 * (module.cpp:300-311). */
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

/* Host buffers: x = A^{-1} b (or A^{-T} b) with the copies inside the call, (batch, n) C-order.
 * Replaces _core.BorderedBandedBatch{D,Z}.solve (core/bindings/module.cpp:184-206). */
int cng_banded_solve_host(cng_banded* h, const void* b_host, void* x_host, int transpose);

#ifdef __cplusplus
}
#endif

#endif /* CONATUS_GB300_H */
