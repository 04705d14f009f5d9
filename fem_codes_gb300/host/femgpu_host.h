/* Host-side setup helpers of libfemgpu (plain C). */
#ifndef FEMGPU_HOST_H
#define FEMGPU_HOST_H

#include <cuda_runtime_api.h>

#include "femgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Return FEMGPU_E_CUDA from the enclosing function on a CUDA runtime error
 * (CK), or on a launcher's cudaError_t > 0 / pass its FEMGPU_E* < 0 (KR);
 * the message goes to femgpu_last_error(). */
#define CK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) {                   \
	fgh_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));     \
	return FEMGPU_E_CUDA; } } while (0)
#define KR(call) do { int r_ = (call); if (r_ > 0) {                                        \
	fgh_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString((cudaError_t)r_)); \
	return FEMGPU_E_CUDA; }                                                                 \
	if (r_ < 0) { fgh_set_error("%s:%d %s: error %d", __FILE__, __LINE__, #call, r_); return r_; } \
	} while (0)

/* Reverse Cuthill-McKee permutation, perm[new] = old. */
int fgh_symrcm(int n, const int *IA, const int *JA, int *perm);
int fgh_bandwidth(int n, const int *IA, const int *JA);
/* Level schedule of the lower/upper triangle: rows [n], tasks allocated. */
int fgh_levels(int n, const int *IA, const int *JA, int lower, int *rows, int **task,
               int *ntask, int *nlev);
void fgh_set_error(const char *fmt, ...);
int fgh_dmalloc(void **p, size_t bytes);
struct femgpu_transport;
int fgh_transport_gmres(struct femgpu_transport *t, const double *B, double *X, int *iters);

/* Krylov workspace (fg_internal.h fg_krylov) for n unknowns and kmax basis
 * vectors; zmode 0: no FGMRES Z, 1: FP64 Z, 2: FP32 Z. */
struct fg_krylov;
struct fg_linop;
int fgh_kry_alloc(struct fg_krylov *k, int n, int kmax, int zmode, void *stream);
void fgh_kry_free(struct fg_krylov *k);
/* Restart cycles until rho <= eps or lmax cycles; kind -1: left-
 * preconditioned pgmres, 0/1/2: FGMRES mixed mode.  Adds the inner
 * iterations to *iters; FEMGPU_E_NOT_CONVERGED when lmax is reached. */
int fgh_kry_cycles(const struct fg_krylov *k, const struct fg_linop *op, const double *B, double *X,
                   int kind, double eps, int lmax, int *iters);
/* The pieces of fgh_kry_cycles: reset the status for a solve to eps, then
 * run one restart cycle (the solve's cycle-th) and read the status back
 * (k->st_host). */
int fgh_kry_begin(const struct fg_krylov *k, double eps);
int fgh_kry_cycle(const struct fg_krylov *k, const struct fg_linop *op, const double *B, double *X, int kind,
                  int cycle);
/* ||B||^2 on the device, returned to the host (synchronises the stream). */
int fgh_kry_dot_host(const struct fg_krylov *k, const double *a, const double *b, int n, double *out);

/* Symbolic ILU(p) (host/iluk.c): the filled pattern in the reference's row
 * layout (lower ascending, diagonal, upper in elimination order) and the
 * position of each of the matrix's entries in it (malloc'd arrays). */
int fgh_iluk_pattern(int n, const int *IA, const int *JA, int p, int **fIA, int **fJA, int **map);

/* Block CSR storage of an EBE element system with M = 3*ndof equations per
 * element (host/blockcsr.c): the pattern built on the device from the EBE
 * context's lm and incidence lists and, when ilu0, the ILU(0) structure of
 * a transport context (solver: the Krylov solver its sweeps serve,
 * ilu_blocks as femgpu_transport_opts.ilu_blocks). */
struct fg_blockcsr;
struct femgpu_ebe;
int fgh_blockcsr_create(struct fg_blockcsr *b, int M, const struct femgpu_ebe *ebe, int nel, int neq,
                        cudaStream_t s, int ilu0, int solver, int ilu_blocks);
void fgh_blockcsr_destroy(struct fg_blockcsr *b);
/* csr_assembly.c per row from the element matrices ebe->A. */
int fgh_blockcsr_assemble(struct fg_blockcsr *b, int M, const struct femgpu_ebe *ebe, int neq, cudaStream_t s);
/* ILU(0) factorisation (ILUp_precond_setup.c:66-167 at fill level 0) of
 * the current values; FEMGPU_E_ZERO_PIVOT on a zero pivot. */
int fgh_blockcsr_factor(struct fg_blockcsr *b, cudaStream_t s);
void fgh_blockcsr_set_stream(struct fg_blockcsr *b, cudaStream_t s);
/* AMG_precond_setup (amg_precond.c:26-100) on the current values: the
 * hierarchy of the attached AMG context, set up on the host. */
int fgh_blockcsr_amg_setup(struct fg_blockcsr *b, int neq, cudaStream_t s);

#ifdef __cplusplus
}
#endif
#endif
