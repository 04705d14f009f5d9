/*
 * CSR storage of the multi-dof element systems (the Navier-Stokes and Euler
 * drivers' csr_Initialization.c / csr_assembly.c, reordering NOT) and the
 * ILU(0) set-up on it: the pattern is built on the device from the EBE
 * context's equation map and incidence lists, and the ILU(0) engine of
 * csrc/ilu.cu (level schedules, sweep programs, factor storage) runs on a
 * transport context that holds only this CSR system.  Plain C.
 */
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_internal.h"
#include "../csrc/fg_ebe.h"
#include "../csrc/fg_amg.h"

#define DM(ptr, bytes) do { int r_ = fgh_dmalloc((void **)&(ptr), (bytes)); if (r_) return r_; } while (0)

int fgh_blockcsr_create(fg_blockcsr *b, int M, const femgpu_ebe *ebe, int nel, int neq, cudaStream_t s, int ilu0,
                        int solver, int ilu_blocks)
{
	femgpu_transport *t;
	int *hIA = NULL, *hJA = NULL, *err = NULL, rc;
	size_t n1 = (size_t)neq + 1;
	DM(err, sizeof(int));
	CK(cudaMemset(err, 0, sizeof(int)));
	rc = fg_build_csr_m(M, nel, neq, ebe->ri_ptr, ebe->ri, ebe->lm, s, err, &b->IA, &b->JA, &b->sbe, &b->nnz);
	cudaFree(err);
	if (rc) { fgh_set_error("CSR pattern (%d equations per element): %d", M, rc); return rc > 0 ? FEMGPU_E_CUDA : rc; }
	DM(b->AA, sizeof(double) * ((size_t)b->nnz + 1));
	CK(cudaMemset(b->AA, 0, sizeof(double) * ((size_t)b->nnz + 1)));
	if (!ilu0) return 0;
	t = b->ilu = calloc(1, sizeof *t);
	if (!t) return FEMGPU_E_NOMEM;
	femgpu_transport_default_opts(&t->o);
	t->o.precond = FEMGPU_PREC_ILU0;
	t->o.solver = solver;
	t->o.ilu_blocks = ilu_blocks;
	t->neq = neq; t->nnz = b->nnz;
	t->IA = b->IA; t->JA = b->JA; t->A = b->AA;
	t->stream = s;
	DM(t->st, sizeof(fg_status));
	CK(cudaMemset(t->st, 0, sizeof(fg_status)));
	t->ilu.n = neq; t->ilu.nnz = b->nnz;
	DM(t->ilu.LU, sizeof(double) * ((size_t)b->nnz + 1));
	DM(t->ilu.Dinv, sizeof(double) * n1);
	hIA = malloc(sizeof(int) * n1);
	hJA = malloc(sizeof(int) * ((size_t)b->nnz + 1));
	if (!hIA || !hJA) { free(hIA); free(hJA); return FEMGPU_E_NOMEM; }
	rc = (cudaMemcpy(hIA, b->IA, sizeof(int) * n1, cudaMemcpyDeviceToHost) != cudaSuccess ||
	      cudaMemcpy(hJA, b->JA, sizeof(int) * (size_t)b->nnz, cudaMemcpyDeviceToHost) != cudaSuccess)
	     ? FEMGPU_E_CUDA : fg_ilu_prepare(t, hIA, hJA);
	free(hIA); free(hJA);
	if (rc) { fgh_set_error("ILU(0) set-up of the CSR system: %d", rc); return rc > 0 ? FEMGPU_E_CUDA : rc; }
	b->have_ilu = 1;
	return 0;
}

void fgh_blockcsr_destroy(fg_blockcsr *b)
{
	femgpu_transport *t = b->ilu;
	/* the AMG context is the caller's and outlives this one: give it back
	 * its own stream before the owner's stream goes away */
	if (b->amg) femgpu_amg_set_stream(b->amg, NULL);
	if (t) {
		if (b->have_ilu) fg_ilu_free(t);
		if (t->st) cudaFree(t->st);
		if (t->ilu.LU) cudaFree(t->ilu.LU);
		if (t->ilu.Dinv) cudaFree(t->ilu.Dinv);
		free(t);
	}
	if (b->IA) cudaFree(b->IA);
	if (b->JA) cudaFree(b->JA);
	if (b->sbe) cudaFree(b->sbe);
	if (b->AA) cudaFree(b->AA);
	memset(b, 0, sizeof *b);
}

int fgh_blockcsr_assemble(fg_blockcsr *b, int M, const femgpu_ebe *ebe, int neq, cudaStream_t s)
{
	KR(fg_assemble_csr_m(M, neq, b->nnz, b->IA, b->sbe, ebe->ri_ptr, ebe->ri, ebe->A, b->AA, s));
	return 0;
}

int fgh_blockcsr_factor(fg_blockcsr *b, cudaStream_t s)
{
	int err = 0;
	if (!b->ilu) return FEMGPU_E_NOT_BUILT;
	KR(fg_ilu0_factor(b->ilu));
	CK(cudaMemcpyAsync(&err, &b->ilu->st->err, sizeof(int), cudaMemcpyDeviceToHost, s));
	CK(cudaStreamSynchronize(s));
	if (err) { fgh_set_error("ILU(0) factorisation: %d", err); return err; }
	return 0;
}

void fgh_blockcsr_set_stream(fg_blockcsr *b, cudaStream_t s)
{
	if (b->ilu) b->ilu->stream = s;
	if (b->amg) femgpu_amg_set_stream(b->amg, s);
}

int fgh_blockcsr_amg_setup(fg_blockcsr *b, int neq, cudaStream_t s)
{
	int *IA, *JA, rc;
	double *AA;
	if (!b->amg) { fgh_set_error("AMG preconditioner not set"); return FEMGPU_E_NOT_BUILT; }
	IA = malloc(sizeof(int) * ((size_t)neq + 1));
	JA = malloc(sizeof(int) * (size_t)(b->nnz ? b->nnz : 1));
	AA = malloc(sizeof(double) * (size_t)(b->nnz ? b->nnz : 1));
	rc = (IA && JA && AA) ? 0 : FEMGPU_E_NOMEM;
	if (!rc && (cudaMemcpyAsync(IA, b->IA, sizeof(int) * ((size_t)neq + 1), cudaMemcpyDeviceToHost, s) ||
	            cudaMemcpyAsync(JA, b->JA, sizeof(int) * (size_t)b->nnz, cudaMemcpyDeviceToHost, s) ||
	            cudaMemcpyAsync(AA, b->AA, sizeof(double) * (size_t)b->nnz, cudaMemcpyDeviceToHost, s) ||
	            cudaStreamSynchronize(s)))
		rc = FEMGPU_E_CUDA;
	if (!rc) rc = femgpu_amg_setup(b->amg, neq, IA, JA, AA);
	free(IA); free(JA); free(AA);
	return rc;
}
