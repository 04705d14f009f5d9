/* State of a steady Navier-Stokes context (VMS build, 3-dof block EBE
 * storage with the nodal block-diagonal preconditioner, or CSR storage with
 * ILU(0); Krylov workspace, damped Newton vectors).  Plain C; shared by ns_build.cu and host/ns.c.
 * Device layout: x, y [nnodes]; upresc [3*nnodes]; nodal force f [2*nnodes];
 * u, F, s, Fold [neq+1]; element residuals Re [9*nel]; stabilisation state
 * dold, nold [nel]; element matrices in the block-EBE context (A [81*nel]). */
#ifndef FG_NS_H
#define FG_NS_H
#include <cuda_runtime_api.h>
#include "femgpu.h"
#include "fg_internal.h"
#include "fg_ebe.h"

#ifdef __cplusplus
extern "C" {
#endif

struct femgpu_ns {
	femgpu_ns_opts o;
	int nnodes, nel, neq;
	cudaStream_t stream, own_stream;
	femgpu_ebe *ebe;
	double *x, *y, *upresc, *f;
	double *u, *F, *s, *Fold, *Re, *dold, *nold;
	double tol;                    /* current linear tolerance (forcing term) */
	int nbuild;                    /* builds since create / reset             */
	int setup_tag;                 /* precond_setup calls                     */
	int have_bd;
	fg_krylov kry;
	/* CSR storage (scheme FEMGPU_CSR, 9 equations per element) and its
	 * ILU(0) (host/blockcsr.c) */
	fg_blockcsr csr;
};

/* Build_K_F_MS on the device state u: element matrices into ebe->A, F, and
 * the stabilisation state updated (first != 0: the run's first build). */
int fg_ns_build(femgpu_ns *c, int first);
/* y += a x (neq entries). */
int fg_ns_axpy(femgpu_ns *c, double a, const double *x, double *y);

#ifdef __cplusplus
}
#endif
#endif
