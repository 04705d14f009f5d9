/* State of a 2D Euler context (SUPG+CAU build, block EBE storage, nodal
 * block-diagonal preconditioner, Krylov workspace, predictor-multicorrector
 * vectors).  Plain C; shared by euler_build.cu and host/euler.c.
 * Device layout: x, y [nnodes]; upresc [4*nnodes] prescribed conservative
 * values; u, a (= du), R, Da [neq+1]; element residuals Re [12*nel]; the
 * element matrices live in the block-EBE context (A [144*nel]). */
#ifndef FG_EULER_H
#define FG_EULER_H
#include <cuda_runtime_api.h>
#include "femgpu.h"
#include "fg_internal.h"
#include "fg_ebe.h"

#ifdef __cplusplus
extern "C" {
#endif

struct femgpu_euler {
	femgpu_euler_opts o;
	int nnodes, nel, neq;
	cudaStream_t stream, own_stream;
	femgpu_ebe *ebe;               /* vert, node_id, lm, incidence, A, BD, invBD */
	double *x, *y, *upresc;
	double *u, *a, *R, *Da, *Re;
	fg_krylov kry;
	int built, have_bd;
	fg_blockcsr csr;               /* scheme FEMGPU_CSR: 12 equations per element */
	/* slip walls (femgpu_euler_set_slip): per node flag and the cos / sin of
	 * its wall angle, and the elements with a slip vertex */
	int *slip_flag, *slip_el, nslip_el;
	double *slip_cs, *slip_sn;
	double *dold;                  /* YZBeta, DD: each element's previous delta  */
	double *uB;                    /* DD: the element bubbles (4 per element)    */
	double alpha_build, dt_build;  /* the builds' Alpha_Build, DeltaT_Build      */
	double *u1, *u2, *uold;        /* BDF / TR-BDF2 history (neq+1 each)         */
	cudaEvent_t ev[4];
	double times[3];               /* build, precond setup, solve (s)            */
};

/* Build_M_K_F_SUPG: element matrices into e->ebe->A, residual into R, from
 * the nodal state (u, du) (device vectors of neq+1). */
int fg_euler_build(femgpu_euler *c, const double *u, const double *du);
/* u += c_pred a, a = 0 (Predictor_Old.c:57-62). */
int fg_euler_predict(femgpu_euler *c, double c_pred);
/* a += Da, u += c_corr Da (Predictor_Old.c:115-116). */
int fg_euler_correct(femgpu_euler *c, double c_corr);
/* u = cp p - cq q, a = 0 (u may be p): Predictor_Old_BDF.c:119-123,
 * Predictor_Old_TRBDF2.c:118-122. */
int fg_euler_lin(femgpu_euler *c, const double *p, const double *q, double cp, double cq);

#ifdef __cplusplus
}
#endif
#endif
