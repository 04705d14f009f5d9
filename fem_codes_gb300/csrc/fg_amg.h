/* Device state of the double-pairwise AMG preconditioner (host/amg.c sets it
 * up, amg.cu runs the V-cycle).  Plain C header. */
#ifndef FG_AMG_H
#define FG_AMG_H

#include <cuda_runtime_api.h>

#include "femgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A run of consecutive SOR levels: `wide` levels are launched one grid each,
 * a narrow run goes to one thread block that walks its levels in order. */
typedef struct { int l0, l1, wide; } fg_amg_seg;

typedef struct fg_amg_level {
	int n, nnz;
	/* device: CSR and diagonal (even levels: the ones that are smoothed) */
	int *ptr, *col;
	double *val, *diag;
	double *f, *u;
	/* SOR schedules: rows in processing order, level offsets, segments */
	int *fw_rows, *fw_lev, *bw_rows, *bw_lev;
	int fw_nlev, bw_nlev;
	int *h_fw_lev, *h_bw_lev;
	fg_amg_seg *fw_seg, *bw_seg;
	int fw_nseg, bw_nseg;
	/* even l below the coarsest: restriction to level l+2 (4 fine rows per
	 * level-(l+2) row, -1 where absent) and the composite aggregate map */
	int4 *quad;
	int *agg2;
	int nc2;
	/* host copies: the level's CSR and (l below the coarsest) its matching */
	int *h_ptr, *h_col, *h_match;
	double *h_val;
} fg_amg_level;

struct femgpu_amg {
	int ncl, nr;
	double beta, omega;
	int nlevels;                 /* 2*ncl + 1 matrices */
	fg_amg_level *lv;
	double *qcopy;               /* [n0]: the input when q and z alias */
	cudaStream_t stream, own_stream;
};

/* z = M^-1 q: one V-cycle (dpa_Vcycle_precond, amg_dpa.c:485-506).  Every
 * kernel is skipped while *active == 0 (active may be NULL). */
int fg_amg_vcycle(femgpu_amg *g, const double *q, double *z, const int *active);

#ifdef __cplusplus
}
#endif
#endif
