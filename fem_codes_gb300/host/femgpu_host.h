/* Host-side setup helpers of libfemgpu (plain C). */
#ifndef FEMGPU_HOST_H
#define FEMGPU_HOST_H

#include "femgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Reverse Cuthill-McKee permutation, perm[new] = old. */
int fgh_symrcm(int n, const int *IA, const int *JA, int *perm);
int fgh_bandwidth(int n, const int *IA, const int *JA);
/* Level schedule of the lower/upper triangle: rows [n], tasks allocated. */
int fgh_levels(int n, const int *IA, const int *JA, int lower, int *rows, int **task,
               int *ntask, int *nlev);
void fgh_set_error(const char *fmt, ...);

#ifdef __cplusplus
}
#endif
#endif
