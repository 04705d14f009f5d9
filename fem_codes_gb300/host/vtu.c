/*
 * VTU output of the steady-transport solution: the file Paraview_Output.c
 * (01_SS_Transport_Equation/2D/01_CommonFiles/Paraview_Output.c:5-85)
 * writes, byte for byte -- ASCII UnstructuredGrid, the nodal solution (the
 * equation's value, or the prescribed value at a prescribed node) as point
 * data and as the third coordinate, triangles as cells.
 *
 * The nodal values are gathered on the device (fg_nodal_values) and come
 * back with the coordinates and connectivity in one round of copies; the
 * text is formatted by several host threads into per-chunk buffers that are
 * then written in order (at 2048x1024 cells the reference's single fprintf
 * loop is the whole cost of an output).  Plain C.
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "femgpu.h"
#include "femgpu_host.h"
#include "../csrc/fg_internal.h"

int fg_nodal_values(const double *u, const int *node_id, const double *upresc, int nnodes, double *out,
                    cudaStream_t s);

#define VTU_THREADS 8

typedef struct {
	int kind, i0, i1;               /* 0 values, 1 points, 2 cells, 3 offsets, 4 types */
	const double *x, *y, *v;
	const int *vert;
	char *buf;
	size_t len, cap;
} vtu_chunk;

static int put(vtu_chunk *c, const char *fmt_out, int n)
{
	if (c->len + (size_t)n + 1 > c->cap) {
		size_t cap = 2 * c->cap + (size_t)n + 4096;
		char *b = realloc(c->buf, cap);
		if (!b) return -1;
		c->buf = b;
		c->cap = cap;
	}
	memcpy(c->buf + c->len, fmt_out, (size_t)n);
	c->len += (size_t)n;
	return 0;
}

static void *format_chunk(void *arg)
{
	vtu_chunk *c = arg;
	char line[160];
	int i, n;
	for (i = c->i0; i < c->i1; i++) {
		switch (c->kind) {
		case 0: n = snprintf(line, sizeof line, "\t\t\t\t   %.12f\n", c->v[i]); break;
		case 1: n = snprintf(line, sizeof line, "\t\t\t\t   %.12f\t%.12f\t%.12f\n", c->x[i], c->y[i], c->v[i]); break;
		case 2: n = snprintf(line, sizeof line, "\t\t\t\t   %d\t%d\t%d\n", c->vert[3 * i], c->vert[3 * i + 1],
		                     c->vert[3 * i + 2]); break;
		case 3: n = snprintf(line, sizeof line, "\t\t\t\t   %d\n", (i + 1) * 3); break;
		default: n = snprintf(line, sizeof line, "\t\t\t\t   %d\n", 5); break;
		}
		if (n < 0 || put(c, line, n)) { c->len = (size_t)-1; return NULL; }
	}
	return NULL;
}

/* One section (kind) of count lines, formatted by VTU_THREADS threads and
 * appended to f in order. */
static int section(FILE *f, int kind, int count, const double *x, const double *y, const double *v, const int *vert)
{
	vtu_chunk c[VTU_THREADS];
	pthread_t th[VTU_THREADS];
	int k, started[VTU_THREADS], rc = 0;
	for (k = 0; k < VTU_THREADS; k++) {
		memset(&c[k], 0, sizeof c[k]);
		c[k].kind = kind;
		c[k].i0 = (int)((long long)count * k / VTU_THREADS);
		c[k].i1 = (int)((long long)count * (k + 1) / VTU_THREADS);
		c[k].x = x; c[k].y = y; c[k].v = v; c[k].vert = vert;
		started[k] = pthread_create(&th[k], NULL, format_chunk, &c[k]) == 0;
		if (!started[k]) format_chunk(&c[k]);
	}
	for (k = 0; k < VTU_THREADS; k++) {
		if (started[k]) pthread_join(th[k], NULL);
		if (c[k].len == (size_t)-1) rc = FEMGPU_E_NOMEM;
		else if (!rc && c[k].len && fwrite(c[k].buf, 1, c[k].len, f) != c[k].len) rc = FEMGPU_E_ARG;
		free(c[k].buf);
	}
	return rc;
}

int femgpu_transport_write_vtu(femgpu_transport *t, const char *path, const double *u_host)
{
	double *d_val = NULL, *d_u = NULL, *x = NULL, *y = NULL, *v = NULL;
	int *vert = NULL, rc = 0, nn, ne;
	FILE *f = NULL;
	if (!t || !path) return FEMGPU_E_ARG;
	nn = t->nnodes;
	ne = t->nel;
	x = malloc(sizeof(double) * (size_t)nn);
	y = malloc(sizeof(double) * (size_t)nn);
	v = malloc(sizeof(double) * (size_t)nn);
	vert = malloc(sizeof(int) * 3 * (size_t)ne);
	if (!x || !y || !v || !vert) { rc = FEMGPU_E_NOMEM; goto out; }
	if (fgh_dmalloc((void **)&d_val, sizeof(double) * (size_t)nn)) { rc = FEMGPU_E_NOMEM; goto out; }
	if (u_host) {
		if (fgh_dmalloc((void **)&d_u, sizeof(double) * ((size_t)t->neq + 1))) { rc = FEMGPU_E_NOMEM; goto out; }
		if (cudaMemcpyAsync(d_u, u_host, sizeof(double) * ((size_t)t->neq + 1), cudaMemcpyHostToDevice,
		                    t->stream) != cudaSuccess) { rc = FEMGPU_E_CUDA; goto out; }
	}
	if (fg_nodal_values(u_host ? d_u : t->u, t->node_id, t->upresc, nn, d_val, t->stream) ||
	    cudaMemcpyAsync(v, d_val, sizeof(double) * (size_t)nn, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
	    cudaMemcpyAsync(x, t->x, sizeof(double) * (size_t)nn, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
	    cudaMemcpyAsync(y, t->y, sizeof(double) * (size_t)nn, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
	    cudaMemcpyAsync(vert, t->vert, sizeof(int) * 3 * (size_t)ne, cudaMemcpyDeviceToHost, t->stream) !=
	        cudaSuccess ||
	    cudaStreamSynchronize(t->stream) != cudaSuccess) {
		fgh_set_error("write_vtu: device copies failed");
		rc = FEMGPU_E_CUDA;
		goto out;
	}
	f = fopen(path, "w");
	if (!f) { fgh_set_error("write_vtu: cannot open %s", path); rc = FEMGPU_E_ARG; goto out; }
	fprintf(f, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n");
	fprintf(f, "\t<UnstructuredGrid>\n");
	fprintf(f, "\t\t<Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", nn, ne);
	fprintf(f, "\t\t\t<PointData Scalars=\"scalars\">\n");
	fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" Name=\"solucao\" Format=\"ascii\">\n");
	if (!rc) rc = section(f, 0, nn, x, y, v, vert);
	fprintf(f, "\t\t\t\t</DataArray>\n");
	fprintf(f, "\t\t\t</PointData>\n");
	fprintf(f, "\t\t\t<Points>\n");
	fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n");
	if (!rc) rc = section(f, 1, nn, x, y, v, vert);
	fprintf(f, "\t\t\t\t</DataArray>\n");
	fprintf(f, "\t\t\t</Points>\n");
	fprintf(f, "\t\t\t<Cells>\n");
	fprintf(f, "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n");
	if (!rc) rc = section(f, 2, ne, x, y, v, vert);
	fprintf(f, "\t\t\t\t</DataArray>\n");
	fprintf(f, "\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n");
	if (!rc) rc = section(f, 3, ne, x, y, v, vert);
	fprintf(f, "\t\t\t\t</DataArray>\n");
	fprintf(f, "\t\t\t\t<DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n");
	if (!rc) rc = section(f, 4, ne, x, y, v, vert);
	fprintf(f, "\t\t\t\t</DataArray>\n");
	fprintf(f, "\t\t\t</Cells>\n");
	fprintf(f, "\t\t</Piece>\n");
	fprintf(f, "\t</UnstructuredGrid>\n");
	fprintf(f, "</VTKFile>\n");
	if (fclose(f) != 0 && !rc) rc = FEMGPU_E_ARG;
out:
	if (d_val) cudaFree(d_val);
	if (d_u) cudaFree(d_u);
	free(x); free(y); free(v); free(vert);
	return rc;
}
