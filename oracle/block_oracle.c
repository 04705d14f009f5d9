/*
 * Test infrastructure only -- CPU oracle for the multi-dof EBE operators of
 * the Euler (4 dof/node) and Navier-Stokes (3 dof/node) drivers, restated in
 * this project's own code with the reference's evaluation order:
 *   ebemvNDOF4.c:5-112 / ebemvNDOF3.c:3-86      element-by-element product
 *   ebe2mvNDOF4.c:4-79                           off-diagonal node blocks only
 *   BlockDiag_precond_EBE_setup.c:6-145,         nodal diagonal blocks, their
 *   BlockDiagDOF3_precond_EBE_setup.c           closed-form inverses, F := D^-1 F
 *   BlockDiag_precond.c, BlockDiagDOF3_precond.c, BlockDiag2_precond.c,
 *   NOBlockDiag2_precond.c                       nodal block applications
 * Element matrices are A[e][m*m] row-major (m = 3*ndof); lm[e][ndof*a+k] is
 * the equation of dof k of vertex a (neq when prescribed, Fill_LM.c).
 */
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

void orc_fill_lm_blk(int ndof, int nel, const int *vert, const int *node_id, int neq, int *lm)
{
	int e, a, k, m = 3 * ndof;
	for (e = 0; e < nel; e++)
		for (a = 0; a < 3; a++)
			for (k = 0; k < ndof; k++) {
				int id = node_id[ndof * vert[3 * e + a] + k];
				lm[e * m + ndof * a + k] = (id == -1) ? neq : id;
			}
}

/* Q = A P, element by element (ebemvNDOF4 / ebemvNDOF3). */
void orc_ebemv_blk(int ndof, int neq, int nel, const int *lm, const double *A, double *P, double *Q)
{
	int e, a, b, m = 3 * ndof;
	double p[12];
	for (a = 0; a < neq; a++) Q[a] = 0;
	P[neq] = 0;
	Q[neq] = 0;
	for (e = 0; e < nel; e++) {
		const int *l = lm + (size_t)e * m;
		const double *Ae = A + (size_t)e * m * m;
		for (b = 0; b < m; b++) p[b] = P[l[b]];
		for (a = 0; a < m; a++) {
			double s = Ae[a * m] * p[0];
			for (b = 1; b < m; b++) s = s + Ae[a * m + b] * p[b];
			Q[l[a]] += s;
		}
		Q[neq] = 0.0;
	}
}

/* Id[node][k] of BlockDiag_precond_EBE_setup.c:35-61: equation or neq. */
static int blk_id(const int *node_id, int ndof, int neq, int node, int k)
{
	int id = node_id[ndof * node + k];
	return id < 0 ? neq : id;
}

/* Nodal diagonal blocks summed over the elements in element order. */
void orc_blockdiag_assemble(int ndof, int nnodes, int nel, const int *vert, const double *A, double *BD)
{
	int e, a, I, J, m = 3 * ndof, d2 = ndof * ndof;
	memset(BD, 0, sizeof(double) * (size_t)nnodes * d2);
	for (e = 0; e < nel; e++)
		for (I = 0; I < ndof; I++)
			for (J = 0; J < ndof; J++)
				for (a = 0; a < 3; a++)
					BD[(size_t)vert[3 * e + a] * d2 + ndof * I + J] +=
						A[(size_t)e * m * m + (size_t)(ndof * a + I) * m + ndof * a + J];
}

/* Closed-form inverse by cofactors: 4x4 of BlockDiag_precond_EBE_setup.c:88-145,
 * 3x3 of BlockDiagDOF3_precond_EBE_setup.c:90-120 (the adjugate over the
 * determinant, expanded in the same order). */
void orc_inverse4(const double *B, double *V)
{
	double a = B[0], b = B[1], c = B[2], d = B[3], e = B[4], f = B[5], g = B[6], h = B[7];
	double i = B[8], j = B[9], k = B[10], l = B[11], m = B[12], n = B[13], o = B[14], p = B[15];
	double det = (a*f*k*p - a*f*l*o - a*g*j*p + a*g*l*n + a*h*j*o - a*h*k*n
		-b*e*k*p  + b*e*l*o + b*g*i*p - b*g*l*m - b*h*i*o + b*h*k*m +
		c*(e*j*p - e*l*n - f*i*p + f*l*m + h*i*n - h*j*m) +
		d*(-e*j*o + e*k*n + f*i*o - f*k*m - g*i*n + g*j*m));
	double q = 1.0/det;
	V[0] = q*(-h*k*n + g*l*n + h*j*o - f*l*o - g*j*p + f*k*p);
	V[1] = q*(d*k*n - c*l*n - d*j*o + b*l*o + c*j*p - b*k*p);
	V[2] = q*(-d*g*n + c*h*n + d*f*o - b*h*o - c*f*p + b*g*p);
	V[3] = q*(d*g*j - c*h*j - d*f*k + b*h*k + c*f*l - b*g*l);
	V[4] = q*(h*k*m - g*l*m - h*i*o + e*l*o + g*i*p - e*k*p);
	V[5] = q*(-d*k*m + c*l*m + d*i*o - a*l*o - c*i*p + a*k*p);
	V[6] = q*(d*g*m - c*h*m - d*e*o + a*h*o + c*e*p - a*g*p);
	V[7] = q*(-d*g*i + c*h*i + d*e*k - a*h*k - c*e*l + a*g*l);
	V[8] = q*(-h*j*m + f*l*m + h*i*n - e*l*n - f*i*p + e*j*p);
	V[9] = q*(d*j*m - b*l*m - d*i*n + a*l*n + b*i*p - a*j*p);
	V[10] = q*(-d*f*m + b*h*m + d*e*n - a*h*n - b*e*p + a*f*p);
	V[11] = q*(d*f*i - b*h*i - d*e*j + a*h*j + b*e*l - a*f*l);
	V[12] = q*(g*j*m - f*k*m - g*i*n + e*k*n + f*i*o - e*j*o);
	V[13] = q*(-c*j*m + b*k*m + c*i*n - a*k*n - b*i*o + a*j*o);
	V[14] = q*(c*j*m - b*g*m - c*e*n + a*g*n + b*e*o - a*f*o);
	V[15] = q*(-c*f*i + b*g*i + c*e*j - a*g*j - b*e*k + a*f*k);
}

void orc_inverse3(const double *B, double *V)
{
	double a = B[0], b = B[1], c = B[2], d = B[3], e = B[4], f = B[5], g = B[6], h = B[7], i = B[8];
	double det = a*e*i - a*f*h - b*d*i + b*f*g + c*d*h - c*e*g;
	double q = 1.0/det;
	V[0] = q*(e*i-f*h); V[1] = q*(c*h-b*i); V[2] = q*(b*f-c*e);
	V[3] = q*(f*g-d*i); V[4] = q*(a*i-c*g); V[5] = q*(c*d-a*f);
	V[6] = q*(d*h-e*g); V[7] = q*(b*g-a*h); V[8] = q*(a*e-b*d);
}

/* z = D^-1 p node by node (BlockDiag_precond.c / BlockDiagDOF3_precond.c);
 * p may equal z. */
void orc_blockdiag_apply(int ndof, int nnodes, int neq, const int *node_id, const double *invBD,
                         const double *p, double *z)
{
	int I, r, c, d2 = ndof * ndof;
	for (I = 0; I < nnodes; I++) {
		double v[4];
		for (c = 0; c < ndof; c++) v[c] = p[blk_id(node_id, ndof, neq, I, c)];
		for (r = 0; r < ndof; r++) {
			const double *row = invBD + (size_t)I * d2 + ndof * r;
			double s = row[0] * v[0];
			for (c = 1; c < ndof; c++) s = s + row[c] * v[c];
			z[blk_id(node_id, ndof, neq, I, r)] = s;
		}
		z[neq] = 0;
	}
}

/* Set-up: assemble, invert, F := D^-1 F. */
void orc_blockdiag_setup(int ndof, int nnodes, int nel, int neq, const int *vert, const int *node_id,
                         const double *A, double *BD, double *invBD, double *F)
{
	int I, d2 = ndof * ndof;
	orc_blockdiag_assemble(ndof, nnodes, nel, vert, A, BD);
	for (I = 0; I < nnodes; I++) {
		if (ndof == 4) orc_inverse4(BD + (size_t)I * d2, invBD + (size_t)I * d2);
		else orc_inverse3(BD + (size_t)I * d2, invBD + (size_t)I * d2);
	}
	if (F) orc_blockdiag_apply(ndof, nnodes, neq, node_id, invBD, F, F);
}

/* ebe2mvNDOF4.c:15-79: off-diagonal node blocks of every element, then
 * with_inverse ? Q = P + D^-1 Q (BlockDiag2_precond.c) : Q += D P
 * (NOBlockDiag2_precond.c). */
void orc_ebe2mv4(int nnodes, int neq, int nel, const int *lm, const int *node_id, const double *A,
                 const double *BD, const double *invBD, int with_inverse, double *P, double *Q)
{
	int e, a, b, I, r, c;
	double p[12];
	for (a = 0; a < neq; a++) Q[a] = 0;
	P[neq] = 0;
	Q[neq] = 0;
	for (e = 0; e < nel; e++) {
		const int *l = lm + (size_t)e * 12;
		const double *Ae = A + (size_t)e * 144;
		for (b = 0; b < 12; b++) p[b] = P[l[b]];
		for (a = 0; a < 12; a++) {
			int first = 1;
			double s = 0.0;
			for (b = 0; b < 12; b++) {
				if (b / 4 == a / 4) continue;
				if (first) { s = Ae[a * 12 + b] * p[b]; first = 0; }
				else s = s + Ae[a * 12 + b] * p[b];
			}
			Q[l[a]] += s;
		}
		Q[neq] = 0.0;
	}
	for (I = 0; I < nnodes; I++) {
		double v[4];
		const double *B = (with_inverse ? invBD : BD) + (size_t)I * 16;
		for (c = 0; c < 4; c++) v[c] = with_inverse ? Q[blk_id(node_id, 4, neq, I, c)] : P[blk_id(node_id, 4, neq, I, c)];
		for (r = 0; r < 4; r++) {
			int id = blk_id(node_id, 4, neq, I, r);
			if (with_inverse) {           /* p + i0 a + i1 b + i2 c + i3 d, left to right */
				double s = P[id];
				for (c = 0; c < 4; c++) s = s + B[4 * r + c] * v[c];
				Q[id] = s;
			} else {
				double s = B[4 * r] * v[0] + B[4 * r + 1] * v[1] + B[4 * r + 2] * v[2] + B[4 * r + 3] * v[3];
				Q[id] += s;
			}
		}
		Q[neq] = 0;
	}
}
