/*
 * Test infrastructure only: the 6-argument GMRES the Euler and Navier-Stokes
 * drivers call (solver(P, M, FS, FF, B, X), EulerEquations.h:168,
 * SSNavierStokesEquations.h:152).  The shipped 00_CommonFiles/.../pgmres.c
 * only has the steady-transport 4-argument form, so those drivers do not link
 * as shipped; this is the documented adapter: the same algorithm and
 * arithmetic as pgmres.c:4-211 (left preconditioned, modified Gram-Schmidt,
 * Givens; the reference's ddot), taking B and X as arguments and
 * FemFunctions->mv as the product.  Included by the harnesses after their
 * equation header.
 */
double ddot(int, double *, double *);

/* pgmres.c:4-211 in the 6-argument form (B, X given). */
static int gmres6(ParametersType *P, MatrixDataType *M, FemStructsType *FS, FemFunctionsType *FF,
                  double *B, double *X)
{
	int i, j, k, l, cont, kmax = P->KrylovBasisVectorsQuantity, lmax = P->LinearMaxIter, neq = P->neq;
	double normb, eps, rho, r, h1, h2, soma;
	double **u = calloc(kmax + 1, sizeof(double *)), **h = calloc(kmax + 1, sizeof(double *));
	double *e = calloc(kmax + 1, sizeof(double)), *c = calloc(kmax, sizeof(double));
	double *s = calloc(kmax, sizeof(double)), *y = calloc(kmax, sizeof(double));
	double *v = calloc(neq + 1, sizeof(double));
	for (i = 0; i <= kmax; i++) { u[i] = calloc(neq + 1, sizeof(double)); h[i] = calloc(kmax + 1, sizeof(double)); }
	for (k = 0; k < neq; k++) X[k] = 0;
	normb = sqrt(ddot(neq, B, B));
	eps = P->SolverTolerance * normb;
	l = 0; cont = 0;
	do {
		i = 0;
		for (j = 0; j < kmax; j++) memset(u[j], 0, sizeof(double) * neq);
		memcpy(v, X, sizeof(double) * neq);
		FF->mv(P, M, FS, v, u[0]);
		FF->precond(P, M, FS, u[0], u[0]);
		for (k = 0; k < neq; k++) u[0][k] += -1.0 * B[k];
		for (k = 0; k < neq; k++) u[0][k] = -1.0 * u[0][k];
		e[0] = sqrt(ddot(neq, u[0], u[0]));
		{ double sc = 1.0 / e[0]; for (k = 0; k < neq; k++) u[0][k] = sc * u[0][k]; }
		rho = e[0];
		do {
			cont++;
			memcpy(v, u[i], sizeof(double) * neq);
			FF->mv(P, M, FS, v, u[i+1]);
			FF->precond(P, M, FS, u[i+1], u[i+1]);
			for (j = 0; j <= i; j++) {
				h[j][i] = ddot(neq, u[j], u[i+1]);
				for (k = 0; k < neq; k++) u[i+1][k] += -h[j][i] * u[j][k];
			}
			h[i+1][i] = sqrt(ddot(neq, u[i+1], u[i+1]));
			{ double sc = 1.0 / h[i+1][i]; for (k = 0; k < neq; k++) u[i+1][k] = sc * u[i+1][k]; }
			for (j = 0; j <= i - 1; j++) {
				h1 = c[j]*h[j][i] + s[j]*h[j+1][i];
				h2 = -s[j]*h[j][i] + c[j]*h[j+1][i];
				h[j][i] = h1; h[j+1][i] = h2;
			}
			r = sqrt(h[i][i]*h[i][i] + h[i+1][i]*h[i+1][i]);
			c[i] = h[i][i] / r; s[i] = h[i+1][i] / r;
			h[i][i] = r; h[i+1][i] = 0.0;
			e[i+1] = -s[i]*e[i]; e[i] = c[i]*e[i];
			rho = fabs(e[i+1]);
			i++;
		} while (rho > eps && i < kmax);
		i--;
		y[i] = e[i] / h[i][i];
		for (j = i - 1; j >= 0; j--) {
			soma = 0.0;
			for (k = j + 1; k <= i; k++) soma = soma + h[j][k]*y[k];
			y[j] = (e[j] - soma) / h[j][j];
		}
		for (j = 0; j <= i; j++) for (k = 0; k < neq; k++) X[k] = X[k] + u[j][k]*y[j];
		l++;
	} while (rho > eps && l < lmax);
	P->iterations += cont;
	for (i = 0; i <= kmax; i++) { free(u[i]); free(h[i]); }
	free(u); free(h); free(e); free(c); free(s); free(y); free(v);
	return 0;
}

