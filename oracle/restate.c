/* Oracle: plain-C restatement of the reference algorithms on the projection
 * hot path. TEST INFRASTRUCTURE ONLY (see restate.h): the product library
 * never links it; tests, the smoke check and the benchmark's CPU-baseline
 * leg use it as the checker. Every function names the reference lines it
 * restates. Compiled with -ffp-contract=off so each a*b+c rounds twice, as
 * the reference's x86 build does. */
#include "restate.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SMALL 1e-10 /* lib/type_define.hpp */

/* ------------------------------------------------------------ BLAS-1 --- */
/* BLAS_Level1.hpp:499-544: leading (n-1)%5+1 terms one by one, then the rest
 * five at a time, each group added left to right onto the running sum. */
double rs_dot(int n, const double* sx, const double* sy) {
	double dot = 0.0;
	if (n <= 0) return dot;
	int m = (n - 1) % 5;
	for (int i = 0; i <= m; ++i) dot = dot + sx[i] * sy[i];
	if (n <= 5) return dot;
	for (int i = m + 1; i < n; i += 5) {
		dot = dot + sx[i] * sy[i] + sx[i + 1] * sy[i + 1]
				+ sx[i + 2] * sy[i + 2] + sx[i + 3] * sy[i + 3]
				+ sx[i + 4] * sy[i + 4];
	}
	return dot;
}

/* BLAS_Level1.hpp:556-577: sqrt of the sum of squares of x[0..n-2]; the last
 * element is left out, zeros are skipped, n == 1 gives |x[0]|. */
double rs_nrm2(int n, const double* x) {
	double norm = 0.0;
	if (n <= 0) return norm;
	if (n == 1) return fabs(x[0]);
	for (int i = 0; i < n - 1; ++i) {
		if (x[i] != 0.0) norm += x[i] * x[i];
	}
	return sqrt(norm);
}

/* threaded variants for the CPU baseline: fixed static partition, partial sums
 * combined in thread order (deterministic for a given thread count) */
static double par_dot(int n, const double* x, const double* y, int th) {
	if (th <= 1) return rs_dot(n, x, y);
	double part[256];
	if (th > 256) th = 256;
	memset(part, 0, sizeof part);
#pragma omp parallel num_threads(th)
	{
#ifdef _OPENMP
		int t = omp_get_thread_num(), nt = omp_get_num_threads();
#else
		int t = 0, nt = 1;
#endif
		long lo = (long)n * t / nt, hi = (long)n * (t + 1) / nt;
		double s = 0.0;
		for (long i = lo; i < hi; ++i) s += x[i] * y[i];
		part[t] = s;
	}
	double s = 0.0;
	for (int t = 0; t < th; ++t) s += part[t];
	return s;
}
static double par_nrm2(int n, const double* x, int th) {
	if (th <= 1) return rs_nrm2(n, x);
	if (n == 1) return fabs(x[0]);
	return sqrt(par_dot(n - 1, x, x, th));
}

/* MatrixSCR_::operator* (matrix_SparCompRow.hpp:236-249): per row, from 0,
 * res += x[col] * val in stored order. */
static void spmv(int n, const unsigned* rp, const unsigned* ci,
		const double* va, const double* x, double* y, int th) {
#pragma omp parallel for num_threads(th) if (th > 1) schedule(static)
	for (int i = 0; i < n; ++i) {
		double s = 0.0;
		for (unsigned k = rp[i]; k < rp[i + 1]; ++k) s += x[ci[k]] * va[k];
		y[i] = s;
	}
}

/* carpio::Residual (solver_matrix.hpp:583-597): nrm2(b - A x) / nrm2(b),
 * normb = 1 when it is 0, with nrm2's drop-last quirk (full != 0: every
 * element counted). */
double rs_residual(int n, const unsigned* rp, const unsigned* ci,
		const double* va, const double* x, const double* b, int full) {
	double* r = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
	spmv(n, rp, ci, va, x, r, 1);
	for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
	double normb, nr;
	if (full && n > 1) {
		double sb = 0.0, sr = 0.0;
		for (int i = 0; i < n; ++i) { sb += b[i] * b[i]; sr += r[i] * r[i]; }
		normb = sqrt(sb);
		nr = sqrt(sr);
	} else {
		normb = rs_nrm2(n, b);
		nr = rs_nrm2(n, r);
	}
	free(r);
	if (normb == 0.0) normb = 1;
	return nr / normb;
}

#define VLOOP(n, th) \
	_Pragma("omp parallel for num_threads(th) if (th > 1) schedule(static)") \
	for (int i = 0; i < (n); ++i)

/* ----------------------------------------------------------- solvers --- */
static int find_diag(int n, const unsigned* rp, const unsigned* ci,
		const double* va, double* d, int inv) {
	/* DiaPre (preconditioner.hpp:182-229): inv 1 -> 1/diag, inv 2 -> diag;
	 * a zero or missing diagonal is a failure (the reference exits) */
	for (int i = 0; i < n; ++i) {
		d[i] = 0.0;
		for (unsigned k = rp[i]; k < rp[i + 1]; ++k) {
			if ((int)ci[k] == i) {
				if (va[k] == 0.0) return RS_EZERODIAG;
				d[i] = inv == 1 ? 1. / va[k] : va[k];
				break;
			}
		}
		if (d[i] == 0.0) return RS_EZERODIAG;
	}
	return 0;
}

static void hist_push(double* h, int cap, int* len, double v) {
	if (*len < cap && h) h[*len] = v;
	(*len)++;
}

/* solver_matrix.hpp:264-316 */
static int cg(int n, const unsigned* rp, const unsigned* ci, const double* va,
		const double* b, double* x, int* max_iter, double* tol, double* h,
		int cap, int* hl, int th) {
	double* r = malloc(sizeof(double) * n);
	double* p = malloc(sizeof(double) * n);
	double* q = malloc(sizeof(double) * n);
	double* t = malloc(sizeof(double) * n);
	double resid, alpha, beta, rho, rho_1 = 0.0;
	int ret = 1;
	double normb = par_nrm2(n, b, th);
	spmv(n, rp, ci, va, x, t, th);
	VLOOP(n, th) r[i] = b[i] - t[i];
	if (normb == 0.0) normb = 1;
	if ((resid = par_nrm2(n, r, th) / normb) <= *tol) {
		*tol = resid;
		*max_iter = 0;
		ret = 0;
		goto done;
	}
	for (int it = 1; it <= *max_iter; ++it) {
		rho = par_dot(n, r, r, th); /* z = r */
		if (it == 1) {
			VLOOP(n, th) p[i] = r[i];
		} else {
			beta = rho / rho_1;
			VLOOP(n, th) { double tt = beta * p[i]; p[i] = r[i] + tt; }
		}
		spmv(n, rp, ci, va, p, q, th);
		alpha = rho / par_dot(n, p, q, th);
		VLOOP(n, th) { double tt = alpha * p[i]; x[i] += tt; }
		VLOOP(n, th) { double tt = alpha * q[i]; r[i] -= tt; }
		resid = par_nrm2(n, r, th) / normb;
		hist_push(h, cap, hl, resid);
		if (resid <= *tol) {
			*tol = resid;
			*max_iter = it;
			ret = 0;
			goto done;
		}
		rho_1 = rho;
	}
	*tol = resid;
done:
	free(r); free(p); free(q); free(t);
	return ret;
}

/* solver_matrix.hpp:192-260 */
static int jacobi(int n, const unsigned* rp, const unsigned* ci,
		const double* va, const double* b, double* x, int* max_iter,
		double* tol, double* h, int cap, int* hl, int th) {
	unsigned nz = rp[n];
	double* T = malloc(sizeof(double) * (nz ? nz : 1));
	double* C = malloc(sizeof(double) * n);
	double* nx = malloc(sizeof(double) * n);
	double* r = malloc(sizeof(double) * n);
	double* t = malloc(sizeof(double) * n);
	double resid;
	int ret = 1;
	memcpy(T, va, sizeof(double) * nz);
	for (int i = 0; i < n; ++i) C[i] = 1.0 / SMALL;
	double normb = par_nrm2(n, b, th);
	spmv(n, rp, ci, va, x, t, th);
	VLOOP(n, th) r[i] = b[i] - t[i];
	if (normb == 0.0) normb = 1;
	if ((resid = par_nrm2(n, r, th) / normb) <= *tol) {
		*tol = resid;
		*max_iter = 0;
		ret = 0;
		goto done;
	}
	for (int i = 0; i < n; ++i) {
		double dv = 0.0;
		long flag = -1;
		for (unsigned k = rp[i]; k < rp[i + 1]; ++k) {
			if ((int)ci[k] == i) { flag = k; dv = T[k]; T[k] = 0; break; }
		}
		if (flag < 0 || dv == 0.0) { ret = RS_EZERODIAG; goto done; }
		for (unsigned k = rp[i]; k < rp[i + 1]; ++k) {
			if ((long)k == flag) C[i] = b[ci[k]] / dv;
			else T[k] = -T[k] / dv;
		}
	}
	for (int it = 1; it <= *max_iter; ++it) {
		spmv(n, rp, ci, T, x, t, th);
		VLOOP(n, th) nx[i] = t[i] + C[i];
		spmv(n, rp, ci, va, nx, t, th);
		VLOOP(n, th) r[i] = b[i] - t[i];
		resid = par_nrm2(n, r, th) / normb;
		hist_push(h, cap, hl, resid);
		if (resid <= *tol) {
			*tol = resid;
			*max_iter = it;
			ret = 0;
			goto done; /* x keeps the previous iterate, as in the reference */
		}
		memcpy(x, nx, sizeof(double) * n);
	}
	*tol = resid;
done:
	free(T); free(C); free(nx); free(r); free(t);
	return ret;
}

/* solver_matrix.hpp:599-672 (inv = 1, Dia_BiCGSTAB) and 674-745 (inv = 2,
 * BiCGSTAB). The two differ in the preconditioner and in whether the early
 * exit on |s| and the initial check append to the residual list. */
static int bicgstab(int inv, int n, const unsigned* rp, const unsigned* ci,
		const double* va, const double* b, double* x, int* max_iter,
		double* tol, double* h, int cap, int* hl, int th) {
	double* d = malloc(sizeof(double) * n);
	double* r = malloc(sizeof(double) * n);
	double* rt = malloc(sizeof(double) * n);
	double* p = malloc(sizeof(double) * n);
	double* ph = malloc(sizeof(double) * n);
	double* s = malloc(sizeof(double) * n);
	double* sh = malloc(sizeof(double) * n);
	double* t = malloc(sizeof(double) * n);
	double* v = malloc(sizeof(double) * n);
	double resid, rho_1, rho_2 = 0, alpha = 0, beta, omega = 0;
	int ret = find_diag(n, rp, ci, va, d, inv);
	if (ret) goto done;
	ret = 1;
	double normb = par_nrm2(n, b, th);
	spmv(n, rp, ci, va, x, t, th);
	VLOOP(n, th) r[i] = b[i] - t[i];
	memcpy(rt, r, sizeof(double) * n);
	if (normb == 0.0) normb = 1;
	if ((resid = par_nrm2(n, r, th) / normb) <= *tol) {
		*tol = resid;
		*max_iter = 0;
		if (inv == 1) hist_push(h, cap, hl, resid);
		ret = 0;
		goto done;
	}
	for (int it = 1; it <= *max_iter; ++it) {
		rho_1 = par_dot(n, rt, r, th);
		if (rho_1 == 0) {
			*tol = par_nrm2(n, r, th) / normb;
			ret = 2;
			goto done;
		}
		if (it == 1) {
			memcpy(p, r, sizeof(double) * n);
		} else {
			beta = (rho_1 / rho_2) * (alpha / omega);
			VLOOP(n, th) {
				double t1 = omega * v[i];
				double t2 = p[i] - t1;
				double t3 = beta * t2;
				p[i] = r[i] + t3;
			}
		}
		VLOOP(n, th) ph[i] = p[i] * d[i];
		spmv(n, rp, ci, va, ph, v, th);
		alpha = rho_1 / par_dot(n, rt, v, th);
		VLOOP(n, th) { double t1 = alpha * v[i]; s[i] = r[i] - t1; }
		if ((resid = par_nrm2(n, s, th) / normb) < *tol) {
			VLOOP(n, th) { double t1 = alpha * ph[i]; x[i] += t1; }
			*tol = resid;
			if (inv == 1) hist_push(h, cap, hl, resid);
			ret = 0; /* max_iter left unchanged, as in the reference */
			goto done;
		}
		VLOOP(n, th) sh[i] = s[i] * d[i];
		spmv(n, rp, ci, va, sh, t, th);
		omega = par_dot(n, t, s, th) / par_dot(n, t, t, th);
		VLOOP(n, th) {
			double t1 = alpha * ph[i];
			double t2 = omega * sh[i];
			double t3 = t1 + t2;
			x[i] += t3;
		}
		VLOOP(n, th) { double t1 = omega * t[i]; r[i] = s[i] - t1; }
		rho_2 = rho_1;
		resid = par_nrm2(n, r, th) / normb;
		hist_push(h, cap, hl, resid);
		if (resid < *tol) {
			*tol = resid;
			*max_iter = it;
			ret = 0;
			goto done;
		}
		if (omega == 0) {
			*tol = par_nrm2(n, r, th) / normb;
			ret = 3;
			goto done;
		}
	}
	*tol = resid;
done:
	free(d); free(r); free(rt); free(p); free(ph); free(s); free(sh);
	free(t); free(v);
	return ret;
}

/* ICPre (preconditioner.hpp:97-177): the upper triangle with the diagonal,
 * columns ascending per row, factored as ICFactor (:20-48) does */
typedef struct { unsigned* pntr; unsigned* indx; double* val; } IcF;

typedef struct { unsigned c; double v; } ColVal;
static int colval_cmp(const void* a, const void* b) {
	unsigned x = ((const ColVal*)a)->c, y = ((const ColVal*)b)->c;
	return x < y ? -1 : (x > y ? 1 : 0);
}

static int ic_build(int n, const unsigned* rp, const unsigned* ci, const double* va, IcF* f) {
	unsigned nz = 0;
	for (int k = 0; k < n; ++k)
		for (unsigned j = rp[k]; j < rp[k + 1]; ++j)
			if (ci[j] >= (unsigned)k) ++nz;
	f->pntr = malloc(sizeof(unsigned) * (n + 1));
	f->indx = malloc(sizeof(unsigned) * (nz + 1));   /* + a sentinel */
	f->val = malloc(sizeof(double) * (nz ? nz : 1));
	ColVal* tmp = malloc(sizeof(ColVal) * (n + 1));   /* a row has at most n entries */
	f->pntr[0] = 0;
	for (int k = 0; k < n; ++k) {
		unsigned m = 0, base = f->pntr[k];
		for (unsigned j = rp[k]; j < rp[k + 1]; ++j)
			if (ci[j] >= (unsigned)k) { tmp[m].c = ci[j]; tmp[m].v = va[j]; ++m; }
		qsort(tmp, m, sizeof(ColVal), colval_cmp);
		for (unsigned e = 0; e < m; ++e) { f->indx[base + e] = tmp[e].c; f->val[base + e] = tmp[e].v; }
		f->pntr[k + 1] = base + m;
		if (m == 0 || tmp[0].c != (unsigned)k) { free(tmp); return RS_EZERODIAG; }
	}
	free(tmp);
	f->indx[nz] = 0;
	unsigned* pntr = f->pntr;
	unsigned* indx = f->indx;
	double* val = f->val;
	for (int k = 0; k < n - 1; ++k) {
		unsigned d = pntr[k];
		double z = val[d] = sqrt(val[d]);
		for (unsigned i = d + 1; i < pntr[k + 1]; ++i) val[i] /= z;
		for (unsigned i = d + 1; i < pntr[k + 1]; ++i) {
			z = val[i];
			unsigned h = indx[i], g = i;
			for (unsigned j = pntr[h]; j < pntr[h + 1]; ++j)
				for (; g < pntr[k + 1] && indx[g + 1] <= indx[j]; ++g)
					if (indx[g] == indx[j]) val[j] -= z * val[g];
		}
	}
	val[pntr[n - 1]] = sqrt(val[pntr[n - 1]]);
	return 0;
}

/* ICPre::solve: forward column sweep, then backward sweep */
static void ic_solve(int n, const IcF* f, const double* x, double* y) {
	for (int i = 0; i < n; ++i) y[i] = x[i];
	for (int i = 0; i < n; ++i) {
		double z = y[i] / f->val[f->pntr[i]];
		y[i] = z;
		for (unsigned j = f->pntr[i] + 1; j < f->pntr[i + 1]; ++j) y[f->indx[j]] -= z * f->val[j];
	}
	for (int i = n - 1; i >= 0; --i) {
		double z = 0;
		for (unsigned j = f->pntr[i] + 1; j < f->pntr[i + 1]; ++j) z += y[f->indx[j]] * f->val[j];
		y[i] = (y[i] - z) / f->val[f->pntr[i]];
	}
}

/* solver_matrix.hpp:318-374 (cgs = 0) and 376-438 (cgs = 1) */
static int ic_krylov(int cgs, int n, const unsigned* rp, const unsigned* ci,
		const double* va, const double* b, double* x, int* max_iter, double* tol,
		double* h, int cap, int* hl) {
	IcF f;
	int rc = ic_build(n, rp, ci, va, &f);
	if (rc) { free(f.pntr); free(f.indx); free(f.val); return rc; }
	double* w[12];
	for (int k = 0; k < 12; ++k) w[k] = malloc(sizeof(double) * n);
	double *r = w[0], *rt = w[1], *p = w[2], *ph = w[3], *q = w[4], *qh = w[5],
		   *vh = w[6], *u = w[7], *uh = w[8], *z = w[9], *t = w[10], *s = w[11];
	double resid, alpha, beta, rho_1 = 0.0, rho_2 = 0.0;
	int ret = 1;
	double normb = rs_nrm2(n, b);
	spmv(n, rp, ci, va, x, t, 1);
	for (int i = 0; i < n; ++i) r[i] = b[i] - t[i];
	for (int i = 0; i < n; ++i) rt[i] = r[i];
	if (normb == 0.0) normb = 1;
	if ((resid = rs_nrm2(n, r) / normb) <= *tol) {
		*tol = resid;
		*max_iter = 0;
		ret = 0;
		goto done;
	}
	for (int it = 1; it <= *max_iter; ++it) {
		if (!cgs) {
			ic_solve(n, &f, r, z);
			double rho = rs_dot(n, r, z);
			if (it == 1) {
				for (int i = 0; i < n; ++i) p[i] = z[i];
			} else {
				beta = rho / rho_1;
				for (int i = 0; i < n; ++i) { double tt = beta * p[i]; p[i] = z[i] + tt; }
			}
			spmv(n, rp, ci, va, p, q, 1);
			alpha = rho / rs_dot(n, p, q);
			for (int i = 0; i < n; ++i) { double tt = alpha * p[i]; x[i] += tt; }
			for (int i = 0; i < n; ++i) { double tt = alpha * q[i]; r[i] -= tt; }
			resid = rs_nrm2(n, r) / normb;
			hist_push(h, cap, hl, resid);
			if (resid <= *tol) { *tol = resid; *max_iter = it; ret = 0; goto done; }
			rho_1 = rho;
			continue;
		}
		rho_1 = rs_dot(n, rt, r);
		if (rho_1 == 0) { *tol = rs_nrm2(n, r) / normb; ret = 2; goto done; }
		if (it == 1) {
			for (int i = 0; i < n; ++i) { u[i] = r[i]; p[i] = u[i]; }
		} else {
			beta = rho_1 / rho_2;
			for (int i = 0; i < n; ++i) { double tt = beta * q[i]; u[i] = r[i] + tt; }
			for (int i = 0; i < n; ++i) {
				double t1 = beta * p[i];
				double t2 = q[i] + t1;
				double t3 = beta * t2;
				p[i] = u[i] + t3;
			}
		}
		ic_solve(n, &f, p, ph);
		spmv(n, rp, ci, va, ph, vh, 1);
		alpha = rho_1 / rs_dot(n, rt, vh);
		for (int i = 0; i < n; ++i) { double tt = alpha * vh[i]; q[i] = u[i] - tt; }
		for (int i = 0; i < n; ++i) s[i] = u[i] + q[i];
		ic_solve(n, &f, s, uh);
		for (int i = 0; i < n; ++i) { double tt = alpha * uh[i]; x[i] += tt; }
		spmv(n, rp, ci, va, uh, qh, 1);
		for (int i = 0; i < n; ++i) { double tt = alpha * qh[i]; r[i] -= tt; }
		rho_2 = rho_1;
		resid = rs_nrm2(n, r) / normb;
		hist_push(h, cap, hl, resid);
		if (resid < *tol) { *tol = resid; *max_iter = it; ret = 0; goto done; }
	}
	*tol = resid;
done:
	for (int k = 0; k < 12; ++k) free(w[k]);
	free(f.pntr); free(f.indx); free(f.val);
	return ret;
}

int rs_krylov_csr(int kind, int n, const unsigned* rowptr, const unsigned* col,
		const double* val, const double* b, double* x, int* max_iter,
		double* tol, double* hist, int hist_cap, int* hist_len, int threads) {
	int hl = 0, ret;
	if (threads < 1) threads = 1;
	switch (kind) {
	case RS_CG:
		ret = cg(n, rowptr, col, val, b, x, max_iter, tol, hist, hist_cap,
				&hl, threads);
		break;
	case RS_JACOBI:
		ret = jacobi(n, rowptr, col, val, b, x, max_iter, tol, hist, hist_cap,
				&hl, threads);
		break;
	case RS_DIA_BICGSTAB:
		ret = bicgstab(1, n, rowptr, col, val, b, x, max_iter, tol, hist,
				hist_cap, &hl, threads);
		break;
	case RS_BICGSTAB:
		ret = bicgstab(2, n, rowptr, col, val, b, x, max_iter, tol, hist,
				hist_cap, &hl, threads);
		break;
	case RS_IC_CGS:
	case RS_IC_CG:
		ret = ic_krylov(kind == RS_IC_CGS, n, rowptr, col, val, b, x, max_iter, tol,
				hist, hist_cap, &hl);
		break;
	default:
		return -1;
	}
	if (hist_len) *hist_len = hl;
	return ret;
}

/* -------------------------------------------------------------- grid --- */
void rs_grid_uniform(int n, int gl, double lo, double hi, double* c,
		double* s) {
	/* s_grid.hpp:372-395 */
	int N = n + 2 * gl;
	double ds = (hi - lo) / n;
	double csum = 0.0, llg = 0.0;
	for (int i = 0; i < N; ++i) s[i] = ds;
	for (int i = 0; i < N; ++i) {
		c[i] = csum + 0.5 * s[i];
		csum += s[i];
	}
	for (int i = 0; i < gl; ++i) llg += s[i];
	double sh = lo - llg;
	for (int i = 0; i < N; ++i) c[i] += sh;
}

void rs_grid_sizes(int n, int gl, double lo, const double* cs, double* c,
		double* s) {
	/* s_grid.hpp:397-434: ghost cells take the size of the nearest normal
	 * cell; centres are running sums, shifted so the first normal cell
	 * starts at lo */
	int N = n + 2 * gl;
	double csum = 0.0, llg = 0.0;
	for (int i = 0; i < N; ++i) s[i] = i < gl ? cs[0] : (i - gl >= n ? cs[n - 1] : cs[i - gl]);
	for (int i = 0; i < N; ++i) {
		c[i] = csum + 0.5 * s[i];
		csum += s[i];
	}
	for (int i = 0; i < gl; ++i) llg += s[i];
	double sh = lo - llg;
	for (int i = 0; i < N; ++i) c[i] += sh;
}

/* field accessors: cell (i, j) of a (nx+2gl) x (ny+2gl) array, i, j in
 * normal-cell coordinates (ghosts negative / >= n) */
#define AT(f, i, j) (f)[(size_t)((i) + gl) * NJ + (size_t)((j) + gl)]
#define CX(i) cx[(i) + gl]
#define CY(j) cy[(j) + gl]
#define SX(i) sx[(i) + gl]
#define SY(j) sy[(j) + gl]

/* ---------------------------------------------------------- assembly --- */
typedef struct {
	int i, j;     /* term index */
	int e;        /* exponent: 0 constant, 1 unknown */
	double c;
} term;

/* Polynomial_ key order (polynomial.hpp:44-57 with Index_compare_,
 * s_define.hpp:227-241): two constants are the same key; otherwise by index
 * (x then y), then exponent. */
static int key_cmp(const term* a, int i, int j, int e) {
	if (a->e == 0 && e == 0) return 0;
	if (a->i != i) return a->i < i ? -1 : 1;
	if (a->j != j) return a->j < j ? -1 : 1;
	if (a->e != e) return a->e < e ? -1 : 1;
	return 0;
}
/* Polynomial_::insert (polynomial.hpp:199-219): add onto an existing key */
static void poly_insert(term* row, int* len, double c, int i, int j, int e) {
	int k = 0;
	for (; k < *len; ++k) {
		int r = key_cmp(&row[k], i, j, e);
		if (r == 0) { row[k].c = row[k].c + c; return; }
		if (r > 0) break;
	}
	memmove(&row[k + 1], &row[k], sizeof(term) * (*len - k));
	row[k].i = i; row[k].j = j; row[k].e = e; row[k].c = c;
	(*len)++;
}

/* the rows of StencilPoisson_ (helm 0) or StencilHelmholtz_ (helm 1,
 * s_poisson.hpp:185-260: centre coec + s_x s_y alpha, source s_x s_y f) */
static int assemble_rows(int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const rs_bc* bc,
		double beta, const double* src, double src_value, unsigned* rowptr,
		unsigned* col, double* val, double* b, const double* bfield, int helm,
		double alpha) {
	const int NJ = ny + 2 * gl;
	int nz = 0;
	rowptr[0] = 0;
	for (int j = 0; j < ny; ++j) {
		for (int i = 0; i < nx; ++i) {
			term row[16];
			int len = 0;
			/* StencilPoisson_::_coe_other (s_poisson.hpp:109-114):
			 * -betaf * a / d, with a the face area (s_y for x faces, s_x for
			 * y faces) and d the centre distance */
			double ax = SY(j) * 1.0, ay = 1.0 * SX(i);
			/* a beta field: _build_default_beta (s_poisson.hpp:144-164), the
			 * face value from the cell and its + neighbour, weighted by
			 * Grid_::df_ = |half size - centre| of the cell and of its
			 * neighbour on the face's side */
			double bxp = beta, bxm = beta, byp = beta, bym = beta;
			if (bfield) {
#define DFX(k) fabs(SX(k) * 0.5 - CX(k))
#define DFY(k) fabs(SY(k) * 0.5 - CY(k))
				double v = AT(bfield, i, j), vx = AT(bfield, i + 1, j), vy = AT(bfield, i, j + 1);
				bxp = (DFX(i) * v + DFX(i + 1) * vx) / (DFX(i) + DFX(i + 1));
				bxm = (DFX(i) * v + DFX(i - 1) * vx) / (DFX(i) + DFX(i - 1));
				byp = (DFY(j) * v + DFY(j + 1) * vy) / (DFY(j) + DFY(j + 1));
				bym = (DFY(j) * v + DFY(j - 1) * vy) / (DFY(j) + DFY(j - 1));
#undef DFX
#undef DFY
			}
			double cxp = (-bxp) * ax / fabs(CX(i) - CX(i + 1));
			double cxm = (-bxm) * ax / fabs(CX(i) - CX(i - 1));
			double cyp = (-byp) * ay / fabs(CY(j) - CY(j + 1));
			double cym = (-bym) * ay / fabs(CY(j) - CY(j - 1));
			/* coe_row (s_poisson.hpp:85-102) */
			poly_insert(row, &len, cxp, i + 1, j, 1);
			poly_insert(row, &len, cxm, i - 1, j, 1);
			poly_insert(row, &len, cyp, i, j + 1, 1);
			poly_insert(row, &len, cym, i, j - 1, 1);
			double coec = 0;
			coec += -cxm;
			coec += -cxp;
			coec += -cym;
			coec += -cyp;
			/* StencilHelmholtz_::coe_row inserts coec + v alpha, v = s_x s_y */
			double v = 1.0;
			v *= SX(i);
			v *= helm ? SY(j) : SX(i);
			if (helm) coec = coec + v * alpha;
			poly_insert(row, &len, coec, i, j, 1);
			/* src (s_poisson.hpp:75-83): s_(0)^DIM * source; Helmholtz:
			 * s_x s_y * source */
			double f = src ? AT(src, i, j) : src_value;
			poly_insert(row, &len, v * f, i, j, 0);
			/* GhostRegular_::substitute (s_ghost.hpp:334-357), in key order */
			for (int k = 0; k < len;) {
				term tk = row[k];
				int gx = tk.i < 0 || tk.i >= nx;
				int gy = tk.j < 0 || tk.j >= ny;
				if (tk.e == 1 && (gx || gy)) {
					memmove(&row[k], &row[k + 1], sizeof(term) * (len - k - 1));
					len--;
					if (tk.c != 0) {
						/* Ghost_::_substitute_ghost (s_ghost.hpp:140-179) */
						int seg, a, oi = tk.i, oj = tk.j, ori;
						if (gx) { a = 0; seg = tk.i < 0 ? 0 : 1; ori = tk.i < 0 ? 0 : 1; oi = tk.i < 0 ? 0 : nx - 1; }
						else { a = 1; seg = tk.j < 0 ? 2 : 3; ori = tk.j < 0 ? 0 : 1; oj = tk.j < 0 ? 0 : ny - 1; }
						double c0 = a == 0 ? CX(tk.i) : CY(tk.j);
						double c1 = a == 0 ? CX(oi) : CY(oj);
						double hs = (a == 0 ? SX(oi) : SY(oj)) * 0.5;
						double cf = ori == 1 ? c1 + hs : c1 - hs;
						double dl = fabs(c1 - c0);
						double d0 = fabs(cf - c0);
						double d1 = fabs(c1 - cf);
						double bv = bc->value[seg];
						if (bc->type[seg] == 1) {
							poly_insert(row, &len, -tk.c * d0 / d1, oi, oj, 1);
							poly_insert(row, &len, tk.c * dl * bv / d1, oi, oj, 0);
						} else {
							poly_insert(row, &len, tk.c, oi, oj, 1);
							poly_insert(row, &len, -bv * dl * tk.c, oi, oj, 0);
						}
					}
					/* the entry was erased; the next entry now sits at k,
					 * unless an insert landed before it (never: inserts hit
					 * the centre and constant, which sort after W and S) */
					k = 0;
					continue;
				}
				++k;
			}
			/* concise: trim_zero + merge_const (polynomial.hpp:288-330) */
			int fconst = 0;
			double bconst = 0.0;
			for (int k = 0; k < len; ++k) {
				if (row[k].c == 0) continue;
				if (row[k].e == 0) {
					fconst = 1;
					bconst = -row[k].c; /* s_solver.hpp:122 */
				} else {
					col[nz] = (unsigned)(row[k].i + row[k].j * nx);
					val[nz] = row[k].c;
					nz++;
				}
			}
			b[i + j * nx] = fconst ? bconst : 0.0;
			rowptr[i + j * nx + 1] = (unsigned)nz;
		}
	}
	return nz;
}

int rs_assemble_poisson(int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const rs_bc* bc,
		double beta, const double* src, double src_value, unsigned* rowptr,
		unsigned* col, double* val, double* b, const double* bfield) {
	return assemble_rows(nx, ny, gl, cx, sx, cy, sy, bc, beta, src, src_value,
			rowptr, col, val, b, bfield, 0, 0.0);
}

int rs_assemble_helmholtz(int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const rs_bc* bc,
		double alpha, double beta, const double* src, unsigned* rowptr,
		unsigned* col, double* val, double* b) {
	return assemble_rows(nx, ny, gl, cx, sx, cy, sy, bc, beta, src, 0.0,
			rowptr, col, val, b, NULL, 1, alpha);
}

/* ------------------------------------------------------------ ghosts --- */
void rs_apply_bc(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const rs_bc* bc, double* f) {
	rs_apply_bc_gv(nx, ny, gl, cx, sx, cy, sy, bc, NULL, f);
}

void rs_apply_bc_gv(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const rs_bc* bc, const double* gv,
		double* f) {
	/* Equation_::apply_bc (s_equation.hpp:340-378): every ghost cell in the
	 * IJK order of begin_IJK (x fastest), in place, so a corner reads the
	 * neighbouring ghost row as it stands when the corner is visited. gv
	 * (optional, a cell field) holds the boundary value of each ghost cell
	 * (BC::get_val at the ghost's face point) in place of bc->value. */
	const int NI = nx + 2 * gl, NJ = ny + 2 * gl;
	for (int J = 0; J < NJ; ++J) {
		for (int I = 0; I < NI; ++I) {
			int i = I - gl, j = J - gl;
			int gx = i < 0 || i >= nx, gy = j < 0 || j >= ny;
			if (!gx && !gy) continue;
			int seg, a, oi = i, oj = j, ori;
			if (gx) { a = 0; seg = i < 0 ? 0 : 1; ori = i < 0 ? 0 : 1; oi = i < 0 ? 0 : nx - 1; }
			else { a = 1; seg = j < 0 ? 2 : 3; ori = j < 0 ? 0 : 1; oj = j < 0 ? 0 : ny - 1; }
			double val = gv ? AT(gv, i, j) : bc->value[seg];
			double cg = a == 0 ? CX(i) : CY(j);
			double co = a == 0 ? CX(oi) : CY(oj);
			double dl = fabs(cg - co);
			if (bc->type[seg] == 1) {
				/* Interp_::Linear (arithmetic.hpp:427-430) through the face */
				double hs = (a == 0 ? SX(oi) : SY(oj)) * 0.5;
				double cf = ori == 1 ? co + hs : co - hs;
				double u = (cg - cf) / (co - cf);
				AT(f, i, j) = (val * (1.0 - u)) + (AT(f, oi, oj) * u);
			} else {
				double po = AT(f, oi, oj);
				AT(f, i, j) = po - val * dl;
			}
		}
	}
}

/* --------------------------------------------------------- operators --- */
void rs_grad(int nx, int ny, int gl, const double* cx, const double* cy,
		const double* phi, double* gx, double* gy) {
	/* Operation_::Grad (s_operation.hpp:46-72) into zeroed face fields */
	const int NJ = ny + 2 * gl;
	size_t N = (size_t)(nx + 2 * gl) * NJ;
	memset(gx, 0, sizeof(double) * N);
	memset(gy, 0, sizeof(double) * N);
	for (int j = 0; j < ny; ++j) {
		for (int i = 0; i < nx; ++i) {
			double vc = AT(phi, i, j);
			AT(gx, i, j) = (AT(phi, i + 1, j) - vc) / (CX(i + 1) - CX(i));
			if (i == 0) AT(gx, i - 1, j) = (AT(phi, i - 1, j) - vc) / (CX(i - 1) - CX(i));
			AT(gy, i, j) = (AT(phi, i, j + 1) - vc) / (CY(j + 1) - CY(j));
			if (j == 0) AT(gy, i, j - 1) = (AT(phi, i, j - 1) - vc) / (CY(j - 1) - CY(j));
		}
	}
}

void rs_div(int nx, int ny, int gl, const double* sx, const double* sy,
		const double* fx, const double* fy, double* div) {
	/* Operation_::Div(VecF) (s_operation.hpp:100-120) into a zeroed field */
	const int NJ = ny + 2 * gl;
	memset(div, 0, sizeof(double) * (size_t)(nx + 2 * gl) * NJ);
	for (int j = 0; j < ny; ++j) {
		for (int i = 0; i < nx; ++i) {
			double d = 0;
			d += (AT(fx, i, j) - AT(fx, i - 1, j)) / SX(i);
			d += (AT(fy, i, j) - AT(fy, i, j - 1)) / SY(j);
			AT(div, i, j) = d;
		}
	}
}

void rs_f2c(int nx, int ny, int gl, const double* fx, const double* fy,
		double* cxo, double* cyo) {
	/* Operation_::InterpolateF2C (s_operation.hpp:141-164) into zeroed fields */
	const int NJ = ny + 2 * gl;
	size_t N = (size_t)(nx + 2 * gl) * NJ;
	memset(cxo, 0, sizeof(double) * N);
	memset(cyo, 0, sizeof(double) * N);
	for (int j = 0; j < ny; ++j) {
		for (int i = 0; i < nx; ++i) {
			AT(cxo, i, j) = (AT(fx, i, j) + AT(fx, i - 1, j)) * 0.5;
			AT(cyo, i, j) = (AT(fy, i, j) + AT(fy, i, j - 1)) * 0.5;
		}
	}
}

void rs_c2f(int nx, int ny, int gl, const double* sx, const double* sy,
		const double* u, const double* v, double* fx, double* fy) {
	/* Operation_::InterpolateC2F(VecC, VecF) (s_operation.hpp:166-187):
	 * writes the normal faces and the low wall face, leaves the rest */
	const int NJ = ny + 2 * gl;
	for (int j = 0; j < ny; ++j) {
		for (int i = 0; i < nx; ++i) {
			double vc = AT(u, i, j);
			double hs = SX(i) * 0.5, hsp = SX(i + 1) * 0.5;
			AT(fx, i, j) = (AT(u, i + 1, j) * hs + vc * hsp) / (hs + hsp);
			if (i == 0) {
				double hsm = SX(i - 1) * 0.5;
				AT(fx, i - 1, j) = (AT(u, i - 1, j) * hs + vc * hsm) / (hs + hsm);
			}
			vc = AT(v, i, j);
			hs = SY(j) * 0.5;
			hsp = SY(j + 1) * 0.5;
			AT(fy, i, j) = (AT(v, i, j + 1) * hs + vc * hsp) / (hs + hsp);
			if (j == 0) {
				double hsm = SY(j - 1) * 0.5;
				AT(fy, i, j - 1) = (AT(v, i, j - 1) * hs + vc * hsm) / (hs + hsm);
			}
		}
	}
}

/* NablaMuNabla(Vt mu, ...) (s_operation.hpp:664-688) at one cell */
static double nmn(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, double mu, const double* f, int i,
		int j) {
	const int NJ = ny + 2 * gl;
	double t0, t1;
	{
		double dm = mu * (AT(f, i, j) - AT(f, i - 1, j)) / (CX(i) - CX(i - 1));
		double dp = mu * (AT(f, i + 1, j) - AT(f, i, j)) / (CX(i + 1) - CX(i));
		t0 = (dp - dm) / SX(i);
	}
	{
		double dm = mu * (AT(f, i, j) - AT(f, i, j - 1)) / (CY(j) - CY(j - 1));
		double dp = mu * (AT(f, i, j + 1) - AT(f, i, j)) / (CY(j + 1) - CY(j));
		t1 = (dp - dm) / SY(j);
	}
	double res = 0.0;
	res += t0;
	res += t1;
	return res;
}

void rs_diffusion(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, double mu, const double* f,
		double* out) {
	const int NJ = ny + 2 * gl;
	memset(out, 0, sizeof(double) * (size_t)(nx + 2 * gl) * NJ);
	for (int j = 0; j < ny; ++j)
		for (int i = 0; i < nx; ++i)
			AT(out, i, j) = nmn(nx, ny, gl, cx, sx, cy, sy, mu, f, i, j);
}

/* NablaMuNabla(const Scalar& mu, ...) (s_operation.hpp:630-662) at one
 * cell: face mu from the cell and its neighbour weighted by the half sizes */
static double nmn_var(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const double* mu, const double* f,
		int i, int j) {
	const int NJ = ny + 2 * gl;
	double t[2];
	for (int d = 0; d < 2; ++d) {
		int ip = d == 0 ? i + 1 : i, jp = d == 0 ? j : j + 1;
		int im = d == 0 ? i - 1 : i, jm = d == 0 ? j : j - 1;
		double hs = (d == 0 ? SX(i) : SY(j)) * 0.5;
		double hsp = (d == 0 ? SX(ip) : SY(jp)) * 0.5;
		double hsm = (d == 0 ? SX(im) : SY(jm)) * 0.5;
		double c = d == 0 ? CX(i) : CY(j);
		double cp = d == 0 ? CX(ip) : CY(jp);
		double cm = d == 0 ? CX(im) : CY(jm);
		double mufp = (hs * AT(mu, ip, jp) + hsp * AT(mu, i, j)) / (hsp + hs);
		double mufm = (hs * AT(mu, im, jm) + hsm * AT(mu, i, j)) / (hsm + hs);
		double dp = mufp * (AT(f, ip, jp) - AT(f, i, j)) / (cp - c);
		double dm = mufm * (AT(f, i, j) - AT(f, im, jm)) / (c - cm);
		t[d] = (dp - dm) / (d == 0 ? SX(i) : SY(j));
	}
	double res = 0.0;
	res += t[0];
	res += t[1];
	return res;
}

void rs_diffusion_var(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const double* mu, const double* f,
		double* out) {
	const int NJ = ny + 2 * gl;
	memset(out, 0, sizeof(double) * (size_t)(nx + 2 * gl) * NJ);
	for (int j = 0; j < ny; ++j)
		for (int i = 0; i < nx; ++i)
			AT(out, i, j) = nmn_var(nx, ny, gl, cx, sx, cy, sy, mu, f, i, j);
}

/* std::min / std::max semantics ((b < a) ? b : a, (a < b) ? b : a) */
static double smin(double a, double b) { return (b < a) ? b : a; }
static double smax(double a, double b) { return (a < b) ? b : a; }

/* limiters (s_operation.hpp:501-541, 598-600; minmod from
 * src/calculation/advection.hpp:1079-1081) */
static double limiter(int sch, double r, double R) {
	switch (sch) {
	case RS_VANLEER: return 0.5 * R * (r + fabs(r)) / (R - 1 + r);
	case RS_SUPERBEE: return smax(smax(0.0, smin(R * r, 1.0)), smin(r, R));
	case RS_WAHYD:
		if (r <= 1.0) return 0.5 * R * (r + fabs(r)) / (R - 1 + r);
		return smin((r + R * r * fabs(r)) / (R + r * r), R);
	case RS_QUICK: return 0.75 * r + 0.25;
	case RS_CUI: return 2.0 / 3.0 * r + 1.0 / 3.0;
	case RS_UPWIND2: return r;
	case RS_MINMOD: return smax(0.0, smin(1.0, r));
	}
	return 0.0;
}

/* one axis of the advection operators at cell (i, j); d = 0 x, 1 y.
 * Cells along the axis are addressed with k relative offsets. */
static double adv_axis(int sch, int d, int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const double* uf,
		const double* vf, const double* f, int i, int j) {
	const int NJ = ny + 2 * gl;
	const double* face = d == 0 ? uf : vf;
#define F(k) (d == 0 ? AT(f, i + (k), j) : AT(f, i, j + (k)))
#define C(k) (d == 0 ? CX(i + (k)) : CY(j + (k)))
#define S(k) (d == 0 ? SX(i + (k)) : SY(j + (k)))
#define FACE(k) (d == 0 ? AT(face, i + (k), j) : AT(face, i, j + (k)))
	double veo = (FACE(0) + FACE(-1)) * 0.5;
	switch (sch) {
	case RS_UPWIND1: /* s_operation.hpp:400-422 */
		if (veo > 0.0) return veo * (F(0) - F(-1)) / (C(0) - C(-1));
		if (veo < 0.0) return veo * (F(1) - F(0)) / (C(1) - C(0));
		return 0.0;
	case RS_CENTER: /* :442-459 */
		return veo * (F(1) - F(-1)) / (C(1) - C(-1));
	case RS_CENTER4: { /* :461-482 (no velocity factor, as in the reference) */
		double din = (F(1) - F(-1)) / (C(1) - C(-1));
		double dout = (F(2) - F(-2)) / (C(2) - C(-2));
		return (4.0 * din - dout) / 3.0;
	}
	default: { /* VdotNabla_TVD :549-596 */
		int Cm, Um, Dm, Cp, Up, Dp;
		if (veo >= 0.0) {
			Dm = 0; Cm = -1; Um = -2;
			Dp = 1; Cp = 0; Up = -1;
		} else {
			Dm = -1; Cm = 0; Um = 1;
			Dp = 0; Cp = 1; Up = 2;
		}
		/* NaN veo takes neither branch in the reference and leaves the
		 * indices as constructed (all zero) */
		if (!(veo >= 0.0) && !(veo < 0.0)) { Dm = Cm = Um = Dp = Cp = Up = 0; }
		double R, r, fp, fm;
		R = (S(Dp) + S(Cp)) / S(Cp);
		r = (F(Cp) - F(Up)) * (S(Dp) + S(Cp)) / (F(Dp) - F(Cp) + SMALL)
				/ (S(Cp) + S(Up));
		fp = F(Cp) + limiter(sch, r, R) / R * (F(Dp) - F(Cp));
		R = (S(Dm) + S(Cm)) / S(Cm);
		r = (F(Cm) - F(Um)) * (S(Dm) + S(Cm)) / (F(Dm) - F(Cm) + SMALL)
				/ (S(Cm) + S(Um));
		fm = F(Cm) + limiter(sch, r, R) / R * (F(Dm) - F(Cm));
		return (FACE(0) * fp - FACE(-1) * fm) / S(0);
	}
	}
#undef F
#undef C
#undef S
#undef FACE
}

static double adv_cell(int sch, int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const double* uf,
		const double* vf, const double* f, int i, int j) {
	double a0 = adv_axis(sch, 0, nx, ny, gl, cx, sx, cy, sy, uf, vf, f, i, j);
	double a1 = adv_axis(sch, 1, nx, ny, gl, cx, sx, cy, sy, uf, vf, f, i, j);
	double s = 0.0;
	s += a0;
	s += a1;
	return s;
}

void rs_advection(int scheme, int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const double* uf,
		const double* vf, const double* f, double* out) {
	const int NJ = ny + 2 * gl;
	memset(out, 0, sizeof(double) * (size_t)(nx + 2 * gl) * NJ);
	for (int j = 0; j < ny; ++j)
		for (int i = 0; i < nx; ++i)
			AT(out, i, j) = adv_cell(scheme, nx, ny, gl, cx, sx, cy, sy, uf, vf,
					f, i, j);
}

void rs_advect_run(int scheme, int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const rs_bc* bc,
		const double* gv, const double* uf, const double* vf, double dt,
		int steps, double* phi) {
	/* Advection_::run_one_step (s_advection.hpp:185-212), `steps` times: the
	 * ghosts of phi refilled, then every normal cell in Ijk order (x
	 * fastest) updated in place, phi - dt * VdotNabla, so a cell reads the
	 * new values of the cells visited before it. (The step also refills the
	 * ghosts of the cell velocities, which no later computation reads.) */
	const int NJ = ny + 2 * gl;
	for (int st = 0; st < steps; ++st) {
		rs_apply_bc_gv(nx, ny, gl, cx, sx, cy, sy, bc, gv, phi);
		for (int j = 0; j < ny; ++j)
			for (int i = 0; i < nx; ++i) {
				double adv = adv_cell(scheme, nx, ny, gl, cx, sx, cy, sy, uf, vf,
						phi, i, j);
				double phin = AT(phi, i, j);
				AT(phi, i, j) = phin - dt * adv;
			}
	}
}

double rs_max_magnitude(int nx, int ny, int gl, const double* u,
		const double* v) {
	/* VectorCenter_::max_magnitude (s_vector.hpp:89-103) */
	const int NJ = ny + 2 * gl;
	double mx = 0;
	for (int j = 0; j < ny; ++j) {
		for (int i = 0; i < nx; ++i) {
			double s = 0;
			s += AT(u, i, j) * AT(u, i, j);
			s += AT(v, i, j) * AT(v, i, j);
			mx = smax(mx, sqrt(s));
		}
	}
	return mx;
}

/* ------------------------------------------------------------ NS run --- */
int rs_ns_run(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const rs_bc* bc_u,
		const rs_bc* bc_v, const rs_ns_cfg* cfg, int steps, double* dt,
		double* u, double* v, double* uf, double* vf, double* phi, double* p,
		double* step_dt, int* step_iters, double* step_resid) {
	const int NI = nx + 2 * gl, NJ = ny + 2 * gl;
	const size_t N = (size_t)NI * NJ;
	const int n = nx * ny;
	double* us = calloc(N, sizeof(double));
	double* vs = calloc(N, sizeof(double));
	double* usf = calloc(N, sizeof(double));
	double* vsf = calloc(N, sizeof(double));
	double* div = calloc(N, sizeof(double));
	double* gx = calloc(N, sizeof(double));
	double* gy = calloc(N, sizeof(double));
	double* gcx = calloc(N, sizeof(double));
	double* gcy = calloc(N, sizeof(double));
	unsigned* rp = malloc(sizeof(unsigned) * (n + 1));
	unsigned* ci = malloc(sizeof(unsigned) * 5 * n);
	double* va = malloc(sizeof(double) * 5 * n);
	double* b = malloc(sizeof(double) * n);
	double* x = malloc(sizeof(double) * n);
	rs_bc bc_phi;
	for (int s = 0; s < 4; ++s) { bc_phi.type[s] = 2; bc_phi.value[s] = 0.0; }
	int ret = 0;
	double mins = 1.79769313486231570815e308;
	for (int I = 0; I < NI; ++I) mins = smin(mins, sx[I]);
	for (int J = 0; J < NJ; ++J) mins = smin(mins, sy[J]);
	double minx = 1.79769313486231570815e308, miny = minx;
	for (int I = 0; I < NI; ++I) minx = smin(minx, sx[I]);
	for (int J = 0; J < NJ; ++J) miny = smin(miny, sy[J]);
	for (int st = 0; st < steps; ++st) {
		/* NS_::restrict_time (s_ns.hpp:146-169) */
		double maxmag = rs_max_magnitude(nx, ny, gl, u, v);
		double rdt = cfg->cfl * mins / maxmag;
		double rdt2 = *dt;
		if (cfg->diff_number < 100) {
			double den = 0.0;
			den += 1.0 / (minx * minx);
			den += 1.0 / (miny * miny);
			rdt2 = cfg->diff_number / cfg->diff_coef / den;
		}
		if (*dt > smin(rdt, rdt2)) *dt = smin(rdt, rdt2);
		const double DT = *dt;
		/* _veo_star_center (s_ns_explicit.hpp:173-229) */
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, bc_u, u);
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, bc_v, v);
		for (int c = 0; c < 2; ++c) {
			const double* s = c == 0 ? u : v;
			double* ss = c == 0 ? us : vs;
			for (int j = 0; j < ny; ++j) {
				for (int i = 0; i < nx; ++i) {
					double adv = adv_cell(cfg->scheme, nx, ny, gl, cx, sx, cy,
							sy, uf, vf, s, i, j);
					/* __diffusion_term (s_ns_explicit.hpp:235-241): the mu
					 * field when set_mu replaced the uniform mu */
					double dif = cfg->mu_field
							? nmn_var(nx, ny, gl, cx, sx, cy, sy, cfg->mu_field, s, i, j)
							: nmn(nx, ny, gl, cx, sx, cy, sy, cfg->mu, s, i, j);
					double src = 0;
					AT(ss, i, j) = (-adv + (dif + src) / cfg->rho) * DT + AT(s, i, j);
				}
			}
		}
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, bc_u, us);
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, bc_v, vs);
		/* run_one_step (s_ns_explicit.hpp:118-155) */
		rs_c2f(nx, ny, gl, sx, sy, us, vs, usf, vsf);
		rs_div(nx, ny, gl, sx, sy, usf, vsf, div);
		/* projection: Poisson_::run with set_depend(phi, -, div), the
		 * CG + mean-removal drop-in solver (proj_kind / proj_nomean: another
		 * carpio:: solver, and the shipped solvers' no removal) */
		rs_assemble_poisson(nx, ny, gl, cx, sx, cy, sy, &bc_phi, 1.0, div, 0.0,
				rp, ci, va, b, NULL);
		for (int j = 0; j < ny; ++j)
			for (int i = 0; i < nx; ++i) x[i + j * nx] = AT(phi, i, j);
		double m = 0;
		if (!cfg->proj_nomean) {
			for (int k = 0; k < n; ++k) m += b[k];
			m = m / (double)n;
			for (int k = 0; k < n; ++k) b[k] = b[k] - m;
		}
		int mi = cfg->cg_max_iter;
		double tol = cfg->cg_tol;
		int r = rs_krylov_csr(cfg->proj_kind, n, rp, ci, va, b, x, &mi, &tol, NULL, 0,
				NULL, cfg->threads);
		if (r && !ret) ret = r;
		if (!cfg->proj_nomean) {
			m = 0;
			for (int k = 0; k < n; ++k) m += x[k];
			m = m / (double)n;
			for (int k = 0; k < n; ++k) x[k] = x[k] - m;
		}
		for (int j = 0; j < ny; ++j)
			for (int i = 0; i < nx; ++i) AT(phi, i, j) = x[i + j * nx];
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, &bc_phi, phi);
		rs_grad(nx, ny, gl, cx, cy, phi, gx, gy);
		/* p = phi (all cells), then p *= 1/dt on normal cells */
		memcpy(p, phi, sizeof(double) * N);
		{
			double inv = 1.0 / DT;
			for (int j = 0; j < ny; ++j)
				for (int i = 0; i < nx; ++i) AT(p, i, j) = AT(p, i, j) * inv;
		}
		for (size_t k = 0; k < N; ++k) usf[k] = usf[k] - gx[k];
		for (size_t k = 0; k < N; ++k) vsf[k] = vsf[k] - gy[k];
		rs_f2c(nx, ny, gl, gx, gy, gcx, gcy);
		for (size_t k = 0; k < N; ++k) us[k] = us[k] - gcx[k];
		for (size_t k = 0; k < N; ++k) vs[k] = vs[k] - gcy[k];
		memcpy(u, us, sizeof(double) * N);
		memcpy(v, vs, sizeof(double) * N);
		memcpy(uf, usf, sizeof(double) * N);
		memcpy(vf, vsf, sizeof(double) * N);
		if (step_dt) step_dt[st] = DT;
		if (step_iters) step_iters[st] = mi;
		if (step_resid) step_resid[st] = tol;
	}
	free(us); free(vs); free(usf); free(vsf); free(div); free(gx); free(gy);
	free(gcx); free(gcy); free(rp); free(ci); free(va); free(b); free(x);
	return ret;
}

/* ------------------------------------------------------------ NS_kim_ --- */
/* Jacobi on an assembled system from x0 (the reference's Solver_Jacobi_
 * gives the same iterate as carpio::Jacobi) */
static int solve_rows(int kind, int nx, int ny, int gl, const unsigned* rp,
		const unsigned* ci, const double* va, const double* b, double* x,
		double* f, int mi, double tol, int nomean, int threads, int* its,
		double* res) {
	const int NJ = ny + 2 * gl;
	const int n = nx * ny;
	double* bb = malloc(sizeof(double) * n);
	memcpy(bb, b, sizeof(double) * n);
	for (int j = 0; j < ny; ++j)
		for (int i = 0; i < nx; ++i) x[i + j * nx] = AT(f, i, j);
	double m = 0;
	if (!nomean) {
		for (int k = 0; k < n; ++k) m += bb[k];
		m = m / (double)n;
		for (int k = 0; k < n; ++k) bb[k] = bb[k] - m;
	}
	int r = rs_krylov_csr(kind, n, rp, ci, va, bb, x, &mi, &tol, NULL, 0, NULL, threads);
	if (!nomean) {
		m = 0;
		for (int k = 0; k < n; ++k) m += x[k];
		m = m / (double)n;
		for (int k = 0; k < n; ++k) x[k] = x[k] - m;
	}
	for (int j = 0; j < ny; ++j)
		for (int i = 0; i < nx; ++i) AT(f, i, j) = x[i + j * nx];
	if (its) *its = mi;
	if (res) *res = tol;
	free(bb);
	return r;
}

int rs_kim_run(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const rs_bc* bc_u,
		const rs_bc* bc_v, const rs_ns_cfg* cfg, int steps, int first, double dt,
		double* u, double* v, double* uf, double* vf, double* phi, double* p,
		double* us, double* vs, double* usf, double* vsf, int* step_iters,
		double* step_resid) {
	/* NS_kim_::run_one_step (s_ns_kim.hpp:130-187, predictor :228-280): no
	 * restrict_time; um/umf copied from u/uf before the ghosts are refilled;
	 * per component the AB2 source and a Helmholtz predictor (alpha 1, beta
	 * dt 0.5 / rho, Neumann 0, default Jacobi 1000 / 1e-4, x0 = the star
	 * field); projection as NS_explicit_; p = phi / dt - NablaMuNabla(mu,
	 * phi) 0.5 / rho. */
	const int NJ = ny + 2 * gl;
	const size_t N = (size_t)(nx + 2 * gl) * NJ;
	const int n = nx * ny;
	double* um = malloc(sizeof(double) * N);
	double* vm = malloc(sizeof(double) * N);
	double* umf = malloc(sizeof(double) * N);
	double* vmf = malloc(sizeof(double) * N);
	double* scr = calloc(N, sizeof(double));
	double* div = calloc(N, sizeof(double));
	double* gx = calloc(N, sizeof(double));
	double* gy = calloc(N, sizeof(double));
	double* gcx = calloc(N, sizeof(double));
	double* gcy = calloc(N, sizeof(double));
	unsigned* rp = malloc(sizeof(unsigned) * (n + 1));
	unsigned* ci = malloc(sizeof(unsigned) * 5 * (size_t)n);
	double* va = malloc(sizeof(double) * 5 * (size_t)n);
	double* b = malloc(sizeof(double) * n);
	double* x = malloc(sizeof(double) * n);
	rs_bc bc_n;
	for (int k = 0; k < 4; ++k) { bc_n.type[k] = 2; bc_n.value[k] = 0.0; }
	const double rho = cfg->rho, mu = cfg->mu;
	int ret = 0;
	for (int st = 0; st < steps; ++st) {
		const int step0 = first && st == 0;
		memcpy(um, u, sizeof(double) * N);
		memcpy(vm, v, sizeof(double) * N);
		memcpy(umf, uf, sizeof(double) * N);
		memcpy(vmf, vf, sizeof(double) * N);
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, bc_u, u);
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, bc_v, v);
		for (int d = 0; d < 2; ++d) {
			double* f = d == 0 ? u : v;
			double* fm = d == 0 ? um : vm;
			double* fs = d == 0 ? us : vs;
			for (int j = 0; j < ny; ++j)
				for (int i = 0; i < nx; ++i) {
					double advn = adv_cell(cfg->scheme, nx, ny, gl, cx, sx, cy, sy,
							uf, vf, f, i, j);
					double advnm1 = adv_cell(cfg->scheme, nx, ny, gl, cx, sx, cy, sy,
							umf, vmf, fm, i, j);
					double adv = 1.5 * advn - 0.5 * advnm1;
					double dif = nmn(nx, ny, gl, cx, sx, cy, sy, mu, f, i, j);
					double src = 0.0;
					double veos;
					if (step0) veos = (advn - (0.5 * dif + src) / rho) * dt - AT(f, i, j);
					else veos = (adv - (0.5 * dif + src) / rho) * dt - AT(f, i, j);
					AT(scr, i, j) = veos;
				}
			const double smu = dt * 0.5 / rho;
			assemble_rows(nx, ny, gl, cx, sx, cy, sy, &bc_n, smu, scr, 0.0, rp, ci,
					va, b, NULL, 1, 1.0);
			solve_rows(RS_JACOBI, nx, ny, gl, rp, ci, va, b, x, fs, 1000, 1e-4, 1,
					1, NULL, NULL);
		}
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, bc_u, us);
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, bc_v, vs);
		rs_c2f(nx, ny, gl, sx, sy, us, vs, usf, vsf);
		rs_div(nx, ny, gl, sx, sy, usf, vsf, div);
		assemble_rows(nx, ny, gl, cx, sx, cy, sy, &bc_n, 1.0, div, 0.0, rp, ci, va,
				b, NULL, 0, 0.0);
		int its = 0;
		double res = 0;
		int r = solve_rows(cfg->proj_kind, nx, ny, gl, rp, ci, va, b, x, phi,
				cfg->cg_max_iter, cfg->cg_tol, cfg->proj_nomean, cfg->threads, &its, &res);
		if (r && !ret) ret = r;
		rs_apply_bc(nx, ny, gl, cx, sx, cy, sy, &bc_n, phi);
		rs_grad(nx, ny, gl, cx, cy, phi, gx, gy);
		memcpy(p, phi, sizeof(double) * N);
		{
			double inv = 1.0 / dt;
			for (int j = 0; j < ny; ++j)
				for (int i = 0; i < nx; ++i) AT(p, i, j) = AT(p, i, j) * inv;
			for (int j = 0; j < ny; ++j)
				for (int i = 0; i < nx; ++i) {
					double lap = nmn(nx, ny, gl, cx, sx, cy, sy, mu, phi, i, j);
					lap = lap * (0.5 / rho);
					AT(p, i, j) = AT(p, i, j) - lap;
				}
		}
		for (size_t k = 0; k < N; ++k) usf[k] = usf[k] - gx[k];
		for (size_t k = 0; k < N; ++k) vsf[k] = vsf[k] - gy[k];
		rs_f2c(nx, ny, gl, gx, gy, gcx, gcy);
		for (size_t k = 0; k < N; ++k) us[k] = us[k] - gcx[k];
		for (size_t k = 0; k < N; ++k) vs[k] = vs[k] - gcy[k];
		memcpy(u, us, sizeof(double) * N);
		memcpy(v, vs, sizeof(double) * N);
		memcpy(uf, usf, sizeof(double) * N);
		memcpy(vf, vsf, sizeof(double) * N);
		if (step_iters) step_iters[st] = its;
		if (step_resid) step_resid[st] = res;
	}
	free(um); free(vm); free(umf); free(vmf); free(scr); free(div); free(gx);
	free(gy); free(gcx); free(gcy); free(rp); free(ci); free(va); free(b); free(x);
	return ret;
}
