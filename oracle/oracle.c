/*
 * oracle.c -- CPU oracle (FP64) for the shape_atrophy forward model.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, never part of
 * the product.  Build: oracle/build_oracle.py (gcc -O2 -fopenmp
 * -ffp-contract=off -DDIM=2|3).  -ffp-contract=off keeps x86 and Arm
 * results identical (no implicit FMA contraction).
 *
 * Citations are reference file:line, relative to the reference's CUDA/
 * folder ("2D/" = 2D_frame/, "3D/" = 3D_frame/, "inc/" = include/).
 * Expressions keep the reference's operand order so that FP64 results
 * match the reference's own code run on the CPU bit for bit.
 */
#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <omp.h>
#include "oracle.h"

#ifndef DIM
#error "compile with -DDIM=2 or -DDIM=3"
#endif

#if DIM == 2
#define VTX 3
#define NPAIR 6
#else
#define VTX 4
#define NPAIR 10
#endif

#define SUMBLK 512   /* inc/constants.h:22 SUMBLKDIM */

/* ------------------------------------------------------------------ */
/* small vector helpers (inc/matvec.h)                                 */
/* ------------------------------------------------------------------ */
typedef struct { double c[DIM]; } vec;
typedef struct { double m[DIM][DIM]; } mat;   /* m[row][col] = matrix.row.col */

static inline vec getv(const double *a, int idx, int num)
{ /* inc/matvec.h:18-24 (2D), 291-298 (3D): SoA column-major */
	vec v; for (int d = 0; d < DIM; ++d) v.c[d] = a[d * num + idx]; return v;
}
static inline void setv(double *a, vec v, int idx, int num)
{ for (int d = 0; d < DIM; ++d) a[d * num + idx] = v.c[d]; }
static inline vec vsub(vec a, vec b) { vec r; for (int d = 0; d < DIM; ++d) r.c[d] = a.c[d] - b.c[d]; return r; }
static inline double vdot(vec a, vec b)
{ /* inc/matvec.h:154-157, 498-501: left-to-right sum */
	double s = a.c[0] * b.c[0];
	for (int d = 1; d < DIM; ++d) s = s + a.c[d] * b.c[d];
	return s;
}
static inline double vnorm(vec a) { return sqrt(vdot(a, a)); }   /* eucnorm */
static inline double vdist2(vec a, vec b)
{ /* eucdistSqu: inc/matvec.h:176-180, 521-526 */
	double s = (a.c[0] - b.c[0]) * (a.c[0] - b.c[0]);
	for (int d = 1; d < DIM; ++d) s = s + (a.c[d] - b.c[d]) * (a.c[d] - b.c[d]);
	return s;
}
#if DIM == 3
static inline vec vcross(vec x, vec y)
{ /* inc/matvec.h:503-510 */
	vec r;
	r.c[0] =  x.c[1] * y.c[2] - x.c[2] * y.c[1];
	r.c[1] = -x.c[0] * y.c[2] + x.c[2] * y.c[0];
	r.c[2] =  x.c[0] * y.c[1] - x.c[1] * y.c[0];
	return r;
}
#endif

static inline double detQ(const vec *q)
{
#if DIM == 2
	/* det(xVec, yVec): inc/matvec.h:250-253 */
	return q[0].c[0] * q[1].c[1] - q[0].c[1] * q[1].c[0];
#else
	/* det(x, y, z): inc/matvec.h:592-600 */
	vec x = q[0], y = q[1], z = q[2];
	return  x.c[0] * y.c[1] * z.c[2]
	      + x.c[1] * y.c[2] * z.c[0]
	      + x.c[2] * y.c[0] * z.c[1]
	      - x.c[0] * y.c[2] * z.c[1]
	      - x.c[1] * y.c[0] * z.c[2]
	      - x.c[2] * y.c[1] * z.c[0];
#endif
}

static inline mat invQ(const vec *q)
{
	mat r;
#if DIM == 2
	/* matInv(inv, xVec, yVec): inc/matvec.h:267-277 */
	vec x = q[0], y = q[1];
	double detVal = x.c[0] * y.c[1] - x.c[1] * y.c[0];
	r.m[0][0] =  y.c[1] / detVal;
	r.m[0][1] = -y.c[0] / detVal;
	r.m[1][0] = -x.c[1] / detVal;
	r.m[1][1] =  x.c[0] / detVal;
#else
	/* matInv(inv, xVec, yVec, zVec): inc/matvec.h:627-649 */
	vec x = q[0], y = q[1], z = q[2];
	double detVal =   x.c[0] * y.c[1] * z.c[2]
	                + x.c[1] * y.c[2] * z.c[0]
	                + x.c[2] * y.c[0] * z.c[1]
	                - x.c[0] * y.c[2] * z.c[1]
	                - x.c[1] * y.c[0] * z.c[2]
	                - x.c[2] * y.c[1] * z.c[0];
	r.m[0][0] =  (y.c[1] * z.c[2] - y.c[2] * z.c[1]) / detVal;
	r.m[0][1] = -(y.c[0] * z.c[2] - y.c[2] * z.c[0]) / detVal;
	r.m[0][2] =  (y.c[0] * z.c[1] - y.c[1] * z.c[0]) / detVal;
	r.m[1][0] = -(x.c[1] * z.c[2] - x.c[2] * z.c[1]) / detVal;
	r.m[1][1] =  (x.c[0] * z.c[2] - x.c[2] * z.c[0]) / detVal;
	r.m[1][2] = -(x.c[0] * z.c[1] - x.c[1] * z.c[0]) / detVal;
	r.m[2][0] =  (x.c[1] * y.c[2] - x.c[2] * y.c[1]) / detVal;
	r.m[2][1] = -(x.c[0] * y.c[2] - x.c[2] * y.c[0]) / detVal;
	r.m[2][2] =  (x.c[0] * y.c[1] - x.c[1] * y.c[0]) / detVal;
#endif
	return r;
}

static inline vec matvec(mat A, vec b)
{ /* matVecMul: inc/matvec.h:217-223, 551-558 */
	vec r;
	for (int i = 0; i < DIM; ++i) {
		double s = A.m[i][0] * b.c[0];
		for (int j = 1; j < DIM; ++j) s = s + A.m[i][j] * b.c[j];
		r.c[i] = s;
	}
	return r;
}
static inline mat matmul(mat A, mat B)
{ /* matMatMul: inc/matvec.h:279-288, 651-666 */
	mat R;
	for (int i = 0; i < DIM; ++i)
		for (int j = 0; j < DIM; ++j) {
			double s = A.m[i][0] * B.m[0][j];
			for (int k = 1; k < DIM; ++k) s = s + A.m[i][k] * B.m[k][j];
			R.m[i][j] = s;
		}
	return R;
}

static inline double elm_volume(double det)
{ /* computeVolume: inc/utility.h:11-29 */
#if DIM == 2
	return 0.5 * fabs(det);
#else
	return fabs(det) / 6.0;
#endif
}

/* edges of element e from an edge array (getEdge, inc/matvec.h:84-93, 407-421) */
static inline void get_edges(const double *edg, int e, int E, vec *q)
{
	for (int k = 0; k < DIM; ++k)
		for (int d = 0; d < DIM; ++d) q[k].c[d] = edg[(k * DIM + d) * E + e];
}

/* ------------------------------------------------------------------ */
/* reference dense BLAS/LAPACK stand-ins (textbook order)              */
/* ------------------------------------------------------------------ */
static double ddot(const double *x, const double *y, int n)
{
	double s = 0.0;
	for (int i = 0; i < n; ++i) s += x[i] * y[i];
	return s;
}

static void axpby(double *out, double a, const double *x, double b, const double *y, long n)
{ /* 2D/vectoraxpby.cu:3-10 */
	#pragma omp parallel for schedule(static)
	for (long i = 0; i < n; ++i) out[i] = a * x[i] + b * y[i];
}

/* lower Cholesky in place, column-major A[col*n+row]: L_ij = (A_ij - sum_k L_ik L_jk) / L_jj */
static int potrf_lower(double *A, int n)
{
	/* row-major scratch copy of the lower triangle for contiguous dots */
	double *L = (double *) malloc(sizeof(double) * (size_t) n * n);
	if (!L) return -1;
	int bad = 0;
	for (int j = 0; j < n; ++j) {
		double s = A[(size_t) j * n + j];
		const double *Lj = L + (size_t) j * n;
		for (int k = 0; k < j; ++k) s -= Lj[k] * Lj[k];
		if (!(s > 0.0)) bad = 1;
		double ljj = sqrt(s);
		L[(size_t) j * n + j] = ljj;
		#pragma omp parallel for schedule(static)
		for (int i = j + 1; i < n; ++i) {
			const double *Li = L + (size_t) i * n;
			double t = A[(size_t) j * n + i];
			for (int k = 0; k < j; ++k) t -= Li[k] * Lj[k];
			L[(size_t) i * n + j] = t / ljj;
		}
	}
	for (int j = 0; j < n; ++j)
		for (int i = j; i < n; ++i) A[(size_t) j * n + i] = L[(size_t) i * n + j];
	free(L);
	return bad;
}

/* solve L L^T x = b for one right-hand side (column-major lower factor) */
static void potrs_lower(const double *L, int n, double *b)
{
	for (int i = 0; i < n; ++i) {           /* forward: L y = b */
		double s = b[i];
		for (int k = 0; k < i; ++k) s -= L[(size_t) k * n + i] * b[k];
		b[i] = s / L[(size_t) i * n + i];
	}
	for (int i = n - 1; i >= 0; --i) {      /* backward: L^T x = y */
		double s = b[i];
		const double *Li = L + (size_t) i * n;   /* column i of L = row i of L^T */
		for (int k = i + 1; k < n; ++k) s -= Li[k] * b[k];
		b[i] = s / Li[i];
	}
}

/* y = alpha * A x + beta * y, A column-major n x n (cublasDgemv CUBLAS_OP_N) */
static void gemv(int n, double alpha, const double *A, const double *x, double beta, double *y)
{
	#pragma omp parallel for schedule(static)
	for (int i = 0; i < n; ++i) {
		double s = 0.0;
		for (int j = 0; j < n; ++j) s += A[(size_t) j * n + i] * x[j];
		y[i] = (beta == 0.0 ? alpha * s : alpha * s + beta * y[i]);   /* BLAS: y not read when beta = 0 */
	}
}

/* dsum: 2D/dsum.cu:6-73 (shared-memory tree over 512-wide blocks) */
static double tree512(const double *v, int len)
{
	double s[SUMBLK];
	for (int t = 0; t < SUMBLK; ++t) s[t] = (t < len ? v[t] : 0.0);
	for (int stride = SUMBLK >> 1; stride > 0; stride >>= 1)
		for (int t = 0; t < stride; ++t) s[t] += s[t + stride];
	return s[0];
}

double orc_dsum(const double *vec, int len)
{
	if (len < SUMBLK) return tree512(vec, len);
	double buf[SUMBLK];
	memset(buf, 0, sizeof(buf));
	int runNum = (len - 1) / (SUMBLK * SUMBLK) + 1;
	for (int runIdx = 0; runIdx < runNum; ++runIdx) {
		int lenNow = (runIdx == runNum - 1 ? len - runIdx * SUMBLK * SUMBLK : SUMBLK * SUMBLK);
		int blkNum = (lenNow - 1) / SUMBLK + 1;
		const double *v = vec + (size_t) runIdx * SUMBLK * SUMBLK;
		for (int b = 0; b < blkNum; ++b) {
			int n = lenNow - b * SUMBLK; if (n > SUMBLK) n = SUMBLK;
			buf[b] += tree512(v + (size_t) b * SUMBLK, n);
		}
	}
	return tree512(buf, SUMBLK);
}

/* ------------------------------------------------------------------ */
/* activity functions (inc/activity.h)                                 */
/* ------------------------------------------------------------------ */
static double yank_template(double tauVal, double dWidth)
{ /* inc/activity.h:4-38 */
	double a = 3.0 * (dWidth - 2.0) / (dWidth * dWidth * dWidth * (6.0 + dWidth * (-6.0 + dWidth)));
	double b = (6.0 + dWidth * (-15.0 + 8 * dWidth)) / (3.0 * (dWidth - 2.0));
	double c = 6.0 / (6.0 + dWidth * (-6.0 + dWidth));
	if (tauVal < -1.0 || tauVal >= 1.0) return 0.0;
	if (tauVal >= -1.0 && tauVal < -1.0 + dWidth)
		return a * (tauVal + 1.0) * (tauVal + 1.0) * (tauVal + 1.0) * (tauVal - b);
	if (tauVal >= -1.0 + dWidth && tauVal < 1.0 - dWidth)
		return -c * tauVal * tauVal + 1.0;
	return a * (-tauVal + 1.0) * (-tauVal + 1.0) * (-tauVal + 1.0) * (-tauVal - b);
}

static double reac_template(double tauVal, double dWidth, double hatVal)
{ /* inc/activity.h:106-167 */
	double a  = hatVal;
	double b1 = 8.0 * (6.0 * (a - 1.0) + a * dWidth * (-6.0 + dWidth))
	            / (3.0 * dWidth * dWidth * dWidth * dWidth);
	double b2 =  -(144.0 * (a - 1.0) + dWidth * (24.0 * (5.0 - 11.0 * a) + dWidth * (156.0 * a - dWidth * 29.0 * a)))
	            / (24.0 * (6.0 * (a - 1.0) + a * dWidth * (-6.0 + dWidth)));
	double c1 = -(24.0 * (a - 1.0) + a * dWidth * (-12.0 + dWidth)) / (9.0 * dWidth * dWidth * dWidth);
	double c2 = -(24.0 * (a - 1.0) + dWidth * (12.0 * (2.0 - 3.0 * a) + a * dWidth * (13.0 + dWidth * 2.0)))
	            / (3.0 * dWidth * dWidth * dWidth);
	double c3 = -((dWidth - 1.0) * (dWidth - 1.0) * (24.0 * (a - 1.0) + a * dWidth * (-12.0 + dWidth)))
	            / (3.0 * dWidth * dWidth * dWidth);
	double c4 = -(24.0 * (a - 1.0)
	              + dWidth * (12.0 * (6.0 - 7.0 * a)
	                          + dWidth * (-72.0 + 109.0 * a
	                                      + dWidth * (3.0 * (5.0 - 21.0 * a)
	                                                  + a * dWidth * (15.0 - dWidth)))))
	            / (9.0 * dWidth * dWidth * dWidth);
	if (tauVal < -1.0 || tauVal >= 1.0) return 0.0;
	if (tauVal >= -1.0 && tauVal < -1.0 + 0.5 * dWidth)
		return b1 * (tauVal + 1.0) * (tauVal + 1.0) * (tauVal + 1.0) * (tauVal - b2);
	if (tauVal >= -1.0 + 0.5 * dWidth && tauVal < -1.0 + dWidth)
		return c4 + tauVal * (c3 + tauVal * (c2 + tauVal * c1));
	if (tauVal >= -1.0 + dWidth && tauVal < 1.0 - dWidth)
		return -a * tauVal * tauVal + 1.0;
	if (tauVal >= 1.0 - dWidth && tauVal < 1.0 - 0.5 * dWidth)
		return c4 + tauVal * (-c3 + tauVal * (c2 - tauVal * c1));
	return b1 * (-tauVal + 1.0) * (-tauVal + 1.0) * (-tauVal + 1.0) * (-tauVal - b2);
}

void orc_yank_activity(const orc_problem *P, const double *tau, double *f, int n)
{
	const double *p = P->ynkActPrmVec;
	if (P->elaType == ORC_ISOTROPIC) {
		/* layered model: atrophy eigenstrain f(u) = c * u */
		for (int i = 0; i < n; ++i) f[i] = p[0] * tau[i];
		return;
	}
	/* 2D/yankTauActivity.cu:4-33, inc/activity.h:81-89 */
	double tauMin = p[0], tauMax = p[1], actMax = p[2], dWidth = p[3];
	for (int i = 0; i < n; ++i) {
		double tauStd = -1.0 + 2.0 * (tau[i] - tauMin) / (tauMax - tauMin);
		f[i] = yank_template(tauStd, dWidth) * actMax;
	}
}

void orc_reaction_activity(const orc_problem *P, const double *tau, double *f, int n)
{
	const double *p = P->reaActPrmVec;
	if (P->elaType == ORC_ISOTROPIC) {
		/* Fisher-KPP reaction R(u) = rate * u * (1 - u) */
		for (int i = 0; i < n; ++i) f[i] = p[0] * tau[i] * (1.0 - tau[i]);
		return;
	}
	/* 2D/reactionTauActivity.cu:4-35, inc/activity.h:239-249 */
	double tauMin = p[0], tauMax = p[1], actMax = p[2], dWidth = p[3], hatVal = p[4];
	for (int i = 0; i < n; ++i) {
		double tauStd = -1.0 + 2.0 * (tau[i] - tauMin) / (tauMax - tauMin);
		f[i] = reac_template(tauStd, dWidth, hatVal) * actMax;
	}
}

/* ------------------------------------------------------------------ */
/* initial chemical                                                    */
/* ------------------------------------------------------------------ */
static double intpow(double bseVal, int expInt)
{ /* 2D/tauInitial.cu:4-22 */
	double outVal = 1;
	double powVal = bseVal;
	do {
		int quoInt = expInt >> 1;
		int remInt = expInt - 2 * quoInt;
		if (remInt == 1) outVal *= powVal;
		powVal *= powVal;
		expInt = quoInt;
	} while (expInt != 0);
	return outVal;
}

void orc_initial_tau(const orc_problem *P, const double *tv, double *tau)
{
	int N = P->lmkNum;
	const double *x = P->lmkIniMat;
	if (P->elaType == ORC_ISOTROPIC) {
		/* Gaussian bump h * exp(-|x - c|^2 / (2 sigma^2)); tauVar = [c, h, sigma] */
		double h = tv[DIM], sg = tv[DIM + 1];
		for (int i = 0; i < N; ++i) {
			double r2 = 0.0;
			for (int d = 0; d < DIM; ++d) { double t = x[d * N + i] - tv[d]; r2 += t * t; }
			tau[i] = h * exp(-r2 / (2.0 * sg * sg));
		}
		return;
	}
#if DIM == 2
	/* 2D/tauInitial.cu:24-64: tauVar = [cx, cy, h, R], tauPrm = [p] */
	double cx = tv[0], cy = tv[1], hgt = tv[2], rad = tv[3];
	int pw = (int) P->tauPrmVec[0];
	for (int i = 0; i < N; ++i) {
		double tauRad2 = rad * rad;
		double xDif = x[i] - cx, yDif = x[N + i] - cy;
		double radSqu = (xDif * xDif + yDif * yDif) / tauRad2;
		double tmpVal = (radSqu - 1.0) * (radSqu - 1.0);
		double pre = (radSqu < 1.0 ? 1.0 - intpow(1.0 - tmpVal, pw) : 0.0);
		tau[i] = hgt * pre;
	}
#else
	/* 3D/tauInitial.cu:24-66: tauVar = [cx, cy, cz, h], tauPrm = [R, p] */
	double cx = tv[0], cy = tv[1], cz = tv[2], hgt = tv[3];
	double rad = P->tauPrmVec[0];
	int pw = (int) P->tauPrmVec[1];
	for (int i = 0; i < N; ++i) {
		double tauRad2 = rad * rad;
		double xDif = x[i] - cx, yDif = x[N + i] - cy, zDif = x[2 * N + i] - cz;
		double radSqu = (xDif * xDif + yDif * yDif + zDif * zDif) / tauRad2;
		double tmpVal = (radSqu - 1.0) * (radSqu - 1.0);
		double pre = (radSqu < 1.0 ? 1.0 - intpow(1.0 - tmpVal, pw) : 0.0);
		tau[i] = hgt * pre;
	}
#endif
}

/* ------------------------------------------------------------------ */
/* geometry                                                            */
/* ------------------------------------------------------------------ */
void orc_edges(const orc_problem *P, const double *lmk, double *edg)
{ /* 2D/vertexToEdge.cu:4-27, 3D/vertexToEdge.cu:4-30 */
	int N = P->lmkNum, E = P->elmNum;
	#pragma omp parallel for schedule(static)
	for (int e = 0; e < E; ++e) {
		vec q0 = getv(lmk, P->elmVtxMat[e], N);
		for (int k = 1; k < VTX; ++k) {
			vec qk = getv(lmk, P->elmVtxMat[k * E + e], N);
			vec dq = vsub(qk, q0);
			for (int d = 0; d < DIM; ++d) edg[((k - 1) * DIM + d) * E + e] = dq.c[d];
		}
	}
}

void orc_frame(const orc_problem *P, const double *lmk, double *frmA, double *tsvMat)
{
	int N = P->lmkNum, E = P->elmNum;
	#pragma omp parallel for schedule(static)
	for (int e = 0; e < E; ++e) {
		vec s; for (int d = 0; d < DIM; ++d) s.c[d] = 0.0;
#if DIM == 2
		/* frameTanKernel 2D/computeFrame.cu:4-35 */
		for (int t = 0; t < 2; ++t) {
			vec l = getv(lmk, P->frmVtxMat[(2 * t) * E + e], N);
			vec r = getv(lmk, P->frmVtxMat[(2 * t + 1) * E + e], N);
			vec df = vsub(r, l);
			double len = vnorm(df);
			for (int d = 0; d < DIM; ++d) s.c[d] += df.c[d] / len;
		}
#else
		/* frameNmlKernel 3D/computeFrame.cu:6-44 */
		for (int t = 0; t < 2; ++t) {
			vec q0 = getv(lmk, P->frmVtxMat[(3 * t) * E + e], N);
			vec q1 = getv(lmk, P->frmVtxMat[(3 * t + 1) * E + e], N);
			vec q2 = getv(lmk, P->frmVtxMat[(3 * t + 2) * E + e], N);
			vec c = vcross(vsub(q1, q0), vsub(q2, q0));
			double len = vnorm(c);
			for (int d = 0; d < DIM; ++d) s.c[d] += c.c[d] / len;
		}
#endif
		double sl = vnorm(s);
		for (int d = 0; d < DIM; ++d) frmA[d * E + e] = s.c[d] / sl;

		/* frameTsvKernel 2D/computeFrame.cu:37-68, 3D/computeFrame.cu:46-78 */
		vec u; for (int d = 0; d < DIM; ++d) u.c[d] = 0.0;
		int tsvNum = (DIM == 2 ? 2 : 3);
		for (int t = 0; t < tsvNum; ++t) {
			vec dw = getv(lmk, P->tsvVtxMat[(2 * t) * E + e], N);
			vec up = getv(lmk, P->tsvVtxMat[(2 * t + 1) * E + e], N);
			vec df = vsub(up, dw);
			double len = vnorm(df);
			for (int d = 0; d < DIM; ++d) u.c[d] += df.c[d] / len;
		}
		double ul = vnorm(u);
		for (int d = 0; d < DIM; ++d) tsvMat[d * E + e] = u.c[d] / ul;
	}
}

/* gradient row a (0..DIM) of the barycentric coordinates: g_0 = -sum, g_a = row a-1 of Q^{-1} */

/* ------------------------------------------------------------------ */
/* mass and diffusion element matrices (assembleFemMatrix)             */
/* ------------------------------------------------------------------ */
static void fem_elements(const orc_problem *P, const double *edg, const double *frmA,
                         const double *tsvMat, double *ppdElm, double *ggdElm)
{
	int E = P->elmNum;
	#pragma omp parallel for schedule(static)
	for (int e = 0; e < E; ++e) {
		vec q[DIM]; get_edges(edg, e, E, q);
		double absDetQ = fabs(detQ(q));
		mat QI = invQ(q);
		double G[VTX][DIM];    /* gradients of barycentric coordinates */
		for (int d = 0; d < DIM; ++d) {
			double s = -QI.m[0][d];
			for (int a = 1; a < DIM; ++a) s = s - QI.m[a][d];
			G[0][d] = s;
			for (int a = 0; a < DIM; ++a) G[a + 1][d] = QI.m[a][d];
		}
		if (P->elaType == ORC_ISOTROPIC) {
			double Dl = P->spdLyrVec[P->elmLyrVec[e]];
#if DIM == 2
			double mvol = 0.5 * absDetQ;
			ppdElm[e] = absDetQ / 24.0;
#else
			double mvol = absDetQ / 6.0;
			ppdElm[e] = absDetQ / 120.0;
#endif
			int k = 0;
			for (int a = 0; a < VTX; ++a)
				for (int b = a; b < VTX; ++b, ++k) {
					double gg = G[a][0] * G[b][0];
					for (int d = 1; d < DIM; ++d) gg = gg + G[a][d] * G[b][d];
					ggdElm[k * E + e] = mvol * (Dl * gg);
				}
			continue;
		}
#if DIM == 2
		/* femMatComputeKernel 2D/assembleFemMatrix.cu:5-59 */
		vec tan = getv(frmA, e, E), tsv = getv(tsvMat, e, E);
		vec QIt = matvec(QI, tan), QIs = matvec(QI, tsv);
		double tG[3] = { -QIt.c[0] - QIt.c[1], QIt.c[0], QIt.c[1] };
		double sG[3] = { -QIs.c[0] - QIs.c[1], QIs.c[0], QIs.c[1] };
		ppdElm[e] = absDetQ / 24.0;
		int k = 0;
		for (int a = 0; a < 3; ++a)
			for (int b = a; b < 3; ++b, ++k)
				ggdElm[k * E + e] = 0.5 * absDetQ * (  P->spdTanVal * tG[a] * tG[b]
				                                     + P->spdTsvVal * sG[a] * sG[b] );
#else
		/* femMatComputeKernel 3D/assembleFemMatrix.cu:5-118 */
		vec nml = getv(frmA, e, E), tsv = getv(tsvMat, e, E);
		vec QIn = matvec(QI, nml), QIs = matvec(QI, tsv);
		double eG[3][4], nG[4], sG[4];
		for (int d = 0; d < 3; ++d) {
			eG[d][0] = -QI.m[0][d] - QI.m[1][d] - QI.m[2][d];
			eG[d][1] = QI.m[0][d]; eG[d][2] = QI.m[1][d]; eG[d][3] = QI.m[2][d];
		}
		nG[0] = -QIn.c[0] - QIn.c[1] - QIn.c[2]; nG[1] = QIn.c[0]; nG[2] = QIn.c[1]; nG[3] = QIn.c[2];
		sG[0] = -QIs.c[0] - QIs.c[1] - QIs.c[2]; sG[1] = QIs.c[0]; sG[2] = QIs.c[1]; sG[3] = QIs.c[2];
		ppdElm[e] = absDetQ / 120.0;
		int k = 0;
		for (int a = 0; a < 4; ++a)
			for (int b = a; b < 4; ++b, ++k)
				ggdElm[k * E + e] = absDetQ / 6.0 * (  P->spdTanVal * (   eG[0][a] * eG[0][b]
				                                                       + eG[1][a] * eG[1][b]
				                                                       + eG[2][a] * eG[2][b]
				                                                       - nG[a] * nG[b] )
				                                     + P->spdTsvVal * sG[a] * sG[b] );
#endif
	}
}

/* femMatGatherKernel 2D/assembleFemMatrix.cu:61-92: values per femVtxMat slot */
static void fem_gather_csr(const orc_problem *P, const double *ppdElm, const double *ggdElm,
                           double *ppdVal, double *ggdVal)
{
	int Z = P->nzrNum;
	const int *ifo = P->femIfoMat;
	#pragma omp parallel for schedule(static)
	for (int z = 0; z < Z; ++z) {
		double ppd = 0.0, ggd = 0.0;
		int adjNum = ifo[z];
		double mulVal = ifo[Z + z];
		for (int a = 0; a < adjNum; ++a) {
			int e = ifo[(2 + 2 * a) * Z + z];
			int g = ifo[(2 + 2 * a + 1) * Z + z];
			ppd += mulVal * ppdElm[e];
			ggd += ggdElm[g];
		}
		ppdVal[z] = ppd; ggdVal[z] = ggd;
	}
}

void orc_fem_csr(const orc_problem *P, const double *lmk, double *ppdVal, double *ggdVal)
{
	int E = P->elmNum;
	double *edg = malloc(sizeof(double) * E * DIM * DIM);
	double *frmA = malloc(sizeof(double) * E * DIM), *tsv = malloc(sizeof(double) * E * DIM);
	double *ppdElm = malloc(sizeof(double) * E), *ggdElm = malloc(sizeof(double) * E * NPAIR);
	orc_edges(P, lmk, edg);
	if (P->elaType == ORC_FRAME) orc_frame(P, lmk, frmA, tsv);
	fem_elements(P, edg, frmA, tsv, ppdElm, ggdElm);
	fem_gather_csr(P, ppdElm, ggdElm, ppdVal, ggdVal);
	free(edg); free(frmA); free(tsv); free(ppdElm); free(ggdElm);
}

/* consistent-mass load vector: 2D/assembleFemVector.cu:5-54, 3D :5-57 */
static void fem_vector(const orc_problem *P, const double *edg, const double *f,
                       double *rpdElm, double *rpd)
{
	int E = P->elmNum, N = P->lmkNum;
	#pragma omp parallel for schedule(static)
	for (int e = 0; e < E; ++e) {
		vec q[DIM]; get_edges(edg, e, E, q);
		double absDetQ = fabs(detQ(q));
		double fv[VTX];
		for (int k = 0; k < VTX; ++k) fv[k] = f[P->elmVtxMat[k * E + e]];
#if DIM == 2
		rpdElm[e]         = (2.0 * fv[0] +       fv[1] +       fv[2]) * absDetQ / 24.0;
		rpdElm[E + e]     = (      fv[0] + 2.0 * fv[1] +       fv[2]) * absDetQ / 24.0;
		rpdElm[2 * E + e] = (      fv[0] +       fv[1] + 2.0 * fv[2]) * absDetQ / 24.0;
#else
		rpdElm[e]         = (2.0 * fv[0] +       fv[1] +       fv[2] +       fv[3]) * absDetQ / 120.0;
		rpdElm[E + e]     = (      fv[0] + 2.0 * fv[1] +       fv[2] +       fv[3]) * absDetQ / 120.0;
		rpdElm[2 * E + e] = (      fv[0] +       fv[1] + 2.0 * fv[2] +       fv[3]) * absDetQ / 120.0;
		rpdElm[3 * E + e] = (      fv[0] +       fv[1] +       fv[2] + 2.0 * fv[3]) * absDetQ / 120.0;
#endif
	}
	const int *ve = P->vtxElmMat;
	#pragma omp parallel for schedule(static)
	for (int i = 0; i < N; ++i) {
		double s = 0.0;
		int adjNum = ve[i];
		for (int a = 0; a < adjNum; ++a) {
			int e = ve[(1 + 2 * a) * N + i], l = ve[(2 + 2 * a) * N + i];
			s += rpdElm[l * E + e];
		}
		rpd[i] = s;
	}
}

/* ------------------------------------------------------------------ */
/* elasticity                                                          */
/* ------------------------------------------------------------------ */
/* computePreMat, frame: 2D/applyFrameElasticOperator.cu:7-39, 3D :7-111 */
static mat pre_frame(const orc_problem *P, vec a, vec s, mat ep)
{
	mat pm;
	const double *mv = P->modVec;
#if DIM == 2
	double muTan = mv[0], muTsv = mv[1], muAng = mv[2];
	vec t = a;
	vec evS = matvec(ep, s);
	/* vecMatVecMul inc/matvec.h:233-237 */
	double TvT = t.c[0] * (ep.m[0][0] * t.c[0] + ep.m[0][1] * t.c[1])
	           + t.c[1] * (ep.m[1][0] * t.c[0] + ep.m[1][1] * t.c[1]);
	double SvS = vdot(s, evS);
	double TvS = vdot(t, evS);
	pm.m[0][0]  = muTan * (t.c[0] * t.c[0]) * TvT;
	pm.m[0][1]  = muTan * (t.c[0] * t.c[1]) * TvT;
	pm.m[1][0]  = muTan * (t.c[1] * t.c[0]) * TvT;
	pm.m[1][1]  = muTan * (t.c[1] * t.c[1]) * TvT;
	pm.m[0][0] += muTsv * (s.c[0] * s.c[0]) * SvS;
	pm.m[0][1] += muTsv * (s.c[0] * s.c[1]) * SvS;
	pm.m[1][0] += muTsv * (s.c[1] * s.c[0]) * SvS;
	pm.m[1][1] += muTsv * (s.c[1] * s.c[1]) * SvS;
	pm.m[0][0] += muAng * (2.0 * t.c[0] * s.c[0]) * TvS;
	pm.m[0][1] += muAng * (t.c[0] * s.c[1] + s.c[0] * t.c[1]) * TvS;
	pm.m[1][0] += muAng * (t.c[1] * s.c[0] + s.c[1] * t.c[0]) * TvS;
	pm.m[1][1] += muAng * (2.0 * t.c[1] * s.c[1]) * TvS;
#else
	double ldTan = mv[0], muTan = mv[1], muTsv = mv[2], muAng = mv[3];
	vec n = a;
	vec evN = matvec(ep, n), evS = matvec(ep, s);
	double NvN = vdot(n, evN), SvS = vdot(s, evS), NvS = vdot(n, evS);
	double ldv = (ep.m[0][0] + ep.m[1][1] + ep.m[2][2]) - NvN;   /* trace - NvN */
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			pm.m[i][j] = ldTan * (i == j ? 1.0 - n.c[i] * n.c[j] : -n.c[i] * n.c[j]) * ldv;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) {
			if (i == j)
				pm.m[i][j] += muTan * (  ep.m[i][j] - (2.0 * evN.c[i] * n.c[j])
				                       + NvN * n.c[i] * n.c[j] );
			else
				pm.m[i][j] += muTan * (  ep.m[i][j] - (evN.c[i] * n.c[j] + n.c[i] * evN.c[j])
				                       + NvN * n.c[i] * n.c[j] );
		}
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			pm.m[i][j] += muTsv * SvS * s.c[i] * s.c[j];
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) {
			if (i == j)
				pm.m[i][j] += muAng * (  2.0 * evS.c[i] * s.c[j]
				                       - NvS * 2.0 * n.c[i] * s.c[j] );
			else
				pm.m[i][j] += muAng * (  (evS.c[i] * s.c[j] + s.c[i] * evS.c[j])
				                       - NvS * (n.c[i] * s.c[j] + s.c[i] * n.c[j]) );
		}
#endif
	return pm;
}

/* isotropic layered stress sigma = lambda tr(eps) I + 2 mu eps */
static mat pre_iso(const orc_problem *P, int e, mat ep)
{
	int l = P->elmLyrVec[e];
	double lam = P->modVec[2 * l], mu = P->modVec[2 * l + 1];
	double tr = ep.m[0][0];
	for (int d = 1; d < DIM; ++d) tr = tr + ep.m[d][d];
	mat pm;
	for (int i = 0; i < DIM; ++i)
		for (int j = 0; j < DIM; ++j)
			pm.m[i][j] = 2.0 * mu * ep.m[i][j] + (i == j ? lam * tr : 0.0);
	return pm;
}

/* element forces (strain 2D/computeStrainTensor.cu:4-44, compute kernel
 * 2D/applyFrameElasticOperator.cu:41-85) then gather (:87-111) */
static void elastic_apply(const orc_problem *P, const double *edg, const double *frmA,
                          const double *tsvMat, const double *v, double *elYElm, double *y)
{
	int N = P->lmkNum, E = P->elmNum;
	#pragma omp parallel for schedule(static)
	for (int e = 0; e < E; ++e) {
		vec q[DIM]; get_edges(edg, e, E, q);
		vec v0 = getv(v, P->elmVtxMat[e], N);
		mat V;
		for (int k = 0; k < DIM; ++k) {
			vec vk = getv(v, P->elmVtxMat[(k + 1) * E + e], N);
			vec dv = vsub(vk, v0);
			for (int d = 0; d < DIM; ++d) V.m[d][k] = dv.c[d];   /* columns2Mat */
		}
		mat QI = invQ(q);
		mat Dv = matmul(V, QI);
		mat ep;
#if DIM == 2
		ep.m[0][0] = Dv.m[0][0];
		ep.m[0][1] = 0.5 * (Dv.m[0][1] + Dv.m[1][0]);
		ep.m[1][0] = 0.5 * (Dv.m[0][1] + Dv.m[1][0]);
		ep.m[1][1] = Dv.m[1][1];
#else
		/* 3D/computeStrainTensor.cu:41-49 */
		ep.m[0][0] = Dv.m[0][0];
		ep.m[0][1] = 0.5 * (Dv.m[0][1] + Dv.m[1][0]);
		ep.m[0][2] = 0.5 * (Dv.m[0][2] + Dv.m[2][0]);
		ep.m[1][0] = 0.5 * (Dv.m[1][0] + Dv.m[0][1]);
		ep.m[1][1] = Dv.m[1][1];
		ep.m[1][2] = 0.5 * (Dv.m[1][2] + Dv.m[2][1]);
		ep.m[2][0] = 0.5 * (Dv.m[2][0] + Dv.m[0][2]);
		ep.m[2][1] = 0.5 * (Dv.m[2][1] + Dv.m[1][2]);
		ep.m[2][2] = Dv.m[2][2];
#endif
		double volVal = elm_volume(detQ(q));
		mat pm;
		if (P->elaType == ORC_ISOTROPIC) pm = pre_iso(P, e, ep);
		else pm = pre_frame(P, getv(frmA, e, E), getv(tsvMat, e, E), ep);
		mat dvE = matmul(QI, pm);
		double f[VTX][DIM];
		for (int d = 0; d < DIM; ++d) {
			double s = -dvE.m[0][d];
			for (int a = 1; a < DIM; ++a) s = s - dvE.m[a][d];
			f[0][d] = s * volVal;
			for (int a = 0; a < DIM; ++a) f[a + 1][d] = dvE.m[a][d] * volVal;
		}
		for (int k = 0; k < VTX; ++k)
			for (int d = 0; d < DIM; ++d) elYElm[(k * DIM + d) * E + e] = f[k][d];
	}
	const int *ve = P->vtxElmMat;
	#pragma omp parallel for schedule(static)
	for (int i = 0; i < N; ++i) {
		double s[DIM]; for (int d = 0; d < DIM; ++d) s[d] = 0.0;
		int adjNum = ve[i];
		for (int a = 0; a < adjNum; ++a) {
			int e = ve[(1 + 2 * a) * N + i], l = ve[(2 + 2 * a) * N + i];
			for (int d = 0; d < DIM; ++d) s[d] = s[d] + elYElm[l * E * DIM + d * E + e];
		}
		for (int d = 0; d < DIM; ++d) y[d * N + i] = s[d];
	}
}

/* bottom penalty: 2D/applyPenaltyOperator.cu:4-63, 3D :4-69.  The
 * gathered value lands at node index btmLmkIdx (bottom nodes are the first
 * btmLmkNum nodes), exactly as penaltyGatherKernel writes it. */
static double btm_face_measure(const orc_problem *P, const vec *qb)
{
#if DIM == 2
	(void) P;
	return vnorm(vsub(qb[1], qb[0]));
#else
	if (P->elaType == ORC_FRAME)   /* 3D/applyPenaltyOperator.cu:13-14: projected (x,y) area */
		return 0.5 * fabs(  (qb[1].c[0] - qb[0].c[0]) * (qb[2].c[1] - qb[0].c[1])
		                  - (qb[1].c[1] - qb[0].c[1]) * (qb[2].c[0] - qb[0].c[0]));
	/* layered model: true face area */
	return 0.5 * vnorm(vcross(vsub(qb[1], qb[0]), vsub(qb[2], qb[0])));
#endif
}

static void penalty_apply(const orc_problem *P, const double *lmk, const double *v, double *y)
{
	int N = P->lmkNum, B = P->btmElmNum, Nb = P->btmLmkNum;
	double *pnl = malloc(sizeof(double) * (size_t) B * DIM * (VTX - 1));
	#pragma omp parallel for schedule(static)
	for (int b = 0; b < B; ++b) {
		vec qb[VTX - 1];
		for (int k = 0; k < VTX - 1; ++k) qb[k] = getv(lmk, P->btmVtxMat[k * B + b], N);
		double m = btm_face_measure(P, qb);
		for (int k = 0; k < VTX - 1; ++k) {
			vec vk = getv(v, P->btmVtxMat[k * B + b], N);
			for (int d = 0; d < DIM; ++d)
				pnl[(k * DIM + d) * B + b] = vk.c[d] * m / (VTX - 1.0);
		}
	}
	for (long i = 0; i < (long) N * DIM; ++i) y[i] = 0.0;
	const int *vb = P->vtxBtmMat;
	for (int i = 0; i < Nb; ++i) {
		double s[DIM]; for (int d = 0; d < DIM; ++d) s[d] = 0.0;
		int adjNum = vb[i];
		for (int a = 0; a < adjNum; ++a) {
			int b = vb[(1 + 2 * a) * Nb + i], l = vb[(2 + 2 * a) * Nb + i];
			for (int d = 0; d < DIM; ++d) s[d] = s[d] + pnl[l * B * DIM + d * B + b];
		}
		for (int d = 0; d < DIM; ++d) y[d * N + i] = s[d];
	}
	free(pnl);
}

/* yank load: 2D/computeExternalYank.cu:5-47 (compute) and :86-122 (gather) */
static void yank_apply(const orc_problem *P, const double *edg, const double *f,
                       double *exYElm, double *b)
{
	int N = P->lmkNum, E = P->elmNum;
	#pragma omp parallel for schedule(static)
	for (int e = 0; e < E; ++e) {
		vec q[DIM]; get_edges(edg, e, E, q);
		double volVal = elm_volume(detQ(q));
		mat QI = invQ(q);
		double fs = f[P->elmVtxMat[e]];
		for (int k = 1; k < VTX; ++k) fs = fs + f[P->elmVtxMat[k * E + e]];
		double fcVal = fs / VTX;
		double g[VTX][DIM];
		for (int d = 0; d < DIM; ++d) {
			double s = -QI.m[0][d];
			for (int a = 1; a < DIM; ++a) s = s - QI.m[a][d];
			g[0][d] = -fcVal * s * volVal;
			for (int a = 0; a < DIM; ++a) g[a + 1][d] = -fcVal * QI.m[a][d] * volVal;
		}
		for (int k = 0; k < VTX; ++k)
			for (int d = 0; d < DIM; ++d) exYElm[(k * DIM + d) * E + e] = g[k][d];
	}
	const int *ve = P->vtxElmMat;
	#pragma omp parallel for schedule(static)
	for (int i = 0; i < N; ++i) {
		double s[DIM]; for (int d = 0; d < DIM; ++d) s[d] = 0.0;
		int adjNum = ve[i];
		for (int a = 0; a < adjNum; ++a) {
			int e = ve[(1 + 2 * a) * N + i], l = ve[(2 + 2 * a) * N + i];
			for (int d = 0; d < DIM; ++d) s[d] = s[d] + exYElm[l * E * DIM + d * E + e];
		}
		for (int d = 0; d < DIM; ++d) b[d * N + i] = s[d];
	}
}

/* ------------------------------------------------------------------ */
/* RKHS kernel (computeKernel)                                         */
/* ------------------------------------------------------------------ */
#if DIM == 2
/* rational-approximation coefficients of inc/besselk.h:4-180 */
static const double P01[6] = { 2.4708152720399552679e+03,  5.9169059852270512312e+03,
                               4.6850901201934832188e+02,  1.1999463724910714109e+01,
                               1.3166052564989571850e-01,  5.8599221412826100000e-04};
static const double Q01[3] = { 2.1312714303849120380e+04, -2.4994418972832303646e+02, 1};
static const double P02[4] = {-4.0320340761145482298e+05, -1.7733784684952985886e+04,
                              -2.9601657892958843866e+02, -1.6414452837299064100e+00};
static const double Q02[4] = {-1.6128136304458193998e+06,  2.9865713163054025489e+04,
                              -2.5064972445877992730e+02,  1};
static const double P03[10] = { 1.1600249425076035558e+02,  2.3444738764199315021e+03,
                                1.8321525870183537725e+04,  7.1557062783764037541e+04,
                                1.5097646353289914539e+05,  1.7398867902565686251e+05,
                                1.0577068948034021957e+05,  3.1075408980684392399e+04,
                                3.6832589957340267940e+03,  1.1394980557384778174e+02};
static const double Q03[11] = { 9.2556599177304839811e+01,  1.8821890840982713696e+03,
                                1.4847228371802360957e+04,  5.8824616785857027752e+04,
                                1.2689839587977598727e+05,  1.5144644673520157801e+05,
                                9.7418829762268075784e+04,  3.1474655750295278825e+04,
                                4.4329628889746408858e+03,  2.0013443064949242491e+02, 1};
static const double P11[6] = {-2.2149374878243304548e+06,  7.1938920065420586101e+05,
                               1.7733324035147015630e+05,  7.1885382604084798576e+03,
                               9.9991373567429309922e+01,  4.8127070456878442310e-01};
static const double Q11[4] = {-2.2149374878243304548e+06,  3.7264298672067697862e+04,
                              -2.8143915754538725829e+02,  1};
static const double P12[5] = {-1.3531161492785421328e+06, -1.4758069205414222471e+05,
                              -4.5051623763436087023e+03, -5.3103913335180275253e+01,
                              -2.2795590826955002390e-01};
static const double Q12[4] = {-2.7062322985570842656e+06,  4.3117653211351080007e+04,
                              -3.0507151578787595807e+02,  1};
static const double P13[11] = { 2.2196792496874548962e+00,  4.4137176114230414036e+01,
                                3.4122953486801312910e+02,  1.3319486433183221990e+03,
                                2.8590657697910288226e+03,  3.4540675585544584407e+03,
                                2.3123742209168871550e+03,  8.1094256146537402173e+02,
                                1.3182609918569941308e+02,  7.5584584631176030810e+00,
                                6.4257745859173138767e-02};
static const double Q13[10] = { 1.7710478032601086579e+00,  3.4552228452758912848e+01,
                                2.5951223655579051357e+02,  9.6929165726802648634e+02,
                                1.9448440788918006154e+03,  2.1181000487171943810e+03,
                                1.2082692316002348638e+03,  3.3031020088765390854e+02,
                                3.6001069306861518855e+01,  1};
static const double XMAX = 700.0;   /* inc/besselk.h:182 */

static double polyval(int deg, const double *c, double x)
{ /* inc/polybesselk.h:8-15 (Horner from the top coefficient) */
	double v = c[deg];
	for (int i = deg - 1; i >= 0; --i) v = v * x + c[i];
	return v;
}

static double p0fcn(double x)
{ /* inc/polybesselk.h:17-54: x^2 K0(x) */
	if (x < DBL_EPSILON || x > XMAX) return 0.0;
	if (x <= 1.0) {
		double xs = x * x, lx = log(x);
		double PQ01 = polyval(5, P01, xs) / polyval(2, Q01, xs);
		double PQ02 = polyval(3, P02, xs) / polyval(3, Q02, xs);
		return xs * (PQ01 - lx * (xs * PQ02 + 1.0));
	}
	double xi = 1.0 / x;
	double PQ03 = polyval(9, P03, xi) / polyval(10, Q03, xi);
	return x * sqrt(x) * exp(-x) * PQ03;
}

static double p1fcn(double x)
{ /* inc/polybesselk.h:56-99: x K1(x) */
	if (x < DBL_EPSILON) return 1.0;
	if (x > XMAX) return 0.0;
	if (x <= 1.0) {
		double xs = x * x, lx = log(x);
		double PQ11 = polyval(5, P11, xs) / polyval(3, Q11, xs);
		double PQ12 = polyval(4, P12, xs) / polyval(3, Q12, xs);
		return PQ11 + xs * lx * PQ12;
	}
	double xi = 1.0 / x;
	double PQ13 = polyval(10, P13, xi) / polyval(9, Q13, xi);
	return sqrt(x) * exp(-x) * PQ13;
}
#endif

void orc_besselk(double x, double *f0, double *f1)
{
#if DIM == 2
	*f0 = p0fcn(x); *f1 = p1fcn(x);
#else
	(void) x; *f0 = 0.0; *f1 = 0.0;
#endif
}

static double kernel_value(int order, double w, vec qi, vec qj)
{
#if DIM == 2
	/* 2D/computeKernel.cu:30-168 */
	if (order == -1) {
		double dijSqu = vdist2(qi, qj) / (w * w);
		return exp(-dijSqu);
	}
	double dij = sqrt(vdist2(qi, qj)) / w;
	double dsq = dij * dij;
	double f0 = 0.0, f1 = p1fcn(dij);
	if (order > 0) f0 = p0fcn(dij);
	switch (order) {
	case 0: return f1;
	case 1: return 0.5 * (f0 + 2.0 * f1);
	case 2: return (4.0 * f0 + (8.0 + dsq) * f1) / 8.0;
	case 3: return ((24.0 + dsq) * f0 + 8.0 * (6.0 + dsq) * f1) / 48.0;
	case 4: return (12.0 * (16.0 + dsq) * f0 + (384.0 + dsq * (72.0 + dsq)) * f1) / 384.0;
	}
	return 0.0;
#else
	/* 3D/computeKernel.cu:5-113 */
	if (order == -1) {
		double dstSqu = vdist2(qi, qj);
		dstSqu /= w * w;
		return exp(-dstSqu);
	}
	double r = sqrt(vdist2(qi, qj));
	r /= w;
	switch (order) {
	case 0: return exp(-r);
	case 1: return (1.0 + r) * exp(-r);
	case 2: return (3.0 + r * (3.0 + r)) / 3.0 * exp(-r);
	case 3: return (15.0 + r * (15.0 + r * (6.0 + r))) / 15.0 * exp(-r);
	case 4: return (105.0 + r * (105.0 + r * (45.0 + r * (10.0 + r)))) / 105.0 * exp(-r);
	}
	return 0.0;
#endif
}

void orc_kernel_matrix(const orc_problem *P, const double *lmk, double *K)
{
	int N = P->lmkNum;
	#pragma omp parallel for schedule(static)
	for (int j = 0; j < N; ++j) {
		vec qj = getv(lmk, j, N);
		for (int i = 0; i < N; ++i)
			K[(size_t) j * N + i] = kernel_value(P->knlOrder, P->knlWidth, getv(lmk, i, N), qj);
	}
}

/* ------------------------------------------------------------------ */
/* solver state                                                        */
/* ------------------------------------------------------------------ */
typedef struct {
	const orc_problem *P;
	double *edg, *frmA, *tsv;   /* geometry at the current time */
	double *lmk;                /* current node positions */
	double *elYElm, *elY, *pnl;
	double *knlMat, *knLMat;    /* frame K-PCG */
	double *diag;               /* isotropic: inverse node blocks (block-Jacobi) */
} vstate;

/* y = E x + btmWgt P x */
static void second_mult(vstate *S, const double *x, double *y)
{ /* 2D/ipcgSecondMatrixMultiplication.cu:8-24 */
	const orc_problem *P = S->P;
	long n = (long) P->lmkNum * DIM;
	elastic_apply(P, S->edg, S->frmA, S->tsv, x, S->elYElm, S->elY);
	penalty_apply(P, S->lmk, x, S->pnl);
	axpby(y, 1.0, S->elY, P->btmWgt, S->pnl, n);
}

/* KX = K X (cublasDgemm N x N times N x D, 2D/ipcgKernelMultiplication.cu:5-17) */
static void kernel_mult(vstate *S, const double *X, double *KX)
{
	int N = S->P->lmkNum;
	for (int d = 0; d < DIM; ++d)
		gemv(N, 1.0, S->knlMat, X + (size_t) d * N, 0.0, KX + (size_t) d * N);
}

/* K-preconditioned CG: 2D/ipcg.cu:11-100 */
static int ipcg(vstate *S, double *x, const double *b, int *itrOut)
{
	const orc_problem *P = S->P;
	int N = P->lmkNum; long n = (long) N * DIM;
	double *Ad = malloc(sizeof(double) * n), *Bd = malloc(sizeof(double) * n);
	double *Kid = malloc(sizeof(double) * n), *r = malloc(sizeof(double) * n);
	double *Kr = malloc(sizeof(double) * n), *dv = malloc(sizeof(double) * n);
	int status = 1, itr = 0;
	double bSqu = ddot(b, b, n);
	if (bSqu == 0.0) { memset(x, 0, sizeof(double) * n); status = 0; goto done; }
	double relTolSqu = bSqu * P->cgTolSqu;
	/* ipcgWholeMatrixMultiplication 2D/ipcgWholeMatrixMultiplication.cu:21-45 */
	{
		double *Kiv = malloc(sizeof(double) * n);
		memcpy(Kiv, x, sizeof(double) * n);
		for (int d = 0; d < DIM; ++d) potrs_lower(S->knLMat, N, Kiv + (size_t) d * N);
		elastic_apply(P, S->edg, S->frmA, S->tsv, x, S->elYElm, S->elY);
		penalty_apply(P, S->lmk, x, S->pnl);
		for (long i = 0; i < n; ++i) Ad[i] = P->ldmWgt * Kiv[i] + S->elY[i] + P->btmWgt * S->pnl[i];
		free(Kiv);
	}
	axpby(r, 1.0, b, -1.0, Ad, n);
	double rSquNow = ddot(r, r, n);
	if (rSquNow < relTolSqu) { status = 0; goto done; }
	memcpy(Kid, r, sizeof(double) * n);
	kernel_mult(S, r, Kr);
	memcpy(dv, Kr, sizeof(double) * n);
	double rKrNow = ddot(r, Kr, n);
	if (rKrNow == 0.0) goto done;
	for (itr = 0; itr < P->cgItrMax; ++itr) {
		second_mult(S, dv, Bd);
		axpby(Ad, P->ldmWgt, Kid, 1.0, Bd, n);
		double dAd = ddot(dv, Ad, n);
		if (dAd == 0.0) goto done;
		double xStp = rKrNow / dAd;
		axpby(x, 1.0, x, xStp, dv, n);
		axpby(r, 1.0, r, -xStp, Ad, n);
		double rSquNxt = ddot(r, r, n);
		if (rSquNxt < relTolSqu) { status = 0; ++itr; goto done; }
		kernel_mult(S, r, Kr);
		double rKrNxt = ddot(r, Kr, n);
		if (rKrNxt == 0.0) goto done;
		double dStp = rKrNxt / rKrNow;
		axpby(Kid, 1.0, r, dStp, Kid, n);
		axpby(dv, 1.0, Kr, dStp, dv, n);
		rSquNow = rSquNxt;
		rKrNow = rKrNxt;
	}
done:
	if (itrOut) *itrOut = itr;
	free(Ad); free(Bd); free(Kid); free(r); free(Kr); free(dv);
	return status;
}

/* Jacobi-PCG (layered model): same stopping rule as the reference's ipcg
 * (|r|^2 < tol^2 |b|^2, b = 0 gives x = 0).  The preconditioner is block-Jacobi
 * over node blocks of bdim components: pinv holds the inverse of every node's
 * bdim x bdim diagonal block of the operator, entry (a, c) of node i at
 * pinv[(a * bdim + c) * N + i] (bdim = 1: the inverse diagonal, point Jacobi). */
typedef void (*apply_fn)(void *ctx, const double *x, double *y);
static void prec_apply(const double *pinv, int N, int bdim, const double *r, double *z)
{
	#pragma omp parallel for schedule(static)
	for (int i = 0; i < N; ++i)
		for (int a = 0; a < bdim; ++a) {
			double t = pinv[(size_t) (a * bdim) * N + i] * r[i];
			for (int c = 1; c < bdim; ++c) t += pinv[(size_t) (a * bdim + c) * N + i] * r[(size_t) c * N + i];
			z[(size_t) a * N + i] = t;
		}
}

static int jpcg(apply_fn A, void *ctx, const double *pinv, int N, int bdim, double *x, const double *b,
                int itrMax, double tolSqu, int *itrOut)
{
	long n = (long) N * bdim;
	double *r = malloc(sizeof(double) * n), *z = malloc(sizeof(double) * n);
	double *p = malloc(sizeof(double) * n), *q = malloc(sizeof(double) * n);
	int status = 1, itr = 0;
	double bSqu = ddot(b, b, n);
	if (bSqu == 0.0) { memset(x, 0, sizeof(double) * n); status = 0; goto done; }
	double relTolSqu = bSqu * tolSqu;
	A(ctx, x, q);
	for (long i = 0; i < n; ++i) r[i] = b[i] - q[i];
	double rr = ddot(r, r, n);
	if (rr < relTolSqu) { status = 0; goto done; }
	prec_apply(pinv, N, bdim, r, z);
	for (long i = 0; i < n; ++i) p[i] = z[i];
	double rz = ddot(r, z, n);
	for (itr = 0; itr < itrMax; ++itr) {
		A(ctx, p, q);
		double pq = ddot(p, q, n);
		if (!(pq > 0.0)) goto done;
		double alpha = rz / pq;
		for (long i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
		rr = ddot(r, r, n);
		if (rr < relTolSqu) { status = 0; ++itr; goto done; }
		prec_apply(pinv, N, bdim, r, z);
		double rzn = ddot(r, z, n);
		double beta = rzn / rz;
		for (long i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
		rz = rzn;
	}
done:
	if (itrOut) *itrOut = itr;
	free(r); free(z); free(p); free(q);
	return status;
}

static void velocity_apply(void *ctx, const double *x, double *y) { second_mult((vstate *) ctx, x, y); }

/* node blocks of E + btmWgt P for the layered model: entry (r, c) of node i's
 * DIM x DIM diagonal block at blk[(r * DIM + c) * N + i].  Element e adds
 * vol ((lam + mu) g_k g_k^T + mu |g_k|^2 I) to its vertex k (g_k the P1 shape
 * gradient, the a = b term of the element stiffness); the bottom penalty is a
 * scalar per node (P applied to the all-ones field) on the block's diagonal. */
static void elastic_blocks_state(const orc_problem *P, const double *lmk, const double *edg, double *blk)
{
	int N = P->lmkNum, E = P->elmNum;
	const int DD = DIM * DIM;
	double *bElm = malloc(sizeof(double) * (size_t) E * VTX * DD);
	#pragma omp parallel for schedule(static)
	for (int e = 0; e < E; ++e) {
		vec q[DIM]; get_edges(edg, e, E, q);
		double volVal = elm_volume(detQ(q));
		mat QI = invQ(q);
		int l = P->elmLyrVec[e];
		double lam = P->modVec[2 * l], mu = P->modVec[2 * l + 1];
		double G[VTX][DIM];
		for (int d = 0; d < DIM; ++d) {
			double s = -QI.m[0][d];
			for (int a = 1; a < DIM; ++a) s = s - QI.m[a][d];
			G[0][d] = s;
			for (int a = 0; a < DIM; ++a) G[a + 1][d] = QI.m[a][d];
		}
		for (int k = 0; k < VTX; ++k) {
			double g2 = G[k][0] * G[k][0];
			for (int d = 1; d < DIM; ++d) g2 = g2 + G[k][d] * G[k][d];
			for (int r = 0; r < DIM; ++r)
				for (int c = 0; c < DIM; ++c)
					bElm[(size_t) (k * DD + r * DIM + c) * E + e] =
						volVal * ((lam + mu) * G[k][r] * G[k][c] + (r == c ? mu * g2 : 0.0));
		}
	}
	const int *ve = P->vtxElmMat;
	#pragma omp parallel for schedule(static)
	for (int i = 0; i < N; ++i) {
		double s[DIM * DIM]; for (int d = 0; d < DD; ++d) s[d] = 0.0;
		int adjNum = ve[i];
		for (int a = 0; a < adjNum; ++a) {
			int e = ve[(1 + 2 * a) * N + i], l = ve[(2 + 2 * a) * N + i];
			for (int d = 0; d < DD; ++d) s[d] += bElm[(size_t) (l * DD + d) * E + e];
		}
		for (int d = 0; d < DD; ++d) blk[(size_t) d * N + i] = s[d];
	}
	free(bElm);
	if (P->btmWgt != 0.0) {
		double *one = malloc(sizeof(double) * (size_t) N * DIM), *pd = malloc(sizeof(double) * (size_t) N * DIM);
		for (long i = 0; i < (long) N * DIM; ++i) one[i] = 1.0;
		penalty_apply(P, lmk, one, pd);
		for (int i = 0; i < N; ++i)
			for (int d = 0; d < DIM; ++d) blk[(size_t) (d * DIM + d) * N + i] += P->btmWgt * pd[(size_t) d * N + i];
		free(one); free(pd);
	}
}

/* in place: every node block replaced by its inverse (cofactors over the determinant) */
static void invert_node_blocks(double *blk, int N)
{
	#pragma omp parallel for schedule(static)
	for (int i = 0; i < N; ++i) {
		double a[DIM][DIM], v[DIM][DIM];
		for (int r = 0; r < DIM; ++r)
			for (int c = 0; c < DIM; ++c) a[r][c] = blk[(size_t) (r * DIM + c) * N + i];
#if DIM == 2
		double det = a[0][0] * a[1][1] - a[0][1] * a[1][0];
		v[0][0] = a[1][1] / det; v[0][1] = -a[0][1] / det;
		v[1][0] = -a[1][0] / det; v[1][1] = a[0][0] / det;
#else
		for (int r = 0; r < 3; ++r)
			for (int c = 0; c < 3; ++c) {
				/* cofactor of a[c][r] (the adjugate is the transposed cofactor matrix) */
				int r0 = (c + 1) % 3, r1 = (c + 2) % 3, c0 = (r + 1) % 3, c1 = (r + 2) % 3;
				v[r][c] = a[r0][c0] * a[r1][c1] - a[r0][c1] * a[r1][c0];
			}
		double det = a[0][0] * v[0][0] + a[0][1] * v[1][0] + a[0][2] * v[2][0];
		for (int r = 0; r < 3; ++r)
			for (int c = 0; c < 3; ++c) v[r][c] = v[r][c] / det;
#endif
		for (int r = 0; r < DIM; ++r)
			for (int c = 0; c < DIM; ++c) blk[(size_t) (r * DIM + c) * N + i] = v[r][c];
	}
}

/* node blocks (blk[(r * DIM + c) * N + i]) and, with inverse != 0, their inverses: the
 * block-Jacobi preconditioner of the layered velocity solve */
void orc_elastic_blocks(const orc_problem *P, const double *lmk, int inverse, double *blk)
{
	int E = P->elmNum;
	if (P->elaType == ORC_FRAME || !P->elmLyrVec) {     /* layered model only: zeros otherwise */
		memset(blk, 0, sizeof(double) * (size_t) P->lmkNum * DIM * DIM);
		return;
	}
	double *edg = malloc(sizeof(double) * (size_t) E * DIM * DIM);
	orc_edges(P, lmk, edg);
	elastic_blocks_state(P, lmk, edg, blk);
	if (inverse) invert_node_blocks(blk, P->lmkNum);
	free(edg);
}

void orc_elastic_diag(const orc_problem *P, const double *lmk, double *diag)
{
	int E = P->elmNum;
	int N = P->lmkNum;
	double *edg = malloc(sizeof(double) * (size_t) E * DIM * DIM);
	double *blk = malloc(sizeof(double) * (size_t) N * DIM * DIM);
	orc_edges(P, lmk, edg);
	elastic_blocks_state(P, lmk, edg, blk);
	for (int d = 0; d < DIM; ++d)
		memcpy(diag + (size_t) d * N, blk + (size_t) (d * DIM + d) * N, sizeof(double) * N);
	free(edg); free(blk);
}

/* CSR matrix apply for the reaction-diffusion system */
typedef struct { const orc_problem *P; const double *val; } csrctx;
static void csr_apply(void *ctx, const double *x, double *y)
{
	csrctx *C = (csrctx *) ctx;
	const orc_problem *P = C->P;
	int N = P->lmkNum, Z = P->nzrNum;
	const int *fv = P->femVtxMat;
	for (int i = 0; i < N; ++i) y[i] = 0.0;
	/* femVtxMat is sorted by (row, col): accumulate row by row in column order */
	for (int z = 0; z < Z; ++z) y[fv[z]] += C->val[z] * x[fv[Z + z]];
}

/* ------------------------------------------------------------------ */
/* operator-level exports                                              */
/* ------------------------------------------------------------------ */
void orc_elastic_apply(const orc_problem *P, const double *lmk, const double *v, double *y)
{
	int E = P->elmNum;
	double *edg = malloc(sizeof(double) * (size_t) E * DIM * DIM);
	double *frmA = malloc(sizeof(double) * (size_t) E * DIM), *tsv = malloc(sizeof(double) * (size_t) E * DIM);
	double *elYElm = malloc(sizeof(double) * (size_t) E * DIM * VTX);
	orc_edges(P, lmk, edg);
	if (P->elaType == ORC_FRAME) orc_frame(P, lmk, frmA, tsv);
	elastic_apply(P, edg, frmA, tsv, v, elYElm, y);
	free(edg); free(frmA); free(tsv); free(elYElm);
}

void orc_penalty_apply(const orc_problem *P, const double *lmk, const double *v, double *y)
{ penalty_apply(P, lmk, v, y); }

void orc_yank(const orc_problem *P, const double *lmk, const double *tau, double *b)
{
	int E = P->elmNum, N = P->lmkNum;
	double *edg = malloc(sizeof(double) * (size_t) E * DIM * DIM);
	double *f = malloc(sizeof(double) * N), *ex = malloc(sizeof(double) * (size_t) E * DIM * VTX);
	orc_edges(P, lmk, edg);
	orc_yank_activity(P, tau, f, N);
	yank_apply(P, edg, f, ex, b);
	free(edg); free(f); free(ex);
}

void orc_reaction_load(const orc_problem *P, const double *lmk, const double *tau, double *r)
{
	int E = P->elmNum, N = P->lmkNum;
	double *edg = malloc(sizeof(double) * (size_t) E * DIM * DIM);
	double *f = malloc(sizeof(double) * N), *re = malloc(sizeof(double) * (size_t) E * VTX);
	orc_edges(P, lmk, edg);
	orc_reaction_activity(P, tau, f, N);
	fem_vector(P, edg, f, re, r);
	free(edg); free(f); free(re);
}

/* ------------------------------------------------------------------ */
/* varifold (2D/varifold.cu, 3D/varifold.cu)                           */
/* ------------------------------------------------------------------ */
static double geo_fun(char type, double w, vec c1, vec c2, vec *d1K)
{ /* geometricFunction: 2D/varifold.cu:38-88 ('M' is the layered model's Matern-3/2) */
	double dstSqu = vdist2(c1, c2), k = 0.0, d1 = 0.0;
	if (type == 'G') { k = exp(-dstSqu / (w * w)); d1 = -2.0 * k / (w * w); }
	else if (type == 'C') { k = 1.0 / (1.0 + dstSqu / (w * w)); d1 = -2.0 * k * k / (w * w); }
	else if (type == 'M') {
		double r = sqrt(dstSqu) / w;
		double ex = exp(-r);
		k = (1.0 + r) * ex;
		d1 = -ex / (w * w);          /* d/dc1 (1+r)e^{-r} = -(r e^{-r}) (c1-c2)/(r w^2) */
	}
	if (d1K) for (int d = 0; d < DIM; ++d) d1K->c[d] = d1 * (c1.c[d] - c2.c[d]);
	return k;
}

static double grass_fun(char type, double w, vec v1, vec v2, double v1Vol, vec *d1K)
{ /* grassmanFunction: 2D/varifold.cu:90-179 (v1Vol is n1Len in 3D) */
	double ang = vdot(v1, v2), k = 0.0, d1 = 0.0;
	if (type == 'B') { k = ang * ang; d1 = 2.0 * ang; }
	else if (type == 'L') { k = ang; d1 = 1.0; }
	else if (type == 'O') { k = exp(2.0 * (ang - 1.0) / (w * w)); d1 = 2.0 * k / (w * w); }
	else if (type == 'U') { k = exp(2.0 * (ang * ang - 1.0) / (w * w)); d1 = 4.0 * ang * k / (w * w); }
	if (d1K) for (int d = 0; d < DIM; ++d) d1K->c[d] = d1 / v1Vol * (-ang * v1.c[d] + v2.c[d]);
	return k;
}

double orc_varifold(const orc_problem *P, const double *lmk, double *grad)
{
	int N = P->lmkNum, Nd = P->vfdElmNum, Nt = P->tgtElmNum;
	char ck = P->cenKnlType, dk = P->dirKnlType;
	double cw = P->cenKnlWidth, dw = P->dirKnlWidth;
	double *cen = malloc(sizeof(double) * (size_t) Nd * DIM), *dir = malloc(sizeof(double) * (size_t) Nd * DIM);
	double *vol = malloc(sizeof(double) * Nd), *vfd = malloc(sizeof(double) * (size_t) (Nd + Nt));
	double *dc = grad ? malloc(sizeof(double) * (size_t) Nd * DIM) : NULL;
	double *dt = grad ? malloc(sizeof(double) * (size_t) Nd * DIM) : NULL;
	const double *tc = P->tgtCenPosMat, *tu = P->tgtUniDirMat, *tv = P->tgtElmVolVec;
	/* landmarksToVarifoldKernel 2D :9-36, 3D :9-43 */
	for (int e = 0; e < Nd; ++e) {
		vec q0 = getv(lmk, P->vfdVtxMat[e], N), q1 = getv(lmk, P->vfdVtxMat[Nd + e], N);
		vec c, u; double v;
#if DIM == 2
		for (int d = 0; d < 2; ++d) c.c[d] = 0.5 * (q0.c[d] + q1.c[d]);
		u = vsub(q1, q0);
		v = vnorm(u);
		for (int d = 0; d < 2; ++d) u.c[d] /= v;
		vol[e] = v;
#else
		vec q2 = getv(lmk, P->vfdVtxMat[2 * Nd + e], N);
		for (int d = 0; d < 3; ++d) c.c[d] = (q0.c[d] + q1.c[d] + q2.c[d]) / 3.0;
		u = vcross(vsub(q1, q0), vsub(q2, q0));
		v = vnorm(u);
		for (int d = 0; d < 3; ++d) u.c[d] /= v;
		vol[e] = 0.5 * v;
#endif
		setv(cen, c, e, Nd); setv(dir, u, e, Nd);
	}
	int ddFirst = (grad != NULL) || (Nd >= Nt);
	/* rows over deformed elements: DD - 2 DT (vfd_DD_DT_Kernel :181-239 / dqVfd_DD_DT_Kernel :359-433) */
	#pragma omp parallel for schedule(dynamic, 16)
	for (int i = 0; i < Nd; ++i) {
		vec ci = getv(cen, i, Nd), ui = getv(dir, i, Nd);
		double vi = vol[i], s = 0.0;
		vec dci, dti;
		for (int d = 0; d < DIM; ++d) { dci.c[d] = 0.0; dti.c[d] = 0.0; }
#if DIM == 2
		double nLen = vi;
		double half = 1.0;
#else
		double nLen = 2.0 * vi;
		double half = 0.5;
#endif
		for (int j = 0; j < Nd; ++j) {
			vec dK, tK;
			double ckv = geo_fun(ck, cw, ci, getv(cen, j, Nd), grad ? &dK : NULL);
			double dkv = grass_fun(dk, dw, ui, getv(dir, j, Nd), nLen, grad ? &tK : NULL);
			s += ckv * dkv * vi * vol[j];
			if (grad) for (int d = 0; d < DIM; ++d) {
				dci.c[d] += 2.0 * dK.c[d] * dkv * vi * vol[j];
				dti.c[d] += 2.0 * ckv * (tK.c[d] * vi + dkv * half * ui.c[d]) * vol[j];
			}
		}
		for (int j = 0; j < Nt; ++j) {
			vec dK, tK;
			double ckv = geo_fun(ck, cw, ci, getv(tc, j, Nt), grad ? &dK : NULL);
			double dkv = grass_fun(dk, dw, ui, getv(tu, j, Nt), nLen, grad ? &tK : NULL);
			s -= 2.0 * ckv * dkv * vi * tv[j];
			if (grad) for (int d = 0; d < DIM; ++d) {
				dci.c[d] -= 2.0 * dK.c[d] * dkv * vi * tv[j];
				dti.c[d] -= 2.0 * ckv * (tK.c[d] * vi + dkv * half * ui.c[d]) * tv[j];
			}
		}
		if (ddFirst) vfd[i] = s; else vfd[Nt + i] = s;
		if (grad) { setv(dc, dci, i, Nd); setv(dt, dti, i, Nd); }
	}
	if (!ddFirst) {
		/* vfd_TT_TD_Kernel :270-327 (DD rows then only carry DD; recompute) */
		#pragma omp parallel for schedule(dynamic, 16)
		for (int i = 0; i < Nd; ++i) {
			vec ci = getv(cen, i, Nd), ui = getv(dir, i, Nd);
			double vi = vol[i], s = 0.0;
			for (int j = 0; j < Nd; ++j)
				s += geo_fun(ck, cw, ci, getv(cen, j, Nd), NULL) * grass_fun(dk, dw, ui, getv(dir, j, Nd), 1.0, NULL)
				     * vi * vol[j];
			vfd[Nt + i] = s;   /* vfd_DD_Kernel :329-357 */
		}
	}
	/* target rows: TT (vfd_TT_Kernel :241-268) or TT - 2 TD */
	#pragma omp parallel for schedule(dynamic, 16)
	for (int i = 0; i < Nt; ++i) {
		vec ci = getv(tc, i, Nt), ui = getv(tu, i, Nt);
		double vi = tv[i], s = 0.0;
		for (int j = 0; j < Nt; ++j)
			s += geo_fun(ck, cw, ci, getv(tc, j, Nt), NULL) * grass_fun(dk, dw, ui, getv(tu, j, Nt), 1.0, NULL)
			     * vi * tv[j];
		if (!ddFirst)
			for (int j = 0; j < Nd; ++j)
				s -= 2.0 * geo_fun(ck, cw, ci, getv(cen, j, Nd), NULL)
				         * grass_fun(dk, dw, ui, getv(dir, j, Nd), 1.0, NULL) * vi * vol[j];
		if (ddFirst) vfd[Nd + i] = s; else vfd[i] = s;
	}
	double obj = orc_dsum(vfd, Nd + Nt);
	if (grad) {
		/* dqVfdGatherKernel 2D :435-466, 3D :492-528 */
		const int *gi = P->vfdIfoMat;
		int C = P->vfdIfoCols;
		(void) C;
		for (int i = 0; i < N; ++i) {
			double s[DIM]; for (int d = 0; d < DIM; ++d) s[d] = 0.0;
			int adjNum = gi[i];
			for (int a = 0; a < adjNum; ++a) {
#if DIM == 2
				int e = gi[(1 + 2 * a) * N + i], sg = gi[(2 + 2 * a) * N + i];
				vec c = getv(dc, e, Nd), t = getv(dt, e, Nd);
				for (int d = 0; d < 2; ++d) s[d] += 0.5 * c.c[d] + sg * t.c[d];
#else
				int e = gi[(1 + 3 * a) * N + i], qa = gi[(2 + 3 * a) * N + i], qb = gi[(3 + 3 * a) * N + i];
				vec c = getv(dc, e, Nd), t = getv(dt, e, Nd);
				vec ab = vsub(getv(lmk, qa, N), getv(lmk, qb, N));
				vec x = vcross(t, ab);
				for (int d = 0; d < 3; ++d) s[d] += c.c[d] / 3.0 + x.c[d];
#endif
			}
			for (int d = 0; d < DIM; ++d) grad[d * N + i] = s[d];
		}
	}
	free(cen); free(dir); free(vol); free(vfd);
	if (dc) free(dc);
	if (dt) free(dt);
	return obj;
}

/* ------------------------------------------------------------------ */
/* forward model: 2D/deform.cu:22-119, 2D/objfcn.cu:23-123             */
/* ------------------------------------------------------------------ */
int orc_forward(const orc_problem *P, const double *tauVarVec,
                double *lmkStk, double *tauMat, double *objPtr, int *cgItr)
{
	return orc_forward_timed(P, tauVarVec, lmkStk, tauMat, objPtr, cgItr, NULL);
}

int orc_forward_timed(const orc_problem *P, const double *tauVarVec, double *lmkStk, double *tauMat,
                      double *objPtr, int *cgItr, double *stepSec)
{
	int N = P->lmkNum, E = P->elmNum, Z = P->nzrNum, T = P->timeNum;
	long nd = (long) N * DIM;
	double dt = P->timeStp;
	int frame = (P->elaType == ORC_FRAME);
	/* frame mode always runs the reference's K-preconditioned CG; the
	 * layered model uses it only when the LDDMM term is switched on */
	int useK = frame || (P->ldmWgt != 0.0);
	int status = 0;

	double *edgNow = malloc(sizeof(double) * (size_t) E * DIM * DIM);
	double *edgNxt = malloc(sizeof(double) * (size_t) E * DIM * DIM);
	double *frmNow = malloc(sizeof(double) * (size_t) E * DIM), *frmNxt = malloc(sizeof(double) * (size_t) E * DIM);
	double *tsvNow = malloc(sizeof(double) * (size_t) E * DIM), *tsvNxt = malloc(sizeof(double) * (size_t) E * DIM);
	double *ppdElm = malloc(sizeof(double) * E), *ggdElm = malloc(sizeof(double) * (size_t) E * NPAIR);
	double *ynk = malloc(sizeof(double) * N), *rea = malloc(sizeof(double) * N);
	double *exY = malloc(sizeof(double) * nd), *exYElm = malloc(sizeof(double) * (size_t) E * DIM * VTX);
	double *rpdElm = malloc(sizeof(double) * (size_t) E * VTX), *rpd = malloc(sizeof(double) * N);
	double *vlc = calloc((size_t) nd, sizeof(double));
	double *vlcHist = calloc((size_t) nd * 5, sizeof(double));     /* up to 5 earlier velocities */
	vstate S; memset(&S, 0, sizeof(S));
	S.P = P;
	S.elYElm = malloc(sizeof(double) * (size_t) E * DIM * VTX);
	S.elY = malloc(sizeof(double) * nd); S.pnl = calloc((size_t) nd, sizeof(double));
	/* dense matrices (frame mode, as the reference) or CSR values (layered) */
	double *ppdNow = NULL, *ppdNxt = NULL, *ggdNxt = NULL, *femLft = NULL;
	double *ppdValNow = NULL, *ppdValNxt = NULL, *ggdValNxt = NULL, *lftVal = NULL;
	if (frame) {
		size_t nn = (size_t) N * N;
		ppdNow = malloc(sizeof(double) * nn); ppdNxt = malloc(sizeof(double) * nn);
		ggdNxt = malloc(sizeof(double) * nn); femLft = malloc(sizeof(double) * nn);
	} else {
		ppdValNow = malloc(sizeof(double) * Z); ppdValNxt = malloc(sizeof(double) * Z);
		ggdValNxt = malloc(sizeof(double) * Z); lftVal = malloc(sizeof(double) * Z);
		S.diag = malloc(sizeof(double) * nd * DIM);
	}
	if (useK) {
		S.knlMat = malloc(sizeof(double) * (size_t) N * N);
		S.knLMat = malloc(sizeof(double) * (size_t) N * N);
	}
	const int *fv = P->femVtxMat;

	memcpy(lmkStk, P->lmkIniMat, sizeof(double) * nd);
	orc_initial_tau(P, tauVarVec, tauMat);
	orc_edges(P, P->lmkIniMat, edgNow);
	if (frame) orc_frame(P, P->lmkIniMat, frmNow, tsvNow);
	fem_elements(P, edgNow, frmNow, tsvNow, ppdElm, ggdElm);
	if (frame) memset(ppdNow, 0, sizeof(double) * (size_t) N * N);
	{
		/* the initial diffusion matrix (2D/deform.cu:41-42) is never used */
		double *pv = malloc(sizeof(double) * Z), *gv = malloc(sizeof(double) * Z);
		fem_gather_csr(P, ppdElm, ggdElm, pv, gv);
		if (frame) for (int z = 0; z < Z; ++z) ppdNow[(size_t) fv[Z + z] * N + fv[z]] = pv[z];
		else memcpy(ppdValNow, pv, sizeof(double) * Z);
		free(pv); free(gv);
	}

	for (int t = 0; t < T - 1; ++t) {
		double tStep = omp_get_wtime();
		double *lmkNow = lmkStk + (size_t) t * nd, *lmkNxt = lmkStk + (size_t) (t + 1) * nd;
		double *tauNow = tauMat + (size_t) t * N, *tauNxt = tauMat + (size_t) (t + 1) * N;
		S.lmk = lmkNow; S.edg = edgNow; S.frmA = frmNow; S.tsv = tsvNow;

		orc_yank_activity(P, tauNow, ynk, N);
		orc_reaction_activity(P, tauNow, rea, N);
		if (useK) {
			orc_kernel_matrix(P, lmkNow, S.knlMat);
			for (int i = 0; i < N; ++i) S.knlMat[(size_t) i * N + i] += P->knlEps;   /* 2D/addEpsIdentity.cu */
			memcpy(S.knLMat, S.knlMat, sizeof(double) * (size_t) N * N);
			potrf_lower(S.knLMat, N);
		}
		yank_apply(P, edgNow, ynk, exYElm, exY);

		int itr = 0, st;
		if (!useK && !frame && P->velocityGuess > 0) {
			/* layered model: start from the degree-q polynomial through the last q + 1 velocities,
			 * evaluated one step ahead, q = min(velocityGuess, t - 1); then shift the history */
			static const double cb[6][6] = {{1, 0, 0, 0, 0, 0}, {2, -1, 0, 0, 0, 0}, {3, -3, 1, 0, 0, 0},
			                                {4, -6, 4, -1, 0, 0}, {5, -10, 10, -5, 1, 0}, {6, -15, 20, -15, 6, -1}};
			const int depth = P->velocityGuess < 5 ? P->velocityGuess : 5;
			int q = t - 1 < depth ? t - 1 : depth;
			if (q < 0) q = 0;
			for (long i = 0; i < nd; ++i) {
				double h[6];
				h[0] = vlc[i];
				for (int j = 1; j <= depth; ++j) h[j] = vlcHist[(size_t) (j - 1) * nd + i];
				if (q > 0) {
					double s = 0.0;
					for (int j = 0; j <= q; ++j) s += cb[q][j] * h[j];
					vlc[i] = s;
				}
				for (int j = depth - 1; j >= 1; --j) vlcHist[(size_t) j * nd + i] = h[j];
				vlcHist[i] = h[0];
			}
		}
		if (useK) st = ipcg(&S, vlc, exY, &itr);
		else {
			/* block-Jacobi over the DIM x DIM node blocks */
			elastic_blocks_state(P, lmkNow, edgNow, S.diag);
			invert_node_blocks(S.diag, N);
			st = jpcg(velocity_apply, &S, S.diag, N, DIM, vlc, exY, P->cgItrMax, P->cgTolSqu, &itr);
		}
		if (cgItr) cgItr[t] = itr;
		if (st != 0) { status = 1; break; }

		/* x_{t+1} = x_t + dt v_t (2D/deform.cu:81-82); v_t warm-starts the next solve */
		axpby(lmkNxt, 1.0, lmkNow, dt, vlc, nd);

		orc_edges(P, lmkNxt, edgNxt);
		if (frame) orc_frame(P, lmkNxt, frmNxt, tsvNxt);
		fem_elements(P, edgNxt, frmNxt, tsvNxt, ppdElm, ggdElm);
		double *pv = malloc(sizeof(double) * Z), *gv = malloc(sizeof(double) * Z);
		fem_gather_csr(P, ppdElm, ggdElm, pv, gv);
		/* reaction load on the current geometry (2D/deform.cu:89) */
		fem_vector(P, edgNow, rea, rpdElm, rpd);
		if (frame) {
			size_t nn = (size_t) N * N;
			memset(ppdNxt, 0, sizeof(double) * nn); memset(ggdNxt, 0, sizeof(double) * nn);
			for (int z = 0; z < Z; ++z) {
				size_t o = (size_t) fv[Z + z] * N + fv[z];
				ppdNxt[o] = pv[z]; ggdNxt[o] = gv[z];
			}
			/* 2D/deform.cu:91-104: (M' + dt G') tau' = M tau + dt rpd, dense Cholesky */
			axpby(femLft, 1.0, ppdNxt, dt, ggdNxt, (long) nn);
			gemv(N, 1.0, ppdNow, tauNow, dt, rpd);
			potrf_lower(femLft, N);
			memcpy(tauNxt, rpd, sizeof(double) * N);
			potrs_lower(femLft, N, tauNxt);
			double *sw = ppdNow; ppdNow = ppdNxt; ppdNxt = sw;
		} else {
			memcpy(ppdValNxt, pv, sizeof(double) * Z); memcpy(ggdValNxt, gv, sizeof(double) * Z);
			for (int z = 0; z < Z; ++z) lftVal[z] = 1.0 * ppdValNxt[z] + dt * ggdValNxt[z];
			/* rhs = M_t tau_t + dt rpd */
			double *Mt = malloc(sizeof(double) * N);
			csrctx C0 = { P, ppdValNow };
			csr_apply(&C0, tauNow, Mt);
			for (int i = 0; i < N; ++i) rpd[i] = 1.0 * Mt[i] + dt * rpd[i];
			free(Mt);
			double *dinv = malloc(sizeof(double) * N);
			for (int z = 0; z < Z; ++z) if (fv[z] == fv[Z + z]) dinv[fv[z]] = 1.0 / lftVal[z];
			if (P->velocityGuess != 0 && t >= 1)       /* extrapolated start: 2 tau_t - tau_t-1 */
				for (int i = 0; i < N; ++i) tauNxt[i] = 2.0 * tauNow[i] - tauNow[i - N];
			else
				memcpy(tauNxt, tauNow, sizeof(double) * N);   /* warm start */
			csrctx C1 = { P, lftVal };
			int rdItr = 0;
			if (jpcg(csr_apply, &C1, dinv, N, 1, tauNxt, rpd, P->rdItrMax, P->rdTolSqu, &rdItr) != 0) {
				free(dinv); free(pv); free(gv); status = 1; break;
			}
			free(dinv);
			double *sw = ppdValNow; ppdValNow = ppdValNxt; ppdValNxt = sw;
		}
		free(pv); free(gv);
		double *sw;
		sw = edgNow; edgNow = edgNxt; edgNxt = sw;
		sw = frmNow; frmNow = frmNxt; frmNxt = sw;
		sw = tsvNow; tsvNow = tsvNxt; tsvNxt = sw;
		if (stepSec) stepSec[t] = omp_get_wtime() - tStep;
	}

	if (objPtr) {
		if (status != 0) *objPtr = DBL_MAX;
		else *objPtr = orc_varifold(P, lmkStk + (size_t) (T - 1) * nd, NULL);
	}

	free(edgNow); free(edgNxt); free(frmNow); free(frmNxt); free(tsvNow); free(tsvNxt);
	free(ppdElm); free(ggdElm); free(ynk); free(rea); free(exY); free(exYElm);
	free(rpdElm); free(rpd); free(vlc); free(vlcHist); free(S.elYElm); free(S.elY); free(S.pnl);
	free(ppdNow); free(ppdNxt); free(ggdNxt); free(femLft);
	free(ppdValNow); free(ppdValNxt); free(ggdValNxt); free(lftVal); free(S.diag);
	free(S.knlMat); free(S.knLMat);
	return status;
}
