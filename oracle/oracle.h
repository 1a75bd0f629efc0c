/*
 * oracle.h -- CPU oracle for the shape_atrophy forward model and objective.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product (shape_atrophy_gb300) never links or calls it.
 *
 * It is a plain-C FP64 restatement of the reference's algorithm, compiled
 * once per dimension (-DDIM=2 / -DDIM=3) exactly as the reference builds
 * its 2D_frame / 3D_frame trees with -DDIM2 / -DDIM3.  Every routine cites
 * the reference file:line it follows (paths relative to the reference's
 * CUDA/ folder).  Frame mode follows the reference operation by operation
 * (dense N x N mass/diffusion matrices, dense Cholesky of the RKHS kernel
 * and of the reaction-diffusion matrix, K-preconditioned CG); the
 * isotropic-layer mode restates the same element loops with the layered
 * physics (Lame stress, isotropic diffusion, Fisher-KPP, Gaussian bump,
 * Jacobi-PCG) that the reference's MATLAB wrapper reserves an empty branch
 * for (deformation.m:12-13,22-24).
 *
 * Parity pin: the frame-mode restatement is checked against the
 * reference's own CUDA sources executed on the CPU through an emulation
 * shim (oracle/ref_shim, built by oracle/build_ref.py into oracle/_ref/)
 * and against the golden vectors in tests/golden/ that the shim produced.
 */
#ifndef SA_ORACLE_H
#define SA_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_FRAME = 0, ORC_ISOTROPIC = 1 };

typedef struct orc_problem {
	int dim;                 /* must equal DIM of the build */
	int lmkNum, elmNum, nzrNum;
	int btmLmkNum, btmElmNum;
	int vfdElmNum, tgtElmNum;
	int vtxElmCols;          /* 1 + 2*maxAdj: columns of vtxElmMat (N x cols) */
	int vtxBtmCols;          /* columns of vtxBtmMat (Nb x cols) */
	int femIfoCols;          /* columns of femIfoMat (nzr x cols) */
	int vfdIfoCols;          /* columns of vfdIfoMat (N x cols), gradient only */

	const double *lmkIniMat; /* N x D, column-major (x-block then y-block ...) */
	const int *elmVtxMat;    /* E x V */
	const int *vtxElmMat;    /* N x vtxElmCols */
	const int *frmVtxMat;    /* 2D: tanVtxMat E x 4; 3D: nmlVtxMat E x 6 */
	const int *tsvVtxMat;    /* 2D: E x 4; 3D: E x 6 */
	const int *btmVtxMat;    /* Bt x (V-1) */
	const int *vtxBtmMat;    /* Nb x vtxBtmCols */
	const int *femVtxMat;    /* nzr x 2 */
	const int *femIfoMat;    /* nzr x femIfoCols */
	const int *vfdVtxMat;    /* Vd x (V-1) */
	const int *vfdIfoMat;    /* N x vfdIfoCols (gradient gather) */
	const double *tgtCenPosMat; /* Vt x D */
	const double *tgtUniDirMat; /* Vt x D */
	const double *tgtElmVolVec; /* Vt */
	char cenKnlType, dirKnlType;
	double cenKnlWidth, dirKnlWidth;

	int elaType;             /* ORC_FRAME or ORC_ISOTROPIC */
	int lyrNum;              /* isotropic: number of material layers */
	const int *elmLyrVec;    /* isotropic: E layer ids in [0, lyrNum) */
	const double *modVec;    /* frame: 3 (2D) / 4 (3D); isotropic: lambda,mu pairs */
	const double *spdLyrVec; /* isotropic: lyrNum diffusivities */
	double spdTanVal, spdTsvVal;
	const double *ynkActPrmVec; /* frame: 4; isotropic: [coefficient] */
	const double *reaActPrmVec; /* frame: 5; isotropic: [rate] */
	const double *tauPrmVec;    /* frame 2D: [p]; frame 3D: [R, p]; isotropic: unused */
	double ldmWgt;
	int knlOrder;
	double knlWidth, knlEps;
	double btmWgt, timeStp;
	int timeNum, cgItrMax;
	double cgTolSqu;
	int rdItrMax;            /* isotropic reaction-diffusion Jacobi-PCG */
	double rdTolSqu;
	int velocityGuess;       /* isotropic: velocity PCG start, the degree-k polynomial through the last k + 1
	                            velocities (k = 0 .. 5; 0: the previous velocity) */
} orc_problem;

/* Full forward model (reference deform(), 2D/deform.cu:22-119) and, when
 * objPtr is not NULL, the varifold objective of the final shape
 * (2D/objfcn.cu:119-120).  lmkStk: N*D*timeNum, tauMat: N*timeNum.
 * cgItr (optional, timeNum-1 ints) receives the velocity CG iteration
 * counts.  Returns 0 on success, 1 when a CG solve failed (objective set to
 * DBL_MAX as the reference does). */
int orc_forward(const orc_problem *P, const double *tauVarVec,
                double *lmkStk, double *tauMat, double *objPtr, int *cgItr);

/* orc_forward that also records, in stepSec (timeNum-1 doubles, optional),
 * the wall time of every time step (omp_get_wtime), for the CPU timing of
 * a sample of steps after warm-up steps. */
int orc_forward_timed(const orc_problem *P, const double *tauVarVec, double *lmkStk, double *tauMat,
                      double *objPtr, int *cgItr, double *stepSec);

/* Single operators, for operator-level parity tests. */
void orc_initial_tau(const orc_problem *P, const double *tauVarVec, double *tau);
void orc_frame(const orc_problem *P, const double *lmk, double *frmA, double *tsv);
void orc_edges(const orc_problem *P, const double *lmk, double *edg);
/* y = E v (elastic operator at geometry lmk) */
void orc_elastic_apply(const orc_problem *P, const double *lmk, const double *v, double *y);
/* y = P v (bottom penalty at geometry lmk) */
void orc_penalty_apply(const orc_problem *P, const double *lmk, const double *v, double *y);
/* diagonal of E + btmWgt P (isotropic mode Jacobi preconditioner) */
void orc_elastic_diag(const orc_problem *P, const double *lmk, double *diag);
void orc_elastic_blocks(const orc_problem *P, const double *lmk, int inverse, double *blk);
/* yank right-hand side b from nodal tau */
void orc_yank(const orc_problem *P, const double *lmk, const double *tau, double *b);
/* reaction load vector from nodal tau (consistent mass) */
void orc_reaction_load(const orc_problem *P, const double *lmk, const double *tau, double *r);
/* mass and diffusion matrix values in femVtxMat (CSR) order */
void orc_fem_csr(const orc_problem *P, const double *lmk, double *ppdVal, double *ggdVal);
/* dense RKHS kernel matrix (N x N column-major) without the eps shift */
void orc_kernel_matrix(const orc_problem *P, const double *lmk, double *knlMat);
/* pointwise activity / reaction functions */
void orc_yank_activity(const orc_problem *P, const double *tau, double *f, int n);
void orc_reaction_activity(const orc_problem *P, const double *tau, double *f, int n);
/* varifold objective of shape lmk against the target; when grad != NULL it
 * also returns d(obj)/d(lmk) (N x D) through the reference's gradient
 * kernels (2D/varifold.cu:359-498,545-576; 3D/varifold.cu:372-530,577-608). */
double orc_varifold(const orc_problem *P, const double *lmk, double *grad);
/* reference dsum tree reduction (2D/dsum.cu:6-73) */
double orc_dsum(const double *vec, int len);
/* 2D Matern helper functions x^2 K0(x) ... (inc/polybesselk.h) */
void orc_besselk(double x, double *f0, double *f1);

#ifdef __cplusplus
}
#endif
#endif
