/*
 * shape_atrophy_gb300.h -- C-ABI of the GB300 forward shape-evolution model.
 *
 * Drop-in boundary for the reference's four MEX binaries
 * (deformation_{2D,3D}_frame, computeObjfcn_{2D,3D}_frame built by
 * CUDA/compile.m): the positional entry points below take the gateways'
 * prhs arguments in the same order and meaning
 * (CUDA/2D_frame/deformation.cu:24-63, CUDA/2D_frame/computeObjfcn.cu:25-65,
 * and the 3D_frame copies), with the sizes the gateways read from
 * mxGPUGetDimensions passed explicitly.  Plain pointers and sizes only.
 *
 * Memory: every array argument may live in host memory or in device memory
 * of the context's GPU (detected per pointer with cudaPointerGetAttributes),
 * so a MATLAB gateway can pass gpuArray data zero-copy and a C caller can
 * pass host arrays.  Outputs follow the same rule.
 *
 * Array layouts are the reference's: an "R x C" matrix is column-major
 * (element (r, c) at c*R + r); index arrays are int32, 0-based, and the
 * adjacency matrices hold a count in column 0 followed by index pairs,
 * exactly as CUDA/generateElementObject2D.m / generateElementObject3D.m
 * produce them.
 *
 * Errors: functions return SA_OK (0) or an SA_ERR_* code; the message of
 * the last failure is available from sa_error_message().  A velocity CG
 * solve that fails does not raise an error: like the reference
 * (CUDA/2D_frame/deform.cu:68-73) that parameter column gets objective
 * DBL_MAX and the call returns SA_OK.
 *
 * Threading: one context per host thread, or serialise calls on a shared
 * context.  Calls are synchronous; all device work runs on the context's
 * own stream.
 */
#ifndef SHAPE_ATROPHY_GB300_H
#define SHAPE_ATROPHY_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SA_OK                 0
#define SA_ERR_ARG            1   /* invalid argument, size or index */
#define SA_ERR_CUDA           2   /* CUDA error or device allocation failure */
#define SA_ERR_UNSUPPORTED    3   /* option combination not supported */
#define SA_ERR_NOT_CONVERGED  4   /* per-solve status: CG hit its iteration cap */
#define SA_ERR_BREAKDOWN      5   /* per-solve status: CG breakdown (zero curvature) */
#define SA_ERR_NONFINITE      6   /* per-solve status: NaN/Inf in a solve */
#define SA_ERR_TIMEOUT        7   /* a bounded device-side wait (grid barrier) gave up */

#define SA_ELA_FRAME          0   /* reference frame elasticity, K-preconditioned CG */
#define SA_ELA_ISOTROPIC      1   /* layered isotropic elasticity, block-Jacobi PCG */

#define SA_PREC_FP64          0   /* all arithmetic in FP64 */
#define SA_PREC_MIXED         1   /* FP32 operators, FP64 dots/residuals + refinement */

#define SA_CG_AUTO            0   /* persistent CG kernel (row state in registers when the grid fits one CTA
                                     per SM, else vectors in global memory), two kernels when neither fits */
#define SA_CG_PERSISTENT      1   /* same as AUTO */
#define SA_CG_TWO_KERNEL      2   /* matvec + vector kernel per iteration */
#define SA_CG_PERSISTENT_GLOBAL 3 /* the persistent kernel with vectors in global memory at any size */

/* sa_params.velocityGuess: where each step's velocity CG starts (layered model) */
#define SA_GUESS_PREVIOUS     0   /* the previous step's velocity (the reference's warm start) */
#define SA_GUESS_EXTRAPOLATE  1   /* 2 v_t-1 - v_t-2 from the third step on: same answer to the CG tolerance,
                                     about a third fewer iterations on the layered shell */
#define SA_GUESS_QUADRATIC    2   /* 3 v_t-1 - 3 v_t-2 + v_t-3 from the fourth step on (linear at the third) */
#define SA_GUESS_CUBIC        3   /* 4 v_t-1 - 6 v_t-2 + 4 v_t-3 - v_t-4 (lower degrees in the first steps) */
#define SA_GUESS_MAX_ORDER    5   /* velocityGuess k = 1 .. 5: the degree-k polynomial through the last k + 1
                                     velocities, evaluated one step ahead (lower degrees in the first steps) */
#define SA_GUESS_DEFAULT      SA_GUESS_CUBIC   /* fewest iterations on the layered workloads; the positional
                                                  isotropic entry points use it */

typedef struct sa_context sa_context;

/* Element object: the fields of the reference's elmObj struct
 * (generateElementObject2D.m:137-150, generateElementObject3D.m:115-127),
 * plus the layer id array of the layered model and the varifold gradient
 * gather table.  frmVtxMat is tanVtxMat (E x 4) in 2D and nmlVtxMat
 * (E x 6) in 3D; tsvVtxMat is E x 4 / E x 6. */
typedef struct sa_element_object {
	int dim;                       /* 2 or 3 */
	int lmkNum, elmNum;            /* N, E */
	const int *elmVtxMat;          /* E x (dim+1) */
	const int *vtxElmMat;  int vtxElmCols;   /* N x cols */
	const int *frmVtxMat;          /* E x 4 (2D) / E x 6 (3D); frame model only (the isotropic model
	                                  neither reads nor checks it; may be NULL there) */
	const int *tsvVtxMat;          /* E x 4 (2D) / E x 6 (3D); frame model only, as frmVtxMat */
	const int *bdrVtxMat;  int bdrElmNum;    /* unused by the model; may be NULL */
	const int *vtxBdrMat;  int vtxBdrCols;   /* unused by the model; may be NULL */
	const int *btmVtxMat;  int btmElmNum;    /* Bt x dim */
	const int *vtxBtmMat;  int btmLmkNum; int vtxBtmCols;   /* Nb x cols */
	const int *femVtxMat;  int nzrNum;       /* nzr x 2, sorted by (row, col) */
	const int *femIfoMat;  int femIfoCols;   /* nzr x cols */
	const int *vfdVtxMat;  int vfdElmNum;    /* Vd x dim (objective only) */
	const int *vfdIfoMat;  int vfdIfoCols;   /* N x cols (gradient only; may be NULL) */
	const int *elmLyrVec;          /* E layer ids (isotropic only) */
} sa_element_object;

/* Model parameters in the reference's argument vocabulary
 * (CUDA/deformation.m:1-5), plus the layered-model tables. */
typedef struct sa_params {
	int elaType;                   /* SA_ELA_FRAME or SA_ELA_ISOTROPIC */
	int precision;                 /* SA_PREC_FP64 or SA_PREC_MIXED */
	const double *tauPrmVec; int tauPrmNum;
	double ldmWgt; int knlOrder; double knlWidth; double knlEps;
	const double *modVec; int modNum;   /* frame: 3 (2D) / 4 (3D); isotropic: lambda,mu per layer */
	double spdTanVal, spdTsvVal;        /* frame diffusion speeds */
	const double *spdLyrVec; int lyrNum;/* isotropic: diffusivity per layer */
	const double *ynkActPrmVec;         /* frame: 4 values; isotropic: [coefficient c], f(u) = c u */
	const double *reaActPrmVec;         /* frame: 5 values; isotropic: [rate], R(u) = rate u (1-u) */
	double btmWgt, timeStp;
	int timeNum, cgItrMax;
	double cgTolSqu;
	int rdItrMax;                       /* isotropic reaction-diffusion PCG (frame: same as cgItrMax) */
	double rdTolSqu;                    /* isotropic RD PCG tolerance squared (frame: 1e-28) */
	int cgKernel;                       /* SA_CG_AUTO (0), SA_CG_PERSISTENT, SA_CG_TWO_KERNEL, SA_CG_PERSISTENT_GLOBAL */
	int velocityGuess;                  /* layered model's velocity CG start: a polynomial order 0 .. 5
	                                       (SA_GUESS_PREVIOUS = 0 is the reference's warm start, SA_GUESS_DEFAULT
	                                       the cubic); the frame model always uses 0 */
} sa_params;

/* Varifold target and kernels (computeObjfcn prhs[13..20]). */
typedef struct sa_target {
	const double *cenPosMat;   /* Vt x dim */
	const double *uniDirMat;   /* Vt x dim */
	const double *elmVolVec;   /* Vt */
	int tgtElmNum;
	char cenKnlType;           /* 'G' Gaussian, 'C' Cauchy, 'M' Matern-3/2 */
	double cenKnlWidth;
	char dirKnlType;           /* 'B' Binet, 'L' linear, 'O' oriented, 'U' unoriented Gaussian */
	double dirKnlWidth;
} sa_target;

/* Per-call diagnostics (optional output). */
typedef struct sa_solve_info {
	int status;                /* SA_OK or the per-solve status of the last column */
	int cgIterTotal;           /* velocity CG iterations, all steps of the last column */
	int rdIterTotal;           /* reaction-diffusion CG iterations, all steps */
	int cgIterMax;             /* largest per-step velocity iteration count */
	int invertedElements;      /* elements whose orientation flipped (Jacobian sign check) */
	double elapsedMs;          /* device time of the solves (sessions: of the last step call) */
	long long kernelLaunches;  /* CUDA kernels launched by the solve (sessions: since creation) */
} sa_solve_info;

int sa_create(sa_context **ctx, int device);
int sa_destroy(sa_context *ctx);
const char *sa_error_message(const sa_context *ctx);

/* Forward model for every column of tauVarMat (tauVarNum x objNum).
 * lmkStk ((N*dim) x timeNum), tauMat (N x timeNum): trajectory of the last
 * column, as the reference returns it (may be NULL).  objVec (objNum):
 * objective when tgt != NULL, else 0; DBL_MAX where the CG failed.
 * Replaces deform()/objfcn() (CUDA/2D_frame/deform.cu:22-119,
 * CUDA/2D_frame/objfcn.cu:23-123). */
int sa_forward(sa_context *ctx, const sa_element_object *obj, const double *lmkIniMat,
               const sa_params *prm, const sa_target *tgt,
               const double *tauVarMat, int tauVarNum, int objNum,
               double *lmkStk, double *tauMat, double *objVec, sa_solve_info *info);

/* Varifold objective of one shape against a target, and optionally its
 * node gradient (N x dim) through the reference's gradient formulas
 * (CUDA/2D_frame/varifold.cu:359-498,545-576; 3D_frame :372-530,577-608).
 * Replaces varifold() (CUDA/2D_frame/varifold.cu:500-543). */
int sa_varifold(sa_context *ctx, const sa_element_object *obj, const double *lmkMat,
                const sa_target *tgt, int precision, double *obj_out, double *gradMat);

/* Objective and its gradient with respect to the bump parameters (no
 * reference counterpart; the reference's computeObjfcn returns objectives
 * only).  Layered model (elaType isotropic, ldmWgt 0), one parameter
 * vector tauVarVec = [c (dim values), h, sigma]: runs the forward solve with
 * the tangent-linear model of every time step for each of the dim + 2
 * parameters (one extra velocity and reaction-diffusion solve per parameter
 * and step, on the operators of the forward step) and returns
 * objOut = J(x_T) and gradOut[k] = dJ/dp_k, k = 0 .. dim + 1.  The gradient
 * is that of the discrete model (exact up to the CG tolerances).  With
 * prm->precision SA_PREC_MIXED the velocity solves (forward and tangent) run
 * as FP32 inner CG with FP64 refinement and the objective in FP32 pair sums
 * (the reaction-diffusion solves stay FP64, as in the forward model).  A failed
 * solve gives objOut = DBL_MAX, NaN gradient and its status in info;
 * info->cgIterMax holds the iterations of all tangent solves.  Needs the
 * element object's vfdIfoMat (varifold gradient). */
int sa_objective_gradient(sa_context *ctx, const sa_element_object *obj, const double *lmkIniMat,
                          const sa_params *prm, const sa_target *tgt, const double *tauVarVec, int tauVarNum,
                          double *objOut, double *gradOut, sa_solve_info *info);

/* Objective and its gradient by the discrete adjoint (no reference
 * counterpart; the reference ships derivative kernels it never calls,
 * 2D_frame/varifold.cu:359-498, tauInitial.cu:68-116, inc/activity.h).  One
 * parameter vector: the forward solve keeps the trajectory and the
 * velocities on the device (N x dim x timeNum doubles twice; the frame model
 * also K^{-1} v), then one backward sweep solves two adjoint systems per step
 * (the forward operators are symmetric: the same CG as the forward solves,
 * FP64) and accumulates the gradient with respect to every parameter at
 * once, at a cost independent of the parameter count:
 *   gradBump  (optional): layered model (elaType isotropic, ldmWgt 0):
 *             dJ/d[c (dim), h, sigma] (dim + 2 values), as
 *             sa_objective_gradient; frame model: dJ/d tauVarVec, 4 values
 *             (2D [cx, cy, h, R], 3D [cx, cy, cz, h]);
 *   gradLayer (3 x lyrNum, optional, layered model): dJ/d(lambda_l, mu_l, D_l)
 *             per material layer, in that order per layer;
 *   gradTau0  (N, optional): dJ/dtau_0 at every node (the initial
 *             concentration as free parameters);
 *   gradX0    (N x dim column-major, optional): dJ/d(initial node positions),
 *             including the bump's dependence on them.
 * The frame model's sweep differentiates its frames (built from other
 * nodes), frame stress, anisotropic diffusion, projected 3D penalty, activity
 * templates and the dense RKHS term ldmWgt K^{-1}.  prm->precision is
 * ignored (FP64 throughout).  A failed solve gives objOut = DBL_MAX, NaN
 * gradients and its status in info; info->cgIterMax holds the iterations of
 * all adjoint solves.  Needs vfdIfoMat. */
int sa_objective_adjoint(sa_context *ctx, const sa_element_object *obj, const double *lmkIniMat,
                         const sa_params *prm, const sa_target *tgt, const double *tauVarVec, int tauVarNum,
                         double *objOut, double *gradBump, double *gradLayer, double *gradTau0, double *gradX0,
                         sa_solve_info *info);

/* Varifold objective without any device allocation (no counterpart in the
 * reference).  For callers that must not allocate while they evaluate the
 * objective: an optimiser's line search that calls it hundreds of times on
 * a GPU whose memory is managed by someone else (MATLAB's gpuArray pool, a
 * serving process with a fixed budget), where cudaMalloc can fail and
 * cudaFree synchronises the whole device.  Same value as sa_varifold.
 *   - All inputs must already be memory of the current device (nodes:
 *     N x dim column-major; vfdVtxMat: Vd x dim int32; target Vt x dim,
 *     Vt); host pointers and other GPUs' memory are rejected with
 *     SA_ERR_ARG (nothing is copied).
 *   - Limit: vfdElmNum and tgtElmNum at most 32768 each; larger sizes
 *     return SA_ERR_ARG.  The scratch is a fixed ~2.4 MB device array that
 *     every GPU loading the library holds until the process exits.
 *   - A vfdVtxMat entry outside [0, lmkNum) is found on the device (the
 *     element is skipped, nothing outside the arrays is read) and the call
 *     returns SA_ERR_ARG.  cenKnlWidth, and dirKnlWidth for the 'O' and
 *     'U' direction kernels, must be finite and > 0.
 *   - The first call on a device looks the array's device address up
 *     (cudaGetSymbolAddress) and keeps it for later calls; make that first
 *     call before any stream capture.  cudaDeviceReset invalidates the
 *     kept address: do not call this function after resetting the device.
 *   - Runs on the given stream (NULL: the legacy default stream) of the
 *     current device and returns only when the objective has been written
 *     to objOut: it waits for that stream.
 *   - All calls share the one array and each leaves its contents behind:
 *     calls that overlap on the GPU (other threads, other streams) race;
 *     serialise them.
 *   - objOut may be host or device memory. */
int sa_varifold_noalloc(int dim, int lmkNum, const double *lmkMat, int vfdElmNum, const int *vfdVtxMat,
                        int tgtElmNum, const double *tgtCenPosMat, const double *tgtUniDirMat,
                        const double *tgtElmVolVec, char cenKnlType, double cenKnlWidth, char dirKnlType,
                        double dirKnlWidth, void *stream, double *objOut);

/* Stepwise solve of one parameter vector (no reference counterpart: the
 * reference runs all timeNum-1 steps inside one call).  A session keeps
 * mesh, state and solver work device-resident; sa_session_step advances up
 * to nsteps time steps (never past timeNum-1, stopping early on a failed
 * solve), sa_session_state copies the current nodes (N x dim) and
 * concentration (N), sa_session_objective evaluates the varifold objective
 * of the current shape (needs a target at creation).  sa_session_profile
 * switches CUDA-event timing of the velocity CG's dominant kernel on or off
 * (the persistent CG kernel, or the matvec kernel on the two-kernel path;
 * enable = -1 leaves it as it is) and returns, since it was last switched,
 * the kernel's accumulated device time, its launch count and the
 * algorithmic bytes and flops of those launches. */
typedef struct sa_session sa_session;
int sa_session_create(sa_context *ctx, const sa_element_object *obj, const double *lmkIniMat,
                      const sa_params *prm, const sa_target *tgt, const double *tauVarVec, int tauVarNum,
                      sa_session **out);
int sa_session_step(sa_session *s, int nsteps, int *stepsDone);
int sa_session_state(sa_session *s, double *lmkMat, double *tauVec, int *step);
/* Streamed trajectory (no reference counterpart: deformation's lmkStk keeps
 * every step on the device and copies it at the end).  Advances up to nsteps
 * steps (like sa_session_step) and writes the state after every step whose
 * session step number is a multiple of stride, at most maxSnapshots of them,
 * in order: snapshot k to lmkOut + k * N * dim (the lmkStk column layout:
 * dim blocks of N) and tauOut + k * N.  lmkOut and tauOut are host memory
 * (either may be NULL); each snapshot is copied to pinned memory on a
 * second stream while the following steps run.  *snapshotsWritten,
 * *stepsDone: counts (may be NULL). */
int sa_session_stream(sa_session *s, int nsteps, int stride, double *lmkOut, double *tauOut, int maxSnapshots,
                      int *snapshotsWritten, int *stepsDone);
int sa_session_objective(sa_session *s, double *obj);
int sa_session_info(sa_session *s, sa_solve_info *info);
int sa_session_profile(sa_session *s, int enable, double *kernelMs, long long *launches, double *bytes,
                       double *flops);
int sa_session_destroy(sa_session *s);

/* Serving (no reference counterpart: the reference solves one request per
 * MEX call).  A server owns a loop thread and its own stream on the
 * context's GPU and runs layered-model forward solves (elaType
 * SA_ELA_ISOTROPIC, one parameter vector each) with continuous batching:
 * requests are admitted in arrival order while their device footprint fits
 * hbmBudgetBytes and fewer than maxInstances run; every running instance
 * keeps its mesh, state and CG vectors on the device; each tick advances all
 * running instances one time step, with one batched persistent CG launch for
 * all their velocity solves (per precision and dimension) and one for all
 * their reaction-diffusion solves.  Finished instances free their memory at
 * the end of a tick; queued requests enter at the start of the next.  A
 * request's result does not depend on which other requests run with it.
 *
 * sa_server_submit copies every input (host or device memory) before it
 * returns.  sa_server_result returns, once the request is DONE, the final
 * node positions (lmkNum x dim, column-major), the final concentration
 * (lmkNum), the varifold objective (0 without a target; DBL_MAX when a solve
 * failed, with info->status telling which), the solve diagnostics
 * (info->elapsedMs = admission to completion) and the latency from
 * submission to completion; it releases the request.  A FAILED request
 * (invalid input, device error) returns its error code and message.
 * sa_server_destroy finishes the queued and running requests first. */
#define SA_REQ_QUEUED   0
#define SA_REQ_RUNNING  1
#define SA_REQ_DONE     2
#define SA_REQ_FAILED   3

typedef struct sa_server sa_server;
typedef struct sa_server_counters {
	long long submitted, completed, failed;
	int queued, running;
	double bytesInUse, peakBytes;   /* device bytes held by running instances (now, peak) */
	long long ticks;                /* batched time steps executed */
	double busyMs;                  /* host wall time spent in ticks */
} sa_server_counters;

int sa_server_create(sa_context *ctx, double hbmBudgetBytes, int maxInstances, sa_server **out);
int sa_server_submit(sa_server *sv, const sa_element_object *obj, const double *lmkIniMat, const sa_params *prm,
                     const sa_target *tgt, const double *tauVarVec, int tauVarNum, long long *requestId);
int sa_server_poll(sa_server *sv, long long requestId, int *state);
int sa_server_wait(sa_server *sv, long long requestId, double timeoutMs, int *state);   /* timeoutMs < 0: no limit */
int sa_server_result(sa_server *sv, long long requestId, double *lmkMat, double *tauVec, double *objOut,
                     sa_solve_info *info, double *latencyMs);
int sa_server_stats(sa_server *sv, sa_server_counters *stats);
int sa_server_destroy(sa_server *sv);

/* Element-object builders (host code, no device needed): the arrays of
 * CUDA/generateElementObject2D.m, CUDA/generateElementObject3D.m and
 * CUDA/tri2tetra.m, bit for bit (same orders: column-major find lists,
 * sortrows pattern, femIfoMat element lists ascending), built in
 * O(E log E) instead of the MATLAB find-per-node loops.  The object owns its
 * arrays; sa_elmobj_view fills an sa_element_object that points into them
 * (valid until sa_elmobj_free) and can be passed to every entry point.
 * vfdIfoMat (the varifold gradient gather table) is included.  tri2tetra:
 * triVtxMat T x 3 -> tetVtxMat E x 4, nmlVtxMat E x 6, tsvVtxMat E x 6,
 * E = 3 T (lyrCntNum - 1), arrays allocated by the caller.  2D: periodic != 0
 * closes every node layer into a ring (annulus). */
typedef struct sa_elmobj sa_elmobj;
int sa_tri2tetra(const int *triVtxMat, int triNum, int lyrCntNum, int *tetVtxMat, int *nmlVtxMat, int *tsvVtxMat);
int sa_build_element_object_3d(const int *tetVtxMat, int elmNum, const int *btmVtxMat, int btmElmNum,
                               const int *nmlVtxMat, const int *tsvVtxMat, const int *vfdLyrVec, int vfdLyrNum,
                               sa_elmobj **out);
int sa_build_element_object_2d(int lyrLmkNum, int lyrCntNum, const int *vfdLyrVec, int vfdLyrNum, int periodic,
                               sa_elmobj **out);
int sa_elmobj_view(const sa_elmobj *obj, sa_element_object *view);
int sa_elmobj_layers(const sa_elmobj *obj, int *lyrLmkNum, int *lyrCntNum, int *elmPerLayer);
int sa_elmobj_free(sa_elmobj *obj);

/* Launch-shape tuning (process-wide; no reference counterpart).  Names:
 * "persistMaxWarps" (1..20, warps per CTA cap of the persistent CG),
 * "batchBlock" (128 or 256, threads per CTA of the batched CG),
 * "batchSlicesPerWarp" (1..16, 32-row slices per warp when a batched solve's
 * CTAs are sized), "vfdCtasPerSm" (1..32, CTAs per SM of the varifold pair
 * sums), "mixedInnerFloor" (4..16: mixed precision's FP32 inner solves stop at
 * a squared relative residual of 10^-k at the lowest), "kernelMatrixFree" (0 or
 * 1: the frame model's RKHS products evaluate each kernel-matrix entry from
 * the node positions instead of reading the stored N x N matrix, the same
 * bits at ~15x the cost; automatic when the matrix would exceed 96 GiB or
 * three quarters of the free device memory).  shape_atrophy_gb300/autotune.py measures them on the GPU and writes
 * shape_atrophy_gb300/tuning.json, which the Python API applies; the compiled
 * defaults are the values measured best on GB300.  They change how partial
 * sums are grouped: results are reproducible for a given setting.  Set them
 * before creating sessions or servers. */
int sa_set_tuning(const char *name, int value);
int sa_get_tuning(const char *name, int *value);
/* Name and SM count of a CUDA device (the key of the tuning table). */
int sa_device_name(int device, char *buf, int len, int *smCount);

/* Self-test of the bounded device-side waits (no reference counterpart).
 * Launches two cooperative CTAs on a grid barrier whose arrival count can
 * never reach its target; each CTA must give up after the 1 s limit the CG
 * kernels use, set the abort flag and return, leaving the context usable.
 * *ctasGaveUp = CTAs that gave up (2 when the mechanism works). */
int sa_selftest_wait_timeout(sa_context *ctx, int *ctasGaveUp, double *elapsedMs);

/* Accuracy check of the FP64 exponential (fn = 0: table-driven) and square
 * root (fn = 1: Newton iteration from the FP32 reciprocal square root) that
 * the varifold pair sums use (no reference counterpart): for n host values
 * x, y[k] = that function of x[k] and yref[k] = CUDA's exp(x[k]) or
 * sqrt(x[k]), both evaluated on the device. */
int sa_selftest_math(sa_context *ctx, int fn, long n, const double *x, double *y, double *yref);

/* FMA throughput of the device's FP64 (fp64 = 1) or FP32 (fp64 = 0) pipe
 * (no reference counterpart): independent FMA chains per thread (4 or 8 in
 * FP64, 8 or 16 in FP32), 256-thread CTAs, 2, 4 or 8 CTAs per SM, the best
 * of two timed launches of each after a warm-up.  *tflops: TFLOP/s by CUDA
 * events; *smMhz (optional): the SM clock during that launch (clock64 over
 * %globaltimer in the kernel); *flopsPerClockSm (optional): the rate per SM
 * per clock cycle, independent of the clock.  The denominator of the pipe
 * fractions the benchmark reports. */
int sa_selftest_fma_peak(sa_context *ctx, int fp64, double *tflops, double *flopsPerClockSm, double *smMhz);

/* Drop-in for the MEX binaries deformation_2D_frame (dim 2) and
 * deformation_3D_frame (dim 3): arguments in prhs order
 * (CUDA/2D_frame/deformation.cu:24-50), outputs plhs[0..2]
 * (:57-63): lmkStk (N*dim x timeNum), tauMat (N x timeNum), objVec (1 x objTotNum). */
int sa_deformation_frame(sa_context *ctx, int dim,
	const double *tauVarMat, int tauVarNum, int objTotNum,  /* prhs[0]  tauVarNum x objTotNum     */
	const double *tauPrmVec, int tauPrmNum,                 /* prhs[1]                            */
	const double *lmkIniMat, int lmkNum,                    /* prhs[2]  N x dim                   */
	const int *elmVtxMat, int elmNum,                       /* prhs[3]  E x (dim+1)               */
	const int *vtxElmMat, int vtxElmCols,                   /* prhs[4]  N x cols                  */
	const int *frmVtxMat,                                   /* prhs[5]  tanVtxMat / nmlVtxMat     */
	const int *tsvVtxMat,                                   /* prhs[6]                            */
	const int *bdrVtxMat, int bdrElmNum,                    /* prhs[7]                            */
	const int *vtxBdrMat, int vtxBdrCols,                   /* prhs[8]                            */
	const int *btmVtxMat, int btmElmNum,                    /* prhs[9]  Bt x dim                  */
	const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols,    /* prhs[10] Nb x cols                 */
	const int *femVtxMat, int nzrNum,                       /* prhs[11] nzr x 2                   */
	const int *femIfoMat, int femIfoCols,                   /* prhs[12] nzr x cols                */
	double ldmWgt, int knlOrder, double knlWidth, double knlEps,   /* prhs[13..16]               */
	const double *modVec,                                   /* prhs[17] 3 (2D) / 4 (3D) values    */
	double spdTanVal, double spdTsvVal,                     /* prhs[18..19]                       */
	const double *ynkActPrmVec, const double *reaActPrmVec, /* prhs[20..21] 4 and 5 values        */
	double btmWgt, double timeStp, int timeNum,             /* prhs[22..24]                       */
	int cgItrMax, double cgTolSqu,                          /* prhs[25..26]                       */
	double *lmkStk, double *tauMat, double *objVec);        /* plhs[0..2]                         */

/* Drop-in for computeObjfcn_2D_frame / computeObjfcn_3D_frame: prhs order
 * of CUDA/2D_frame/computeObjfcn.cu:25-59; output plhs[0] objVec. */
int sa_computeObjfcn_frame(sa_context *ctx, int dim,
	const double *tauVarMat, int tauVarNum, int objTotNum,  /* prhs[0]                            */
	const double *tauPrmVec, int tauPrmNum,                 /* prhs[1]                            */
	const double *lmkIniMat, int lmkNum,                    /* prhs[2]                            */
	const int *elmVtxMat, int elmNum,                       /* prhs[3]                            */
	const int *vtxElmMat, int vtxElmCols,                   /* prhs[4]                            */
	const int *frmVtxMat,                                   /* prhs[5]                            */
	const int *tsvVtxMat,                                   /* prhs[6]                            */
	const int *bdrVtxMat, int bdrElmNum,                    /* prhs[7]                            */
	const int *vtxBdrMat, int vtxBdrCols,                   /* prhs[8]                            */
	const int *btmVtxMat, int btmElmNum,                    /* prhs[9]                            */
	const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols,    /* prhs[10]                           */
	const int *femVtxMat, int nzrNum,                       /* prhs[11]                           */
	const int *femIfoMat, int femIfoCols,                   /* prhs[12]                           */
	const int *vfdVtxMat, int vfdElmNum,                    /* prhs[13] Vd x dim                  */
	const double *tgtCenPosMat, const double *tgtUniDirMat, /* prhs[14..15] Vt x dim              */
	const double *tgtElmVolVec, int tgtElmNum,              /* prhs[16] Vt                        */
	double cenKnlType, double cenKnlWidth,                  /* prhs[17..18] (char code as double) */
	double dirKnlType, double dirKnlWidth,                  /* prhs[19..20]                       */
	double ldmWgt, int knlOrder, double knlWidth, double knlEps,   /* prhs[21..24]               */
	const double *modVec,                                   /* prhs[25]                           */
	double spdTanVal, double spdTsvVal,                     /* prhs[26..27]                       */
	const double *ynkActPrmVec, const double *reaActPrmVec, /* prhs[28..29]                       */
	double btmWgt, double timeStp, int timeNum,             /* prhs[30..32]                       */
	int cgItrMax, double cgTolSqu,                          /* prhs[33..34]                       */
	double *objVec);                                        /* plhs[0]                            */

/* The layered (isotropic) model through the positional surface of the
 * frame entry points: the branch that CUDA/deformation.m:12-13,22-24 and
 * CUDA/computeObjfcn.m:12-13,22-24 parse (d_modMat = reshape(h_modVec, 2,
 * [])') and leave empty.  Arguments are those of sa_deformation_frame with
 * three changes: elmLyrVec (E int32, the 0-based material layer of each
 * element) follows femIfoMat; modMat (lyrNum x 2 column-major: lambda in
 * column 0, mu in column 1; host or device memory) replaces modVec; and
 * spdLyrVec (lyrNum per-layer diffusivities, the wrapper's spdTanVal)
 * replaces spdTanVal, spdTsvVal.  ynkActPrmVec = [c] (load -c u I),
 * reaActPrmVec = [rate] (Fisher-KPP rate u (1 - u)), tauVarMat columns are
 * the bump [centre (dim), height, sigma].  tanVtxMat/nmlVtxMat and
 * tsvVtxMat are not used by this model and may be NULL.  FP64, velocity CG
 * started from SA_GUESS_DEFAULT; outputs as sa_deformation_frame. */
int sa_deformation_isotropic(sa_context *ctx, int dim,
	const double *tauVarMat, int tauVarNum, int objTotNum,  /* prhs[0]                            */
	const double *tauPrmVec, int tauPrmNum,                 /* prhs[1]                            */
	const double *lmkIniMat, int lmkNum,                    /* prhs[2]  N x dim                   */
	const int *elmVtxMat, int elmNum,                       /* prhs[3]                            */
	const int *vtxElmMat, int vtxElmCols,                   /* prhs[4]                            */
	const int *frmVtxMat,                                   /* prhs[5]  unused here (may be NULL) */
	const int *tsvVtxMat,                                   /* prhs[6]  unused here (may be NULL) */
	const int *bdrVtxMat, int bdrElmNum,                    /* prhs[7]                            */
	const int *vtxBdrMat, int vtxBdrCols,                   /* prhs[8]                            */
	const int *btmVtxMat, int btmElmNum,                    /* prhs[9]                            */
	const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols,    /* prhs[10]                           */
	const int *femVtxMat, int nzrNum,                       /* prhs[11]                           */
	const int *femIfoMat, int femIfoCols,                   /* prhs[12]                           */
	const int *elmLyrVec,                                   /* prhs[13] E                         */
	double ldmWgt, int knlOrder, double knlWidth, double knlEps,   /* prhs[14..17]               */
	const double *modMat, int lyrNum,                       /* prhs[18] lyrNum x 2 (lambda, mu)   */
	const double *spdLyrVec,                                /* prhs[19] lyrNum                    */
	const double *ynkActPrmVec, const double *reaActPrmVec, /* prhs[20..21] 1 value each          */
	double btmWgt, double timeStp, int timeNum,             /* prhs[22..24]                       */
	int cgItrMax, double cgTolSqu,                          /* prhs[25..26]                       */
	double *lmkStk, double *tauMat, double *objVec);        /* plhs[0..2]                         */

/* computeObjfcn for the layered model: the arguments of
 * sa_computeObjfcn_frame with the three changes of sa_deformation_isotropic
 * (elmLyrVec after femIfoMat, modMat, spdLyrVec). */
int sa_computeObjfcn_isotropic(sa_context *ctx, int dim,
	const double *tauVarMat, int tauVarNum, int objTotNum,  /* prhs[0]                            */
	const double *tauPrmVec, int tauPrmNum,                 /* prhs[1]                            */
	const double *lmkIniMat, int lmkNum,                    /* prhs[2]                            */
	const int *elmVtxMat, int elmNum,                       /* prhs[3]                            */
	const int *vtxElmMat, int vtxElmCols,                   /* prhs[4]                            */
	const int *frmVtxMat,                                   /* prhs[5]  unused here (may be NULL) */
	const int *tsvVtxMat,                                   /* prhs[6]  unused here (may be NULL) */
	const int *bdrVtxMat, int bdrElmNum,                    /* prhs[7]                            */
	const int *vtxBdrMat, int vtxBdrCols,                   /* prhs[8]                            */
	const int *btmVtxMat, int btmElmNum,                    /* prhs[9]                            */
	const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols,    /* prhs[10]                           */
	const int *femVtxMat, int nzrNum,                       /* prhs[11]                           */
	const int *femIfoMat, int femIfoCols,                   /* prhs[12]                           */
	const int *elmLyrVec,                                   /* prhs[13] E                         */
	const int *vfdVtxMat, int vfdElmNum,                    /* prhs[14] Vd x dim                  */
	const double *tgtCenPosMat, const double *tgtUniDirMat, /* prhs[15..16] Vt x dim              */
	const double *tgtElmVolVec, int tgtElmNum,              /* prhs[17] Vt                        */
	double cenKnlType, double cenKnlWidth,                  /* prhs[18..19] (char code as double) */
	double dirKnlType, double dirKnlWidth,                  /* prhs[20..21]                       */
	double ldmWgt, int knlOrder, double knlWidth, double knlEps,   /* prhs[22..25]               */
	const double *modMat, int lyrNum,                       /* prhs[26] lyrNum x 2                */
	const double *spdLyrVec,                                /* prhs[27] lyrNum                    */
	const double *ynkActPrmVec, const double *reaActPrmVec, /* prhs[28..29]                       */
	double btmWgt, double timeStp, int timeNum,             /* prhs[30..32]                       */
	int cgItrMax, double cgTolSqu,                          /* prhs[33..34]                       */
	double *objVec);                                        /* plhs[0]                            */

#ifdef __cplusplus
}
#endif
#endif
