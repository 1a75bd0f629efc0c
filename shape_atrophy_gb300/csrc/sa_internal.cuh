// sa_internal.cuh -- shared declarations of the shape_atrophy_gb300 CUDA library.
//
// Layout conventions (device):
//   * node vectors are interleaved per node: x[i*D + d] (one 16/24-byte
//     record per node, so element and block-row gathers read one record);
//   * element data is structure-of-arrays over elements: a[k*E + e];
//   * the reference's int32 index matrices are kept in their own
//     column-major layout (entity index fastest), e.g. elmVtx[k*E + e];
//   * the elasticity operator is a block CSR matrix on the femVtxMat
//     pattern (D x D blocks, row-major inside a block), the mass and
//     diffusion matrices are scalar CSR on the same pattern.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cfloat>
#include <string>
#include <vector>
#include "../../include/shape_atrophy_gb300.h"

namespace sa {

constexpr int kBlock = 256;

inline int grid_for(long n, int block = kBlock) { return (int) ((n + block - 1) / block); }

// varifold kernel widths: the centre width always divides, the direction width only for the 'O' and 'U'
// direction kernels (2D_frame/varifold.cu:105-120); a width that divides must be finite and > 0
inline bool kernel_widths_ok(double cenWidth, char dirType, double dirWidth)
{
	auto pos = [](double w) { return w > 0.0 && w < DBL_MAX; };     // false for NaN and Inf
	return pos(cenWidth) && ((dirType != 'O' && dirType != 'U') || pos(dirWidth));
}

// --------------------------------------------------------------------------
// small fixed-size vector math (mirrors inc/matvec.h operation order)
// --------------------------------------------------------------------------
template <int D> struct Vec { double c[D]; };
template <int D> struct Mat { double m[D][D]; };

template <int D> __device__ __forceinline__ Vec<D> vsub(const Vec<D> &a, const Vec<D> &b)
{ Vec<D> r; for (int d = 0; d < D; ++d) r.c[d] = a.c[d] - b.c[d]; return r; }

template <int D> __device__ __forceinline__ double vdot(const Vec<D> &a, const Vec<D> &b)
{ double s = a.c[0] * b.c[0]; for (int d = 1; d < D; ++d) s = s + a.c[d] * b.c[d]; return s; }

template <int D> __device__ __forceinline__ Vec<D> load_node(const double *x, int i)
{ Vec<D> v; for (int d = 0; d < D; ++d) v.c[d] = x[(long) i * D + d]; return v; }

__device__ __forceinline__ Vec<3> vcross(const Vec<3> &x, const Vec<3> &y)
{   // inc/matvec.h:503-510
	Vec<3> r;
	r.c[0] =  x.c[1] * y.c[2] - x.c[2] * y.c[1];
	r.c[1] = -x.c[0] * y.c[2] + x.c[2] * y.c[0];
	r.c[2] =  x.c[0] * y.c[1] - x.c[1] * y.c[0];
	return r;
}

template <int D> __device__ __forceinline__ double det_edges(const Vec<D> *q);
template <> __device__ __forceinline__ double det_edges<2>(const Vec<2> *q)
{ return q[0].c[0] * q[1].c[1] - q[0].c[1] * q[1].c[0]; }                 // inc/matvec.h:250-253
template <> __device__ __forceinline__ double det_edges<3>(const Vec<3> *q)
{   // inc/matvec.h:592-600
	const Vec<3> &x = q[0], &y = q[1], &z = q[2];
	return  x.c[0] * y.c[1] * z.c[2] + x.c[1] * y.c[2] * z.c[0] + x.c[2] * y.c[0] * z.c[1]
	      - x.c[0] * y.c[2] * z.c[1] - x.c[1] * y.c[0] * z.c[2] - x.c[2] * y.c[1] * z.c[0];
}

// inverse of Q = [q1-q0, q2-q0 (, q3-q0)] given the edge vectors and det(Q)
template <int D> __device__ __forceinline__ Mat<D> inv_edges(const Vec<D> *q, double det);
template <> __device__ __forceinline__ Mat<2> inv_edges<2>(const Vec<2> *q, double det)
{   // inc/matvec.h:267-277
	Mat<2> r;
	r.m[0][0] =  q[1].c[1] / det; r.m[0][1] = -q[1].c[0] / det;
	r.m[1][0] = -q[0].c[1] / det; r.m[1][1] =  q[0].c[0] / det;
	return r;
}
template <> __device__ __forceinline__ Mat<3> inv_edges<3>(const Vec<3> *q, double det)
{   // inc/matvec.h:627-649
	const Vec<3> &x = q[0], &y = q[1], &z = q[2];
	Mat<3> r;
	r.m[0][0] =  (y.c[1] * z.c[2] - y.c[2] * z.c[1]) / det;
	r.m[0][1] = -(y.c[0] * z.c[2] - y.c[2] * z.c[0]) / det;
	r.m[0][2] =  (y.c[0] * z.c[1] - y.c[1] * z.c[0]) / det;
	r.m[1][0] = -(x.c[1] * z.c[2] - x.c[2] * z.c[1]) / det;
	r.m[1][1] =  (x.c[0] * z.c[2] - x.c[2] * z.c[0]) / det;
	r.m[1][2] = -(x.c[0] * z.c[1] - x.c[1] * z.c[0]) / det;
	r.m[2][0] =  (x.c[1] * y.c[2] - x.c[2] * y.c[1]) / det;
	r.m[2][1] = -(x.c[0] * y.c[2] - x.c[2] * y.c[0]) / det;
	r.m[2][2] =  (x.c[0] * y.c[1] - x.c[1] * y.c[0]) / det;
	return r;
}

// inverse of a small dense matrix by cofactors (diagonal blocks of the operator; SPD, well away from 0)
template <int D> __device__ __forceinline__ Mat<D> mat_inverse(const Mat<D> &a);
template <> __device__ __forceinline__ Mat<2> mat_inverse<2>(const Mat<2> &a)
{
	Mat<2> r;
	double det = a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0];
	r.m[0][0] = a.m[1][1] / det; r.m[0][1] = -a.m[0][1] / det;
	r.m[1][0] = -a.m[1][0] / det; r.m[1][1] = a.m[0][0] / det;
	return r;
}
template <> __device__ __forceinline__ Mat<3> mat_inverse<3>(const Mat<3> &a)
{
	Mat<3> r;
	double c00 = a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1];
	double c01 = a.m[1][2] * a.m[2][0] - a.m[1][0] * a.m[2][2];
	double c02 = a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0];
	double det = a.m[0][0] * c00 + a.m[0][1] * c01 + a.m[0][2] * c02;
	r.m[0][0] = c00 / det;
	r.m[1][0] = c01 / det;
	r.m[2][0] = c02 / det;
	r.m[0][1] = (a.m[0][2] * a.m[2][1] - a.m[0][1] * a.m[2][2]) / det;
	r.m[1][1] = (a.m[0][0] * a.m[2][2] - a.m[0][2] * a.m[2][0]) / det;
	r.m[2][1] = (a.m[0][1] * a.m[2][0] - a.m[0][0] * a.m[2][1]) / det;
	r.m[0][2] = (a.m[0][1] * a.m[1][2] - a.m[0][2] * a.m[1][1]) / det;
	r.m[1][2] = (a.m[0][2] * a.m[1][0] - a.m[0][0] * a.m[1][2]) / det;
	r.m[2][2] = (a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]) / det;
	return r;
}

// --------------------------------------------------------------------------
// activity functions (inc/activity.h:4-38, 106-167)
// --------------------------------------------------------------------------
__device__ __forceinline__ double yank_template(double t, double w)
{
	double a = 3.0 * (w - 2.0) / (w * w * w * (6.0 + w * (-6.0 + w)));
	double b = (6.0 + w * (-15.0 + 8 * w)) / (3.0 * (w - 2.0));
	double c = 6.0 / (6.0 + w * (-6.0 + w));
	if (t < -1.0 || t >= 1.0) return 0.0;
	if (t < -1.0 + w) return a * (t + 1.0) * (t + 1.0) * (t + 1.0) * (t - b);
	if (t < 1.0 - w) return -c * t * t + 1.0;
	return a * (-t + 1.0) * (-t + 1.0) * (-t + 1.0) * (-t - b);
}

__device__ __forceinline__ double reac_template(double t, double w, double a)
{
	double b1 = 8.0 * (6.0 * (a - 1.0) + a * w * (-6.0 + w)) / (3.0 * w * w * w * w);
	double b2 = -(144.0 * (a - 1.0) + w * (24.0 * (5.0 - 11.0 * a) + w * (156.0 * a - w * 29.0 * a)))
	            / (24.0 * (6.0 * (a - 1.0) + a * w * (-6.0 + w)));
	double c1 = -(24.0 * (a - 1.0) + a * w * (-12.0 + w)) / (9.0 * w * w * w);
	double c2 = -(24.0 * (a - 1.0) + w * (12.0 * (2.0 - 3.0 * a) + a * w * (13.0 + w * 2.0))) / (3.0 * w * w * w);
	double c3 = -((w - 1.0) * (w - 1.0) * (24.0 * (a - 1.0) + a * w * (-12.0 + w))) / (3.0 * w * w * w);
	double c4 = -(24.0 * (a - 1.0) + w * (12.0 * (6.0 - 7.0 * a)
	              + w * (-72.0 + 109.0 * a + w * (3.0 * (5.0 - 21.0 * a) + a * w * (15.0 - w)))))
	            / (9.0 * w * w * w);
	if (t < -1.0 || t >= 1.0) return 0.0;
	if (t < -1.0 + 0.5 * w) return b1 * (t + 1.0) * (t + 1.0) * (t + 1.0) * (t - b2);
	if (t < -1.0 + w) return c4 + t * (c3 + t * (c2 + t * c1));
	if (t < 1.0 - w) return -a * t * t + 1.0;
	if (t < 1.0 - 0.5 * w) return c4 + t * (-c3 + t * (c2 - t * c1));
	return b1 * (-t + 1.0) * (-t + 1.0) * (-t + 1.0) * (-t - b2);
}

// derivatives of the two templates with respect to t (inc/activity.h:40-79, 169-237)
__device__ __forceinline__ double yank_template_d(double t, double w)
{
	double a = 3.0 * (w - 2.0) / (w * w * w * (6.0 + w * (-6.0 + w)));
	double b = (6.0 + w * (-15.0 + 8 * w)) / (3.0 * (w - 2.0));
	double c = 6.0 / (6.0 + w * (-6.0 + w));
	if (t < -1.0 || t >= 1.0) return 0.0;
	if (t < -1.0 + w) return a * (t + 1.0) * (t + 1.0) * (3.0 * (t - b) + (t + 1.0));
	if (t < 1.0 - w) return -2.0 * c * t;
	return -a * (-t + 1.0) * (-t + 1.0) * (3.0 * (-t - b) + (-t + 1.0));
}

__device__ __forceinline__ double reac_template_d(double t, double w, double a)
{
	double b1 = 8.0 * (6.0 * (a - 1.0) + a * w * (-6.0 + w)) / (3.0 * w * w * w * w);
	double b2 = -(144.0 * (a - 1.0) + w * (24.0 * (5.0 - 11.0 * a) + w * (156.0 * a - w * 29.0 * a)))
	            / (24.0 * (6.0 * (a - 1.0) + a * w * (-6.0 + w)));
	double c1 = -(24.0 * (a - 1.0) + a * w * (-12.0 + w)) / (9.0 * w * w * w);
	double c2 = -(24.0 * (a - 1.0) + w * (12.0 * (2.0 - 3.0 * a) + a * w * (13.0 + w * 2.0))) / (3.0 * w * w * w);
	double c3 = -((w - 1.0) * (w - 1.0) * (24.0 * (a - 1.0) + a * w * (-12.0 + w))) / (3.0 * w * w * w);
	if (t < -1.0 || t >= 1.0) return 0.0;
	if (t < -1.0 + 0.5 * w) return b1 * (t + 1.0) * (t + 1.0) * (3.0 * (t - b2) + (t + 1.0));
	if (t < -1.0 + w) return c3 + t * (2.0 * c2 + t * 3.0 * c1);
	if (t < 1.0 - w) return -2.0 * a * t;
	if (t < 1.0 - 0.5 * w) return -c3 + t * (2.0 * c2 - t * 3.0 * c1);
	return -b1 * (-t + 1.0) * (-t + 1.0) * (3.0 * (-t - b2) + (-t + 1.0));
}

// --------------------------------------------------------------------------
// host-side structures
// --------------------------------------------------------------------------
struct Status {            // device-resident solver status (one per solve)
	int code;              // SA_OK or an error code
	int iters;             // iterations of the last CG solve
	int done;              // current CG solve finished
	int inverted;          // count of elements whose orientation flipped
};

struct Mesh {              // device copy of one element object + derived tables
	int dim, V, N, E, Z, Bt, Nb, Vd;
	int vtxElmCols, vtxBtmCols, femIfoCols, vfdIfoCols, frmCols, tsvCols;
	int *elmVtx = nullptr, *vtxElm = nullptr, *frmVtx = nullptr, *tsvVtx = nullptr;
	int *btmVtx = nullptr, *vtxBtm = nullptr, *femVtx = nullptr, *femIfo = nullptr;
	int *vfdVtx = nullptr, *vfdIfo = nullptr, *elmLyr = nullptr;
	int *rowPtr = nullptr;     // N+1 (from femVtxMat rows)
	int *diagSlot = nullptr;   // N
	// sliced layout of the operators: slices of 32 consecutive rows; inside a
	// slice, block slot k of row (32 s + lane) sits at off[s] + 32 k + lane
	int nslice = 0;
	long slTotal = 0;          // slots including padding
	int *slWidth = nullptr;    // nslice: longest row of the slice
	int *slOff = nullptr;      // nslice: first slot of the slice
	std::vector<int> slOffHost;  // host copy of slOff plus slTotal at the end (per-CTA column spans)
	int *slCol = nullptr;      // slTotal: column (node) of each slot; padding points at the row itself
	int *slDest = nullptr;     // Z: sliced slot of each femVtxMat slot
	int *transZ = nullptr;     // Z: femVtxMat slot of the transposed entry (j, i)
	int *asmOrder = nullptr;   // nAsm: slots assembled (diagonal slots, then i < j)
	int nAsm = 0;
	int *asmTab = nullptr;     // femIfoCols/2-1 x Z: e*16 + a*4 + b, femIfo order
	int asmCols = 0;
	signed char *sign0 = nullptr;  // initial orientation of each element
	std::vector<void *> owned;
};

// Per-element geometry record, one aligned record per element so that an
// assembly contribution reads one cache line: gradients of the barycentric
// coordinates (a = 0..D, component c at a*D + c), then the element volume
// and |det Q|.  128 bytes in 3D, 64 bytes in 2D.
template <int D> constexpr int rec_len() { return D == 3 ? 16 : 8; }
template <int D> constexpr int rec_vol() { return (D + 1) * D; }
template <int D> constexpr int rec_det() { return (D + 1) * D + 1; }

struct Geom {              // per-element geometry of one configuration
	double *rec = nullptr;     // rec_len<D>() x E, element-major
	double *frm = nullptr;     // D x E frame: tangent (2D) / normal (3D)
	double *tsv = nullptr;     // D x E transverse direction
};

// the full parameter set of one forward solve (device pointers resolved)
struct Model {
	int dim, frame;            // frame = reference frame elasticity, else layered isotropic
	int lyrNum;
	double mod[4];             // frame moduli
	const double *lyrMod = nullptr;   // device: lambda,mu per layer
	const double *lyrSpd = nullptr;   // device: D per layer
	double spdTan, spdTsv;
	double ynk[4], rea[5];
	double tauPrm[2];
	double ldmWgt; int knlOrder; double knlWidth, knlEps;
	double btmWgt, timeStp; int timeNum, cgItrMax; double cgTolSqu;
	int rdItrMax; double rdTolSqu;
	char cenKnl, dirKnl; double cenWidth, dirWidth;
	int precision;             // SA_PREC_FP64 or SA_PREC_MIXED
	int cgKernel = 0;          // SA_CG_AUTO / SA_CG_PERSISTENT / SA_CG_TWO_KERNEL
	int velocityGuess = 0;     // layered model: SA_GUESS_PREVIOUS or SA_GUESS_EXTRAPOLATE
	int kernelFree = 0;        // RKHS matrix evaluated on the fly instead of stored (too large, or requested)
};

// ---------------------------------------------------------------------------
// frame stress laws (used by the assembly and by the adjoint)
// ---------------------------------------------------------------------------
struct FrameMod { double m[4]; };

// computePreMat 2D (2D_frame/applyFrameElasticOperator.cu:7-39)
__device__ __forceinline__ void pre_frame(Mat<2> &pm, const Vec<2> &t, const Vec<2> &s, const FrameMod &md,
                                          const Mat<2> &ep)
{
	double muT = md.m[0], muS = md.m[1], muA = md.m[2];
	Vec<2> evS;
	evS.c[0] = ep.m[0][0] * s.c[0] + ep.m[0][1] * s.c[1];
	evS.c[1] = ep.m[1][0] * s.c[0] + ep.m[1][1] * s.c[1];
	double TvT = t.c[0] * (ep.m[0][0] * t.c[0] + ep.m[0][1] * t.c[1]) + t.c[1] * (ep.m[1][0] * t.c[0] + ep.m[1][1] * t.c[1]);
	double SvS = vdot(s, evS), TvS = vdot(t, evS);
	for (int i = 0; i < 2; ++i)
		for (int j = 0; j < 2; ++j) {
			double v = muT * (t.c[i] * t.c[j]) * TvT;
			v += muS * (s.c[i] * s.c[j]) * SvS;
			v += muA * (i == j ? 2.0 * t.c[i] * s.c[j] : t.c[i] * s.c[j] + s.c[i] * t.c[j]) * TvS;
			pm.m[i][j] = v;
		}
}

// computePreMat 3D (3D_frame/applyFrameElasticOperator.cu:7-111)
__device__ __forceinline__ void pre_frame(Mat<3> &pm, const Vec<3> &n, const Vec<3> &s, const FrameMod &md,
                                          const Mat<3> &ep)
{
	double ldT = md.m[0], muT = md.m[1], muS = md.m[2], muA = md.m[3];
	Vec<3> evN, evS;
	for (int i = 0; i < 3; ++i) {
		evN.c[i] = ep.m[i][0] * n.c[0] + ep.m[i][1] * n.c[1] + ep.m[i][2] * n.c[2];
		evS.c[i] = ep.m[i][0] * s.c[0] + ep.m[i][1] * s.c[1] + ep.m[i][2] * s.c[2];
	}
	double NvN = vdot(n, evN), SvS = vdot(s, evS), NvS = vdot(n, evS);
	double ldv = (ep.m[0][0] + ep.m[1][1] + ep.m[2][2]) - NvN;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) {
			double v = ldT * (i == j ? 1.0 - n.c[i] * n.c[j] : -n.c[i] * n.c[j]) * ldv;
			if (i == j) v += muT * (ep.m[i][j] - (2.0 * evN.c[i] * n.c[j]) + NvN * n.c[i] * n.c[j]);
			else v += muT * (ep.m[i][j] - (evN.c[i] * n.c[j] + n.c[i] * evN.c[j]) + NvN * n.c[i] * n.c[j]);
			v += muS * SvS * s.c[i] * s.c[j];
			if (i == j) v += muA * (2.0 * evS.c[i] * s.c[j] - NvS * 2.0 * n.c[i] * s.c[j]);
			else v += muA * ((evS.c[i] * s.c[j] + s.c[i] * evS.c[j]) - NvS * (n.c[i] * s.c[j] + s.c[i] * n.c[j]));
			pm.m[i][j] = v;
		}
}

// --------------------------------------------------------------------------
// sliced block-row matvec.  Slots are numbered slice by slice (slot idx of
// lane l = idx % 32 in a 32-slot group starting at idx - l); entry e of the
// row-major B x B block of slot idx sits at val[(idx - l) B^2 + 32 e + l].
// For a fixed block slot and entry, the 32 lanes of a warp (32 consecutive
// rows) therefore read 32 consecutive values: every load instruction of the
// matvec is one fully used 256-byte (FP64) or 128-byte (FP32) span.
// --------------------------------------------------------------------------
struct SellOp {
	int N;
	long total;
	const int *width, *off, *col;
};

inline SellOp sell_of(const Mesh &m) { return SellOp{m.N, m.slTotal, m.slWidth, m.slOff, m.slCol}; }

template <int B> constexpr int sell_vals() { return B * B; }

__device__ __forceinline__ long sell_pos(long idx, int e, int BB)
{
	long lane = idx & 31;
	return (idx - lane) * BB + 32L * e + lane;
}

template <int B, typename TM>
__device__ __forceinline__ void load_block(const TM *__restrict__ val, long, long idx, TM (&a)[B * B])
{
	const TM *p = val + sell_pos(idx, 0, B * B);
#pragma unroll
	for (int e = 0; e < B * B; ++e) a[e] = __ldg(p + 32 * e);
}

// store one assembled block into the sliced layout
template <int B>
__device__ __forceinline__ void store_block(double *val, long, long idx, const double (&a)[B][B])
{
	double *p = val + sell_pos(idx, 0, B * B);
	for (int r = 0; r < B; ++r)
		for (int c = 0; c < B; ++c) p[32 * (r * B + c)] = a[r][c];
}

// acc = row i of A x
template <int B, typename TM, typename TV>
__device__ __forceinline__ void sell_row(const SellOp &A, const TM *__restrict__ val, int i,
                                         const TV *__restrict__ x, TV (&acc)[B])
{
	for (int r = 0; r < B; ++r) acc[r] = (TV) 0;
	int s = i >> 5, lane = i & 31;
	int w = __ldg(A.width + s);
	long base = __ldg(A.off + s) + lane;
#pragma unroll 2
	for (int k = 0; k < w; ++k) {
		long idx = base + ((long) k << 5);
		int j = __ldg(A.col + idx);
		TV xj[B];
		for (int c = 0; c < B; ++c) xj[c] = x[(long) j * B + c];
		TM a[B * B];
		load_block<B, TM>(val, A.total, idx, a);
		for (int r = 0; r < B; ++r)
			for (int c = 0; c < B; ++c) acc[r] += (TV) a[r * B + c] * xj[c];
	}
}

// --------------------------------------------------------------------------
// kernels and launchers (defined in the .cu files)
// --------------------------------------------------------------------------
template <int D> void launch_elem_geom(const Mesh &m, const Model &md, const double *x, Geom &g,
                                       Status *st, bool check, cudaStream_t s);
template <int D> void launch_activity(const Mesh &m, const Model &md, const double *tau, double *fy,
                                      double *fr, cudaStream_t s);
template <int D> void launch_tau_initial(const Mesh &m, const Model &md, const double *tauVar,
                                         const double *x, double *tau, cudaStream_t s);
template <int D> void launch_yank_rhs(const Mesh &m, const Geom &g, const double *fy, double *b,
                                      cudaStream_t s);
template <int D> void launch_penalty_diag(const Mesh &m, const Model &md, const double *x, double *pd,
                                          cudaStream_t s);
// binv64 / binv32 (each optional, N x D x D): FP64 / FP32 inverses of the diagonal blocks (the block-Jacobi
// preconditioner of the FP64 velocity solves / of the FP32 inner solves of mixed precision)
template <int D> void launch_assemble_elastic(const Mesh &m, const Model &md, const Geom &g,
                                              const double *pd, double *blk, double *dinv, double *binv64,
                                              float *binv32, cudaStream_t s);
template <int D> void launch_assemble_rd(const Mesh &m, const Model &md, const Geom &g, double dt,
                                         double *Mval, double *Lval, double *dinv, cudaStream_t s);
template <int D> void launch_rd_rhs(const Mesh &m, const Geom &gNow, const double *Mnow, const double *tau,
                                    const double *fr, double dt, double *rhs, cudaStream_t s);
template <int D> void launch_advance(int N, const double *x, const double *v, double dt, double *xn,
                                     double *trajSlot, cudaStream_t s);
void launch_soa_to_aos(int N, int D, const double *soa, double *aos, cudaStream_t s);
// tangent-linear kernels of the layered model (sa_tangent.cu)
void launch_axpy64(long n, const double *x, double a, const double *y, double *out, cudaStream_t s);
// accuracy check of the varifold's FP64 exponential and square root (sa_varifold.cu): fn 0: y = exp_tab(x),
// yref = exp(x); fn 1: y = sqrt_nr(x), yref = sqrt(x)
void math_check(int fn, long n, const double *x, double *y, double *yref, cudaStream_t s);
void launch_extrap_poly(long n, int order, int t, double *v, double *hist, cudaStream_t s);
void launch_lin_extrap(long n, const double *a, const double *b, double *out, cudaStream_t s);
template <int D> void launch_geom_tan(const Mesh &m, const double *rec, const double *dx, double *drec, cudaStream_t s);
template <int D> void launch_penalty_tan(const Mesh &m, const double *x, const double *dx, double *dpd, cudaStream_t s);
template <int D> void launch_vel_tan_rhs(const Mesh &m, const Model &md, const double *rec, const double *drec,
                                         const double *fy, const double *dfy, const double *v, const double *dpd,
                                         double *out, cudaStream_t s);
template <int D> void launch_rd_tan_rhs(const Mesh &m, const Model &md, const double *Mnow, const double *recNow,
                                        const double *drecNow, const double *recNext, const double *drecNext,
                                        const double *tau, const double *fr, const double *dtau,
                                        const double *tauNext, double *out, cudaStream_t s);
template <int D> void launch_tau0_tan(const Mesh &m, const double *x, const double *tau0, const double *tv, int k,
                                      double *dtau, cudaStream_t s);
void launch_aos_to_soa(int N, int D, const double *aos, double *soa, cudaStream_t s);
// discrete adjoint kernels of the layered model (sa_adjoint.cu)
template <int D> void launch_adj_velocity(const Mesh &m, const Model &md, const double *rec, const double *fy,
                                          const double *x, const double *v, const double *nu, double *ax,
                                          double *atau, cudaStream_t s);
template <int D> void launch_adj_rd(const Mesh &m, const Model &md, const double *rec, const double *mu,
                                    const double *w, double sgnM, double sgnG, double *ax, cudaStream_t s);
template <int D> void launch_adj_moduli(const Mesh &m, const double *rec, const double *v, const double *nu,
                                        double *accLam, double *accMu, cudaStream_t s);
template <int D> void launch_adj_diffusivity(const Mesh &m, const Model &md, const double *rec, const double *mu,
                                             const double *tau, double *accD, cudaStream_t s);
void launch_adj_tau(const Mesh &m, const Model &md, const double *Mval, const double *mu, const double *tau,
                    double *atau, cudaStream_t s);
template <int D> void launch_adj_tau0_x(const Mesh &m, const double *x, const double *tau0, const double *atau,
                                        const double *tv, double *ax, cudaStream_t s);
void launch_adj_axpy(long n, const double *a, double sc, const double *b, double *out, cudaStream_t s);
template <int D> void launch_adj_velocity_frame(const Mesh &m, const Model &md, const Geom &g, const double *fy,
                                                const double *fyd, const double *x, const double *v,
                                                const double *nu, double *ax, double *atau, double *gF, double *gS,
                                                cudaStream_t s);
template <int D> void launch_adj_rd_frame(const Mesh &m, const Model &md, const Geom &g, const double *mu,
                                          const double *w, double sgnM, double sgnG, double *ax, double *gF,
                                          double *gS, cudaStream_t s);
template <int D> void launch_adj_frame_scatter(const Mesh &m, const int *rowPtr, const int *ent, const double *x,
                                               const double *gF, const double *gS, double *ax, cudaStream_t s);
void launch_act_deriv(const Mesh &m, const Model &md, const double *tau, double *fyd, double *frd, cudaStream_t s);
void launch_adj_tau_d(const Mesh &m, const Model &md, const double *Mval, const double *mu, const double *frd,
                      double *atau, cudaStream_t s);
template <int D> void launch_adj_bump_poly(const Mesh &m, const Model &md, const double *x, const double *atau,
                                           const double *tv, double *out, double *ax, cudaStream_t s);


// --------------------------------------------------------------------------
// CG solvers
// --------------------------------------------------------------------------
constexpr int kGridBarBytes = 512;   // device memory of the persistent CG's grid barrier

// Launch shapes chosen by the autotuner (shape_atrophy_gb300/autotune.py, which writes
// shape_atrophy_gb300/tuning.json; the Python API applies it with sa_set_tuning).  The defaults are the
// values it measured best on GB300.  They change how partial sums are grouped, so results are
// reproducible for a given setting.
struct Tuning {
	int persistMaxWarps = 20;      // warps per CTA cap of the persistent CG (CTAs per SM follow)
	int batchBlock = 256;          // threads per CTA of the batched (serving) CG: 128 or 256
	int batchSlicesPerWarp = 2;    // 32-row slices per warp when a batched solve's CTAs are sized
	int vfdCtasPerSm = 8;          // CTAs per SM of the varifold pair sums (column chunks)
	int mixedInnerFloor = 10;      // mixed precision: inner FP32 solves stop at 10^-k squared relative residual
	int kernelMatrixFree = 0;      // frame model: 1 = evaluate the RKHS matrix on the fly at every size
};
Tuning &tuning();

struct CgWork {            // scratch of the Jacobi CG (Chronopoulos-Gear form)
	double *r, *u, *w, *p, *sv;   // n each
	double *part;                 // partial sums: 3 x maxBlocks
	double *scal;                 // device scalars
	int maxBlocks;
	int smCount = 1;              // SMs of the device (grid of the vector kernels)
	int cgKernel = 0;             // SA_CG_AUTO / SA_CG_PERSISTENT / SA_CG_TWO_KERNEL
	void *bar = nullptr;          // grid barrier of the persistent CG kernel (kGridBarBytes, device)
	double profBytes = 0.0, profFlops = 0.0;   // algorithmic bytes / flops of the timed launches
	float *blk32 = nullptr;       // FP32 copy of the operator (mixed precision)
	float *binv32 = nullptr;      // FP32 inverses of its diagonal blocks (block-Jacobi, mixed precision)
	double *binv64 = nullptr;     // FP64 inverses of its diagonal blocks (block-Jacobi of the FP64 solves)
	float *f32 = nullptr;         // 7 n FP32 vectors of the inner solve (mixed precision)
	double *xr = nullptr;         // 3 n FP64 refinement scratch
	double *u4 = nullptr;         // 4 N: the persistent CG's gather copy of u (3-component nodes padded to 4)
	// optional CUDA-event timing of the velocity matvec kernel (k_cg_spmv)
	int profileEnabled = 0, profileOn = 0;
	cudaEvent_t ev[64] = {};
	double spmvMs = 0.0;
	long spmvCount = 0;
	long long launches = 0;       // kernel launches issued (CG loops and the time stepper)
	void *pinned = nullptr;       // two host copies of the CG status (chunk pipelining)
	cudaEvent_t chunkEv[2] = {};
	// persistent CG: slices of each CTA's row warps, balanced by slot count (device: slice ids, then column
	// cache offsets, nctas x warps each; host copy kept until its upload has completed)
	int *ctaTab = nullptr;
	long ctaTabCap = 0;           // ints allocated at ctaTab
	int ctaTabWarps = 0, ctaTabCtas = 0;
	size_t ctaTabSmem = 0;        // largest column cache of one CTA, bytes
	std::vector<int> ctaTabHost;

	CgWork() = default;
	CgWork(const CgWork &) = delete;
	CgWork &operator=(const CgWork &) = delete;
	~CgWork()
	{
		for (cudaEvent_t e : ev) if (e) cudaEventDestroy(e);
		for (cudaEvent_t e : chunkEv) if (e) cudaEventDestroy(e);
		if (pinned) cudaFreeHost(pinned);
	}
};

template <int B> int cg_jacobi(const Mesh &m, const double *blk, const double *dinv, const double *b,
                               double *x, int itrMax, double tolSqu, CgWork &w, Status *st,
                               int *itersOut, cudaStream_t s, int precision);

// ---- batched CG (many independent solves in one persistent launch) ----
struct CgJob {                 // one solve of a batched launch (device-visible)
	SellOp A;
	const void *blk, *dinv;    // operator values (TM), Jacobi inverse (TV)
	const void *binv;          // block-Jacobi inverses (TV, B x B per row) or null
	void *x, *r, *u, *w, *p, *s;   // solution (TX) and CG vectors (TV)
	double *part;              // 3 x nctas partial sums
	void *sc, *bar;            // scalars, grid barrier
	int cta0, nctas;           // CTAs of the launch that belong to this solve
};
struct CgState { int code, iters, zero, done; double rr, bb; };   // host copy of a solve's scalars
enum CgVec { kCgFp64, kCgFp32 };     // which vector set of CgWork a batched solve uses
struct BatchSolve { const Mesh *m; CgWork *cw; const void *blk; const void *dinv; void *x; const void *binv; };

// FP64 solve A x = b (x holds the initial guess): q = A x, r = b - q, u = D^-1 r, scalars; zeroes p, s
template <int B> void cg_prepare_fp64(const Mesh &m, const double *blk, const double *dinv, const double *b,
                                      double *x, int itrMax, double tolSqu, CgWork &w, cudaStream_t s);
// mixed precision, outer step: rin = b - A x (FP64 operator), |b|^2 (bb < 0: take it from b) and |rin|^2,
// and the FP32 Jacobi inverse on the first call (first != 0)
template <int B> void cg_mixed_outer(const Mesh &m, const double *blk, const double *dinv, const double *b,
                                     const double *x, double bb, int first, CgWork &w, cudaStream_t s);
// mixed precision, inner FP32 solve A d = rin to the relative tolerance innerTolSqu (d = 0 first)
template <int B> void cg_mixed_inner(const Mesh &m, int itrMax, double innerTolSqu, CgWork &w, cudaStream_t s);
// mixed precision: x += d
void cg_mixed_apply(long n, double *x, const CgWork &w, cudaStream_t s);
// one launch (or several, when the CTAs do not fit at once) over all solves
template <int B, typename TM, typename TV, typename TX>
int cg_batch_run(const std::vector<BatchSolve> &solves, int smCount, CgJob *devJobs, int maxJobs,
                  cudaStream_t s);
// x = 0 where the right-hand side was zero (after a batched FP64 solve)
template <int B> void cg_finish_fp64(const Mesh &m, double *x, CgWork &w, cudaStream_t s);
// host copy of the scalars (synchronises s)
CgState cg_state(const CgWork &w, cudaStream_t s);
size_t cg_scal_bytes();
void cg_states(const std::vector<const CgWork *> &ws, void *pinned, cudaStream_t s, std::vector<CgState> &out);
// bounded grid wait self-test: CTAs that gave up, and the abort flag they left
int barrier_selftest(cudaStream_t s, int *ctasGaveUp, int *abortFlag);
int fma_peak_selftest(cudaStream_t s, int fp64, double *tflops, double *flopsPerClockSm, double *mhz);

// frame mode K-preconditioned CG (2D/ipcg.cu:11-100) with dense K
struct KpcgWork {
	double *Ad, *Kid, *r, *Kr, *dv, *wK;  // wK tracks K^{-1} x
	double *dv2 = nullptr;                // second direction buffer of the persistent K-PCG
	void *bar = nullptr;                  // its grid barrier (kGridBarBytes)
	double *part, *scal;
	int maxBlocks;
	long partLen = 0;                     // doubles in part
};
// K: the stored kernel matrix, or null to evaluate it on the fly from the node positions q (interleaved)
template <int D> int kpcg(const Mesh &m, const Model &md, const double *blk, const double *K, const double *q,
                          const double *b, double *x, KpcgWork &w, Status *st, int *itersOut, cudaStream_t s);
template <int D> void launch_kernel_matrix(const Model &md, int N, const double *x, double *K, cudaStream_t s);
template <int D> void launch_adj_kernel_term(const Model &md, int N, const double *x, const double *alpha,
                                             const double *beta, double *ax, cudaStream_t s);

// the target-target rows of the varifold objective (they depend on the target only), kept between calls
struct VfdTargetCache {
	double *rows = nullptr;    // device, capacity doubles
	int capacity = 0;
	bool valid = false;
	int Vt = 0, precision = -1, ck = 0, dk = 0;
	double cw = 0.0, dw = 0.0;
};

// varifold objective (and node gradient) of a shape; cache (optional) keeps the target-target rows
template <int D> double varifold(const Mesh &m, const Model &md, const double *x, const double *tgtCen,
                                 const double *tgtDir, const double *tgtVol, int Vt, double *grad,
                                 cudaStream_t s, int precision, int *err, VfdTargetCache *cache = nullptr);

// column chunks of the varifold pair sums of a Vd x Vt objective
int vfd_chunk_count(int Vd, int Vt);
// the target-target rows of a Vd x Vt objective into cache.rows on stream s (the objective's own launches);
// part: varifold_target_rows_scratch(D, Vd, Vt, precision) doubles
size_t varifold_target_rows_scratch(int D, int Vd, int Vt, int precision);
template <int D> void varifold_target_rows(const Model &md, int Vd, const double *tgtCen, const double *tgtDir,
                                           const double *tgtVol, int Vt, int precision, double *part,
                                           VfdTargetCache &cache, cudaStream_t s);

// deterministic sum of n doubles on the device (returned via host)
double device_sum(const double *v, long n, double *scratch, cudaStream_t s);

// error helpers
struct CudaError { cudaError_t e; const char *where; };
struct DeviceWaitError { const char *where; };   // a bounded device-side wait gave up
#define SA_CHECK(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) throw ::sa::CudaError{_e, #x}; } while (0)

}  // namespace sa
