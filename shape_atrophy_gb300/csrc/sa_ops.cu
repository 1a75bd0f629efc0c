// sa_ops.cu -- per-step element, assembly and vector kernels.
//
// Reference counterparts (CUDA/ folder of the reference):
//   element geometry + frame   2D_frame/vertexToEdge.cu:4-27, computeFrame.cu:4-78,
//                              3D_frame/computeFrame.cu:6-78
//   activity functions         2D_frame/yankTauActivity.cu:4-33, reactionTauActivity.cu:4-35
//   initial chemical           2D_frame/tauInitial.cu:24-64, 3D_frame/tauInitial.cu:24-66
//   yank right-hand side       2D_frame/computeExternalYank.cu:5-47 (element), :86-122 (gather)
//   elasticity operator        2D_frame/computeStrainTensor.cu:4-44, applyFrameElasticOperator.cu:7-111,
//                              3D_frame/applyFrameElasticOperator.cu:7-190 -- assembled here into
//                              D x D blocks on the femVtxMat pattern (one FP64 block-CSR matvec
//                              per CG iteration instead of three element/gather kernels)
//   bottom penalty             2D_frame/applyPenaltyOperator.cu:4-63, 3D_frame :4-69 (diagonal)
//   mass / diffusion           2D_frame/assembleFemMatrix.cu:5-92, 3D_frame :5-151 (same femIfoMat
//                              gather order; CSR values instead of dense N x N)
//   reaction load + RD rhs     2D_frame/assembleFemVector.cu:5-54, deform.cu:89-97
//   node update                2D_frame/deform.cu:81-82
#include "sa_internal.cuh"

namespace sa {

// ---------------------------------------------------------------------------
// element geometry: gradients of the barycentric coordinates, |det Q|,
// volume, orientation check and (frame mode) the element frame
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_elem_geom(int E, const int *__restrict__ elmVtx, const double *__restrict__ x,
                            double *__restrict__ rec,
                            int frame, const int *__restrict__ frmVtx, const int *__restrict__ tsvVtx,
                            double *__restrict__ frm, double *__restrict__ tsv,
                            const signed char *__restrict__ sign0, int *inverted)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= E) return;
	Vec<D> q0 = load_node<D>(x, elmVtx[e]);
	Vec<D> q[D];
	for (int k = 0; k < D; ++k) q[k] = vsub(load_node<D>(x, elmVtx[(k + 1) * E + e]), q0);
	double det = det_edges<D>(q);
	Mat<D> QI = inv_edges<D>(q, det);
	double r[rec_len<D>()];
	// gradient of phi_0 is minus the column sums of Q^{-1} (reference order: -a - b - c)
	for (int c = 0; c < D; ++c) {
		double s = -QI.m[0][c];
		for (int k = 1; k < D; ++k) s = s - QI.m[k][c];
		r[c] = s;
		for (int k = 0; k < D; ++k) r[(k + 1) * D + c] = QI.m[k][c];
	}
	double ad = fabs(det);
	r[rec_vol<D>()] = (D == 2 ? 0.5 * ad : ad / 6.0);   // inc/utility.h:11-29
	r[rec_det<D>()] = ad;
	for (int k = rec_det<D>() + 1; k < rec_len<D>(); ++k) r[k] = 0.0;
	double2 *o = reinterpret_cast<double2 *>(rec + (long) e * rec_len<D>());
	for (int k = 0; k < rec_len<D>() / 2; ++k) o[k] = make_double2(r[2 * k], r[2 * k + 1]);
	if (sign0) {
		signed char sg = det > 0.0 ? 1 : (det < 0.0 ? -1 : 0);
		if (sg != sign0[e]) atomicAdd(inverted, 1);
	}
	if (!frame) return;
	Vec<D> s; for (int d = 0; d < D; ++d) s.c[d] = 0.0;
	if (D == 2) {
		for (int t = 0; t < 2; ++t) {
			Vec<D> df = vsub(load_node<D>(x, frmVtx[(2 * t + 1) * E + e]), load_node<D>(x, frmVtx[(2 * t) * E + e]));
			double len = sqrt(vdot(df, df));
			for (int d = 0; d < D; ++d) s.c[d] += df.c[d] / len;
		}
	} else {
		for (int t = 0; t < 2; ++t) {
			Vec<3> a0 = load_node<3>(x, frmVtx[(3 * t) * E + e]);
			Vec<3> a1 = load_node<3>(x, frmVtx[(3 * t + 1) * E + e]);
			Vec<3> a2 = load_node<3>(x, frmVtx[(3 * t + 2) * E + e]);
			Vec<3> cr = vcross(vsub(a1, a0), vsub(a2, a0));
			double len = sqrt(vdot(cr, cr));
			for (int d = 0; d < 3; ++d) s.c[d] += cr.c[d] / len;
		}
	}
	double sl = sqrt(vdot(s, s));
	for (int d = 0; d < D; ++d) frm[d * (long) E + e] = s.c[d] / sl;
	Vec<D> u; for (int d = 0; d < D; ++d) u.c[d] = 0.0;
	const int tsvNum = (D == 2 ? 2 : 3);
	for (int t = 0; t < tsvNum; ++t) {
		Vec<D> df = vsub(load_node<D>(x, tsvVtx[(2 * t + 1) * E + e]), load_node<D>(x, tsvVtx[(2 * t) * E + e]));
		double len = sqrt(vdot(df, df));
		for (int d = 0; d < D; ++d) u.c[d] += df.c[d] / len;
	}
	double ul = sqrt(vdot(u, u));
	for (int d = 0; d < D; ++d) tsv[d * (long) E + e] = u.c[d] / ul;
}

template <int D>
void launch_elem_geom(const Mesh &m, const Model &md, const double *x, Geom &g, Status *st, bool check,
                      cudaStream_t s)
{
	k_elem_geom<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, x, g.rec, md.frame, m.frmVtx, m.tsvVtx, g.frm,
	                                                  g.tsv, check ? m.sign0 : nullptr, &st->inverted);
}

// ---------------------------------------------------------------------------
// activity functions: yank f(tau) and reaction R(tau), per node
// ---------------------------------------------------------------------------
struct ActPrm { double y[4]; double r[5]; int frame; };

__global__ void k_activity(int N, const double *__restrict__ tau, double *__restrict__ fy,
                           double *__restrict__ fr, ActPrm p)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double t = tau[i];
	if (p.frame) {
		// inc/activity.h:81-89 and 239-249
		double ty = -1.0 + 2.0 * (t - p.y[0]) / (p.y[1] - p.y[0]);
		fy[i] = yank_template(ty, p.y[3]) * p.y[2];
		double tr = -1.0 + 2.0 * (t - p.r[0]) / (p.r[1] - p.r[0]);
		fr[i] = reac_template(tr, p.r[3], p.r[4]) * p.r[2];
	} else {
		fy[i] = p.y[0] * t;                    // atrophy eigenstrain f(u) = c u
		fr[i] = p.r[0] * t * (1.0 - t);        // Fisher-KPP R(u) = rate u (1 - u)
	}
}

template <int D>
void launch_activity(const Mesh &m, const Model &md, const double *tau, double *fy, double *fr, cudaStream_t s)
{
	ActPrm p;
	for (int k = 0; k < 4; ++k) p.y[k] = md.ynk[k];
	for (int k = 0; k < 5; ++k) p.r[k] = md.rea[k];
	p.frame = md.frame;
	k_activity<<<grid_for(m.N), kBlock, 0, s>>>(m.N, tau, fy, fr, p);
}

// ---------------------------------------------------------------------------
// initial chemical
// ---------------------------------------------------------------------------
__device__ __forceinline__ double intpow(double b, int e)
{   // 2D_frame/tauInitial.cu:4-22
	double out = 1, pw = b;
	do {
		int q = e >> 1, r = e - 2 * q;
		if (r == 1) out *= pw;
		pw *= pw;
		e = q;
	} while (e != 0);
	return out;
}

struct TauPrm { double c[3]; double hgt, rad; int pw; int frame; };

template <int D>
__global__ void k_tau_initial(int N, const double *__restrict__ x, double *__restrict__ tau, TauPrm p)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	Vec<D> q = load_node<D>(x, i);
	if (p.frame) {
		double r2 = p.rad * p.rad;
		double s = (q.c[0] - p.c[0]) * (q.c[0] - p.c[0]);
		for (int d = 1; d < D; ++d) s = s + (q.c[d] - p.c[d]) * (q.c[d] - p.c[d]);
		double radSqu = s / r2;
		double tmp = (radSqu - 1.0) * (radSqu - 1.0);
		double pre = (radSqu < 1.0 ? 1.0 - intpow(1.0 - tmp, p.pw) : 0.0);
		tau[i] = p.hgt * pre;
	} else {
		double r2 = 0.0;
		for (int d = 0; d < D; ++d) { double t = q.c[d] - p.c[d]; r2 += t * t; }
		tau[i] = p.hgt * exp(-r2 / (2.0 * p.rad * p.rad));      // Gaussian bump
	}
}

template <int D>
void launch_tau_initial(const Mesh &m, const Model &md, const double *tv, const double *x, double *tau,
                        cudaStream_t s)
{
	TauPrm p{};
	p.frame = md.frame;
	for (int d = 0; d < D; ++d) p.c[d] = tv[d];
	if (md.frame) {
		if (D == 2) { p.hgt = tv[2]; p.rad = tv[3]; p.pw = (int) md.tauPrm[0]; }   // [cx, cy, h, R], [p]
		else { p.hgt = tv[3]; p.rad = md.tauPrm[0]; p.pw = (int) md.tauPrm[1]; }    // [c, h], [R, p]
	} else {
		p.hgt = tv[D]; p.rad = tv[D + 1];                                            // [c, h, sigma]
	}
	k_tau_initial<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, x, tau, p);
}

// ---------------------------------------------------------------------------
// yank right-hand side b_i = sum_{e ∋ i} -fbar_e vol_e grad(phi_l)
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_yank_rhs(int N, int E, const int *__restrict__ vtxElm, const int *__restrict__ elmVtx,
                           const double *__restrict__ rec, const double *__restrict__ fy, double *__restrict__ b)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	int cnt = vtxElm[i];
	for (int a = 0; a < cnt; ++a) {
		int e = vtxElm[(1 + 2 * a) * (long) N + i], l = vtxElm[(2 + 2 * a) * (long) N + i];
		double fs = fy[elmVtx[e]];
		for (int k = 1; k <= D; ++k) fs = fs + fy[elmVtx[k * (long) E + e]];
		double fc = fs / (D + 1);
		const double *R = rec + (long) e * rec_len<D>();
		double v = R[rec_vol<D>()];
		for (int d = 0; d < D; ++d) acc[d] = acc[d] + -fc * R[l * D + d] * v;
	}
	for (int d = 0; d < D; ++d) b[(long) i * D + d] = acc[d];
}

template <int D>
void launch_yank_rhs(const Mesh &m, const Geom &g, const double *fy, double *b, cudaStream_t s)
{
	k_yank_rhs<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, m.vtxElm, m.elmVtx, g.rec, fy, b);
}

// ---------------------------------------------------------------------------
// bottom penalty diagonal: pd_i = sum over bottom faces of |face| / (V-1).
// As in penaltyGatherKernel the value belongs to node index i of vtxBtmMat,
// which must be the face vertex itself (bottom nodes numbered first);
// other layouts are rejected at set-up.
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_penalty_diag(int N, int Nb, int Bt, const int *__restrict__ vtxBtm,
                               const int *__restrict__ btmVtx, const double *__restrict__ x, int projected,
                               double *__restrict__ pd)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double acc = 0.0;
	if (i < Nb) {
		int cnt = vtxBtm[i];
		for (int a = 0; a < cnt; ++a) {
			int f = vtxBtm[(1 + 2 * a) * (long) Nb + i];
			Vec<D> q0 = load_node<D>(x, btmVtx[f]);
			Vec<D> q1 = load_node<D>(x, btmVtx[Bt + f]);
			double meas;
			if (D == 2) {
				Vec<D> t = vsub(q1, q0);
				meas = sqrt(vdot(t, t));
			} else {
				Vec<3> a0 = load_node<3>(x, btmVtx[f]), a1 = load_node<3>(x, btmVtx[Bt + f]);
				Vec<3> a2 = load_node<3>(x, btmVtx[2 * Bt + f]);
				if (projected)   // 3D_frame/applyPenaltyOperator.cu:13-14: (x, y) projection
					meas = 0.5 * fabs((a1.c[0] - a0.c[0]) * (a2.c[1] - a0.c[1]) - (a1.c[1] - a0.c[1]) * (a2.c[0] - a0.c[0]));
				else {
					Vec<3> cr = vcross(vsub(a1, a0), vsub(a2, a0));
					meas = 0.5 * sqrt(vdot(cr, cr));
				}
			}
			acc += meas / (double) D;     // |face| / (VTXNUM - 1)
		}
	}
	pd[i] = acc;
}

template <int D>
void launch_penalty_diag(const Mesh &m, const Model &md, const double *x, double *pd, cudaStream_t s)
{
	k_penalty_diag<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.Nb, m.Bt, m.vtxBtm, m.btmVtx, x,
	                                                    md.frame, pd);
}

// ---------------------------------------------------------------------------
// elasticity block assembly: one thread per femVtxMat slot (i, j) with
// i <= j, diagonal slots first (Mesh::asmOrder); the contributions are the elements listed for the slot in
// femIfoMat (same order), with ordered local indices (a, b) precomputed in
// asmTab.  The block of (j, i) is the transpose and is written by the same
// thread, so the assembled operator is exactly symmetric.
//   isotropic: K_ab = vol (lambda g_a g_b^T + mu (g_a.g_b) I + mu g_b g_a^T)
//   frame:     column c of K_ab = vol * preMat(sym(e_c (x) g_b))^T g_a
// Diagonal slots add btmWgt * pd_i * I and write the Jacobi inverse.
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_asm_elastic(int Z, int E, int asmCols, const int *__restrict__ femVtx,
                              const int *__restrict__ femIfo, const int *__restrict__ asmTab,
                              const double *__restrict__ rec,
                              int frame, FrameMod fm, const double *__restrict__ frm, const double *__restrict__ tsv,
                              const int *__restrict__ lyr, const double *__restrict__ lyrMod,
                              double btmWgt, const double *__restrict__ pd, int Nb,
                              const int *__restrict__ slDest, const int *__restrict__ transZ, long total,
                              const int *__restrict__ order, int nOrd,
                              double *__restrict__ blk, double *__restrict__ dinv, double *__restrict__ binv64,
                              float *__restrict__ binv32)
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nOrd) return;
	const int z = order[t];
	const int i = femVtx[z], j = femVtx[Z + z];
	if (i > j) return;                       // written by the thread of (j, i)
	double acc[D][D];
	for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) acc[r][c] = 0.0;
	int cnt = femIfo[z];
	for (int k = 0; k < cnt; ++k) {
		int code = asmTab[k * (long) Z + z];
		int e = code >> 4, a = (code >> 2) & 3, b = code & 3;
		const double *R = rec + (long) e * rec_len<D>();
		double v = R[rec_vol<D>()];
		Vec<D> ga, gb;
		for (int c = 0; c < D; ++c) { ga.c[c] = R[a * D + c]; gb.c[c] = R[b * D + c]; }
		if (!frame) {
			int l = lyr[e];
			double vl = v * lyrMod[2 * l], vm = v * lyrMod[2 * l + 1];
			double la[D], ma[D];
			for (int r = 0; r < D; ++r) { la[r] = vl * ga.c[r]; ma[r] = vm * ga.c[r]; }
			double dg = vm * vdot(ga, gb);
			for (int r = 0; r < D; ++r) {
				for (int c = 0; c < D; ++c) acc[r][c] += la[r] * gb.c[c] + gb.c[r] * ma[c];
				acc[r][r] += dg;
			}
		} else {
			Vec<D> fa, sa;
			for (int d = 0; d < D; ++d) { fa.c[d] = frm[d * (long) E + e]; sa.c[d] = tsv[d * (long) E + e]; }
			for (int c = 0; c < D; ++c) {
				Mat<D> ep, pm;
				for (int i2 = 0; i2 < D; ++i2)
					for (int j2 = 0; j2 < D; ++j2)
						ep.m[i2][j2] = 0.5 * ((i2 == c ? gb.c[j2] : 0.0) + (j2 == c ? gb.c[i2] : 0.0));
				pre_frame(pm, fa, sa, fm, ep);
				for (int r = 0; r < D; ++r) {
					double f = 0.0;
					for (int kk = 0; kk < D; ++kk) f += ga.c[kk] * pm.m[kk][r];
					acc[r][c] += v * f;
				}
			}
		}
	}
	if (i == j) {
		double p = (i < Nb) ? btmWgt * pd[i] : 0.0;
		for (int d = 0; d < D; ++d) {
			acc[d][d] += p;
			dinv[(long) i * D + d] = 1.0 / acc[d][d];
		}
		store_block<D>(blk, total, slDest[z], acc);
		if (binv64 || binv32) {            // block-Jacobi preconditioner (FP64 solves, FP32 inner solves)
			Mat<D> a, inv;
			for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) a.m[r][c] = acc[r][c];
			inv = mat_inverse<D>(a);
			for (int r = 0; r < D; ++r)
				for (int c = 0; c < D; ++c) {
					const long k = (long) i * D * D + r * D + c;
					if (binv64) binv64[k] = inv.m[r][c];
					if (binv32) binv32[k] = (float) inv.m[r][c];
				}
		}
		return;
	}
	store_block<D>(blk, total, slDest[z], acc);
	double tr[D][D];
	for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) tr[r][c] = acc[c][r];
	store_block<D>(blk, total, slDest[transZ[z]], tr);
}

template <int D>
void launch_assemble_elastic(const Mesh &m, const Model &md, const Geom &g, const double *pd, double *blk,
                             double *dinv, double *binv64, float *binv32, cudaStream_t s)
{
	FrameMod fm;
	for (int k = 0; k < 4; ++k) fm.m[k] = md.mod[k];
	k_asm_elastic<D><<<grid_for(m.nAsm, 128), 128, 0, s>>>(m.Z, m.E, m.asmCols, m.femVtx, m.femIfo, m.asmTab, g.rec,
	                                                        md.frame, fm, g.frm, g.tsv, m.elmLyr, md.lyrMod, md.btmWgt,
	                                                        pd, m.Nb, m.slDest, m.transZ, m.slTotal, m.asmOrder,
	                                                        m.nAsm, blk, dinv, binv64, binv32);
}

// ---------------------------------------------------------------------------
// reaction-diffusion matrices: M (mass) and L = M + dt G (diffusion), CSR
// values on the femVtxMat pattern, gathered in femIfoMat order
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ double ggd_value(int frame, int e, int E, int a, int b, const double *R,
                                            double absDet, const double *frm, const double *tsv,
                                            double spdTan, double spdTsv, double Dl)
{
	Vec<D> ga, gb;
	for (int c = 0; c < D; ++c) { ga.c[c] = R[a * D + c]; gb.c[c] = R[b * D + c]; }
	if (!frame) {
		double mvol = (D == 2 ? 0.5 * absDet : absDet / 6.0);
		return mvol * (Dl * vdot(ga, gb));
	}
	// frame: projections of the gradients on the frame, with the phi_0
	// projection formed as minus the sum (2D_frame/assembleFemMatrix.cu:28-34)
	Vec<D> f, s;
	for (int d = 0; d < D; ++d) { f.c[d] = frm[d * (long) E + e]; s.c[d] = tsv[d * (long) E + e]; }
	double fP[D + 1], sP[D + 1];
	for (int k = 1; k <= D; ++k) {
		Vec<D> gk;
		for (int c = 0; c < D; ++c) gk.c[c] = R[k * D + c];
		fP[k] = vdot(gk, f); sP[k] = vdot(gk, s);
	}
	fP[0] = -fP[1]; sP[0] = -sP[1];
	for (int k = 2; k <= D; ++k) { fP[0] = fP[0] - fP[k]; sP[0] = sP[0] - sP[k]; }
	if (D == 2)
		return 0.5 * absDet * (spdTan * fP[a] * fP[b] + spdTsv * sP[a] * sP[b]);
	double gg = ga.c[0] * gb.c[0] + ga.c[1] * gb.c[1] + ga.c[2] * gb.c[2];
	return absDet / 6.0 * (spdTan * (gg - fP[a] * fP[b]) + spdTsv * sP[a] * sP[b]);
}

// one thread per slot (i, j) with i <= j; M and G are symmetric (the
// femIfoMat lists of (i, j) and (j, i) hold the same elements in the same
// order), so the thread writes both entries
template <int D>
__global__ void k_asm_rd(int Z, int E, const int *__restrict__ femVtx, const int *__restrict__ femIfo,
                         const int *__restrict__ asmTab, const double *__restrict__ rec, int frame,
                         const double *__restrict__ frm, const double *__restrict__ tsv, double spdTan, double spdTsv,
                         const int *__restrict__ lyr, const double *__restrict__ lyrSpd, double dt,
                         const int *__restrict__ slDest, const int *__restrict__ transZ,
                         const int *__restrict__ order, int nOrd,
                         double *__restrict__ Mval, double *__restrict__ Lval, double *__restrict__ dinv)
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nOrd) return;
	const int z = order[t];
	const int i = femVtx[z], j = femVtx[Z + z];
	if (i > j) return;
	int cnt = femIfo[z];
	double mul = femIfo[Z + z];
	double M = 0.0, Gs = 0.0;
	for (int k = 0; k < cnt; ++k) {
		int code = asmTab[k * (long) Z + z];
		int e = code >> 4, a = (code >> 2) & 3, b = code & 3;
		int lo = a < b ? a : b, hi = a < b ? b : a;
		const double *R = rec + (long) e * rec_len<D>();
		double ad = R[rec_det<D>()];
		M += mul * (ad / (D == 2 ? 24.0 : 120.0));
		double Dl = frame ? 0.0 : lyrSpd[lyr[e]];
		Gs += ggd_value<D>(frame, e, E, lo, hi, R, ad, frm, tsv, spdTan, spdTsv, Dl);
	}
	double L = 1.0 * M + dt * Gs;
	Mval[z] = M;                 // femVtxMat (CSR) order, read by the next step's right-hand side
	Lval[slDest[z]] = L;         // sliced layout, read by the CG matvec
	if (i == j) { dinv[i] = 1.0 / L; return; }
	int zt = transZ[z];
	Mval[zt] = M;
	Lval[slDest[zt]] = L;
}

template <int D>
void launch_assemble_rd(const Mesh &m, const Model &md, const Geom &g, double dt, double *Mval, double *Lval,
                        double *dinv, cudaStream_t s)
{
	k_asm_rd<D><<<grid_for(m.nAsm), kBlock, 0, s>>>(m.Z, m.E, m.femVtx, m.femIfo, m.asmTab, g.rec, md.frame, g.frm,
	                                                 g.tsv, md.spdTan, md.spdTsv, m.elmLyr, md.lyrSpd, dt, m.slDest,
	                                                 m.transZ, m.asmOrder, m.nAsm, Mval, Lval, dinv);
}

// rhs_i = (M_t tau_t)_i + dt * sum_{e ∋ i} (tau-weighted consistent mass load)
template <int D>
__global__ void k_rd_rhs(int N, int E, const int *__restrict__ rowPtr, const int *__restrict__ col,
                         const double *__restrict__ Mnow, const double *__restrict__ tau,
                         const int *__restrict__ vtxElm, const int *__restrict__ elmVtx,
                         const double *__restrict__ rec, const double *__restrict__ fr, double dt,
                         double *__restrict__ rhs)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double mt = 0.0;
	for (int z = rowPtr[i]; z < rowPtr[i + 1]; ++z) mt += Mnow[z] * tau[col[z]];
	double rp = 0.0;
	int cnt = vtxElm[i];
	for (int a = 0; a < cnt; ++a) {
		int e = vtxElm[(1 + 2 * a) * (long) N + i], l = vtxElm[(2 + 2 * a) * (long) N + i];
		double s = 0.0;
		for (int k = 0; k <= D; ++k) {
			double f = fr[elmVtx[k * (long) E + e]];
			s = s + (k == l ? 2.0 * f : f);
		}
		rp += s * rec[(long) e * rec_len<D>() + rec_det<D>()] / (D == 2 ? 24.0 : 120.0);
	}
	rhs[i] = 1.0 * mt + dt * rp;
}

template <int D>
void launch_rd_rhs(const Mesh &m, const Geom &gNow, const double *Mnow, const double *tau, const double *fr,
                   double dt, double *rhs, cudaStream_t s)
{
	k_rd_rhs<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, m.rowPtr, m.femVtx + m.Z, Mnow, tau, m.vtxElm, m.elmVtx,
	                                             gNow.rec, fr, dt, rhs);
}

// ---------------------------------------------------------------------------
// node update and trajectory output
// ---------------------------------------------------------------------------
__global__ void k_advance(int N, int D, const double *__restrict__ x, const double *__restrict__ v, double dt,
                          double *__restrict__ xn, double *__restrict__ traj)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k >= (long) N * D) return;
	double y = 1.0 * x[k] + dt * v[k];
	xn[k] = y;
	if (traj) traj[(k % D) * N + k / D] = y;
}

template <int D>
void launch_advance(int N, const double *x, const double *v, double dt, double *xn, double *trajSlot, cudaStream_t s)
{
	k_advance<<<grid_for((long) N * D), kBlock, 0, s>>>(N, D, x, v, dt, xn, trajSlot);
}

__global__ void k_soa_to_aos(int N, int D, const double *__restrict__ soa, double *__restrict__ aos)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k >= (long) N * D) return;
	aos[k] = soa[(k % D) * N + k / D];
}

void launch_soa_to_aos(int N, int D, const double *soa, double *aos, cudaStream_t s)
{
	k_soa_to_aos<<<grid_for((long) N * D), kBlock, 0, s>>>(N, D, soa, aos);
}

__global__ void k_aos_to_soa(int N, int D, const double *__restrict__ aos, double *__restrict__ soa)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k >= (long) N * D) return;
	soa[(k % D) * N + k / D] = aos[k];
}

void launch_aos_to_soa(int N, int D, const double *aos, double *soa, cudaStream_t s)
{
	k_aos_to_soa<<<grid_for((long) N * D), kBlock, 0, s>>>(N, D, aos, soa);
}

// explicit instantiations
#define SA_INST(D)                                                                                           \
	template void launch_elem_geom<D>(const Mesh &, const Model &, const double *, Geom &, Status *, bool,     \
	                                  cudaStream_t);                                                           \
	template void launch_activity<D>(const Mesh &, const Model &, const double *, double *, double *,          \
	                                 cudaStream_t);                                                            \
	template void launch_tau_initial<D>(const Mesh &, const Model &, const double *, const double *, double *, \
	                                    cudaStream_t);                                                         \
	template void launch_yank_rhs<D>(const Mesh &, const Geom &, const double *, double *, cudaStream_t);      \
	template void launch_penalty_diag<D>(const Mesh &, const Model &, const double *, double *, cudaStream_t); \
	template void launch_assemble_elastic<D>(const Mesh &, const Model &, const Geom &, const double *,        \
	                                         double *, double *, double *, float *, cudaStream_t);             \
	template void launch_assemble_rd<D>(const Mesh &, const Model &, const Geom &, double, double *, double *, \
	                                    double *, cudaStream_t);                                               \
	template void launch_rd_rhs<D>(const Mesh &, const Geom &, const double *, const double *, const double *, \
	                               double, double *, cudaStream_t);                                            \
	template void launch_advance<D>(int, const double *, const double *, double, double *, double *,           \
	                                cudaStream_t);
SA_INST(2)
SA_INST(3)

}  // namespace sa
