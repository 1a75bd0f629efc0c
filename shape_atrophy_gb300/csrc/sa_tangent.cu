// sa_tangent.cu -- tangent-linear (forward sensitivity) kernels of the layered model.
//
// Differentiating one time step of the layered forward model (element
// geometry, isotropic elasticity, bottom penalty, yank load, mass, diffusion,
// Fisher-KPP load) along a direction of the bump parameters gives, per step,
//   K(x_t) dv = db - (dK v) - btmWgt dpd v                 (velocity tangent)
//   L(x_t+1) dtau' = dM_t (tau + dt R) + M_t (dtau + dt R' dtau)
//                    - (dM_t+1 + dt dG_t+1) tau'           (concentration tangent)
//   dx_t+1 = dx_t + dt dv
// with the operators K and L the forward step already assembled.  The kernels
// below form the geometry tangent and the right-hand sides; the solves use the
// same CG as the forward model.  Element formulas (layered model, sa_ops.cu):
//   K_ab = vol (lambda g_a g_b^T + mu (g_a.g_b) I + mu g_b g_a^T),  i.e. (K v)_a = vol sigma(F) g_a with
//          F = sum_b v_b (x) g_b and sigma(F) = lambda tr(F) I + mu (F + F^T)
//   M_ab = (1 + [a == b]) |det| / 24 (2D), / 120 (3D)
//   G_ab = vol D_l g_a.g_b,   b_i = -sum_e fbar_e vol_e g_l,   fbar = mean of y0 tau over the element
// Geometry tangent (P = Q^{-1}, rows g_1..g_D, g_0 = -sum):
//   dg_a = -sum_b (g_a . dX_b) g_b,   dvol = vol sum_a g_a . dX_a,   d|det| = |det| sum_a g_a . dX_a.
#include "sa_internal.cuh"

namespace sa {

__device__ __forceinline__ Vec<3> vadd3(const Vec<3> &a, const Vec<3> &b)
{
	Vec<3> r;
	for (int c = 0; c < 3; ++c) r.c[c] = a.c[c] + b.c[c];
	return r;
}

template <int D>
__global__ void k_geom_tan(int E, const int *__restrict__ elmVtx, const double *__restrict__ rec,
                           const double *__restrict__ dx, double *__restrict__ drec)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= E) return;
	const double *R = rec + (long) e * rec_len<D>();
	double g[D + 1][D], dX[D + 1][D];
	for (int a = 0; a <= D; ++a) {
		for (int c = 0; c < D; ++c) g[a][c] = R[a * D + c];
		Vec<D> q = load_node<D>(dx, elmVtx[(long) a * E + e]);
		for (int c = 0; c < D; ++c) dX[a][c] = q.c[c];
	}
	double s[D + 1][D + 1];                 // s[a][b] = g_a . dX_b
	double tr = 0.0;
	for (int a = 0; a <= D; ++a)
		for (int b = 0; b <= D; ++b) {
			double v = 0.0;
			for (int c = 0; c < D; ++c) v += g[a][c] * dX[b][c];
			s[a][b] = v;
			if (a == b) tr += v;
		}
	double o[rec_len<D>()];
	for (int a = 0; a <= D; ++a)
		for (int c = 0; c < D; ++c) {
			double v = 0.0;
			for (int b = 0; b <= D; ++b) v -= s[a][b] * g[b][c];
			o[a * D + c] = v;
		}
	o[rec_vol<D>()] = R[rec_vol<D>()] * tr;
	o[rec_det<D>()] = R[rec_det<D>()] * tr;
	for (int k = rec_det<D>() + 1; k < rec_len<D>(); ++k) o[k] = 0.0;
	double *out = drec + (long) e * rec_len<D>();
	for (int k = 0; k < rec_len<D>(); ++k) out[k] = o[k];
}

// tangent of the bottom-penalty diagonal pd_i = sum over bottom faces of |face| / D (unprojected)
template <int D>
__global__ void k_penalty_tan(int N, int Nb, int Bt, const int *__restrict__ vtxBtm, const int *__restrict__ btmVtx,
                              const double *__restrict__ x, const double *__restrict__ dx, double *__restrict__ dpd)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double acc = 0.0;
	if (i < Nb) {
		int cnt = vtxBtm[i];
		for (int a = 0; a < cnt; ++a) {
			int f = vtxBtm[(1 + 2 * a) * (long) Nb + i];
			double dm;
			if (D == 2) {
				Vec<D> t = vsub(load_node<D>(x, btmVtx[Bt + f]), load_node<D>(x, btmVtx[f]));
				Vec<D> dt = vsub(load_node<D>(dx, btmVtx[Bt + f]), load_node<D>(dx, btmVtx[f]));
				dm = vdot(t, dt) / sqrt(vdot(t, t));
			} else {
				Vec<3> a0 = load_node<3>(x, btmVtx[f]), a1 = load_node<3>(x, btmVtx[Bt + f]);
				Vec<3> a2 = load_node<3>(x, btmVtx[2 * Bt + f]);
				Vec<3> d0 = load_node<3>(dx, btmVtx[f]), d1 = load_node<3>(dx, btmVtx[Bt + f]);
				Vec<3> d2 = load_node<3>(dx, btmVtx[2 * Bt + f]);
				Vec<3> e1 = vsub(a1, a0), e2 = vsub(a2, a0);
				Vec<3> n = vcross(e1, e2);
				Vec<3> dn = vadd3(vcross(vsub(d1, d0), e2), vcross(e1, vsub(d2, d0)));
				dm = 0.5 * vdot(n, dn) / sqrt(vdot(n, n));
			}
			acc += dm / (double) D;
		}
	}
	dpd[i] = acc;
}

// sigma(F) g = lambda tr(F) g + mu (F + F^T) g
template <int D>
__device__ __forceinline__ void stress_apply(const double (&F)[D][D], double lam, double mu, const double *g,
                                             double (&out)[D])
{
	double tr = 0.0;
	for (int c = 0; c < D; ++c) tr += F[c][c];
	for (int r = 0; r < D; ++r) {
		double v = lam * tr * g[r];
		for (int c = 0; c < D; ++c) v += mu * (F[r][c] + F[c][r]) * g[c];
		out[r] = v;
	}
}

// velocity tangent right-hand side: db - dK v - btmWgt dpd v, node by node over the node's elements
template <int D>
__global__ void k_vel_tan_rhs(int N, int E, int Nb, const int *__restrict__ vtxElm, const int *__restrict__ elmVtx,
                              const double *__restrict__ rec, const double *__restrict__ drec,
                              const int *__restrict__ lyr, const double *__restrict__ lyrMod,
                              const double *__restrict__ fy, const double *__restrict__ dfy,
                              const double *__restrict__ v, const double *__restrict__ dpd, double btmWgt,
                              double *__restrict__ out)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	int cnt = vtxElm[i];
	for (int a = 0; a < cnt; ++a) {
		int e = vtxElm[(1 + 2 * a) * (long) N + i], l = vtxElm[(2 + 2 * a) * (long) N + i];
		const double *R = rec + (long) e * rec_len<D>(), *dR = drec + (long) e * rec_len<D>();
		const double vol = R[rec_vol<D>()], dvol = dR[rec_vol<D>()];
		const int ly = lyr[e];
		const double lam = lyrMod[2 * ly], mu = lyrMod[2 * ly + 1];
		double F[D][D], dF[D][D];
		for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) { F[r][c] = 0.0; dF[r][c] = 0.0; }
		double fs = 0.0, dfs = 0.0;
		for (int b = 0; b <= D; ++b) {
			const int nb = elmVtx[(long) b * E + e];
			fs += fy[nb];
			dfs += dfy[nb];
			const double *vb = v + (long) nb * D;
			for (int r = 0; r < D; ++r)
				for (int c = 0; c < D; ++c) {
					F[r][c] += vb[r] * R[b * D + c];
					dF[r][c] += vb[r] * dR[b * D + c];
				}
		}
		const double fc = fs / (D + 1), dfc = dfs / (D + 1);
		const double *gl = R + l * D, *dgl = dR + l * D;
		double s1[D], s2[D], s3[D];
		stress_apply<D>(F, lam, mu, gl, s1);      // sigma(F) g_l
		stress_apply<D>(dF, lam, mu, gl, s2);     // sigma(dF) g_l
		stress_apply<D>(F, lam, mu, dgl, s3);     // sigma(F) dg_l
		for (int d = 0; d < D; ++d) {
			const double db = -(dfc * vol * gl[d] + fc * dvol * gl[d] + fc * vol * dgl[d]);
			const double dKv = dvol * s1[d] + vol * (s2[d] + s3[d]);
			acc[d] += db - dKv;
		}
	}
	if (i < Nb)
		for (int d = 0; d < D; ++d) acc[d] -= btmWgt * dpd[i] * v[(long) i * D + d];
	for (int d = 0; d < D; ++d) out[(long) i * D + d] = acc[d];
}

// concentration tangent right-hand side
template <int D>
__global__ void k_rd_tan_rhs(int N, int E, const int *__restrict__ rowPtr, const int *__restrict__ col,
                             const double *__restrict__ Mnow, const int *__restrict__ vtxElm,
                             const int *__restrict__ elmVtx, const int *__restrict__ lyr,
                             const double *__restrict__ lyrSpd, const double *__restrict__ recNow,
                             const double *__restrict__ drecNow, const double *__restrict__ recNext,
                             const double *__restrict__ drecNext, const double *__restrict__ tau,
                             const double *__restrict__ fr, const double *__restrict__ dtau,
                             const double *__restrict__ tauNext, double rate, double dt, double *__restrict__ out)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	constexpr double mden = (D == 2 ? 24.0 : 120.0);
	// M_t (dtau + dt R'(tau) dtau), R' = rate (1 - 2 tau)
	double acc = 0.0;
	for (int z = rowPtr[i]; z < rowPtr[i + 1]; ++z) {
		const int j = col[z];
		acc += Mnow[z] * (dtau[j] + dt * rate * (1.0 - 2.0 * tau[j]) * dtau[j]);
	}
	int cnt = vtxElm[i];
	for (int a = 0; a < cnt; ++a) {
		int e = vtxElm[(1 + 2 * a) * (long) N + i], l = vtxElm[(2 + 2 * a) * (long) N + i];
		const double *Rn = recNow + (long) e * rec_len<D>(), *dRn = drecNow + (long) e * rec_len<D>();
		const double *Rx = recNext + (long) e * rec_len<D>(), *dRx = drecNext + (long) e * rec_len<D>();
		const double Dl = lyrSpd[lyr[e]];
		const double volx = Rx[rec_vol<D>()], dvolx = dRx[rec_vol<D>()];
		double mNow = 0.0, mNext = 0.0, gNext = 0.0;
		for (int k = 0; k <= D; ++k) {
			const int nk = elmVtx[(long) k * E + e];
			const double w = (k == l ? 2.0 : 1.0);
			mNow += w * (tau[nk] + dt * fr[nk]);
			mNext += w * tauNext[nk];
			double gg = 0.0, dgg = 0.0;
			for (int c = 0; c < D; ++c) {
				gg += Rx[l * D + c] * Rx[k * D + c];
				dgg += dRx[l * D + c] * Rx[k * D + c] + Rx[l * D + c] * dRx[k * D + c];
			}
			gNext += (dvolx * gg + volx * dgg) * tauNext[nk];
		}
		acc += dRn[rec_det<D>()] / mden * mNow;            // dM_t (tau + dt R)
		acc -= dRx[rec_det<D>()] / mden * mNext;           // dM_t+1 tau'
		acc -= dt * Dl * gNext;                            // dt dG_t+1 tau'
	}
	out[i] = acc;
}

// tangent of the initial concentration tau_0 = h exp(-|x - c|^2 / (2 s^2)) along parameter k of [c, h, s]
template <int D>
__global__ void k_tau0_tan(int N, const double *__restrict__ x, const double *__restrict__ tau0, double cx,
                           double cy, double cz, double h, double sg, int k, double *__restrict__ dtau)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	const double c[3] = {cx, cy, cz};
	double r2 = 0.0;
	for (int d = 0; d < D; ++d) { double t = x[(long) i * D + d] - c[d]; r2 += t * t; }
	const double t0 = tau0[i];
	double v;
	if (k < D) v = t0 * (x[(long) i * D + k] - c[k]) / (sg * sg);
	else if (k == D) v = exp(-r2 / (2.0 * sg * sg));
	else v = t0 * r2 / (sg * sg * sg);
	dtau[i] = v;
}

// Polynomial extrapolation of the next CG start from the previous solutions: v holds x_t-1, hist[j n ..]
// holds x_t-2-j (j < depth).  With q of them usable, v <- sum_{j=0..q} (-1)^j C(q+1, j+1) x_t-1-j (the
// degree-q polynomial through the last q+1 solutions, evaluated one step ahead); then the history shifts.
constexpr int kMaxGuessOrder = 5;
__constant__ double c_binom[kMaxGuessOrder + 1][kMaxGuessOrder + 1] = {
	{1, 0, 0, 0, 0, 0},
	{2, -1, 0, 0, 0, 0},
	{3, -3, 1, 0, 0, 0},
	{4, -6, 4, -1, 0, 0},
	{5, -10, 10, -5, 1, 0},
	{6, -15, 20, -15, 6, -1},
};

__global__ void k_extrap_poly(long n, int q, int depth, double *__restrict__ v, double *__restrict__ hist)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k >= n) return;
	double h[kMaxGuessOrder + 1];
	h[0] = v[k];
	for (int j = 1; j <= depth; ++j) h[j] = hist[(long) (j - 1) * n + k];
	if (q > 0) {
		double s = 0.0;
		for (int j = 0; j <= q; ++j) s += c_binom[q][j] * h[j];
		v[k] = s;
	}
	for (int j = depth - 1; j >= 1; --j) hist[(long) j * n + k] = h[j];
	if (depth > 0) hist[k] = h[0];
}

void launch_extrap_poly(long n, int order, int t, double *v, double *hist, cudaStream_t s)
{
	const int depth = order < kMaxGuessOrder ? order : kMaxGuessOrder;
	int q = t - 1;                       // previous solutions x_0 .. x_t-1: degree at most t - 1
	if (q > depth) q = depth;
	if (q < 0) q = 0;
	if (depth > 0) k_extrap_poly<<<grid_for(n), kBlock, 0, s>>>(n, q, depth, v, hist);
}

// out = 2 a - b (out may alias b)
__global__ void k_lin_extrap(long n, const double *__restrict__ a, const double *b, double *out)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) out[k] = 2.0 * a[k] - b[k];
}

void launch_lin_extrap(long n, const double *a, const double *b, double *out, cudaStream_t s)
{
	k_lin_extrap<<<grid_for(n), kBlock, 0, s>>>(n, a, b, out);
}

__global__ void k_axpy64(long n, const double *__restrict__ x, double a, const double *__restrict__ y,
                         double *__restrict__ out)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) out[k] = x[k] + a * y[k];
}

void launch_axpy64(long n, const double *x, double a, const double *y, double *out, cudaStream_t s)
{
	k_axpy64<<<grid_for(n), kBlock, 0, s>>>(n, x, a, y, out);
}

template <int D>
void launch_geom_tan(const Mesh &m, const double *rec, const double *dx, double *drec, cudaStream_t s)
{
	k_geom_tan<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, rec, dx, drec);
}

template <int D>
void launch_penalty_tan(const Mesh &m, const double *x, const double *dx, double *dpd, cudaStream_t s)
{
	k_penalty_tan<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.Nb, m.Bt, m.vtxBtm, m.btmVtx, x, dx, dpd);
}

template <int D>
void launch_vel_tan_rhs(const Mesh &m, const Model &md, const double *rec, const double *drec, const double *fy,
                        const double *dfy, const double *v, const double *dpd, double *out, cudaStream_t s)
{
	const double bw = (m.Bt > 0 && md.btmWgt != 0.0) ? md.btmWgt : 0.0;
	k_vel_tan_rhs<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, m.Nb, m.vtxElm, m.elmVtx, rec, drec, m.elmLyr,
	                                                   md.lyrMod, fy, dfy, v, dpd, bw, out);
}

template <int D>
void launch_rd_tan_rhs(const Mesh &m, const Model &md, const double *Mnow, const double *recNow,
                       const double *drecNow, const double *recNext, const double *drecNext, const double *tau,
                       const double *fr, const double *dtau, const double *tauNext, double *out, cudaStream_t s)
{
	k_rd_tan_rhs<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, m.rowPtr, m.femVtx + m.Z, Mnow, m.vtxElm, m.elmVtx,
	                                                  m.elmLyr, md.lyrSpd, recNow, drecNow, recNext, drecNext, tau,
	                                                  fr, dtau, tauNext, md.rea[0], md.timeStp, out);
}

template <int D>
void launch_tau0_tan(const Mesh &m, const double *x, const double *tau0, const double *tv, int k, double *dtau,
                     cudaStream_t s)
{
	k_tau0_tan<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, x, tau0, tv[0], tv[1], D == 3 ? tv[2] : 0.0, tv[D],
	                                                tv[D + 1], k, dtau);
}

#define SA_TAN_INST(D)                                                                                           \
	template void launch_geom_tan<D>(const Mesh &, const double *, const double *, double *, cudaStream_t);      \
	template void launch_penalty_tan<D>(const Mesh &, const double *, const double *, double *, cudaStream_t);   \
	template void launch_vel_tan_rhs<D>(const Mesh &, const Model &, const double *, const double *,              \
	                                    const double *, const double *, const double *, const double *, double *, \
	                                    cudaStream_t);                                                            \
	template void launch_rd_tan_rhs<D>(const Mesh &, const Model &, const double *, const double *,               \
	                                   const double *, const double *, const double *, const double *,            \
	                                   const double *, const double *, const double *, double *, cudaStream_t);   \
	template void launch_tau0_tan<D>(const Mesh &, const double *, const double *, const double *, int, double *, \
	                                 cudaStream_t);
SA_TAN_INST(2)
SA_TAN_INST(3)

}  // namespace sa
