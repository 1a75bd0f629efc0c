// sa_adjoint.cu -- discrete adjoint (reverse mode) of the layered forward model.
//
// One step of the layered model (sa_driver.cu Stepper, the element formulas of sa_ops.cu):
//   K(x_t) v_t = b(x_t, tau_t)                       K: isotropic elasticity + btmWgt diag(pd(x_t)),
//                                                    b_i = -sum_e fbar_e vol_e g_e,l(i), fbar = mean y0 tau
//   x_t+1 = x_t + dt v_t
//   L(x_t+1) tau_t+1 = M(x_t) (tau_t + dt R(tau_t))  L = M + dt G, R(u) = rate u (1 - u)
// and J = varifold(x_T), tau_0 = h exp(-|x_0 - c|^2 / (2 sigma^2)).  Going backwards with the adjoint
// states a_x = dJ/dx_t, a_tau = dJ/dtau_t (a_x^T = the varifold gradient, a_tau^T = 0), each step solves
//   L(x_t+1) m = a_tau^t+1                    and then, with a_v = dt (a_x^t+1 - (d(L tau_t+1)/dx_t+1)^T m),
//   K(x_t) n = a_v
// (both operators are symmetric, the same CG as the forward solves) and accumulates
//   a_x^t   = a_x^t+1 - (d(L tau_t+1)/dx_t+1)^T m + (d(M w)/dx_t)^T m + (db/dx_t)^T n - (d(K v_t)/dx_t)^T n
//   a_tau^t = (I + dt diag(R'(tau_t))) M(x_t) m + y0 (db/dfbar)^T n,        w = tau_t + dt R(tau_t).
// The vector-Jacobian products are element formulas: with the basis gradients g_a (rows of Q^-1, g_0 = -sum)
// of an element, dg_a = -sum_c (g_a . dX_c) g_c, dvol = vol sum_c g_c . dX_c, and F = sum_b v_b (x) g_b,
// N = sum_b n_b (x) g_b, sigma(F) = lambda tr(F) I + mu (F + F^T) (self-adjoint):
//   d(n . K v)/dX_c   = vol (<sigma(F), N> g_c - F^T sigma(N) g_c - N^T sigma(F) g_c)
//   d(n . b)/dX_c     = -fbar vol (tr(N) g_c - N^T g_c)
//   d(m . M w)/dX_c   = |det| / mden (m^T Mloc w) g_c              (Mloc_ab = 1 + [a == b])
//   d(m . G w)/dX_c   = D_l vol ((gm . gw) g_c - gm (g_c . gw) - gw (g_c . gm)),  gm = sum_a m_a g_a
// and the bottom penalty adds btmWgt sum_faces (sum_i n_i . v_i) / dim d|face|/dX.  Per-layer moduli:
//   dJ/dlambda_l = -sum_t sum_e in l vol tr(F) tr(N),  dJ/dmu_l = -sum_t sum_e in l vol <F + F^T, N>,
//   dJ/dD_l = -sum_t sum_e in l dt vol_t+1 (gm . gtau_t+1).
// Every kernel gathers per node over its elements (or runs per element): deterministic, no atomics.
#include "sa_internal.cuh"

namespace sa {

template <int D>
__device__ __forceinline__ void load_grads(const double *R, double (&g)[D + 1][D])
{
	for (int a = 0; a <= D; ++a)
		for (int c = 0; c < D; ++c) g[a][c] = R[a * D + c];
}

// F = sum_b u_b (x) g_b for an interleaved nodal vector u
template <int D>
__device__ __forceinline__ void nodal_grad(const int *elmVtx, int E, int e, const double (&g)[D + 1][D],
                                           const double *u, double (&F)[D][D])
{
	for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) F[r][c] = 0.0;
	for (int b = 0; b <= D; ++b) {
		const double *ub = u + (long) elmVtx[(long) b * E + e] * D;
		for (int r = 0; r < D; ++r)
			for (int c = 0; c < D; ++c) F[r][c] += ub[r] * g[b][c];
	}
}

template <int D>
__device__ __forceinline__ void stress(const double (&F)[D][D], double lam, double mu, double (&S)[D][D])
{
	double tr = 0.0;
	for (int c = 0; c < D; ++c) tr += F[c][c];
	for (int r = 0; r < D; ++r)
		for (int c = 0; c < D; ++c) S[r][c] = mu * (F[r][c] + F[c][r]) + (r == c ? lam * tr : 0.0);
}

// a_x_i += d(n . b)/dX_i - d(n . K v)/dX_i over the node's elements (elasticity and yank; penalty separately);
// a_tau_i += y0 d(n . b)/dfy_i
template <int D>
__global__ void k_adj_velocity(int N, int E, const int *__restrict__ vtxElm, const int *__restrict__ elmVtx,
                               const double *__restrict__ rec, const int *__restrict__ lyr,
                               const double *__restrict__ lyrMod, const double *__restrict__ fy, double y0,
                               const double *__restrict__ v, const double *__restrict__ nu,
                               double *__restrict__ ax, double *__restrict__ atau)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double acc[D], at = 0.0;
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	const int cnt = vtxElm[i];
	for (int k = 0; k < cnt; ++k) {
		const int e = vtxElm[(1 + 2 * k) * (long) N + i], l = vtxElm[(2 + 2 * k) * (long) N + i];
		const double *R = rec + (long) e * rec_len<D>();
		double g[D + 1][D];
		load_grads<D>(R, g);
		const double vol = R[rec_vol<D>()];
		const int ly = lyr[e];
		const double lam = lyrMod[2 * ly], mu = lyrMod[2 * ly + 1];
		double F[D][D], Nm[D][D], SF[D][D], SN[D][D];
		nodal_grad<D>(elmVtx, E, e, g, v, F);
		nodal_grad<D>(elmVtx, E, e, g, nu, Nm);
		stress<D>(F, lam, mu, SF);
		stress<D>(Nm, lam, mu, SN);
		double fs = 0.0, sfn = 0.0, trN = 0.0;
		for (int b = 0; b <= D; ++b) fs += fy[elmVtx[(long) b * E + e]];
		const double fbar = fs / (D + 1);
		for (int r = 0; r < D; ++r) {
			trN += Nm[r][r];
			for (int c = 0; c < D; ++c) sfn += SF[r][c] * Nm[r][c];
		}
		const double *gc = g[l];
		for (int d = 0; d < D; ++d) {
			// (F^T sigma(N) g_c)_d = sum_r F[r][d] (sigma(N) g_c)_r; likewise N^T sigma(F) g_c and N^T g_c
			double fsn = 0.0, nsf = 0.0, ng = 0.0;
			for (int r = 0; r < D; ++r) {
				double sng = 0.0, sfg = 0.0;
				for (int c = 0; c < D; ++c) { sng += SN[r][c] * gc[c]; sfg += SF[r][c] * gc[c]; }
				fsn += F[r][d] * sng;
				nsf += Nm[r][d] * sfg;
				ng += Nm[r][d] * gc[r];
			}
			const double dPhi = vol * (sfn * gc[d] - fsn - nsf);
			const double dPsi = -fbar * vol * (trN * gc[d] - ng);
			acc[d] += dPsi - dPhi;
		}
		at += -vol * trN / (D + 1);        // d(n . b)/dfy_i: fy_i enters fbar of each of its elements
	}
	for (int d = 0; d < D; ++d) ax[(long) i * D + d] += acc[d];
	atau[i] += y0 * at;
}

// bottom penalty: a_x_c -= btmWgt sum_{faces f at c} (sum_{i in f} n_i . v_i) / dim d|f|/dX_c
template <int D>
__global__ void k_adj_penalty(int Nb, int Bt, const int *__restrict__ vtxBtm, const int *__restrict__ btmVtx,
                              const double *__restrict__ x, const double *__restrict__ v,
                              const double *__restrict__ nu, double btmWgt, int projected, double *__restrict__ ax)
{
	int c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c >= Nb) return;
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	const int cnt = vtxBtm[c];
	for (int k = 0; k < cnt; ++k) {
		const int f = vtxBtm[(1 + 2 * k) * (long) Nb + c], l = vtxBtm[(2 + 2 * k) * (long) Nb + c];
		int q[D];
		double w = 0.0;
		for (int a = 0; a < D; ++a) {
			q[a] = btmVtx[(long) a * Bt + f];
			const Vec<D> na = load_node<D>(nu, q[a]), va = load_node<D>(v, q[a]);
			w += vdot(na, va);
		}
		double dA[D];
		if (D == 2) {
			Vec<D> t = vsub(load_node<D>(x, q[1]), load_node<D>(x, q[0]));
			const double len = sqrt(vdot(t, t));
			for (int d = 0; d < D; ++d) dA[d] = (l == 1 ? 1.0 : -1.0) * t.c[d] / len;
		} else if (projected) {
			// frame model: area of the face's (x, y) projection (3D_frame/applyPenaltyOperator.cu:13-14)
			Vec<3> a0 = load_node<3>(x, q[0]), a1 = load_node<3>(x, q[1]), a2 = load_node<3>(x, q[2]);
			Vec<3> e1 = vsub(a1, a0), e2 = vsub(a2, a0);
			const double cz = e1.c[0] * e2.c[1] - e1.c[1] * e2.c[0];
			const double sg = cz > 0.0 ? 0.5 : (cz < 0.0 ? -0.5 : 0.0);
			const double d1[2] = {e2.c[1], -e2.c[0]}, d2[2] = {-e1.c[1], e1.c[0]};
			for (int d = 0; d < 2; ++d)
				dA[d] = sg * (l == 1 ? d1[d] : (l == 2 ? d2[d] : -(d1[d] + d2[d])));
			dA[D - 1] = 0.0;
		} else {
			Vec<3> a0 = load_node<3>(x, q[0]), a1 = load_node<3>(x, q[1]), a2 = load_node<3>(x, q[2]);
			Vec<3> e1 = vsub(a1, a0), e2 = vsub(a2, a0);
			Vec<3> n = vcross(e1, e2);
			const double nl = sqrt(vdot(n, n));
			for (int d = 0; d < 3; ++d) n.c[d] /= nl;
			Vec<3> e2n = vcross(e2, n), ne1 = vcross(n, e1);
			for (int d = 0; d < 3; ++d)
				dA[d] = 0.5 * (l == 0 ? -(e2n.c[d] + ne1.c[d]) : (l == 1 ? e2n.c[d] : ne1.c[d]));
		}
		for (int d = 0; d < D; ++d) acc[d] += w / (double) D * dA[d];
	}
	for (int d = 0; d < D; ++d) ax[(long) c * D + d] -= btmWgt * acc[d];
}

// a_x_c += sgnM d(m . M w)/dX_c + sgnG dt d(m . G w)/dX_c over the node's elements (mass and diffusion at
// the geometry rec)
template <int D>
__global__ void k_adj_rd(int N, int E, const int *__restrict__ vtxElm, const int *__restrict__ elmVtx,
                         const double *__restrict__ rec, const int *__restrict__ lyr,
                         const double *__restrict__ lyrSpd, const double *__restrict__ m,
                         const double *__restrict__ w, double sgnM, double sgnG, double dt, double *__restrict__ ax)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	constexpr double mden = (D == 2 ? 24.0 : 120.0);
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	const int cnt = vtxElm[i];
	for (int k = 0; k < cnt; ++k) {
		const int e = vtxElm[(1 + 2 * k) * (long) N + i], l = vtxElm[(2 + 2 * k) * (long) N + i];
		const double *R = rec + (long) e * rec_len<D>();
		double g[D + 1][D];
		load_grads<D>(R, g);
		const double vol = R[rec_vol<D>()], det = R[rec_det<D>()];
		double ms = 0.0, ws = 0.0, mw = 0.0, gm[D], gw[D];
		for (int d = 0; d < D; ++d) { gm[d] = 0.0; gw[d] = 0.0; }
		for (int b = 0; b <= D; ++b) {
			const int nb = elmVtx[(long) b * E + e];
			const double mb = m[nb], wb = w[nb];
			ms += mb; ws += wb; mw += mb * wb;
			for (int d = 0; d < D; ++d) { gm[d] += mb * g[b][d]; gw[d] += wb * g[b][d]; }
		}
		const double mMw = ms * ws + mw;            // m^T Mloc w with Mloc = ones + identity
		double gmw = 0.0, gcw = 0.0, gcm = 0.0;
		for (int d = 0; d < D; ++d) { gmw += gm[d] * gw[d]; gcw += g[l][d] * gw[d]; gcm += g[l][d] * gm[d]; }
		const double Dl = lyrSpd[lyr[e]];
		for (int d = 0; d < D; ++d) {
			const double dM = det / mden * mMw * g[l][d];
			const double dG = Dl * vol * (gmw * g[l][d] - gm[d] * gcw - gw[d] * gcm);
			acc[d] += sgnM * dM + sgnG * dt * dG;
		}
	}
	for (int d = 0; d < D; ++d) ax[(long) i * D + d] += acc[d];
}

// per-element moduli sensitivities, accumulated over the steps: accLam -= vol tr F tr N,
// accMu -= vol <F + F^T, N> (velocity step), accD -= dt vol (gm . gtau') (reaction-diffusion step)
template <int D>
__global__ void k_adj_moduli(int E, const int *__restrict__ elmVtx, const double *__restrict__ rec,
                             const double *__restrict__ v, const double *__restrict__ nu,
                             double *__restrict__ accLam, double *__restrict__ accMu)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= E) return;
	const double *R = rec + (long) e * rec_len<D>();
	double g[D + 1][D];
	load_grads<D>(R, g);
	const double vol = R[rec_vol<D>()];
	double F[D][D], Nm[D][D];
	nodal_grad<D>(elmVtx, E, e, g, v, F);
	nodal_grad<D>(elmVtx, E, e, g, nu, Nm);
	double trF = 0.0, trN = 0.0, s = 0.0;
	for (int r = 0; r < D; ++r) {
		trF += F[r][r];
		trN += Nm[r][r];
		for (int c = 0; c < D; ++c) s += (F[r][c] + F[c][r]) * Nm[r][c];
	}
	accLam[e] -= vol * trF * trN;
	accMu[e] -= vol * s;
}

template <int D>
__global__ void k_adj_diffusivity(int E, const int *__restrict__ elmVtx, const double *__restrict__ rec,
                                  const double *__restrict__ m, const double *__restrict__ tau, double dt,
                                  double *__restrict__ accD)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= E) return;
	const double *R = rec + (long) e * rec_len<D>();
	double s = 0.0, gm[D], gt[D];
	for (int d = 0; d < D; ++d) { gm[d] = 0.0; gt[d] = 0.0; }
	for (int b = 0; b <= D; ++b) {
		const int nb = elmVtx[(long) b * E + e];
		for (int d = 0; d < D; ++d) { gm[d] += m[nb] * R[b * D + d]; gt[d] += tau[nb] * R[b * D + d]; }
	}
	for (int d = 0; d < D; ++d) s += gm[d] * gt[d];
	accD[e] -= dt * R[rec_vol<D>()] * s;
}

// a_tau_i = (1 + dt R'(tau_i)) (M m)_i with M in CSR (symmetric), R' = rate (1 - 2 tau)
__global__ void k_adj_tau(int N, const int *__restrict__ rowPtr, const int *__restrict__ col,
                          const double *__restrict__ Mval, const double *__restrict__ m,
                          const double *__restrict__ tau, double rate, double dt, double *__restrict__ atau)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double s = 0.0;
	for (int z = rowPtr[i]; z < rowPtr[i + 1]; ++z) s += Mval[z] * m[col[z]];
	atau[i] = (1.0 + dt * rate * (1.0 - 2.0 * tau[i])) * s;
}

// the bump's dependence on the initial shape: a_x_i += a_tau_i dtau0_i/dx_i = -a_tau_i tau0_i (x_i - c) / s^2
template <int D>
__global__ void k_adj_tau0_x(int N, const double *__restrict__ x, const double *__restrict__ tau0,
                             const double *__restrict__ atau, double cx, double cy, double cz, double sg,
                             double *__restrict__ ax)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	const double c[3] = {cx, cy, cz};
	for (int d = 0; d < D; ++d)
		ax[(long) i * D + d] -= atau[i] * tau0[i] * (x[(long) i * D + d] - c[d]) / (sg * sg);
}

// out = a + s b (out may alias a)
__global__ void k_adj_axpy(long n, const double *a, double s, const double *__restrict__ b, double *out)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) out[k] = a[k] + s * b[k];
}

// ---------------------------------------------------------------------------
// frame model (the reference's own): frame stress S(eps; f, s) of 2D_frame/ and 3D_frame/
// applyFrameElasticOperator.cu (pre_frame, self-adjoint as a bilinear form), anisotropic diffusion
// T = spdTan f f^T + spdTsv s s^T (2D) or spdTan (I - n n^T) + spdTsv s s^T (3D), frames built from other
// nodes (normalised sums of edge directions, 3D normals of two triangles), activity templates, the dense
// RKHS term (sa_kernel.cu) and the polynomial bump.  With A = sym F, B = sym N:
//   2D: dPhi/df = vol (muT (2 (f.Bf) A f + 2 (f.Af) B f) + 2 muA ((f.Bs) A s + (f.As) B s)),
//       dPhi/ds = vol (muS (2 (s.Bs) A s + 2 (s.As) B s) + 2 muA ((f.Bs) A f + (f.As) B f));
//   3D: dPhi/dn = vol (ldT (-2 A n trp(B) - 2 B n trp(A)) + muT (-2 (AB + BA) n + 2 (n.Bn) A n + 2 (n.An) B n)
//                      - 2 muA ((n.Bs) A s + (n.As) B s)),  trp(A) = tr A - n.An,
//       dPhi/ds = vol (muS (2 (s.Bs) A s + 2 (s.As) B s) + muA (2 (AB + BA) s - 2 (n.Bs) A n - 2 (n.As) B n)).
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void frame_of(const double *frm, const double *tsv, int E, int e, Vec<D> &f, Vec<D> &sv)
{
	for (int d = 0; d < D; ++d) { f.c[d] = frm[d * (long) E + e]; sv.c[d] = tsv[d * (long) E + e]; }
}

template <int D>
__device__ __forceinline__ void frame_stress(const double (&A)[D][D], const Vec<D> &f, const Vec<D> &sv,
                                             const FrameMod &fm, double (&S)[D][D])
{
	Mat<D> ep, pm;
	for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) ep.m[r][c] = A[r][c];
	pre_frame(pm, f, sv, fm, ep);
	for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) S[r][c] = pm.m[r][c];
}

template <int D>
__device__ __forceinline__ void matvec(const double (&A)[D][D], const Vec<D> &x, Vec<D> &y)
{
	for (int r = 0; r < D; ++r) {
		double v = 0.0;
		for (int c = 0; c < D; ++c) v += A[r][c] * x.c[c];
		y.c[r] = v;
	}
}

template <int D>
__device__ __forceinline__ void sym_of(const double (&F)[D][D], double (&A)[D][D])
{
	for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) A[r][c] = 0.5 * (F[r][c] + F[c][r]);
}

// a_x_i += d(n . b)/dX_i - d(n . E v)/dX_i at fixed frames (frame stress), a_tau_i += fyd_i d(n . b)/dfy_i
template <int D>
__global__ void k_adj_velocity_frame(int N, int E, const int *__restrict__ vtxElm, const int *__restrict__ elmVtx,
                                     const double *__restrict__ rec, const double *__restrict__ frm,
                                     const double *__restrict__ tsv, FrameMod fm, const double *__restrict__ fy,
                                     const double *__restrict__ fyd, const double *__restrict__ v,
                                     const double *__restrict__ nu, double *__restrict__ ax, double *__restrict__ atau)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double acc[D], at = 0.0;
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	const int cnt = vtxElm[i];
	for (int k = 0; k < cnt; ++k) {
		const int e = vtxElm[(1 + 2 * k) * (long) N + i], l = vtxElm[(2 + 2 * k) * (long) N + i];
		const double *R = rec + (long) e * rec_len<D>();
		double g[D + 1][D];
		load_grads<D>(R, g);
		const double vol = R[rec_vol<D>()];
		Vec<D> f, sv;
		frame_of<D>(frm, tsv, E, e, f, sv);
		double F[D][D], Nm[D][D], A[D][D], B[D][D], SF[D][D], SN[D][D];
		nodal_grad<D>(elmVtx, E, e, g, v, F);
		nodal_grad<D>(elmVtx, E, e, g, nu, Nm);
		sym_of<D>(F, A);
		sym_of<D>(Nm, B);
		frame_stress<D>(A, f, sv, fm, SF);
		frame_stress<D>(B, f, sv, fm, SN);
		double fs = 0.0, sfn = 0.0, trN = 0.0;
		for (int b = 0; b <= D; ++b) fs += fy[elmVtx[(long) b * E + e]];
		const double fbar = fs / (D + 1);
		for (int r = 0; r < D; ++r) {
			trN += Nm[r][r];
			for (int c = 0; c < D; ++c) sfn += SF[r][c] * Nm[r][c];
		}
		const double *gc = g[l];
		for (int d = 0; d < D; ++d) {
			double fsn = 0.0, nsf = 0.0, ng = 0.0;
			for (int r = 0; r < D; ++r) {
				double sng = 0.0, sfg = 0.0;
				for (int c = 0; c < D; ++c) { sng += SN[r][c] * gc[c]; sfg += SF[r][c] * gc[c]; }
				fsn += F[r][d] * sng;
				nsf += Nm[r][d] * sfg;
				ng += Nm[r][d] * gc[r];
			}
			acc[d] += -fbar * vol * (trN * gc[d] - ng) - vol * (sfn * gc[d] - fsn - nsf);
		}
		at += -vol * trN / (D + 1);
	}
	for (int d = 0; d < D; ++d) ax[(long) i * D + d] += acc[d];
	atau[i] += fyd[i] * at;
}

// per element: sgn d(n . E v)/d(frame vectors), added to gF (tangent / normal) and gS (transverse), D x E
template <int D>
__global__ void k_adj_frame_grads_elastic(int E, const int *__restrict__ elmVtx, const double *__restrict__ rec,
                                          const double *__restrict__ frm, const double *__restrict__ tsv,
                                          FrameMod fm, const double *__restrict__ v, const double *__restrict__ nu,
                                          double sgn, double *__restrict__ gF, double *__restrict__ gS)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= E) return;
	const double *R = rec + (long) e * rec_len<D>();
	double g[D + 1][D];
	load_grads<D>(R, g);
	const double vol = R[rec_vol<D>()];
	Vec<D> f, sv;
	frame_of<D>(frm, tsv, E, e, f, sv);
	double F[D][D], Nm[D][D], A[D][D], B[D][D];
	nodal_grad<D>(elmVtx, E, e, g, v, F);
	nodal_grad<D>(elmVtx, E, e, g, nu, Nm);
	sym_of<D>(F, A);
	sym_of<D>(Nm, B);
	Vec<D> Af, Bf, As, Bs;
	matvec<D>(A, f, Af); matvec<D>(B, f, Bf); matvec<D>(A, sv, As); matvec<D>(B, sv, Bs);
	const double fBf = vdot(f, Bf), fAf = vdot(f, Af), sBs = vdot(sv, Bs), sAs = vdot(sv, As);
	const double fBs = vdot(f, Bs), fAs = vdot(f, As);
	double gf[D], gs[D];
	if (D == 2) {
		const double muT = fm.m[0], muS = fm.m[1], muA = fm.m[2];
		for (int d = 0; d < D; ++d) {
			gf[d] = muT * (2.0 * fBf * Af.c[d] + 2.0 * fAf * Bf.c[d]) + 2.0 * muA * (fBs * As.c[d] + fAs * Bs.c[d]);
			gs[d] = muS * (2.0 * sBs * As.c[d] + 2.0 * sAs * Bs.c[d]) + 2.0 * muA * (fBs * Af.c[d] + fAs * Bf.c[d]);
		}
	} else {
		const double ldT = fm.m[0], muT = fm.m[1], muS = fm.m[2], muA = fm.m[3];
		double trA = -fAf, trB = -fBf;
		for (int r = 0; r < D; ++r) { trA += A[r][r]; trB += B[r][r]; }
		// M = AB + BA applied to n (f) and to s
		Vec<D> ABf, BAf, ABs, BAs;
		matvec<D>(A, Bf, ABf); matvec<D>(B, Af, BAf); matvec<D>(A, Bs, ABs); matvec<D>(B, As, BAs);
		for (int d = 0; d < D; ++d) {
			gf[d] = ldT * (-2.0 * Af.c[d] * trB - 2.0 * Bf.c[d] * trA)
			      + muT * (-2.0 * (ABf.c[d] + BAf.c[d]) + 2.0 * fBf * Af.c[d] + 2.0 * fAf * Bf.c[d])
			      - 2.0 * muA * (fBs * As.c[d] + fAs * Bs.c[d]);
			gs[d] = muS * (2.0 * sBs * As.c[d] + 2.0 * sAs * Bs.c[d])
			      + muA * (2.0 * (ABs.c[d] + BAs.c[d]) - 2.0 * fBs * Af.c[d] - 2.0 * fAs * Bf.c[d]);
		}
	}
	for (int d = 0; d < D; ++d) {
		gF[d * (long) E + e] += sgn * vol * gf[d];
		gS[d * (long) E + e] += sgn * vol * gs[d];
	}
}

// per element: sgn d(m . G w)/d(frame vectors) of the anisotropic diffusion, added to gF, gS
template <int D>
__global__ void k_adj_frame_grads_diff(int E, const int *__restrict__ elmVtx, const double *__restrict__ rec,
                                       const double *__restrict__ frm, const double *__restrict__ tsv, double spdTan,
                                       double spdTsv, const double *__restrict__ m, const double *__restrict__ w,
                                       double sgn, double *__restrict__ gF, double *__restrict__ gS)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= E) return;
	const double *R = rec + (long) e * rec_len<D>();
	const double vol = R[rec_vol<D>()];
	Vec<D> f, sv, gm, gw;
	frame_of<D>(frm, tsv, E, e, f, sv);
	for (int d = 0; d < D; ++d) { gm.c[d] = 0.0; gw.c[d] = 0.0; }
	for (int b = 0; b <= D; ++b) {
		const int nb = elmVtx[(long) b * E + e];
		for (int d = 0; d < D; ++d) { gm.c[d] += m[nb] * R[b * D + d]; gw.c[d] += w[nb] * R[b * D + d]; }
	}
	const double fm_ = vdot(f, gm), fw = vdot(f, gw), sm = vdot(sv, gm), sw = vdot(sv, gw);
	const double cf = D == 2 ? spdTan : -spdTan;        // 3D: the tangential projection removes n n^T
	for (int d = 0; d < D; ++d) {
		gF[d * (long) E + e] += sgn * vol * cf * (fw * gm.c[d] + fm_ * gw.c[d]);
		gS[d * (long) E + e] += sgn * vol * spdTsv * (sw * gm.c[d] + sm * gw.c[d]);
	}
}

// a_x_c += sgnM d(m . M w)/dX_c + sgnG dt d(m . G w)/dX_c at fixed frames, G the anisotropic diffusion
template <int D>
__global__ void k_adj_rd_frame(int N, int E, const int *__restrict__ vtxElm, const int *__restrict__ elmVtx,
                               const double *__restrict__ rec, const double *__restrict__ frm,
                               const double *__restrict__ tsv, double spdTan, double spdTsv,
                               const double *__restrict__ m, const double *__restrict__ w, double sgnM, double sgnG,
                               double dt, double *__restrict__ ax)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	constexpr double mden = (D == 2 ? 24.0 : 120.0);
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	const int cnt = vtxElm[i];
	for (int k = 0; k < cnt; ++k) {
		const int e = vtxElm[(1 + 2 * k) * (long) N + i], l = vtxElm[(2 + 2 * k) * (long) N + i];
		const double *R = rec + (long) e * rec_len<D>();
		double g[D + 1][D];
		load_grads<D>(R, g);
		const double vol = R[rec_vol<D>()], det = R[rec_det<D>()];
		Vec<D> f, sv, gm, gw, gc;
		frame_of<D>(frm, tsv, E, e, f, sv);
		double ms = 0.0, ws = 0.0, mw = 0.0;
		for (int d = 0; d < D; ++d) { gm.c[d] = 0.0; gw.c[d] = 0.0; gc.c[d] = g[l][d]; }
		for (int b = 0; b <= D; ++b) {
			const int nb = elmVtx[(long) b * E + e];
			const double mb = m[nb], wb = w[nb];
			ms += mb; ws += wb; mw += mb * wb;
			for (int d = 0; d < D; ++d) { gm.c[d] += mb * g[b][d]; gw.c[d] += wb * g[b][d]; }
		}
		// T u for T = spdTan f f^T + spdTsv s s^T (2D) or spdTan (I - n n^T) + spdTsv s s^T (3D)
		auto T = [&](const Vec<D> &u, Vec<D> &o) {
			const double fu = vdot(f, u), su = vdot(sv, u);
			for (int d = 0; d < D; ++d)
				o.c[d] = (D == 2 ? spdTan * fu * f.c[d] : spdTan * (u.c[d] - fu * f.c[d])) + spdTsv * su * sv.c[d];
		};
		Vec<D> Tw, Tm;
		T(gw, Tw);
		T(gm, Tm);
		const double mTw = vdot(gm, Tw), cTw = vdot(gc, Tw), cTm = vdot(gc, Tm);
		for (int d = 0; d < D; ++d) {
			const double dM = det / mden * (ms * ws + mw) * gc.c[d];
			const double dG = vol * (mTw * gc.c[d] - cTw * gm.c[d] - cTm * gw.c[d]);
			acc[d] += sgnM * dM + sgnG * dt * dG;
		}
	}
	for (int d = 0; d < D; ++d) ax[(long) i * D + d] += acc[d];
}

// Vector-Jacobian product of the element frames with respect to the nodes that build them.  Node i gathers
// over (element, role) entries: role r of frmVtx (2D: pair r / 2, end r % 2; 3D: triangle r / 3, vertex
// r % 3) or of tsvVtx (pair r / 2, end r % 2), entry code e * 16 + which * 8 + r (which 0: frmVtx, 1: tsvVtx).
// Frame = normalise(sum of unit vectors): with y = S / |S|, the gradient on S is (g - (g.y) y) / |S|, on an
// edge e = p1 - p0 (g_S - (g_S.u) u) / |e|, on a triangle normal c = e1 x e2 (g_S - (g_S.c^) c^) / |c| =: g_c,
// giving e2 x g_c on vertex 1, g_c x e1 on vertex 2 and minus their sum on vertex 0.
template <int D>
__device__ __forceinline__ void norm_sum_grad(const Vec<D> &S, const Vec<D> &g, Vec<D> &gS)
{
	const double sl = sqrt(vdot(S, S));
	double gy = 0.0;
	for (int d = 0; d < D; ++d) gy += g.c[d] * S.c[d] / sl;
	for (int d = 0; d < D; ++d) gS.c[d] = (g.c[d] - gy * S.c[d] / sl) / sl;
}

template <int D>
__device__ __forceinline__ Vec<D> pair_grad(const double *x, const int *pairs, int E, int e, int np, int role,
                                            const Vec<D> &g)
{
	Vec<D> S, ev[3];
	double el[3];
	for (int d = 0; d < D; ++d) S.c[d] = 0.0;
	for (int t = 0; t < np; ++t) {
		ev[t] = vsub(load_node<D>(x, pairs[(2 * t + 1) * (long) E + e]), load_node<D>(x, pairs[(2 * t) * (long) E + e]));
		el[t] = sqrt(vdot(ev[t], ev[t]));
		for (int d = 0; d < D; ++d) S.c[d] += ev[t].c[d] / el[t];
	}
	Vec<D> gS;
	norm_sum_grad<D>(S, g, gS);
	const int t = role >> 1;
	double gu = 0.0;
	for (int d = 0; d < D; ++d) gu += gS.c[d] * ev[t].c[d] / el[t];
	Vec<D> out;
	const double sg = (role & 1) ? 1.0 : -1.0;
	for (int d = 0; d < D; ++d) out.c[d] = sg * (gS.c[d] - gu * ev[t].c[d] / el[t]) / el[t];
	return out;
}

__device__ __forceinline__ Vec<3> normal_grad(const double *x, const int *tri, int E, int e, int role, const Vec<3> &g)
{
	Vec<3> S, c[2], e1[2], e2[2];
	double cl[2];
	for (int d = 0; d < 3; ++d) S.c[d] = 0.0;
	for (int t = 0; t < 2; ++t) {
		Vec<3> a0 = load_node<3>(x, tri[(3 * t) * (long) E + e]), a1 = load_node<3>(x, tri[(3 * t + 1) * (long) E + e]);
		Vec<3> a2 = load_node<3>(x, tri[(3 * t + 2) * (long) E + e]);
		e1[t] = vsub(a1, a0);
		e2[t] = vsub(a2, a0);
		c[t] = vcross(e1[t], e2[t]);
		cl[t] = sqrt(vdot(c[t], c[t]));
		for (int d = 0; d < 3; ++d) S.c[d] += c[t].c[d] / cl[t];
	}
	Vec<3> gS;
	norm_sum_grad<3>(S, g, gS);
	const int t = role / 3, k = role % 3;
	double gu = 0.0;
	for (int d = 0; d < 3; ++d) gu += gS.c[d] * c[t].c[d] / cl[t];
	Vec<3> gc;
	for (int d = 0; d < 3; ++d) gc.c[d] = (gS.c[d] - gu * c[t].c[d] / cl[t]) / cl[t];
	Vec<3> a1 = vcross(e2[t], gc), a2 = vcross(gc, e1[t]), out;
	for (int d = 0; d < 3; ++d) out.c[d] = k == 1 ? a1.c[d] : (k == 2 ? a2.c[d] : -(a1.c[d] + a2.c[d]));
	return out;
}

template <int D>
__global__ void k_adj_frame_scatter(int N, int E, const int *__restrict__ rowPtr, const int *__restrict__ ent,
                                    const int *__restrict__ frmVtx, const int *__restrict__ tsvVtx,
                                    const double *__restrict__ x, const double *__restrict__ gF,
                                    const double *__restrict__ gS, double *__restrict__ ax)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	for (int q = rowPtr[i]; q < rowPtr[i + 1]; ++q) {
		const int code = ent[q], e = code >> 4, which = (code >> 3) & 1, role = code & 7;
		Vec<D> g;
		const double *G = which ? gS : gF;
		for (int d = 0; d < D; ++d) g.c[d] = G[d * (long) E + e];
		Vec<D> c;
		if (which) c = pair_grad<D>(x, tsvVtx, E, e, D == 2 ? 2 : 3, role, g);
		else if (D == 2) c = pair_grad<D>(x, frmVtx, E, e, 2, role, g);
		else {
			Vec<3> g3, c3;
			for (int d = 0; d < 3; ++d) g3.c[d] = g.c[d % D];
			c3 = normal_grad(x, frmVtx, E, e, role, g3);
			for (int d = 0; d < D; ++d) c.c[d] = c3.c[d];
		}
		for (int d = 0; d < D; ++d) acc[d] += c.c[d];
	}
	for (int d = 0; d < D; ++d) ax[(long) i * D + d] += acc[d];
}

// frame-model activity derivatives fyd = d fy / d tau, frd = d fr / d tau (templates on the scaled tau)
__global__ void k_act_deriv(int N, const double *__restrict__ tau, double y0, double y1, double y2, double y3,
                            double r0, double r1, double r2, double r3, double r4, double *__restrict__ fyd,
                            double *__restrict__ frd)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	const double t = tau[i];
	const double ty = -1.0 + 2.0 * (t - y0) / (y1 - y0), tr = -1.0 + 2.0 * (t - r0) / (r1 - r0);
	fyd[i] = yank_template_d(ty, y3) * y2 * 2.0 / (y1 - y0);
	frd[i] = reac_template_d(tr, r3, r4) * r2 * 2.0 / (r1 - r0);
}

// a_tau_i = (1 + dt frd_i) (M m)_i (frame model: the reaction template's derivative per node)
__global__ void k_adj_tau_d(int N, const int *__restrict__ rowPtr, const int *__restrict__ col,
                            const double *__restrict__ Mval, const double *__restrict__ m,
                            const double *__restrict__ frd, double dt, double *__restrict__ atau)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double s = 0.0;
	for (int z = rowPtr[i]; z < rowPtr[i + 1]; ++z) s += Mval[z] * m[col[z]];
	atau[i] = (1.0 + dt * frd[i]) * s;
}

// polynomial bump tau_0 = h (1 - (1 - (q - 1)^2)^p) for q = |x - c|^2 / R^2 < 1 (2D_frame/tauInitial.cu:24-64,
// 3D_frame/tauInitial.cu:24-66): per node the parameter derivatives times a_tau (out: 4 x N, parameters
// [c (dim), h, R in 2D] / [c (3), h] in 3D) and the node-position term added to a_x
template <int D>
__global__ void k_adj_bump_poly(int N, const double *__restrict__ x, const double *__restrict__ atau, double cx,
                                double cy, double cz, double h, double R, int pw, double *__restrict__ out,
                                double *__restrict__ ax)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	const double c[3] = {cx, cy, cz};
	double s = 0.0, dx[D];
	for (int d = 0; d < D; ++d) { dx[d] = x[(long) i * D + d] - c[d]; s += dx[d] * dx[d]; }
	const double q = s / (R * R);
	double pre = 0.0, dpre = 0.0;
	if (q < 1.0) {
		const double tmp = (q - 1.0) * (q - 1.0), base = 1.0 - tmp;
		double pw1 = 1.0;
		for (int k = 1; k < pw; ++k) pw1 *= base;              // base^(p-1)
		pre = 1.0 - pw1 * base;
		dpre = pw * pw1 * 2.0 * (q - 1.0);                      // d pre / d q
	}
	const double a = atau[i];
	for (int d = 0; d < D; ++d) out[d * (long) N + i] = a * h * dpre * (-2.0 * dx[d] / (R * R));
	out[D * (long) N + i] = a * pre;
	if (D == 2) out[3 * (long) N + i] = a * h * dpre * (-2.0 * q / R);
	for (int d = 0; d < D; ++d) ax[(long) i * D + d] += a * h * dpre * 2.0 * dx[d] / (R * R);
}

template <int D>
void launch_adj_velocity(const Mesh &m, const Model &md, const double *rec, const double *fy, const double *x,
                         const double *v, const double *nu, double *ax, double *atau, cudaStream_t s)
{
	k_adj_velocity<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, m.vtxElm, m.elmVtx, rec, m.elmLyr, md.lyrMod, fy,
	                                                    md.ynk[0], v, nu, ax, atau);
	if (m.Bt > 0 && md.btmWgt != 0.0)
		k_adj_penalty<D><<<grid_for(m.Nb), kBlock, 0, s>>>(m.Nb, m.Bt, m.vtxBtm, m.btmVtx, x, v, nu, md.btmWgt, 0,
		                                                    ax);
}

template <int D>
void launch_adj_rd(const Mesh &m, const Model &md, const double *rec, const double *mu, const double *w,
                   double sgnM, double sgnG, double *ax, cudaStream_t s)
{
	k_adj_rd<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, m.vtxElm, m.elmVtx, rec, m.elmLyr, md.lyrSpd, mu, w, sgnM,
	                                              sgnG, md.timeStp, ax);
}

template <int D>
void launch_adj_moduli(const Mesh &m, const double *rec, const double *v, const double *nu, double *accLam,
                       double *accMu, cudaStream_t s)
{
	k_adj_moduli<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, rec, v, nu, accLam, accMu);
}

template <int D>
void launch_adj_diffusivity(const Mesh &m, const Model &md, const double *rec, const double *mu, const double *tau,
                            double *accD, cudaStream_t s)
{
	k_adj_diffusivity<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, rec, mu, tau, md.timeStp, accD);
}

void launch_adj_tau(const Mesh &m, const Model &md, const double *Mval, const double *mu, const double *tau,
                    double *atau, cudaStream_t s)
{
	k_adj_tau<<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.rowPtr, m.femVtx + m.Z, Mval, mu, tau, md.rea[0], md.timeStp,
	                                           atau);
}

template <int D>
void launch_adj_tau0_x(const Mesh &m, const double *x, const double *tau0, const double *atau, const double *tv,
                       double *ax, cudaStream_t s)
{
	k_adj_tau0_x<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, x, tau0, atau, tv[0], tv[1], D == 3 ? tv[2] : 0.0,
	                                                  tv[D + 1], ax);
}

void launch_adj_axpy(long n, const double *a, double sc, const double *b, double *out, cudaStream_t s)
{
	k_adj_axpy<<<grid_for(n), kBlock, 0, s>>>(n, a, sc, b, out);
}

template <int D>
void launch_adj_velocity_frame(const Mesh &m, const Model &md, const Geom &g, const double *fy, const double *fyd,
                               const double *x, const double *v, const double *nu, double *ax, double *atau,
                               double *gF, double *gS, cudaStream_t s)
{
	FrameMod fm;
	for (int k = 0; k < 4; ++k) fm.m[k] = md.mod[k];
	k_adj_velocity_frame<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, m.vtxElm, m.elmVtx, g.rec, g.frm, g.tsv, fm,
	                                                          fy, fyd, v, nu, ax, atau);
	k_adj_frame_grads_elastic<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, g.rec, g.frm, g.tsv, fm, v, nu,
	                                                               -1.0, gF, gS);
	if (m.Bt > 0 && md.btmWgt != 0.0)
		k_adj_penalty<D><<<grid_for(m.Nb), kBlock, 0, s>>>(m.Nb, m.Bt, m.vtxBtm, m.btmVtx, x, v, nu, md.btmWgt, 1,
		                                                    ax);
}

template <int D>
void launch_adj_rd_frame(const Mesh &m, const Model &md, const Geom &g, const double *mu, const double *w,
                         double sgnM, double sgnG, double *ax, double *gF, double *gS, cudaStream_t s)
{
	k_adj_rd_frame<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, m.vtxElm, m.elmVtx, g.rec, g.frm, g.tsv, md.spdTan,
	                                                    md.spdTsv, mu, w, sgnM, sgnG, md.timeStp, ax);
	if (sgnG != 0.0 && gF)
		k_adj_frame_grads_diff<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, g.rec, g.frm, g.tsv, md.spdTan,
		                                                            md.spdTsv, mu, w, sgnG * md.timeStp, gF, gS);
}

template <int D>
void launch_adj_frame_scatter(const Mesh &m, const int *rowPtr, const int *ent, const double *x, const double *gF,
                              const double *gS, double *ax, cudaStream_t s)
{
	k_adj_frame_scatter<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.E, rowPtr, ent, m.frmVtx, m.tsvVtx, x, gF, gS, ax);
}

void launch_act_deriv(const Mesh &m, const Model &md, const double *tau, double *fyd, double *frd, cudaStream_t s)
{
	k_act_deriv<<<grid_for(m.N), kBlock, 0, s>>>(m.N, tau, md.ynk[0], md.ynk[1], md.ynk[2], md.ynk[3], md.rea[0],
	                                             md.rea[1], md.rea[2], md.rea[3], md.rea[4], fyd, frd);
}

void launch_adj_tau_d(const Mesh &m, const Model &md, const double *Mval, const double *mu, const double *frd,
                      double *atau, cudaStream_t s)
{
	k_adj_tau_d<<<grid_for(m.N), kBlock, 0, s>>>(m.N, m.rowPtr, m.femVtx + m.Z, Mval, mu, frd, md.timeStp, atau);
}

template <int D>
void launch_adj_bump_poly(const Mesh &m, const Model &md, const double *x, const double *atau, const double *tv,
                          double *out, double *ax, cudaStream_t s)
{
	double h = D == 2 ? tv[2] : tv[3], R = D == 2 ? tv[3] : md.tauPrm[0];
	int pw = (int) (D == 2 ? md.tauPrm[0] : md.tauPrm[1]);
	k_adj_bump_poly<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, x, atau, tv[0], tv[1], D == 3 ? tv[2] : 0.0, h, R, pw,
	                                                     out, ax);
}

#define SA_ADJ_INST(D)                                                                                            \
	template void launch_adj_velocity<D>(const Mesh &, const Model &, const double *, const double *,             \
	                                     const double *, const double *, const double *, double *, double *,      \
	                                     cudaStream_t);                                                           \
	template void launch_adj_rd<D>(const Mesh &, const Model &, const double *, const double *, const double *,   \
	                               double, double, double *, cudaStream_t);                                       \
	template void launch_adj_moduli<D>(const Mesh &, const double *, const double *, const double *, double *,    \
	                                   double *, cudaStream_t);                                                   \
	template void launch_adj_diffusivity<D>(const Mesh &, const Model &, const double *, const double *,          \
	                                        const double *, double *, cudaStream_t);                              \
	template void launch_adj_tau0_x<D>(const Mesh &, const double *, const double *, const double *,              \
	                                   const double *, double *, cudaStream_t);                                   \
	template void launch_adj_velocity_frame<D>(const Mesh &, const Model &, const Geom &, const double *,         \
	                                           const double *, const double *, const double *, const double *,    \
	                                           double *, double *, double *, double *, cudaStream_t);             \
	template void launch_adj_rd_frame<D>(const Mesh &, const Model &, const Geom &, const double *, const double *, \
	                                     double, double, double *, double *, double *, cudaStream_t);             \
	template void launch_adj_frame_scatter<D>(const Mesh &, const int *, const int *, const double *,             \
	                                          const double *, const double *, double *, cudaStream_t);            \
	template void launch_adj_bump_poly<D>(const Mesh &, const Model &, const double *, const double *,            \
	                                      const double *, double *, double *, cudaStream_t);
SA_ADJ_INST(2)
SA_ADJ_INST(3)

}  // namespace sa
