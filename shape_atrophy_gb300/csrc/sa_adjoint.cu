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
	                                   const double *, double *, cudaStream_t);
SA_ADJ_INST(2)
SA_ADJ_INST(3)

}  // namespace sa
