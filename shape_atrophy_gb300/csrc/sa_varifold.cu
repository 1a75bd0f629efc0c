// sa_varifold.cu -- varifold objective and its node gradient.
//
// Reference: 2D_frame/varifold.cu (3D_frame/varifold.cu):
//   landmarksToVarifoldKernel :9-36 (3D :9-43)      -> k_vfd_elems
//   geometricFunction / grassmanFunction :38-179    -> cen_knl / dir_knl
//   vfd_DD_DT, vfd_TT, vfd_TT_TD, vfd_DD :181-357   -> k_vfd_rows (one thread per row, the
//       same row/column roles and per-row accumulation order, column tiles staged in shared
//       memory so a CTA reads each column record once per tile instead of once per thread)
//   dqVfd_DD_DT + dqVfdGather :359-498 (3D :372-530) -> k_vfd_rows (gradient) + k_vfd_gather
//   dsum (2D_frame/dsum.cu:6-73)                     -> device_sum (same 512-wide tree order)
// The Matern-3/2 centre kernel 'M' (1 + r/w) exp(-r/w) is the layered model's addition.
//
// FP64 pair term: e^x by a table-driven method and the Matern distance by a
// Newton square root (exp_tab, sqrt_nr below), both within about 1 ulp;
// work items (row block, column chunk) taken largest first by a persistent
// grid.
//
// Mixed precision: pair terms in FP32 with compensated (Kahan) FP32 sums
// inside each column tile, tile sums accumulated in FP64 per row, FP64 final
// reduction.  Centres are carried as two floats (value and remainder), so a
// centre difference keeps FP32 precision relative to the difference itself
// rather than to the coordinates (the kernel widths are small against the
// shape's extent).  The near field (kernel product above kNearField) is
// evaluated again in FP64, with both element sets in Morton order so that a
// warp's rows take that branch together (spatial_order).
#include "sa_internal.cuh"
#include <cmath>
#include <algorithm>

namespace sa {

constexpr int kVfdTile = 128;
constexpr float kNearField = 0.01f;     // mixed-precision objective: K_c K_d above this is evaluated in FP64

// 2^(j/256), j = 0 .. 255, each rounded to the nearest double (computed with 60-digit decimal arithmetic)
__constant__ double c_exp2_256[256] = {
	0x1.0000000000000p+0, 0x1.00b1afa5abcbfp+0, 0x1.0163da9fb3335p+0, 0x1.02168143b0281p+0,
	0x1.02c9a3e778061p+0, 0x1.037d42e11bbccp+0, 0x1.04315e86e7f85p+0, 0x1.04e5f72f654b1p+0,
	0x1.059b0d3158574p+0, 0x1.0650a0e3c1f89p+0, 0x1.0706b29ddf6dep+0, 0x1.07bd42b72a836p+0,
	0x1.0874518759bc8p+0, 0x1.092bdf66607e0p+0, 0x1.09e3ecac6f383p+0, 0x1.0a9c79b1f3919p+0,
	0x1.0b5586cf9890fp+0, 0x1.0c0f145e46c85p+0, 0x1.0cc922b7247f7p+0, 0x1.0d83b23395decp+0,
	0x1.0e3ec32d3d1a2p+0, 0x1.0efa55fdfa9c5p+0, 0x1.0fb66affed31bp+0, 0x1.1073028d7233ep+0,
	0x1.11301d0125b51p+0, 0x1.11edbab5e2ab6p+0, 0x1.12abdc06c31ccp+0, 0x1.136a814f204abp+0,
	0x1.1429aaea92de0p+0, 0x1.14e95934f312ep+0, 0x1.15a98c8a58e51p+0, 0x1.166a45471c3c2p+0,
	0x1.172b83c7d517bp+0, 0x1.17ed48695bbc0p+0, 0x1.18af9388c8deap+0, 0x1.1972658375d2fp+0,
	0x1.1a35beb6fcb75p+0, 0x1.1af99f8138a1cp+0, 0x1.1bbe084045cd4p+0, 0x1.1c82f95281c6bp+0,
	0x1.1d4873168b9aap+0, 0x1.1e0e75eb44027p+0, 0x1.1ed5022fcd91dp+0, 0x1.1f9c18438ce4dp+0,
	0x1.2063b88628cd6p+0, 0x1.212be3578a819p+0, 0x1.21f49917ddc96p+0, 0x1.22bdda27912d1p+0,
	0x1.2387a6e756238p+0, 0x1.2451ffb82140ap+0, 0x1.251ce4fb2a63fp+0, 0x1.25e85711ece75p+0,
	0x1.26b4565e27cddp+0, 0x1.2780e341ddf29p+0, 0x1.284dfe1f56381p+0, 0x1.291ba7591bb70p+0,
	0x1.29e9df51fdee1p+0, 0x1.2ab8a66d10f13p+0, 0x1.2b87fd0dad990p+0, 0x1.2c57e39771b2fp+0,
	0x1.2d285a6e4030bp+0, 0x1.2df961f641589p+0, 0x1.2ecafa93e2f56p+0, 0x1.2f9d24abd886bp+0,
	0x1.306fe0a31b715p+0, 0x1.31432edeeb2fdp+0, 0x1.32170fc4cd831p+0, 0x1.32eb83ba8ea32p+0,
	0x1.33c08b26416ffp+0, 0x1.3496266e3fa2dp+0, 0x1.356c55f929ff1p+0, 0x1.36431a2de883bp+0,
	0x1.371a7373aa9cbp+0, 0x1.37f26231e754ap+0, 0x1.38cae6d05d866p+0, 0x1.39a401b7140efp+0,
	0x1.3a7db34e59ff7p+0, 0x1.3b57fbfec6cf4p+0, 0x1.3c32dc313a8e5p+0, 0x1.3d0e544ede173p+0,
	0x1.3dea64c123422p+0, 0x1.3ec70df1c5175p+0, 0x1.3fa4504ac801cp+0, 0x1.40822c367a024p+0,
	0x1.4160a21f72e2ap+0, 0x1.423fb2709468ap+0, 0x1.431f5d950a897p+0, 0x1.43ffa3f84b9d4p+0,
	0x1.44e086061892dp+0, 0x1.45c2042a7d232p+0, 0x1.46a41ed1d0057p+0, 0x1.4786d668b3237p+0,
	0x1.486a2b5c13cd0p+0, 0x1.494e1e192aed2p+0, 0x1.4a32af0d7d3dep+0, 0x1.4b17dea6db7d7p+0,
	0x1.4bfdad5362a27p+0, 0x1.4ce41b817c114p+0, 0x1.4dcb299fddd0dp+0, 0x1.4eb2d81d8abffp+0,
	0x1.4f9b2769d2ca7p+0, 0x1.508417f4531eep+0, 0x1.516daa2cf6642p+0, 0x1.5257de83f4eefp+0,
	0x1.5342b569d4f82p+0, 0x1.542e2f4f6ad27p+0, 0x1.551a4ca5d920fp+0, 0x1.56070dde910d2p+0,
	0x1.56f4736b527dap+0, 0x1.57e27dbe2c4cfp+0, 0x1.58d12d497c7fdp+0, 0x1.59c0827ff07ccp+0,
	0x1.5ab07dd485429p+0, 0x1.5ba11fba87a03p+0, 0x1.5c9268a5946b7p+0, 0x1.5d84590998b93p+0,
	0x1.5e76f15ad2148p+0, 0x1.5f6a320dceb71p+0, 0x1.605e1b976dc09p+0, 0x1.6152ae6cdf6f4p+0,
	0x1.6247eb03a5585p+0, 0x1.633dd1d1929fdp+0, 0x1.6434634ccc320p+0, 0x1.652b9febc8fb7p+0,
	0x1.6623882552225p+0, 0x1.671c1c70833f6p+0, 0x1.68155d44ca973p+0, 0x1.690f4b19e9538p+0,
	0x1.6a09e667f3bcdp+0, 0x1.6b052fa75173ep+0, 0x1.6c012750bdabfp+0, 0x1.6cfdcddd47645p+0,
	0x1.6dfb23c651a2fp+0, 0x1.6ef9298593ae5p+0, 0x1.6ff7df9519484p+0, 0x1.70f7466f42e87p+0,
	0x1.71f75e8ec5f74p+0, 0x1.72f8286ead08ap+0, 0x1.73f9a48a58174p+0, 0x1.74fbd35d7cbfdp+0,
	0x1.75feb564267c9p+0, 0x1.77024b1ab6e09p+0, 0x1.780694fde5d3fp+0, 0x1.790b938ac1cf6p+0,
	0x1.7a11473eb0187p+0, 0x1.7b17b0976cfdbp+0, 0x1.7c1ed0130c132p+0, 0x1.7d26a62ff86f0p+0,
	0x1.7e2f336cf4e62p+0, 0x1.7f3878491c491p+0, 0x1.80427543e1a12p+0, 0x1.814d2add106d9p+0,
	0x1.82589994cce13p+0, 0x1.8364c1eb941f7p+0, 0x1.8471a4623c7adp+0, 0x1.857f4179f5b21p+0,
	0x1.868d99b4492edp+0, 0x1.879cad931a436p+0, 0x1.88ac7d98a6699p+0, 0x1.89bd0a478580fp+0,
	0x1.8ace5422aa0dbp+0, 0x1.8be05bad61778p+0, 0x1.8cf3216b5448cp+0, 0x1.8e06a5e0866d9p+0,
	0x1.8f1ae99157736p+0, 0x1.902fed0282c8ap+0, 0x1.9145b0b91ffc6p+0, 0x1.925c353aa2fe2p+0,
	0x1.93737b0cdc5e5p+0, 0x1.948b82b5f98e5p+0, 0x1.95a44cbc8520fp+0, 0x1.96bdd9a7670b3p+0,
	0x1.97d829fde4e50p+0, 0x1.98f33e47a22a2p+0, 0x1.9a0f170ca07bap+0, 0x1.9b2bb4d53fe0dp+0,
	0x1.9c49182a3f090p+0, 0x1.9d674194bb8d5p+0, 0x1.9e86319e32323p+0, 0x1.9fa5e8d07f29ep+0,
	0x1.a0c667b5de565p+0, 0x1.a1e7aed8eb8bbp+0, 0x1.a309bec4a2d33p+0, 0x1.a42c980460ad8p+0,
	0x1.a5503b23e255dp+0, 0x1.a674a8af46052p+0, 0x1.a799e1330b358p+0, 0x1.a8bfe53c12e59p+0,
	0x1.a9e6b5579fdbfp+0, 0x1.ab0e521356ebap+0, 0x1.ac36bbfd3f37ap+0, 0x1.ad5ff3a3c2774p+0,
	0x1.ae89f995ad3adp+0, 0x1.afb4ce622f2ffp+0, 0x1.b0e07298db666p+0, 0x1.b20ce6c9a8952p+0,
	0x1.b33a2b84f15fbp+0, 0x1.b468415b749b1p+0, 0x1.b59728de5593ap+0, 0x1.b6c6e29f1c52ap+0,
	0x1.b7f76f2fb5e47p+0, 0x1.b928cf22749e4p+0, 0x1.ba5b030a1064ap+0, 0x1.bb8e0b79a6f1fp+0,
	0x1.bcc1e904bc1d2p+0, 0x1.bdf69c3f3a207p+0, 0x1.bf2c25bd71e09p+0, 0x1.c06286141b33dp+0,
	0x1.c199bdd85529cp+0, 0x1.c2d1cd9fa652cp+0, 0x1.c40ab5fffd07ap+0, 0x1.c544778fafb22p+0,
	0x1.c67f12e57d14bp+0, 0x1.c7ba88988c933p+0, 0x1.c8f6d9406e7b5p+0, 0x1.ca3405751c4dbp+0,
	0x1.cb720dcef9069p+0, 0x1.ccb0f2e6d1675p+0, 0x1.cdf0b555dc3fap+0, 0x1.cf3155b5bab74p+0,
	0x1.d072d4a07897cp+0, 0x1.d1b532b08c968p+0, 0x1.d2f87080d89f2p+0, 0x1.d43c8eacaa1d6p+0,
	0x1.d5818dcfba487p+0, 0x1.d6c76e862e6d3p+0, 0x1.d80e316c98398p+0, 0x1.d955d71ff6075p+0,
	0x1.da9e603db3285p+0, 0x1.dbe7cd63a8315p+0, 0x1.dd321f301b460p+0, 0x1.de7d5641c0658p+0,
	0x1.dfc97337b9b5fp+0, 0x1.e11676b197d17p+0, 0x1.e264614f5a129p+0, 0x1.e3b333b16ee12p+0,
	0x1.e502ee78b3ff6p+0, 0x1.e653924676d76p+0, 0x1.e7a51fbc74c83p+0, 0x1.e8f7977cdb740p+0,
	0x1.ea4afa2a490dap+0, 0x1.eb9f4867cca6ep+0, 0x1.ecf482d8e67f1p+0, 0x1.ee4aaa2188510p+0,
	0x1.efa1bee615a27p+0, 0x1.f0f9c1cb6412ap+0, 0x1.f252b376bba97p+0, 0x1.f3ac948dd7274p+0,
	0x1.f50765b6e4540p+0, 0x1.f6632798844f8p+0, 0x1.f7bfdad9cbe14p+0, 0x1.f91d802243c89p+0,
	0x1.fa7c1819e90d8p+0, 0x1.fbdba3692d514p+0, 0x1.fd3c22b8f71f1p+0, 0x1.fe9d96b2a23d9p+0,
};

// e^x in FP64 by Tang's table-driven method (P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989): with
// N = rint(256 x / ln 2) = 256 m + j, r = x - N ln2/256 (|r| <= ln2/512, formed exactly enough by two fused
// multiply-adds with ln2/256 split in a leading and a trailing part),
//     e^x = 2^m * 2^(j/256) * (1 + p(r)),   p(r) = r + r^2/2 + r^3/6 + r^4/24,
// the Taylor remainder r^5/120 staying below 2^-54.  2^(j/256) comes from a 256-entry table in shared
// memory (tab), 2^m is added to the exponent field.  Nine FP64-pipe instructions; |x| >= 700, infinities
// and NaN are passed to exp().  Error about 1 ulp (tests/test_gpu_pair_math.py checks it against exp()).
__device__ __forceinline__ double exp_tab(double x, const double *__restrict__ tab)
{
	const int hx = __double2hiint(x) & 0x7fffffff;
	if (hx >= 0x4085E000) return exp(x);                      // |x| >= 700 (0x4085E000... = 700.0), Inf, NaN
	const double t = fma(x, 0x1.71547652b82fep+8, 0x1.8p52);  // 256/ln2; 1.5 * 2^52 rounds to an integer
	const int N = __double2loint(t);
	const double Nd = t - 0x1.8p52;
	double r = fma(-Nd, 0x1.62e42fefa39efp-9, x);             // ln2/256, leading part
	r = fma(-Nd, 0x1.abc9e3b39803fp-64, r);                   // trailing part
	double p = fma(r, 1.0 / 24.0, 1.0 / 6.0);
	p = fma(p, r, 0.5);
	p = fma(p, r, 1.0);
	p = p * r;
	const double S = tab[N & 255];
	const double y = fma(S, p, S);
	return __hiloint2double(__double2hiint(y) + (int) ((unsigned) (N >> 8) << 20), __double2loint(y));
}

// sqrt(a) in FP64 by Newton's (Heron's) iteration s <- s + (a - s^2) h with h = y / 2 fixed, where y is the
// FP32 reciprocal square root of a (relative error d of a few 1e-8): from s = a y each step multiplies the
// relative error by about d (1.5 d^2 after the first, below 1e-20 after the second), so the result is
// within about 1 ulp of the root.  Six FP64-pipe instructions.  Arguments outside [2^-95, 2^96) (zero
// included) go to sqrt(); tests/test_gpu_pair_math.py checks the result against sqrt().
__device__ __forceinline__ double sqrt_nr(double a)
{
	const unsigned e = (unsigned) __double2hiint(a) >> 20;   // sign and biased exponent
	if (e < 1023u - 95u || e >= 1023u + 96u) return sqrt(a);
	const double y = (double) rsqrtf(__double2float_rn(a));
	const double h = 0.5 * y;
	double s = a * y;
	s = fma(fma(-s, s, a), h, s);
	s = fma(fma(-s, s, a), h, s);
	return s;
}

__device__ __forceinline__ double exp_k(double x, const double *tab) { return exp_tab(x, tab); }
__device__ __forceinline__ float exp_k(float x, const double *) { return exp(x); }
__device__ __forceinline__ double sqrt_k(double x) { return sqrt_nr(x); }
__device__ __forceinline__ float sqrt_k(float x) { return sqrt(x); }

// Kernel values with the widths' reciprocals iw = 1/w, iw2 = 1/w^2 precomputed (no division per pair: FP64
// divisions cost about ten FP64-pipe instructions each on GB300); derivatives d1 only when G (gradient).
// tab: the 2^(j/64) table in shared memory (FP64 exponentials).
template <typename T, bool G>
__device__ __forceinline__ T cen_knl(int type, T iw, T iw2, T d2, T &d1, const double *tab)
{
	if (type == 'G') { T k = exp_k(-d2 * iw2, tab); if (G) d1 = (T) -2.0 * k * iw2; return k; }
	if (type == 'C') { T k = (T) 1.0 / ((T) 1.0 + d2 * iw2); if (G) d1 = (T) -2.0 * k * k * iw2; return k; }
	T r = sqrt_k(d2) * iw, ex = exp_k(-r, tab);   // 'M'
	if (G) d1 = -ex * iw2;
	return fma(r, ex, ex);                          // (1 + r) e^-r
}

// the same for centres already multiplied by 1/w (d2 = |c_i - c_j|^2 / w^2): one multiplication less per pair
template <typename T>
__device__ __forceinline__ T cen_knl_scaled(int type, T d2, const double *tab)
{
	if (type == 'G') return exp_k(-d2, tab);
	if (type == 'C') return (T) 1.0 / ((T) 1.0 + d2);
	T r = sqrt_k(d2), ex = exp_k(-r, tab);          // 'M'
	return fma(r, ex, ex);
}

template <typename T, bool G>
__device__ __forceinline__ T dir_knl(int type, T iw2, T ang, T &d1, const double *tab)
{
	if (type == 'B') { if (G) d1 = (T) 2.0 * ang; return ang * ang; }
	if (type == 'L') { if (G) d1 = (T) 1.0; return ang; }
	if (type == 'O') { T k = exp_k((T) 2.0 * (ang - (T) 1.0) * iw2, tab); if (G) d1 = (T) 2.0 * k * iw2; return k; }
	T k = exp_k((T) 2.0 * (ang * ang - (T) 1.0) * iw2, tab);     // 'U'
	if (G) d1 = (T) 4.0 * ang * k * iw2;
	return k;
}

// exp_tab and exp() (fn 0) or sqrt_nr and sqrt() (fn 1) side by side: accuracy check
__global__ void k_math_check(int fn, long n, const double *__restrict__ x, double *__restrict__ y,
                             double *__restrict__ yref)
{
	__shared__ double tab[256];
	for (int t = threadIdx.x; t < 256; t += blockDim.x) tab[t] = c_exp2_256[t];
	__syncthreads();
	for (long k = blockIdx.x * (long) blockDim.x + threadIdx.x; k < n; k += (long) gridDim.x * blockDim.x) {
		if (fn == 0) { y[k] = exp_tab(x[k], tab); yref[k] = exp(x[k]); }
		else { y[k] = sqrt_nr(x[k]); yref[k] = sqrt(x[k]); }
	}
}

void math_check(int fn, long n, const double *x, double *y, double *yref, cudaStream_t s)
{
	k_math_check<<<4 * 152, 128, 0, s>>>(fn, n, x, y, yref);
	SA_CHECK(cudaGetLastError());
}

template <int D>
__global__ void k_vfd_elems(int N, int Vd, const int *__restrict__ vfdVtx, const double *__restrict__ x,
                            double *__restrict__ cen, double *__restrict__ dir, double *__restrict__ vol)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= Vd) return;
	Vec<D> q0 = load_node<D>(x, vfdVtx[e]), q1 = load_node<D>(x, vfdVtx[Vd + e]);
	Vec<D> c, u;
	double v;
	if (D == 2) {
		for (int d = 0; d < D; ++d) c.c[d] = 0.5 * (q0.c[d] + q1.c[d]);
		u = vsub(q1, q0);
		v = sqrt(vdot(u, u));
		for (int d = 0; d < D; ++d) u.c[d] /= v;
		vol[e] = v;
	} else {
		Vec<3> a0 = load_node<3>(x, vfdVtx[e]), a1 = load_node<3>(x, vfdVtx[Vd + e]);
		Vec<3> a2 = load_node<3>(x, vfdVtx[2 * Vd + e]);
		Vec<3> cr = vcross(vsub(a1, a0), vsub(a2, a0));
		v = sqrt(vdot(cr, cr));
		for (int d = 0; d < 3; ++d) { c.c[d] = (a0.c[d] + a1.c[d] + a2.c[d]) / 3.0; u.c[d] = cr.c[d] / v; }
		vol[e] = 0.5 * v;
	}
	for (int d = 0; d < D; ++d) { cen[d * (long) Vd + e] = c.c[d]; dir[d * (long) Vd + e] = u.c[d]; }
}

struct VfdSet { const double *cen, *dir, *vol; int n; };

// out[i] = sum_j c1 K(i, j) over set A  +  sum_j c2 K(i, j) over set B (B may be empty);
// gradient rows (dc, dt) when G (rows must be the deformed set).  The columns of each set are split
// into C contiguous chunks (more work items than row blocks alone give); the item (row block, chunk c)
// writes its partial row sums at out + c * R.n (dc, dt at + c * D * R.n), summed in chunk order by
// k_vfd_chunks.  With a queue, a persistent grid takes the items from it (see the loop below); without
// one, the grid is (row blocks, C) with one item per CTA.  One chunk: the reference's per-row order.
// symA != 0 (objective only, set A is the row set itself): K is symmetric, so row i takes the pairs
// j >= i of set A with weight 2 (1 on the diagonal) -- the same total with half the pair evaluations.
template <int D, typename T, bool G>
__global__ void k_vfd_rows(VfdSet R, VfdSet A, double cA, VfdSet Bs, double cB, int ck, double cw, int dk,
                           double dw, double *__restrict__ out, double *__restrict__ dc, double *__restrict__ dt,
                           int symA = 0, int C = 0, int *__restrict__ queue = nullptr)
{
	constexpr bool kSplit = sizeof(T) < sizeof(double);     // two-float centres in FP32
	// mixed-precision objective: pairs whose FP32 kernel product K_c K_d exceeds kNearField (the near field,
	// about 6 % of the pairs on the shell workload: Matern r < ~6) are evaluated again in FP64 and summed in
	// FP64; only the far field keeps FP32 terms.  The near field carries most of the objective and of the
	// FP32 rounding (the column volumes' FP32 rounding in particular is systematic and survives the
	// cancellation DD - 2 DT + TT).
	constexpr bool kNear = kSplit && !G;
	constexpr int kN = kNear ? 1 : 0;
	// FP64 objective: centres (rows and tiles) multiplied by 1/w as they are loaded, so the pair term does
	// not scale the squared distance (the gradient keeps unscaled centres for its derivatives)
	constexpr bool kScaled = !kSplit && !G;
	const double cs = kScaled ? 1.0 / cw : 1.0;
	__shared__ T sc[kVfdTile * D], su[kVfdTile * D], sv[kVfdTile], sl[kSplit ? kVfdTile * D : 1];
	__shared__ double sc64[kN * kVfdTile * D + 1], su64[kN * kVfdTile * D + 1], sv64[kN * kVfdTile + 1];
	__shared__ double sExp[(kSplit && !kNear) ? 1 : 256];
	if (!kSplit || kNear)                                     // read after the tile barrier
		for (int t = threadIdx.x; t < 256; t += blockDim.x) sExp[t] = c_exp2_256[t];
	// work items (row block bx, column chunk cy), item = bx C + cy: with a queue, a persistent grid takes items
	// in that order (largest first: a row block's span shrinks with bx in the symmetric half), each item writing
	// its own partial-sum slot, so results do not depend on which CTA ran it; without a queue, the 2D grid
	// (bx, cy) = (blockIdx.x, blockIdx.y) runs one item per CTA
	if (!queue) C = gridDim.y;
	const int rowBlocks = (R.n + blockDim.x - 1) / blockDim.x, nItems = rowBlocks * C;
	__shared__ int sItem;
	double *const out0 = out, *const dc0 = dc, *const dt0 = dt;
	for (int pass = 0;; ++pass) {
	int item;
	if (queue) {
		__syncthreads();                      // the previous item's tile reads are done
		if (threadIdx.x == 0) sItem = atomicAdd(queue, 1);
		__syncthreads();
		item = sItem;
	} else {
		if (pass > 0) break;
		item = blockIdx.x * C + blockIdx.y;
	}
	if (item >= nItems) break;
	const int bx = item / C, cy = item % C;
	int i = bx * blockDim.x + threadIdx.x;
	bool act = i < R.n;
	T ci[D], cl[D], ui[D], vi = 0;
	double ci64[D], ui64[D];
	for (int d = 0; d < D; ++d) {
		double c = act ? R.cen[d * (long) R.n + i] : 0.0;
		ci[d] = (T) (kScaled ? c * cs : c);
		cl[d] = kSplit ? (T) (c - (double) ci[d]) : (T) 0;
		ci64[d] = c;
		ui64[d] = act ? R.dir[d * (long) R.n + i] : 0.0;
		ui[d] = (T) ui64[d];
	}
	const double ciw64 = 1.0 / cw, ciw2_64 = 1.0 / (cw * cw), diw2_64 = 1.0 / (dw * dw);
	if (act) vi = (T) R.vol[i];
	const T nLen = (D == 2 ? vi : (T) 2.0 * vi), half = (D == 2 ? (T) 1.0 : (T) 0.5);
	double acc = 0.0, gc[D], gt[D];
	for (int d = 0; d < D; ++d) { gc[d] = 0.0; gt[d] = 0.0; }
	const T ciw = (T) (1.0 / cw), ciw2 = (T) (1.0 / (cw * cw)), diw2 = (T) (1.0 / (dw * dw));
	out = out0 + (long) cy * R.n;
	if (G) { dc = dc0 + (long) cy * D * R.n; dt = dt0 + (long) cy * D * R.n; }
	for (int set = 0; set < 2; ++set) {
		const VfdSet &S = set == 0 ? A : Bs;
		// row factor coef * vol_i in FP64 from the FP64 volume (applied to each tile's FP32 or FP64 sum)
		const double cv = (set == 0 ? cA : cB) * (act ? R.vol[i] : 0.0);
		const bool sym = set == 0 && symA;
		const int lo = sym ? (int) (bx * blockDim.x) : 0;           // columns below the item's rows: none
		const int span = S.n > lo ? S.n - lo : 0;
		const int jBeg = lo + (int) ((long) span * cy / C), jEnd = lo + (int) ((long) span * (cy + 1) / C);
		// gradient weights of dqVfd_DD_DT: +2 for the deformed-deformed term (both ends move), -2 for
		// the deformed-target term
		T gco = (T) (set == 0 ? 2.0 * cA : cB);
		for (int j0 = jBeg; j0 < jEnd; j0 += kVfdTile) {
			int nt = min(kVfdTile, jEnd - j0);
			__syncthreads();
			for (int t = threadIdx.x; t < nt; t += blockDim.x) {
				for (int d = 0; d < D; ++d) {
					double c = S.cen[d * (long) S.n + j0 + t], u = S.dir[d * (long) S.n + j0 + t];
					sc[t * D + d] = (T) (kScaled ? c * cs : c);
					if (kSplit) sl[t * D + d] = (T) (c - (double) sc[t * D + d]);
					su[t * D + d] = (T) u;
					if (kNear) { sc64[t * D + d] = c; su64[t * D + d] = u; }
				}
				const double v = S.vol[j0 + t];
				sv[t] = (T) v;
				if (kNear) sv64[t] = v;
			}
			__syncthreads();
			if (!act) continue;
			// tile = sum of K_c K_d vol_j over the tile's columns; the row factor coef * vol_i and, for the
			// symmetric half, the weights (2 off the diagonal, 1 on it: 2 tile - diagonal term) are applied
			// once per tile
			T tile = 0, comp = 0, diag = 0, tgc[D], tgt[D];
			double nearSum = 0.0, diag64 = 0.0;                       // FP64 near-field terms (kNear)
			for (int d = 0; d < D; ++d) { tgc[d] = 0; tgt[d] = 0; }
			for (int jj = 0; jj < nt; ++jj) {
				bool onDiag = false;
				if (sym) {
					const int j = j0 + jj;
					if (j < i) continue;
					onDiag = j == i;
				}
				T df[D];
				for (int d = 0; d < D; ++d) {
					df[d] = ci[d] - sc[jj * D + d];
					if (kSplit) df[d] = df[d] + (cl[d] - sl[jj * D + d]);
				}
				T d2 = df[0] * df[0];
				for (int d = 1; d < D; ++d) d2 = d2 + df[d] * df[d];
				T ang = ui[0] * su[jj * D];
				for (int d = 1; d < D; ++d) ang = ang + ui[d] * su[jj * D + d];
				T d1c = 0, d1d = 0;
				T kc = kScaled ? cen_knl_scaled<T>(ck, d2, sExp) : cen_knl<T, G>(ck, ciw, ciw2, d2, d1c, sExp);
				T kd = dir_knl<T, G>(dk, diw2, ang, d1d, sExp);
				T vj = sv[jj];
				const T kv = kd * vj;
				if (kNear && kc * kd > (T) kNearField) {
					double e2 = 0.0, a64 = 0.0, u1 = 0.0, u2 = 0.0;
					for (int d = 0; d < D; ++d) {
						const double df = ci64[d] - sc64[jj * D + d];
						e2 = fma(df, df, e2);
						a64 = fma(ui64[d], su64[jj * D + d], a64);
					}
					const double t64 = cen_knl<double, false>(ck, ciw64, ciw2_64, e2, u1, sExp) *
					                   (dir_knl<double, false>(dk, diw2_64, a64, u2, sExp) * sv64[jj]);
					nearSum += t64;
					if (onDiag) diag64 = t64;
				} else if (kSplit) {           // Kahan: the FP32 tile sum keeps its lost low bits
					if (onDiag) diag = kc * kv;
					T y = kc * kv - comp, t = tile + y;
					comp = (t - tile) - y;
					tile = t;
				} else {
					if (onDiag) diag = kc * kv;
					tile = fma(kc, kv, tile);
				}
				if (G) {
					// geometricFunction/grassmanFunction gradients and dqVfd_DD_DT accumulation
					for (int d = 0; d < D; ++d) {
						T dK = d1c * df[d];
						T tK = d1d / nLen * (-ang * ui[d] + su[jj * D + d]);
						tgc[d] += gco * dK * kd * vi * vj;
						tgt[d] += gco * kc * (tK * vi + kd * half * ui[d]) * vj;
					}
				}
			}
			// Kahan: the FP32 sum with its lost low part, plus the FP64 near-field terms
			const double tsum = ((double) tile - (double) comp) + nearSum;
			acc += cv * (sym ? 2.0 * tsum - ((double) diag + diag64) : tsum);
			if (G) for (int d = 0; d < D; ++d) { gc[d] += (double) tgc[d]; gt[d] += (double) tgt[d]; }
		}
	}
	if (act) {
		out[i] = acc;
		if (G)
			for (int d = 0; d < D; ++d) { dc[d * (long) R.n + i] = gc[d]; dt[d * (long) R.n + i] = gt[d]; }
	}
	}   // items
}

// ---------------------------------------------------------------------------
// Spatial order of a set of boundary elements (mixed-precision objective).
// The FP64 near-field branch of the FP32 pair sums is taken by a warp when
// any of its 32 rows is near the column; in mesh order a warp's rows lie all
// over the surface, so nearly every warp would take it.  Sorted by the Morton
// code of their centres (10 bits per axis in 3D, 15 in 2D, inside the set's
// bounding box; ties broken by index, so the 64-bit keys are distinct and the
// order is deterministic) a warp's rows are neighbours.  The objective is a
// double sum over the sets, so its value does not depend on the order.
// ---------------------------------------------------------------------------
constexpr int kSortBlock = 2048;        // keys per CTA in the shared-memory bitonic stages

template <int D>
__global__ void k_set_bbox(int n, const double *__restrict__ cen, double *__restrict__ box)
{
	__shared__ double lo[256][D], hi[256][D];
	const int t = threadIdx.x;
	for (int d = 0; d < D; ++d) { lo[t][d] = 1e300; hi[t][d] = -1e300; }
	for (int e = t; e < n; e += blockDim.x)
		for (int d = 0; d < D; ++d) {
			const double c = cen[d * (long) n + e];
			lo[t][d] = fmin(lo[t][d], c);
			hi[t][d] = fmax(hi[t][d], c);
		}
	__syncthreads();
	for (int h = 128; h > 0; h >>= 1) {
		if (t < h)
			for (int d = 0; d < D; ++d) {
				lo[t][d] = fmin(lo[t][d], lo[t + h][d]);
				hi[t][d] = fmax(hi[t][d], hi[t + h][d]);
			}
		__syncthreads();
	}
	if (t < D) { box[t] = lo[0][t]; box[D + t] = hi[0][t]; }
}

__device__ __forceinline__ unsigned spread_bits(unsigned v, int D)
{
	unsigned r = 0;
	const int bits = D == 3 ? 10 : 15;
	for (int b = 0; b < bits; ++b) r |= ((v >> b) & 1u) << (b * D);
	return r;
}

template <int D>
__global__ void k_set_keys(int n, int npad, const double *__restrict__ cen, const double *__restrict__ box,
                           unsigned long long *__restrict__ keys)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= npad) return;
	if (k >= n) { keys[k] = ~0ULL; return; }                 // padding sorts last
	const unsigned cells = D == 3 ? 1024u : 32768u;
	unsigned code = 0;
	for (int d = 0; d < D; ++d) {
		const double ext = box[D + d] - box[d];
		const double f = ext > 0.0 ? (cen[d * (long) n + k] - box[d]) / ext : 0.0;
		unsigned q = (unsigned) fmin(fmax(f * (double) cells, 0.0), (double) (cells - 1));
		code |= spread_bits(q, D) << d;
	}
	keys[k] = ((unsigned long long) code << 32) | (unsigned) k;
}

__device__ __forceinline__ void cmp_swap(unsigned long long &a, unsigned long long &b, bool up)
{
	if ((a > b) == up) { const unsigned long long t = a; a = b; b = t; }
}

// bitonic stages with j < kSortBlock inside one CTA's 2048 keys: all sizes k <= kSortBlock when k == 0,
// else the stages j = kSortBlock/2 .. 1 of size k
__global__ void __launch_bounds__(kSortBlock / 2) k_bitonic_local(unsigned long long *__restrict__ keys, int k)
{
	__shared__ unsigned long long s[kSortBlock];
	const int base = blockIdx.x * kSortBlock, t = threadIdx.x;
	s[t] = keys[base + t];
	s[t + kSortBlock / 2] = keys[base + t + kSortBlock / 2];
	__syncthreads();
	const int kLo = k == 0 ? 2 : k, kHi = k == 0 ? kSortBlock : k;
	for (int kk = kLo; kk <= kHi; kk <<= 1)
		for (int j = min(kk, kSortBlock) >> 1; j > 0; j >>= 1) {
			// thread t handles the pair (i, i + j) with i the t-th index whose bit j is clear
			const int i = 2 * t - (t & (j - 1));
			const bool up = ((base + i) & kk) == 0;
			cmp_swap(s[i], s[i + j], up);
			__syncthreads();
		}
	keys[base + t] = s[t];
	keys[base + t + kSortBlock / 2] = s[t + kSortBlock / 2];
}

// one bitonic stage (size k, distance j >= kSortBlock) over all npad keys
__global__ void k_bitonic_global(unsigned long long *__restrict__ keys, int npad, int j, int k)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= npad) return;
	const int l = i ^ j;
	if (l <= i) return;
	unsigned long long a = keys[i], b = keys[l];
	const bool up = (i & k) == 0;
	if ((a > b) == up) { keys[i] = b; keys[l] = a; }
}

template <int D>
__global__ void k_set_gather(int n, const unsigned long long *__restrict__ keys, VfdSet S, double *__restrict__ cen,
                             double *__restrict__ dir, double *__restrict__ vol)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n) return;
	const int e = (int) (keys[k] & 0xffffffffu);
	for (int d = 0; d < D; ++d) {
		cen[d * (long) n + k] = S.cen[d * (long) n + e];
		dir[d * (long) n + k] = S.dir[d * (long) n + e];
	}
	vol[k] = S.vol[e];
}

static int sort_pad(int n)
{
	int p = kSortBlock;
	while (p < n) p <<= 1;
	return p;
}

// doubles of scratch spatial_order needs for a set of n elements
static size_t spatial_order_doubles(int D, int n) { return (size_t) (2 * D + 1) * n + sort_pad(n) + 2 * D + 8; }

// the set S in spatial order, written into scr (spatial_order_doubles(D, S.n) doubles)
template <int D>
static VfdSet spatial_order(const VfdSet &S, double *scr, cudaStream_t s)
{
	if (S.n <= 0) return S;
	const int n = S.n, npad = sort_pad(n);
	double *cen = scr, *dir = cen + (long) D * n, *vol = dir + (long) D * n, *box = vol + n;
	unsigned long long *keys = reinterpret_cast<unsigned long long *>(box + 2 * D + 8);
	k_set_bbox<D><<<1, 256, 0, s>>>(n, S.cen, box);
	k_set_keys<D><<<(npad + 255) / 256, 256, 0, s>>>(n, npad, S.cen, box, keys);
	k_bitonic_local<<<npad / kSortBlock, kSortBlock / 2, 0, s>>>(keys, 0);
	for (int k = 2 * kSortBlock; k <= npad; k <<= 1) {
		for (int j = k >> 1; j >= kSortBlock; j >>= 1)
			k_bitonic_global<<<(npad + 255) / 256, 256, 0, s>>>(keys, npad, j, k);
		k_bitonic_local<<<npad / kSortBlock, kSortBlock / 2, 0, s>>>(keys, k);
	}
	k_set_gather<D><<<grid_for(n), kBlock, 0, s>>>(n, keys, S, cen, dir, vol);
	return VfdSet{cen, dir, vol, n};
}

// row sums of the column chunks of k_vfd_rows, chunk order fixed (K values per row: 1, or 1 + 2D with the
// gradient rows laid out [chunk][d][row])
template <int D>
__global__ void k_vfd_chunks(int n, int C, const double *__restrict__ part, double *__restrict__ out, int grad,
                             const double *__restrict__ pdc, const double *__restrict__ pdt, double *__restrict__ dc,
                             double *__restrict__ dt)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	double a = part[i];
	for (int c = 1; c < C; ++c) a += part[(long) c * n + i];
	out[i] = a;
	if (!grad) return;
	for (int d = 0; d < D; ++d) {
		double x = pdc[(long) d * n + i], y = pdt[(long) d * n + i];
		for (int c = 1; c < C; ++c) {
			x += pdc[((long) c * D + d) * n + i];
			y += pdt[((long) c * D + d) * n + i];
		}
		dc[(long) d * n + i] = x;
		dt[(long) d * n + i] = y;
	}
}

// node gradient gather (2D_frame/varifold.cu:435-466, 3D_frame :492-528)
template <int D>
__global__ void k_vfd_gather(int N, int Vd, const int *__restrict__ ifo, const double *__restrict__ x,
                             const double *__restrict__ dc, const double *__restrict__ dt, double *__restrict__ g)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double s[D];
	for (int d = 0; d < D; ++d) s[d] = 0.0;
	int cnt = ifo[i];
	for (int a = 0; a < cnt; ++a) {
		if (D == 2) {
			int e = ifo[(1 + 2 * a) * (long) N + i], sg = ifo[(2 + 2 * a) * (long) N + i];
			for (int d = 0; d < D; ++d) s[d] += 0.5 * dc[d * (long) Vd + e] + sg * dt[d * (long) Vd + e];
		} else {
			int e = ifo[(1 + 3 * a) * (long) N + i];
			int qa = ifo[(2 + 3 * a) * (long) N + i], qb = ifo[(3 + 3 * a) * (long) N + i];
			Vec<3> t, ab;
			for (int d = 0; d < 3; ++d) {
				t.c[d] = dt[d * (long) Vd + e];
				ab.c[d] = x[(long) qa * 3 + d] - x[(long) qb * 3 + d];
			}
			Vec<3> cr = vcross(t, ab);
			for (int d = 0; d < 3; ++d) s[d] += dc[d * (long) Vd + e] / 3.0 + cr.c[d];
		}
	}
	for (int d = 0; d < D; ++d) g[(long) i * D + d] = s[d];
}

// ---------------------------------------------------------------------------
// reference dsum order: 512-wide shared-memory trees, accumulated per block
// across 512*512 runs, then a final 512 tree (2D_frame/dsum.cu:6-73)
// ---------------------------------------------------------------------------
constexpr int kSum = 512;

__global__ void k_dsum_tree(double *buf, const double *v, int len, int small)
{
	__shared__ double s[kSum];
	int t = threadIdx.x, g = blockIdx.x * blockDim.x + t;
	s[t] = g < len ? v[g] : 0.0;
	__syncthreads();
	for (int stride = blockDim.x >> 1; stride > 0; stride >>= 1) {
		if (t < stride) s[t] += s[t + stride];
		__syncthreads();
	}
	if (t == 0) {
		if (small) buf[0] = s[0];
		else buf[blockIdx.x] += s[0];
	}
}

double device_sum(const double *v, long n, double *scratch, cudaStream_t s)
{
	// scratch: kSum + 1 doubles
	double h = 0.0;
	if (n < kSum) {
		k_dsum_tree<<<1, kSum, 0, s>>>(scratch + kSum, v, (int) n, 1);
	} else {
		SA_CHECK(cudaMemsetAsync(scratch, 0, sizeof(double) * kSum, s));
		long run = (long) kSum * kSum;
		long runNum = (n - 1) / run + 1;
		for (long r = 0; r < runNum; ++r) {
			long lenNow = (r == runNum - 1 ? n - r * run : run);
			int blk = (int) ((lenNow - 1) / kSum + 1);
			k_dsum_tree<<<blk, kSum, 0, s>>>(scratch, v + r * run, (int) lenNow, 0);
		}
		k_dsum_tree<<<1, kSum, 0, s>>>(scratch + kSum, scratch, kSum, 1);
	}
	SA_CHECK(cudaMemcpyAsync(&h, scratch + kSum, sizeof(double), cudaMemcpyDeviceToHost, s));
	SA_CHECK(cudaStreamSynchronize(s));
	return h;
}

constexpr int kVfdBlock = 128;

// persistent grid of k_vfd_rows: as many CTAs as fit on the GPU at once, at most one per work item
template <int D, typename T, bool G>
static int vfd_grid(int items)
{
	int dev = 0, sms = 1, per = 1;
	SA_CHECK(cudaGetDevice(&dev));
	SA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	SA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_vfd_rows<D, T, G>, kVfdBlock, 0));
	return std::max(1, std::min(items, std::max(1, per) * sms));
}

// one k_vfd_rows launch over all (row block, column chunk) items of R, taken from the queue counter (zeroed
// here on the stream)
template <int D, typename T, bool G>
static void launch_vfd_rows(VfdSet R, VfdSet A, double cA, VfdSet B, double cB, int ck, double cw, int dk, double dw,
                            double *out, double *dc, double *dt, int sym, int C, int *queue, cudaStream_t s)
{
	const int items = grid_for(R.n, kVfdBlock) * C;
	SA_CHECK(cudaMemsetAsync(queue, 0, sizeof(int), s));
	k_vfd_rows<D, T, G><<<vfd_grid<D, T, G>(items), kVfdBlock, 0, s>>>(R, A, cA, B, cB, ck, cw, dk, dw, out, dc, dt,
	                                                                     sym, C, queue);
}

// column chunks of the pair sums of a Vd x Vt objective: enough CTAs to fill the GPU (the pair sums are latency
// bound at one CTA per SM), each chunk at least two tiles wide
int vfd_chunk_count(int Vd, int Vt)
{
	int dev = 0, sms = 1;
	SA_CHECK(cudaGetDevice(&dev));
	SA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	const int rowMax = std::max(Vd, Vt), colMin = std::min(Vd, Vt);
	const int perSm = std::max(1, tuning().vfdCtasPerSm);
	const int rowCtas = std::max(1, grid_for(rowMax, kVfdBlock));
	int C = std::max(1, (perSm * sms + rowCtas - 1) / rowCtas);
	C = std::min(C, std::max(1, colMin / (2 * kVfdTile)));
	return std::min(C, 32);
}

// the target-target rows (vfd_TT) of a Vd x Vt objective into cache.rows, launched on stream s: the same
// launches as inside varifold(), so the objective gives the same value whether it finds these rows in the
// cache or computes them itself.  part: varifold_target_rows_scratch(D, Vd, Vt, precision) doubles.
size_t varifold_target_rows_scratch(int D, int Vd, int Vt, int precision)
{
	return (size_t) vfd_chunk_count(Vd, Vt) * Vt + (precision == SA_PREC_MIXED ? spatial_order_doubles(D, Vt) : 0) +
	       1;                                                      // + the work-item counter
}

template <int D>
void varifold_target_rows(const Model &md, int Vd, const double *tgtCen, const double *tgtDir, const double *tgtVol,
                          int Vt, int precision, double *part, VfdTargetCache &cache, cudaStream_t s)
{
	if (!cache.rows || cache.capacity < Vt || Vt <= 0) return;     // not cached: the objective computes them
	const int C = vfd_chunk_count(Vd, Vt);
	VfdSet Ts{tgtCen, tgtDir, tgtVol, Vt}, E0{nullptr, nullptr, nullptr, 0};
	int *queue = reinterpret_cast<int *>(part + varifold_target_rows_scratch(D, Vd, Vt, precision) - 1);
	if (precision == SA_PREC_MIXED) Ts = spatial_order<D>(Ts, part + (size_t) C * Vt, s);
	const int ck = md.cenKnl, dk = md.dirKnl;
	const double cw = md.cenWidth, dw = md.dirWidth;
	if (precision == SA_PREC_MIXED)
		launch_vfd_rows<D, float, false>(Ts, Ts, 1.0, E0, 0.0, ck, cw, dk, dw, part, nullptr, nullptr, 1, C, queue, s);
	else
		launch_vfd_rows<D, double, false>(Ts, Ts, 1.0, E0, 0.0, ck, cw, dk, dw, part, nullptr, nullptr, 1, C, queue, s);
	k_vfd_chunks<D><<<grid_for(Vt), kBlock, 0, s>>>(Vt, C, part, cache.rows, 0, nullptr, nullptr, nullptr, nullptr);
	SA_CHECK(cudaGetLastError());
	cache.valid = true; cache.Vt = Vt; cache.precision = precision;
	cache.ck = ck; cache.dk = dk; cache.cw = cw; cache.dw = dw;
}

template void varifold_target_rows<2>(const Model &, int, const double *, const double *, const double *, int, int,
                                      double *, VfdTargetCache &, cudaStream_t);
template void varifold_target_rows<3>(const Model &, int, const double *, const double *, const double *, int, int,
                                      double *, VfdTargetCache &, cudaStream_t);

template <int D>
double varifold(const Mesh &m, const Model &md, const double *x, const double *tgtCen, const double *tgtDir,
                const double *tgtVol, int Vt, double *grad, cudaStream_t s, int precision, int *err,
                VfdTargetCache *cache)
{
	int Vd = m.Vd;
	*err = SA_OK;
	if (grad && !m.vfdIfo) { *err = SA_ERR_ARG; return 0.0; }
	const int rowMax = std::max(Vd, Vt);
	const int C = vfd_chunk_count(Vd, Vt);
	double *buf = nullptr;
	const size_t rows = (size_t) (Vd + Vt);
	// mixed-precision objective: both sets in spatial order (coherent near-field branch, see spatial_order)
	const bool ordered = precision == SA_PREC_MIXED && !grad;
	const size_t partLen = (size_t) C * rowMax * (1 + (grad ? 2 * D : 0));
	size_t need = (size_t) Vd * (2 * D + 1) + rows + kSum + 1 + (grad ? (size_t) 2 * D * Vd : 0) + partLen +
	              (ordered ? spatial_order_doubles(D, Vd) + spatial_order_doubles(D, Vt) : 0) + 1;
	SA_CHECK(cudaMallocAsync(&buf, sizeof(double) * need, s));
	double *cen = buf, *dir = cen + (long) D * Vd, *vol = dir + (long) D * Vd, *vfd = vol + Vd;
	double *scr = vfd + Vd + Vt, *dc = scr + kSum + 1, *dt = dc + (long) D * Vd;
	double *part = grad ? dt + (long) D * Vd : dc;
	double *pdc = part + (long) C * rowMax, *pdt = pdc + (long) C * D * rowMax;
	double *ordD = part + partLen, *ordT = ordD + (ordered ? spatial_order_doubles(D, Vd) : 0);
	int *queue = reinterpret_cast<int *>(buf + need - 1);          // work-item counter of the pair-sum launches
	k_vfd_elems<D><<<grid_for(Vd), kBlock, 0, s>>>(m.N, Vd, m.vfdVtx, x, cen, dir, vol);
	VfdSet Ds{cen, dir, vol, Vd}, Ts{tgtCen, tgtDir, tgtVol, Vt}, E0{nullptr, nullptr, nullptr, 0};
	// row sets: the deformed set (spatially ordered in the mixed objective); the target set as rows (TT) is
	// ordered when it is needed
	const VfdSet Dr = ordered ? spatial_order<D>(Ds, ordD, s) : Ds;
	auto target_rows = [&]() { return ordered ? spatial_order<D>(Ts, ordT, s) : Ts; };
	int ck = md.cenKnl, dk = md.dirKnl;
	// rows_of: per-row sums of R against A (coefficient cA) and B (cB); the self term R = A uses the
	// symmetric half when no gradient rows are wanted
	auto rows_of = [&](VfdSet R, VfdSet A, double cA, VfdSet B, double cB, double *out, int g) {
		if (R.n == 0) return;
		const int sym = g ? 0 : 1;
		const double cw = md.cenWidth, dw = md.dirWidth;
		if (precision == SA_PREC_MIXED) {
			if (g) launch_vfd_rows<D, float, true>(R, A, cA, B, cB, ck, cw, dk, dw, part, pdc, pdt, sym, C, queue, s);
			else launch_vfd_rows<D, float, false>(R, A, cA, B, cB, ck, cw, dk, dw, part, pdc, pdt, sym, C, queue, s);
		} else {
			if (g) launch_vfd_rows<D, double, true>(R, A, cA, B, cB, ck, cw, dk, dw, part, pdc, pdt, sym, C, queue, s);
			else launch_vfd_rows<D, double, false>(R, A, cA, B, cB, ck, cw, dk, dw, part, pdc, pdt, sym, C, queue, s);
		}
		k_vfd_chunks<D><<<grid_for(R.n), kBlock, 0, s>>>(R.n, C, part, out, g, pdc, pdt, dc, dt);
	};
	if (grad || Vd >= Vt) {
		rows_of(Dr, Dr, 1.0, Ts, -2.0, vfd, grad ? 1 : 0);      // vfd_DD_DT / dqVfd_DD_DT
		// vfd_TT depends on the target only: a cache (same target, same kernels, same precision) keeps
		// its rows between calls
		bool hit = cache && cache->rows && cache->valid && cache->Vt == Vt && cache->precision == precision &&
		           cache->ck == ck && cache->dk == dk && cache->cw == md.cenWidth && cache->dw == md.dirWidth;
		if (hit) {
			SA_CHECK(cudaMemcpyAsync(vfd + Vd, cache->rows, sizeof(double) * Vt, cudaMemcpyDeviceToDevice, s));
		} else {
			const VfdSet Tr = target_rows();
			rows_of(Tr, Tr, 1.0, E0, 0.0, vfd + Vd, 0);
			if (cache && cache->rows && cache->capacity >= Vt) {
				SA_CHECK(cudaMemcpyAsync(cache->rows, vfd + Vd, sizeof(double) * Vt, cudaMemcpyDeviceToDevice, s));
				cache->valid = true; cache->Vt = Vt; cache->precision = precision;
				cache->ck = ck; cache->dk = dk; cache->cw = md.cenWidth; cache->dw = md.dirWidth;
			}
		}
	} else {
		const VfdSet Tr = target_rows();
		rows_of(Tr, Tr, 1.0, Dr, -2.0, vfd, 0);                 // vfd_TT_TD
		rows_of(Dr, Dr, 1.0, E0, 0.0, vfd + Vt, 0);             // vfd_DD
	}
	SA_CHECK(cudaGetLastError());
	double obj = device_sum(vfd, Vd + Vt, scr, s);
	if (grad) k_vfd_gather<D><<<grid_for(m.N), kBlock, 0, s>>>(m.N, Vd, m.vfdIfo, x, dc, dt, grad);
	SA_CHECK(cudaFreeAsync(buf, s));
	return obj;
}

template double varifold<2>(const Mesh &, const Model &, const double *, const double *, const double *,
                            const double *, int, double *, cudaStream_t, int, int *, VfdTargetCache *);
template double varifold<3>(const Mesh &, const Model &, const double *, const double *, const double *,
                            const double *, int, double *, cudaStream_t, int, int *, VfdTargetCache *);

// ---------------------------------------------------------------------------
// Allocation-free variant of the varifold objective (sa_varifold_noalloc).
//
// Its scratch -- boundary-element centres and directions (2 D Vd doubles),
// element volumes (Vd), per-row pair sums (Vd + Vt) and the reduction buffer
// (kSum + 1) -- lives in the file-scope device array below instead of device
// memory obtained per call.  Every GPU that loads the library holds the
// array (about 2.4 MB) until the process exits.  Host code never hands the
// array's name to a kernel: on the host that name is only a stand-in, so the
// device address is looked up once per device with cudaGetSymbolAddress and
// that address is what the kernels receive.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxElm = 32768;                       // max Vd and max Vt
struct BadIndex {};                                         // a vfdVtxMat entry outside [0, N)
constexpr long kNoAllocDoubles = 9L * kNoAllocMaxElm + 1024;
__device__ __align__(256) double g_noallocScratch[kNoAllocDoubles];

// the last double of the scratch array: set (as an int) when an element names a node outside [0, N)
constexpr long kNoAllocFlagSlot = kNoAllocDoubles - 1;

// boundary elements from nodes in the reference's N x D column-major layout.  The caller's indices are not
// checked on the host (they are device memory): an element with a node index outside [0, N) is written as
// zeros and raises *badIndex, and the host turns that into SA_ERR_ARG -- no out-of-range read is made.
template <int D>
__global__ void k_vfd_elems_soa(int N, int Vd, const int *__restrict__ vfdVtx, const double *__restrict__ x,
                                double *__restrict__ cen, double *__restrict__ dir, double *__restrict__ vol,
                                int *__restrict__ badIndex)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= Vd) return;
	int idx[D];
	bool ok = true;
	for (int k = 0; k < D; ++k) {
		idx[k] = vfdVtx[(long) k * Vd + e];
		ok = ok && idx[k] >= 0 && idx[k] < N;
	}
	if (!ok) {
		*badIndex = 1;
		for (int d = 0; d < D; ++d) { cen[d * (long) Vd + e] = 0.0; dir[d * (long) Vd + e] = 0.0; }
		vol[e] = 0.0;
		return;
	}
	Vec<D> q[D];
	for (int k = 0; k < D; ++k)
		for (int d = 0; d < D; ++d) q[k].c[d] = x[(long) d * N + idx[k]];
	Vec<D> c, u;
	double v;
	if (D == 2) {
		for (int d = 0; d < D; ++d) c.c[d] = 0.5 * (q[0].c[d] + q[1].c[d]);
		u = vsub(q[1], q[0]);
		v = sqrt(vdot(u, u));
		for (int d = 0; d < D; ++d) u.c[d] /= v;
		vol[e] = v;
	} else {
		Vec<3> a0, a1, a2;
		for (int d = 0; d < 3; ++d) { a0.c[d] = q[0].c[d]; a1.c[d] = q[1].c[d]; a2.c[d] = q[2].c[d]; }
		Vec<3> cr = vcross(vsub(a1, a0), vsub(a2, a0));
		v = sqrt(vdot(cr, cr));
		for (int d = 0; d < 3; ++d) { c.c[d] = (a0.c[d] + a1.c[d] + a2.c[d]) / 3.0; u.c[d] = cr.c[d] / v; }
		vol[e] = 0.5 * v;
	}
	for (int d = 0; d < D; ++d) { cen[d * (long) Vd + e] = c.c[d]; dir[d * (long) Vd + e] = u.c[d]; }
}

template <int D>
static double varifold_in_scratch(double *scr, int N, const double *x, int Vd, const int *vfdVtx, int Vt,
                                  const double *tc, const double *tu, const double *tv, int ck, double cw, int dk,
                                  double dw, cudaStream_t s)
{
	double *cen = scr, *dir = cen + (long) D * Vd, *vol = dir + (long) D * Vd, *vfd = vol + Vd;
	double *sumScr = vfd + Vd + Vt;
	int *badIndex = (int *) (scr + kNoAllocFlagSlot);
	SA_CHECK(cudaMemsetAsync(badIndex, 0, sizeof(int), s));
	k_vfd_elems_soa<D><<<grid_for(Vd), kBlock, 0, s>>>(N, Vd, vfdVtx, x, cen, dir, vol, badIndex);
	VfdSet Ds{cen, dir, vol, Vd}, Ts{tc, tu, tv, Vt}, E0{nullptr, nullptr, nullptr, 0};
	const int blk = 128;
	// same row/column roles as the allocating path (reference branch on Vd >= Vt)
	if (Vd >= Vt) {
		k_vfd_rows<D, double, false><<<grid_for(Vd, blk), blk, 0, s>>>(Ds, Ds, 1.0, Ts, -2.0, ck, cw, dk, dw, vfd,
		                                                               nullptr, nullptr);
		k_vfd_rows<D, double, false><<<grid_for(Vt, blk), blk, 0, s>>>(Ts, Ts, 1.0, E0, 0.0, ck, cw, dk, dw, vfd + Vd,
		                                                               nullptr, nullptr);
	} else {
		k_vfd_rows<D, double, false><<<grid_for(Vt, blk), blk, 0, s>>>(Ts, Ts, 1.0, Ds, -2.0, ck, cw, dk, dw, vfd,
		                                                               nullptr, nullptr);
		k_vfd_rows<D, double, false><<<grid_for(Vd, blk), blk, 0, s>>>(Ds, Ds, 1.0, E0, 0.0, ck, cw, dk, dw, vfd + Vt,
		                                                               nullptr, nullptr);
	}
	SA_CHECK(cudaGetLastError());
	// device_sum clears the part of its buffer that accumulates before using it (and waits for the stream)
	double v = device_sum(vfd, Vd + Vt, sumScr, s);
	int bad = 0;
	SA_CHECK(cudaMemcpy(&bad, badIndex, sizeof(int), cudaMemcpyDeviceToHost));
	if (bad) throw BadIndex{};
	return v;
}

}  // namespace sa

#include <mutex>

namespace {
std::mutex g_noallocMutex;
double *g_noallocAddr[128] = {};

// device address of the scratch array on device dev (looked up on first use)
int noalloc_scratch(int dev, double **out)
{
	if (dev < 0 || dev >= 128) return SA_ERR_UNSUPPORTED;
	std::lock_guard<std::mutex> lock(g_noallocMutex);
	if (!g_noallocAddr[dev]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, sa::g_noallocScratch);
		if (e != cudaSuccess || !p) { cudaGetLastError(); return SA_ERR_CUDA; }
		g_noallocAddr[dev] = (double *) p;
	}
	*out = g_noallocAddr[dev];
	return SA_OK;
}

// device memory of GPU dev (or managed memory): memory of another GPU is refused, a kernel on this one would
// read it only through peer access
bool on_device(const void *p, int dev)
{
	cudaPointerAttributes a;
	if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
	return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
}
}  // namespace

extern "C" int sa_varifold_noalloc(int dim, int lmkNum, const double *lmkMat, int vfdElmNum, const int *vfdVtxMat,
                                   int tgtElmNum, const double *tgtCenPosMat, const double *tgtUniDirMat,
                                   const double *tgtElmVolVec, char cenKnlType, double cenKnlWidth, char dirKnlType,
                                   double dirKnlWidth, void *stream, double *objOut)
{
	if (dim != 2 && dim != 3) return SA_ERR_ARG;
	if (lmkNum <= 0 || vfdElmNum <= 0 || tgtElmNum <= 0 || !objOut) return SA_ERR_ARG;
	if (vfdElmNum > sa::kNoAllocMaxElm || tgtElmNum > sa::kNoAllocMaxElm) return SA_ERR_ARG;   // scratch limit
	if (cenKnlType != 'G' && cenKnlType != 'C' && cenKnlType != 'M') return SA_ERR_ARG;
	if (dirKnlType != 'B' && dirKnlType != 'L' && dirKnlType != 'O' && dirKnlType != 'U') return SA_ERR_ARG;
	if (!sa::kernel_widths_ok(cenKnlWidth, dirKnlType, dirKnlWidth)) return SA_ERR_ARG;
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return SA_ERR_CUDA; }
	if (!on_device(lmkMat, dev) || !on_device(vfdVtxMat, dev) || !on_device(tgtCenPosMat, dev) ||
	    !on_device(tgtUniDirMat, dev) || !on_device(tgtElmVolVec, dev))
		return SA_ERR_ARG;                     // inputs must already be in this device's memory: nothing is copied
	double *scr = nullptr;
	int rc = noalloc_scratch(dev, &scr);
	if (rc != SA_OK) return rc;
	cudaStream_t s = (cudaStream_t) stream;
	try {
		double v = dim == 2
		    ? sa::varifold_in_scratch<2>(scr, lmkNum, lmkMat, vfdElmNum, vfdVtxMat, tgtElmNum, tgtCenPosMat,
		                                 tgtUniDirMat, tgtElmVolVec, cenKnlType, cenKnlWidth, dirKnlType,
		                                 dirKnlWidth, s)
		    : sa::varifold_in_scratch<3>(scr, lmkNum, lmkMat, vfdElmNum, vfdVtxMat, tgtElmNum, tgtCenPosMat,
		                                 tgtUniDirMat, tgtElmVolVec, cenKnlType, cenKnlWidth, dirKnlType,
		                                 dirKnlWidth, s);
		if (cudaMemcpy(objOut, &v, sizeof(double), cudaMemcpyDefault) != cudaSuccess) {
			cudaGetLastError();
			return SA_ERR_CUDA;
		}
	} catch (const sa::BadIndex &) {
		return SA_ERR_ARG;                     // a node index outside [0, lmkNum): no objective
	} catch (const sa::CudaError &) {
		cudaGetLastError();
		return SA_ERR_CUDA;
	}
	return SA_OK;
}
