// sa_kernel.cu -- RKHS kernel matrix and the K-preconditioned CG of frame mode.
//
// Reference: 2D_frame/computeKernel.cu:7-209 (2D Matern through x^2 K0(x) and
// x K1(x), inc/polybesselk.h:8-99 with the rational-approximation tables of
// inc/besselk.h), 3D_frame/computeKernel.cu:5-153 (closed-form Matern
// n + 1/2), 2D_frame/addEpsIdentity.cu:3-20, and the CG of
// 2D_frame/ipcg.cu:11-100 with ipcgWholeMatrixMultiplication.cu:21-45,
// ipcgSecondMatrixMultiplication.cu:8-24, ipcgKernelMultiplication.cu:5-17.
//
// GB300 changes: scalars and the stopping test stay on the device (the
// reference returns every dot product to the host), and the dense Cholesky
// of K is gone.  The reference needs potrs(K, x0) only for the warm start
// x0 = v_prev; here the solve tracks w = K^{-1} x through the CG recurrences
// (w += alpha K^{-1}d, with K^{-1}d already tracked as KidVec) and starts the
// next step from x0 = K_new w_prev, whose K_new^{-1} x0 = w_prev is known
// exactly.  The converged velocity is the same solution of the same system
// to the CG tolerance.
#include "sa_internal.cuh"
#include "sa_grid.cuh"
#include <cmath>

namespace sa {

// rational-approximation coefficients (inc/besselk.h:4-180), same values
__constant__ double cP01[6] = { 2.4708152720399552679e+03,  5.9169059852270512312e+03,
                                4.6850901201934832188e+02,  1.1999463724910714109e+01,
                                1.3166052564989571850e-01,  5.8599221412826100000e-04};
__constant__ double cQ01[3] = { 2.1312714303849120380e+04, -2.4994418972832303646e+02, 1};
__constant__ double cP02[4] = {-4.0320340761145482298e+05, -1.7733784684952985886e+04,
                               -2.9601657892958843866e+02, -1.6414452837299064100e+00};
__constant__ double cQ02[4] = {-1.6128136304458193998e+06,  2.9865713163054025489e+04,
                               -2.5064972445877992730e+02,  1};
__constant__ double cP03[10] = { 1.1600249425076035558e+02,  2.3444738764199315021e+03,
                                 1.8321525870183537725e+04,  7.1557062783764037541e+04,
                                 1.5097646353289914539e+05,  1.7398867902565686251e+05,
                                 1.0577068948034021957e+05,  3.1075408980684392399e+04,
                                 3.6832589957340267940e+03,  1.1394980557384778174e+02};
__constant__ double cQ03[11] = { 9.2556599177304839811e+01,  1.8821890840982713696e+03,
                                 1.4847228371802360957e+04,  5.8824616785857027752e+04,
                                 1.2689839587977598727e+05,  1.5144644673520157801e+05,
                                 9.7418829762268075784e+04,  3.1474655750295278825e+04,
                                 4.4329628889746408858e+03,  2.0013443064949242491e+02, 1};
__constant__ double cP11[6] = {-2.2149374878243304548e+06,  7.1938920065420586101e+05,
                                1.7733324035147015630e+05,  7.1885382604084798576e+03,
                                9.9991373567429309922e+01,  4.8127070456878442310e-01};
__constant__ double cQ11[4] = {-2.2149374878243304548e+06,  3.7264298672067697862e+04,
                               -2.8143915754538725829e+02,  1};
__constant__ double cP12[5] = {-1.3531161492785421328e+06, -1.4758069205414222471e+05,
                               -4.5051623763436087023e+03, -5.3103913335180275253e+01,
                               -2.2795590826955002390e-01};
__constant__ double cQ12[4] = {-2.7062322985570842656e+06,  4.3117653211351080007e+04,
                               -3.0507151578787595807e+02,  1};
__constant__ double cP13[11] = { 2.2196792496874548962e+00,  4.4137176114230414036e+01,
                                 3.4122953486801312910e+02,  1.3319486433183221990e+03,
                                 2.8590657697910288226e+03,  3.4540675585544584407e+03,
                                 2.3123742209168871550e+03,  8.1094256146537402173e+02,
                                 1.3182609918569941308e+02,  7.5584584631176030810e+00,
                                 6.4257745859173138767e-02};
__constant__ double cQ13[10] = { 1.7710478032601086579e+00,  3.4552228452758912848e+01,
                                 2.5951223655579051357e+02,  9.6929165726802648634e+02,
                                 1.9448440788918006154e+03,  2.1181000487171943810e+03,
                                 1.2082692316002348638e+03,  3.3031020088765390854e+02,
                                 3.6001069306861518855e+01,  1};

__device__ __forceinline__ double polyval(int deg, const double *c, double x)
{
	double v = c[deg];
	for (int i = deg - 1; i >= 0; --i) v = v * x + c[i];
	return v;
}

__device__ double p0fcn(double x)
{   // x^2 K0(x): inc/polybesselk.h:17-54
	if (x < DBL_EPSILON || x > 700.0) return 0.0;
	if (x <= 1.0) {
		double xs = x * x, lx = log(x);
		double PQ01 = polyval(5, cP01, xs) / polyval(2, cQ01, xs);
		double PQ02 = polyval(3, cP02, xs) / polyval(3, cQ02, xs);
		return xs * (PQ01 - lx * (xs * PQ02 + 1.0));
	}
	double xi = 1.0 / x;
	return x * sqrt(x) * exp(-x) * (polyval(9, cP03, xi) / polyval(10, cQ03, xi));
}

__device__ double p1fcn(double x)
{   // x K1(x): inc/polybesselk.h:56-99
	if (x < DBL_EPSILON) return 1.0;
	if (x > 700.0) return 0.0;
	if (x <= 1.0) {
		double xs = x * x, lx = log(x);
		double PQ11 = polyval(5, cP11, xs) / polyval(3, cQ11, xs);
		double PQ12 = polyval(4, cP12, xs) / polyval(3, cQ12, xs);
		return PQ11 + xs * lx * PQ12;
	}
	double xi = 1.0 / x;
	return sqrt(x) * exp(-x) * (polyval(10, cP13, xi) / polyval(9, cQ13, xi));
}

template <int D>
__device__ __forceinline__ double kernel_value(int order, double w, double d2)
{
	if (D == 2) {
		if (order == -1) return exp(-(d2 / (w * w)));
		double dij = sqrt(d2) / w, dsq = dij * dij;
		double f1 = p1fcn(dij), f0 = order > 0 ? p0fcn(dij) : 0.0;
		switch (order) {
		case 0: return f1;
		case 1: return 0.5 * (f0 + 2.0 * f1);
		case 2: return (4.0 * f0 + (8.0 + dsq) * f1) / 8.0;
		case 3: return ((24.0 + dsq) * f0 + 8.0 * (6.0 + dsq) * f1) / 48.0;
		default: return (12.0 * (16.0 + dsq) * f0 + (384.0 + dsq * (72.0 + dsq)) * f1) / 384.0;
		}
	}
	if (order == -1) return exp(-(d2 / (w * w)));
	double r = sqrt(d2) / w, ex = exp(-r);
	switch (order) {
	case 0: return ex;
	case 1: return (1.0 + r) * ex;
	case 2: return (3.0 + r * (3.0 + r)) / 3.0 * ex;
	case 3: return (15.0 + r * (15.0 + r * (6.0 + r))) / 15.0 * ex;
	default: return (105.0 + r * (105.0 + r * (45.0 + r * (10.0 + r)))) / 105.0 * ex;
	}
}

// dk/d(d2), the kernel's derivative with respect to the squared distance (discrete adjoint of the frame
// model).  2D Matern through d(x K1)/dx = -x K0 = -p0 / x and d(x^2 K0)/dx = 2 p0 / x - x p1; every order
// but 0 carries a factor x that cancels dx/d(d2) = 1 / (2 w^2 x).  Not called at d2 = 0.
template <int D>
__device__ __forceinline__ double kernel_dvalue(int order, double w, double d2)
{
	if (order == -1) return -exp(-(d2 / (w * w))) / (w * w);
	const double w2 = w * w;
	if (D == 2) {
		double x = sqrt(d2) / w, xs = x * x;
		double f1 = p1fcn(x), f0 = p0fcn(x);
		switch (order) {
		case 0: return -f0 / (2.0 * w2 * xs);
		case 1: return -0.5 * f1 / (2.0 * w2);
		case 2: return -(2.0 * f1 + f0) / (16.0 * w2);
		case 3: return -(4.0 * f0 + (8.0 + xs) * f1) / (96.0 * w2);
		default: return -((24.0 + xs) * f0 + (48.0 + 8.0 * xs) * f1) / (768.0 * w2);
		}
	}
	double r = sqrt(d2) / w, ex = exp(-r);
	switch (order) {
	case 0: return -ex / (2.0 * w2 * r);
	case 1: return -ex / (2.0 * w2);
	case 2: return -(1.0 + r) * ex / (6.0 * w2);
	case 3: return -(3.0 + r * (3.0 + r)) * ex / (30.0 * w2);
	default: return -(15.0 + r * (15.0 + r * (6.0 + r))) * ex / (210.0 * w2);
	}
}

// a_x_i += ldm sum_{j != i} 2 dk/d(d2)(x_i - x_j) sum_d (alpha_id beta_jd + alpha_jd beta_id): the vector-Jacobian
// product of x -> -ldm n^T K(x)^{-1} v with alpha = K^{-1} n, beta = K^{-1} v (nodal vectors, interleaved).
// One thread per node, the other nodes in shared-memory tiles.
template <int D>
__global__ void k_adj_kernel_term(int N, const double *__restrict__ x, const double *__restrict__ alpha,
                                  const double *__restrict__ beta, int order, double w, double ldm,
                                  double *__restrict__ ax)
{
	__shared__ double tx[128 * D], ta[128 * D], tb[128 * D];
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	Vec<D> xi, ai, bi;
	for (int d = 0; d < D; ++d) {
		xi.c[d] = i < N ? x[(long) i * D + d] : 0.0;
		ai.c[d] = i < N ? alpha[(long) i * D + d] : 0.0;
		bi.c[d] = i < N ? beta[(long) i * D + d] : 0.0;
	}
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	for (int j0 = 0; j0 < N; j0 += 128) {
		const int nt = min(128, N - j0);
		__syncthreads();
		for (int t = threadIdx.x; t < nt * D; t += blockDim.x) {
			tx[t] = x[(long) j0 * D + t];
			ta[t] = alpha[(long) j0 * D + t];
			tb[t] = beta[(long) j0 * D + t];
		}
		__syncthreads();
		if (i >= N) continue;
		for (int jj = 0; jj < nt; ++jj) {
			if (j0 + jj == i) continue;
			double d2 = 0.0, ab = 0.0, dx[D];
			for (int d = 0; d < D; ++d) {
				dx[d] = xi.c[d] - tx[jj * D + d];
				d2 += dx[d] * dx[d];
				ab += ai.c[d] * tb[jj * D + d] + ta[jj * D + d] * bi.c[d];
			}
			const double g = 2.0 * kernel_dvalue<D>(order, w, d2) * ab;
			for (int d = 0; d < D; ++d) acc[d] += g * dx[d];
		}
	}
	if (i < N)
		for (int d = 0; d < D; ++d) ax[(long) i * D + d] += ldm * acc[d];
}

template <int D>
void launch_adj_kernel_term(const Model &md, int N, const double *x, const double *alpha, const double *beta,
                            double *ax, cudaStream_t s)
{
	k_adj_kernel_term<D><<<grid_for(N, 128), 128, 0, s>>>(N, x, alpha, beta, md.knlOrder, md.knlWidth, md.ldmWgt, ax);
}

// One RKHS matrix entry k(|q_i - q_j| / w) (without the eps diagonal).  Compiled once, not inlined: the
// stored matrix and the matrix-free products evaluate it with the same instructions, so the compiler's
// multiply-add fusion cannot differ between the two callers and both give the same bits.  Symmetric bit for
// bit: (a - b)^2 = (b - a)^2 exactly.
template <int D>
__device__ __noinline__ double kernel_entry(int order, double w, Vec<D> qi, Vec<D> qj)
{
	double d2 = (qi.c[0] - qj.c[0]) * (qi.c[0] - qj.c[0]);
	for (int d = 1; d < D; ++d) d2 = d2 + (qi.c[d] - qj.c[d]) * (qi.c[d] - qj.c[d]);
	return kernel_value<D>(order, w, d2);
}

// K[j*N + i] = k(|q_i - q_j| / w) + eps * delta_ij
template <int D>
__global__ void k_kernel_matrix(int N, const double *__restrict__ x, int order, double w, double eps,
                                double *__restrict__ K)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	const Vec<D> qi = load_node<D>(x, i);
	for (int j = blockIdx.y; j < N; j += gridDim.y) {
		double v = kernel_entry<D>(order, w, qi, load_node<D>(x, j));
		if (i == j) v += eps;
		K[(long) j * N + i] = v;
	}
}

template <int D>
void launch_kernel_matrix(const Model &md, int N, const double *x, double *K, cudaStream_t s)
{
	dim3 g(grid_for(N, 128), std::min(N, 65535));
	k_kernel_matrix<D><<<g, 128, 0, s>>>(N, x, md.knlOrder, md.knlWidth, md.knlEps, K);
}

// ---------------------------------------------------------------------------
// dense K X for D interleaved columns: partial sums over column slices
// ---------------------------------------------------------------------------
constexpr int kDenseRows = 128, kDenseSlices = 16, kDenseTile = 128;

template <int D>
__global__ void k_dense_partial(int N, const double *__restrict__ K, const double *__restrict__ X,
                                double *__restrict__ part)
{
	__shared__ double xs[kDenseTile * D];
	int i = blockIdx.x * kDenseRows + threadIdx.x;
	int s = blockIdx.y;
	int per = (N + kDenseSlices - 1) / kDenseSlices;
	int j0 = s * per, j1 = min(N, j0 + per);
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	for (int jt = j0; jt < j1; jt += kDenseTile) {
		int nt = min(kDenseTile, j1 - jt);
		__syncthreads();
		for (int t = threadIdx.x; t < nt * D; t += blockDim.x) xs[t] = X[(long) jt * D + t];
		__syncthreads();
		if (i < N)
			for (int jj = 0; jj < nt; ++jj) {
				double k = K[(long) (jt + jj) * N + i];
				for (int d = 0; d < D; ++d) acc[d] += k * xs[jj * D + d];
			}
	}
	if (i < N)
		for (int d = 0; d < D; ++d) part[((long) s * N + i) * D + d] = acc[d];
}

template <int D>
__global__ void k_dense_sum(int N, const double *__restrict__ part, double *__restrict__ Y)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k >= (long) N * D) return;
	double s = 0.0;
	for (int t = 0; t < kDenseSlices; ++t) s += part[(long) t * N * D + k];
	Y[k] = s;
}

template <int D>
void launch_dense_matvec(int N, const double *K, const double *x, double *y, double *part, cudaStream_t s)
{
	dim3 g(grid_for(N, kDenseRows), kDenseSlices);
	k_dense_partial<D><<<g, kDenseRows, 0, s>>>(N, K, x, part);
	k_dense_sum<D><<<grid_for((long) N * D), kBlock, 0, s>>>(N, part, y);
}

// K X without the stored matrix (meshes whose N x N matrix does not fit): the same slices, tiles and
// summation order as k_dense_partial, each K entry evaluated on the fly by the same kernel_entry as
// k_kernel_matrix, so the result equals the stored-matrix product bit for bit.  Costs one kernel
// evaluation (a square root, an exponential, and for 2D Matern the Bessel rational approximations) per
// matrix entry instead of one 8-byte read.
template <int D>
__global__ void k_kernel_partial(int N, const double *__restrict__ q, int order, double w, double eps,
                                 const double *__restrict__ X, double *__restrict__ part)
{
	__shared__ double xs[kDenseTile * D], qs[kDenseTile * D];
	int i = blockIdx.x * kDenseRows + threadIdx.x;
	int s = blockIdx.y;
	int per = (N + kDenseSlices - 1) / kDenseSlices;
	int j0 = s * per, j1 = min(N, j0 + per);
	Vec<D> qi;
	for (int d = 0; d < D; ++d) qi.c[d] = i < N ? q[(long) i * D + d] : 0.0;
	double acc[D];
	for (int d = 0; d < D; ++d) acc[d] = 0.0;
	for (int jt = j0; jt < j1; jt += kDenseTile) {
		int nt = min(kDenseTile, j1 - jt);
		__syncthreads();
		for (int t = threadIdx.x; t < nt * D; t += blockDim.x) {
			xs[t] = X[(long) jt * D + t];
			qs[t] = q[(long) jt * D + t];
		}
		__syncthreads();
		if (i < N)
			for (int jj = 0; jj < nt; ++jj) {
				Vec<D> qj;
				for (int d = 0; d < D; ++d) qj.c[d] = qs[jj * D + d];
				double k = kernel_entry<D>(order, w, qi, qj);
				if (i == jt + jj) k += eps;
				for (int d = 0; d < D; ++d) acc[d] += k * xs[jj * D + d];
			}
	}
	if (i < N)
		for (int d = 0; d < D; ++d) part[((long) s * N + i) * D + d] = acc[d];
}

// y = K x with K stored (dense) or, when K is null, evaluated from the node positions q
template <int D>
static void kernel_matvec(const Model &md, int N, const double *K, const double *q, const double *x, double *y,
                          double *part, cudaStream_t s)
{
	if (K) {
		launch_dense_matvec<D>(N, K, x, y, part, s);
		return;
	}
	dim3 g(grid_for(N, kDenseRows), kDenseSlices);
	k_kernel_partial<D><<<g, kDenseRows, 0, s>>>(N, q, md.knlOrder, md.knlWidth, md.knlEps, x, part);
	k_dense_sum<D><<<grid_for((long) N * D), kBlock, 0, s>>>(N, part, y);
}


// ---------------------------------------------------------------------------
// K-preconditioned CG (reference ipcg) with device scalars
// ---------------------------------------------------------------------------
struct KScal {
	double bSqu, rSqu, rKr, rKrNew, dAd, alpha, beta, tolSqu, ldmWgt;
	int done, code, iters, itrMax;
	unsigned int counter;
	int pad;
};

constexpr int kKBlock = 256;

template <int K>
__device__ __forceinline__ bool kreduce(double (&v)[K], double *part, unsigned int *counter)
{
	__shared__ double sm[K][kKBlock / 32];
	__shared__ bool last;
	int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int k = 0; k < K; ++k)
		for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
	if (lane == 0) for (int k = 0; k < K; ++k) sm[k][wid] = v[k];
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int k = 0; k < K; ++k) {
			double s = 0.0;
			for (int w = 0; w < kKBlock / 32; ++w) s += sm[k][w];
			part[k * gridDim.x + blockIdx.x] = s;
		}
		__threadfence();
		unsigned int t = atomicAdd(counter, 1u);
		last = (t == gridDim.x - 1);
	}
	__syncthreads();
	return last;
}

template <int K>
__device__ __forceinline__ void kfinish(double (&out)[K], const double *part)
{
	int lane = threadIdx.x & 31;
	for (int k = 0; k < K; ++k) {
		double s = 0.0;
		for (int b = lane; b < (int) gridDim.x; b += 32) s += __ldcg(part + k * gridDim.x + b);
		for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
		out[k] = s;
	}
}

// (b, b): zero rhs gives x = 0, w = 0
template <int D>
__global__ void k_kp_bnorm(int N, const double *__restrict__ b, double *part, KScal *sc)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	double v[1] = {0.0};
	if (i < N) for (int d = 0; d < D; ++d) v[0] += b[(long) i * D + d] * b[(long) i * D + d];
	if (!kreduce<1>(v, part, &sc->counter)) return;
	double o[1]; kfinish<1>(o, part);
	if (threadIdx.x == 0) {
		sc->bSqu = o[0];
		if (!isfinite(o[0])) { sc->code = SA_ERR_NONFINITE; sc->done = 1; }
		else if (o[0] == 0.0) sc->done = 2;          // x = 0
		sc->counter = 0;
	}
}

// r = b - (ldm w + Bx0), (r, r)
template <int D>
__global__ void k_kp_init_r(SellOp A, const double *__restrict__ blk, const double *__restrict__ b,
                            const double *__restrict__ x, const double *__restrict__ w, double *__restrict__ r,
                            double *part, KScal *sc)
{
	if (sc->done) return;
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	const int N = A.N;
	double v[1] = {0.0};
	if (i < N) {
		double acc[D];
		sell_row<D, double, double>(A, blk, i, x, acc);
		for (int d = 0; d < D; ++d) {
			long k = (long) i * D + d;
			double Ax = sc->ldmWgt * w[k] + acc[d];
			double rk = 1.0 * b[k] + -1.0 * Ax;
			r[k] = rk;
			v[0] += rk * rk;
		}
	}
	if (!kreduce<1>(v, part, &sc->counter)) return;
	double o[1]; kfinish<1>(o, part);
	if (threadIdx.x == 0) {
		sc->rSqu = o[0];
		if (!isfinite(o[0])) { sc->code = SA_ERR_NONFINITE; sc->done = 1; }
		else if (o[0] < sc->bSqu * sc->tolSqu) sc->done = 1;
		sc->counter = 0;
	}
}

// (r, Kr) after Kr = K r; first = 1: initialise Kid = r, d = Kr; else beta and the d / Kid updates
template <int D>
__global__ void k_kp_rkr(int N, const double *__restrict__ r, const double *__restrict__ Kr, double *part,
                         KScal *sc, int first)
{
	if (sc->done) return;
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	double v[1] = {0.0};
	if (i < N) for (int d = 0; d < D; ++d) v[0] += r[(long) i * D + d] * Kr[(long) i * D + d];
	if (!kreduce<1>(v, part, &sc->counter)) return;
	double o[1]; kfinish<1>(o, part);
	if (threadIdx.x == 0) {
		if (o[0] == 0.0 || !isfinite(o[0])) {
			sc->code = isfinite(o[0]) ? SA_ERR_BREAKDOWN : SA_ERR_NONFINITE;
			sc->done = 1;
		} else if (first) {
			sc->rKr = o[0];
		} else {
			sc->beta = o[0] / sc->rKr;
			sc->rKr = o[0];
		}
		sc->counter = 0;
	}
}

// Kid = r + beta Kid; d = Kr + beta d (first: Kid = r, d = Kr)
template <int D>
__global__ void k_kp_dir(int N, const double *__restrict__ r, const double *__restrict__ Kr, double *__restrict__ Kid,
                         double *__restrict__ dv, const KScal *sc, int first)
{
	if (sc->done) return;
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k >= (long) N * D) return;
	if (first) { Kid[k] = r[k]; dv[k] = Kr[k]; return; }
	double be = sc->beta;
	Kid[k] = 1.0 * r[k] + be * Kid[k];
	dv[k] = 1.0 * Kr[k] + be * dv[k];
}

// Bd = (E + btm P) d; Ad = ldm Kid + Bd; (d, Ad) -> alpha
template <int D>
__global__ void k_kp_ad(SellOp A, const double *__restrict__ blk, const double *__restrict__ dv,
                        const double *__restrict__ Kid, double *__restrict__ Ad, double *part, KScal *sc)
{
	if (sc->done) return;
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	const int N = A.N;
	double v[1] = {0.0};
	if (i < N) {
		double acc[D];
		sell_row<D, double, double>(A, blk, i, dv, acc);
		for (int d = 0; d < D; ++d) {
			long k = (long) i * D + d;
			double a = sc->ldmWgt * Kid[k] + 1.0 * acc[d];
			Ad[k] = a;
			v[0] += dv[k] * a;
		}
	}
	if (!kreduce<1>(v, part, &sc->counter)) return;
	double o[1]; kfinish<1>(o, part);
	if (threadIdx.x == 0) {
		sc->dAd = o[0];
		if (o[0] == 0.0 || !isfinite(o[0])) {
			sc->code = isfinite(o[0]) ? SA_ERR_BREAKDOWN : SA_ERR_NONFINITE;
			sc->done = 1;
		} else sc->alpha = sc->rKr / o[0];
		sc->counter = 0;
	}
}

// x += alpha d; w += alpha Kid; r -= alpha Ad; (r, r) -> stop test
template <int D>
__global__ void k_kp_step(int N, double *__restrict__ x, double *__restrict__ w, double *__restrict__ r,
                          const double *__restrict__ dv, const double *__restrict__ Kid,
                          const double *__restrict__ Ad, double *part, KScal *sc)
{
	if (sc->done) return;
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	double v[1] = {0.0};
	if (i < N) {
		double al = sc->alpha;
		for (int d = 0; d < D; ++d) {
			long k = (long) i * D + d;
			x[k] = 1.0 * x[k] + al * dv[k];
			w[k] = w[k] + al * Kid[k];
			double rk = 1.0 * r[k] + -al * Ad[k];
			r[k] = rk;
			v[0] += rk * rk;
		}
	}
	if (!kreduce<1>(v, part, &sc->counter)) return;
	double o[1]; kfinish<1>(o, part);
	if (threadIdx.x == 0) {
		sc->rSqu = o[0];
		sc->iters += 1;
		if (!isfinite(o[0])) { sc->code = SA_ERR_NONFINITE; sc->done = 1; }
		else if (o[0] < sc->bSqu * sc->tolSqu) sc->done = 1;
		else if (sc->iters >= sc->itrMax) { sc->code = SA_ERR_NOT_CONVERGED; sc->done = 1; }
		sc->counter = 0;
	}
}

__global__ void k_kp_zero(long n, double *x, double *w, const KScal *sc)
{
	if (sc->done != 2) return;
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) { x[k] = 0.0; w[k] = 0.0; }
}

// ---------------------------------------------------------------------------
// Persistent K-preconditioned CG: one cooperative launch runs all iterations of the loop below (six
// launches per iteration there).  One CTA per SM, kKpWarps warps.  Per iteration three grid-wide exact
// sums (sa_grid.cuh), which are also the grid's barriers:
//   A  rows (grid-stride, one thread per row): Kid = r + beta Kid, d = Kr + beta d and
//      Ad = ldm Kid + (E + btm P) d, with (d, Ad) -> alpha.  A row that gathers a neighbour's d forms it
//      the same way from the neighbour's previous d and Kr (two d buffers alternate), so no barrier
//      separates the direction update from the operator;
//   B  rows: x += alpha d, w += alpha Kid, r -= alpha Ad, with (r, r) -> stop test;
//   C  Kr = K r, with (r, Kr) -> beta.  Each CTA forms the whole rows of its row range: K is symmetric bit
//      for bit (kernel_entry squares differences), so row i is read contiguously, lanes over columns,
//      warps over (row, column segment) units, a fixed shuffle tree per unit and the segments added in a
//      fixed order in shared memory.  The matrix-free form evaluates each entry with the same
//      kernel_entry call the stored matrix was written with, in the same place: both give the same bits.
// Vectors that other CTAs write during the launch are read with __ldcg (L2), never through the
// incoherent L1.  Iterates, stopping rule and status codes are those of the loop below.
// ---------------------------------------------------------------------------
constexpr int kKpWarps = 16;
constexpr int kKpUnits = 512;     // (row, segment) units per chunk of phase C

struct KpVec {
	double *x, *w, *r, *Kr, *Kid, *d0, *d1, *Ad;
};

__device__ __forceinline__ double kp_dir(double kr, double dOld, double be, bool first)
{
	return first ? kr : __fma_rn(be, dOld, kr);
}

template <int D, bool kFree>
__global__ void __launch_bounds__(32 * kKpWarps, 1)
k_kpcg_persist(SellOp A, const double *__restrict__ blk, const double *__restrict__ K, const double *__restrict__ q,
               int order, double kw, double eps, KpVec v, double *part, KScal *sc, GridBar *bar)
{
	__shared__ FxScratch fs;
	__shared__ double segPart[kKpUnits][D];
	if (sc->done) return;                       // set before the launch: the same for every CTA
	const int N = A.N, nctas = gridDim.x, lc = blockIdx.x;
	const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, W = blockDim.x >> 5;
	// rows of phases A and B: 32-row slices dealt round-robin over the CTAs first, so that a small mesh
	// spreads its row work (gathers) over all SMs instead of the first few CTAs
	const int nsl = (N + 31) >> 5, sl0 = blockIdx.x + gridDim.x * wp, slStride = gridDim.x * W;
	const double bSqu = sc->bSqu, tolSqu = sc->tolSqu, ldm = sc->ldmWgt;
	const int itrMax = sc->itrMax;
	double rKr = sc->rKr, rr = sc->rSqu, be = 0.0;
	int it = sc->iters, code = SA_OK;
	bool first = true;
	unsigned int target = 0;
	double *partA = part, *partB = part + nctas, *partC = part + 2 * nctas;
	// phase C's row range and (row, segment) units
	const int r0 = (int) ((long) N * lc / nctas), r1 = (int) ((long) N * (lc + 1) / nctas), R = r1 - r0;
	const int SEG = min(8, max(1, (2 * W + max(R, 1) - 1) / max(R, 1)));
	const int RC = kKpUnits / SEG;
	double *dOld = v.d0, *dNew = v.d1;
	for (;;) {
		// A: direction, operator, (d, Ad)
		double loc[1] = {0.0}, res[1];
		for (int sl = sl0; sl < nsl; sl += slStride) {
			const int i = sl * 32 + lane, ln = lane;
			if (i >= N) continue;
			const int wdt = __ldg(A.width + sl);
			const long base = __ldg(A.off + sl) + ln;
			double acc[D];
			for (int c = 0; c < D; ++c) acc[c] = 0.0;
			for (int k = 0; k < wdt; ++k) {
				const long idx = base + ((long) k << 5);
				const int j = __ldg(A.col + idx);
				double dj[D];
				for (int c = 0; c < D; ++c)
					dj[c] = kp_dir(__ldcg(v.Kr + (long) j * D + c), first ? 0.0 : __ldcg(dOld + (long) j * D + c),
					               be, first);
				double a[D * D];
				load_block<D, double>(blk, A.total, idx, a);
				for (int r = 0; r < D; ++r)
					for (int c = 0; c < D; ++c) acc[r] += a[r * D + c] * dj[c];
			}
			for (int c = 0; c < D; ++c) {
				const long k = (long) i * D + c;
				const double ri = __ldcg(v.r + k);
				const double kid = first ? ri : __fma_rn(be, v.Kid[k], ri);
				const double di = kp_dir(__ldcg(v.Kr + k), first ? 0.0 : __ldcg(dOld + k), be, first);
				const double ad = __fma_rn(ldm, kid, acc[c]);
				v.Kid[k] = kid;
				dNew[k] = di;
				v.Ad[k] = ad;
				loc[0] += di * ad;
			}
		}
		if (!grid_reduce<1, double>(loc, res, partA, lc, nctas, bar, target, fs)) { code = SA_ERR_TIMEOUT; break; }
		const double dAd = res[0];
		if (dAd == 0.0 || !isfinite(dAd)) { code = isfinite(dAd) ? SA_ERR_BREAKDOWN : SA_ERR_NONFINITE; break; }
		const double alpha = rKr / dAd;
		// B: x, w, r and (r, r)
		loc[0] = 0.0;
		for (int sl = sl0; sl < nsl; sl += slStride) {
			const int i = sl * 32 + lane;
			if (i >= N) continue;
			for (int c = 0; c < D; ++c) {
				const long k = (long) i * D + c;
				v.x[k] = __fma_rn(alpha, dNew[k], v.x[k]);
				v.w[k] = __fma_rn(alpha, v.Kid[k], v.w[k]);
				const double rk = __fma_rn(-alpha, v.Ad[k], v.r[k]);
				v.r[k] = rk;
				loc[0] += rk * rk;
			}
		}
		if (!grid_reduce<1, double>(loc, res, partB, lc, nctas, bar, target, fs)) { code = SA_ERR_TIMEOUT; break; }
		rr = res[0];
		++it;
		if (!isfinite(rr)) { code = SA_ERR_NONFINITE; break; }
		if (rr < bSqu * tolSqu) { code = SA_OK; break; }
		if (it >= itrMax) { code = SA_ERR_NOT_CONVERGED; break; }
		// C: Kr = K r over the CTA's rows, (r, Kr)
		loc[0] = 0.0;
		for (int c0 = r0; c0 < r1; c0 += RC) {
			const int rc = min(RC, r1 - c0), units = rc * SEG;
			for (int u = wp; u < units; u += W) {
				const int i = c0 + u / SEG, sg = u % SEG;
				const int j0 = (int) ((long) N * sg / SEG), j1 = (int) ((long) N * (sg + 1) / SEG);
				double acc[D];
				for (int c = 0; c < D; ++c) acc[c] = 0.0;
				Vec<D> qi;
				if constexpr (kFree) qi = load_node<D>(q, i);
#pragma unroll 4
				for (int j = j0 + lane; j < j1; j += 32) {
					double kij;
					if constexpr (kFree) {
						kij = kernel_entry<D>(order, kw, load_node<D>(q, j), qi);   // as K[i N + j] was written
						if (i == j) kij += eps;
					} else {
						kij = __ldg(K + (long) i * N + j);
					}
					for (int c = 0; c < D; ++c) acc[c] += kij * __ldcg(v.r + (long) j * D + c);
				}
				for (int c = 0; c < D; ++c)
					for (int off = 16; off > 0; off >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], off);
				if (lane == 0)
					for (int c = 0; c < D; ++c) segPart[u][c] = acc[c];
			}
			__syncthreads();
			for (int t = threadIdx.x; t < rc * D; t += blockDim.x) {
				const int il = t / D, c = t - il * D;
				double sum = 0.0;
				for (int sg = 0; sg < SEG; ++sg) sum += segPart[il * SEG + sg][c];
				const long k = (long) (c0 + il) * D + c;
				v.Kr[k] = sum;
				loc[0] += v.r[k] * sum;
			}
			__syncthreads();
		}
		if (!grid_reduce<1, double>(loc, res, partC, lc, nctas, bar, target, fs)) { code = SA_ERR_TIMEOUT; break; }
		const double o = res[0];
		if (o == 0.0 || !isfinite(o)) { code = isfinite(o) ? SA_ERR_BREAKDOWN : SA_ERR_NONFINITE; break; }
		be = o / rKr;
		rKr = o;
		first = false;
		double *t = dOld; dOld = dNew; dNew = t;
	}
	if (lc == 0 && threadIdx.x == 0) {
		sc->iters = it; sc->code = code; sc->rSqu = rr; sc->rKr = rKr; sc->done = 1;
	}
}

static int device_sm_count()
{
	int dev = 0, n = 0;
	SA_CHECK(cudaGetDevice(&dev));
	SA_CHECK(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
	return n;
}

// one cooperative launch of the persistent K-PCG when every SM can hold one of its CTAs; false: use the loop
template <int D, bool kFree>
static bool kpcg_persist_launch(const Mesh &m, const Model &md, const double *blk, const double *K, const double *q,
                                double *x, KpcgWork &wk, KScal *sc, cudaStream_t s)
{
	int occ = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_kpcg_persist<D, kFree>, 32 * kKpWarps, 0) !=
	    cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	const int nctas = device_sm_count();
	if (occ < 1 || 3L * nctas > wk.partLen) return false;
	GridBar *bar = (GridBar *) wk.bar;
	SA_CHECK(cudaMemsetAsync(bar, 0, sizeof(GridBar), s));
	SellOp A = sell_of(m);
	KpVec v{x, wk.wK, wk.r, wk.Kr, wk.Kid, wk.dv, wk.dv2, wk.Ad};
	int order = md.knlOrder;
	double kw = md.knlWidth, eps = md.knlEps;
	double *part = wk.part;
	void *args[] = {&A, (void *) &blk, (void *) &K, (void *) &q, &order, &kw, &eps, &v, &part, &sc, &bar};
	SA_CHECK(cudaLaunchCooperativeKernel((const void *) k_kpcg_persist<D, kFree>, dim3(nctas), dim3(32 * kKpWarps),
	                                     args, 0, s));
	return true;
}

template <int D>
int kpcg(const Mesh &m, const Model &md, const double *blk, const double *K, const double *q, const double *b,
         double *x, KpcgWork &wk, Status *st, int *itersOut, cudaStream_t s)
{
	(void) st;
	int N = m.N;
	long n = (long) N * D;
	int nb = grid_for(N, kKBlock);
	KScal h{};
	h.tolSqu = md.cgTolSqu; h.itrMax = md.cgItrMax; h.ldmWgt = md.ldmWgt;
	KScal *sc = (KScal *) wk.scal;
	SA_CHECK(cudaMemcpyAsync(sc, &h, sizeof(KScal), cudaMemcpyHostToDevice, s));
	double *dpart = wk.part + 4 * (long) nb;     // dense matvec slice partials
	k_kp_bnorm<D><<<nb, kKBlock, 0, s>>>(N, b, wk.part, sc);
	// warm start x0 = K w (w = K^{-1} v of the previous step)
	kernel_matvec<D>(md, N, K, q, wk.wK, x, dpart, s);
	k_kp_init_r<D><<<nb, kKBlock, 0, s>>>(sell_of(m), blk, b, x, wk.wK, wk.r, wk.part, sc);
	kernel_matvec<D>(md, N, K, q, wk.r, wk.Kr, dpart, s);
	k_kp_rkr<D><<<nb, kKBlock, 0, s>>>(N, wk.r, wk.Kr, wk.part, sc, 1);
	k_kp_dir<D><<<grid_for(n), kBlock, 0, s>>>(N, wk.r, wk.Kr, wk.Kid, wk.dv, sc, 1);
	const bool persist = md.cgKernel != SA_CG_TWO_KERNEL && wk.bar && wk.dv2 &&
	                     (K ? kpcg_persist_launch<D, false>(m, md, blk, K, q, x, wk, sc, s)
	                        : kpcg_persist_launch<D, true>(m, md, blk, K, q, x, wk, sc, s));
	const int chunk = 8;
	for (int it = 0; !persist && it < md.cgItrMax + chunk; it += chunk) {
		for (int k = 0; k < chunk; ++k) {
			k_kp_ad<D><<<nb, kKBlock, 0, s>>>(sell_of(m), blk, wk.dv, wk.Kid, wk.Ad, wk.part, sc);
			k_kp_step<D><<<nb, kKBlock, 0, s>>>(N, x, wk.wK, wk.r, wk.dv, wk.Kid, wk.Ad, wk.part, sc);
			kernel_matvec<D>(md, N, K, q, wk.r, wk.Kr, dpart, s);
			k_kp_rkr<D><<<nb, kKBlock, 0, s>>>(N, wk.r, wk.Kr, wk.part, sc, 0);
			k_kp_dir<D><<<grid_for(n), kBlock, 0, s>>>(N, wk.r, wk.Kr, wk.Kid, wk.dv, sc, 0);
		}
		SA_CHECK(cudaGetLastError());
		SA_CHECK(cudaMemcpyAsync(&h, sc, sizeof(KScal), cudaMemcpyDeviceToHost, s));
		SA_CHECK(cudaStreamSynchronize(s));
		if (h.done) break;
	}
	k_kp_zero<<<grid_for(n), kBlock, 0, s>>>(n, x, wk.wK, sc);
	SA_CHECK(cudaMemcpyAsync(&h, sc, sizeof(KScal), cudaMemcpyDeviceToHost, s));
	SA_CHECK(cudaStreamSynchronize(s));
	if (itersOut) *itersOut = h.iters;
	return h.code;
}

template void launch_adj_kernel_term<2>(const Model &, int, const double *, const double *, const double *, double *,
                                        cudaStream_t);
template void launch_adj_kernel_term<3>(const Model &, int, const double *, const double *, const double *, double *,
                                        cudaStream_t);
template void launch_kernel_matrix<2>(const Model &, int, const double *, double *, cudaStream_t);
template void launch_kernel_matrix<3>(const Model &, int, const double *, double *, cudaStream_t);
template int kpcg<2>(const Mesh &, const Model &, const double *, const double *, const double *, const double *,
                     double *, KpcgWork &, Status *, int *, cudaStream_t);
template int kpcg<3>(const Mesh &, const Model &, const double *, const double *, const double *, const double *,
                     double *, KpcgWork &, Status *, int *, cudaStream_t);

}  // namespace sa
