// sa_cg.cu -- Jacobi-preconditioned CG on the block-CSR operators.
//
// Replaces the reference's host-driven CG loop (2D_frame/ipcg.cu:11-100:
// four cuBLAS dots with a host round trip each, plus axpby kernels) for the
// layered model and for the reaction-diffusion solve (which the reference
// does by dense Cholesky, 2D_frame/deform.cu:99-104).
//
// Chronopoulos-Gear form: per iteration one matvec w = A u with the dot
// (w, u), and one update of p, s, x, r, u with the dots (r, u) and (r, r).
// Stopping rule as the reference: |r|^2 < tol^2 |b|^2; b = 0 gives x = 0.
// Four implementations of the same recurrences:
//   k_cg_persist   one cooperative launch per solve, one CTA per SM, one
//                  32-row slice per row warp with the row state in
//                  registers, a reducer warp per CTA, the CTA's column
//                  indices in shared memory, grid reductions in exact
//                  128-bit fixed point (sa_fixsum.cuh) behind bounded
//                  arrival-count barriers;
//   k_cg_persist_g the same for operators too large for row state in
//                  registers: vectors in global memory, contiguous slice
//                  ranges per CTA;
//   k_cg_spmv + k_cg_update  two kernels per iteration (fallback), scalars
//                  on the device, the last block of each kernel finishes
//                  its reduction in a fixed order; iterations queued in
//                  chunks of 16 one chunk ahead of the host's status check;
//   k_cg_batch     many independent solves (the server's instances) in one
//                  cooperative launch, each on its own CTA range.
// All results are deterministic (fixed grouping or order-free sums).
//
// Mixed precision (SA_PREC_MIXED): FP32 operator values and FP32 vectors in
// an inner CG (3x3 block-Jacobi) with FP64 dot products, inside an FP64
// iterative-refinement loop whose residual b - A x is recomputed with the
// FP64 operator.
#include "sa_internal.cuh"
#include "sa_fixsum.cuh"
#include "sa_grid.cuh"
#include <algorithm>
#include <cmath>
#include <mutex>
#include <queue>

namespace sa {

struct CgScal {
	double bb, rr, gam, gamPrev, alpha, beta, delta, tolSqu;
	int first, done, code, iters, zero, itrMax;
	unsigned int counter;
	int pad;
};

// FP64 throughput on GB300 is 2 thread-DFMA per clock per SM (a warp
// instruction occupies the SM's FP64 pipe for 16 cycles), so the kernels
// below avoid FP64 work that is not the algorithm's own: in the two-kernel
// path block sums of the dot products go through shared memory and are added
// by one warp, and the vector kernels run on a grid of kVecCtasPerSm CTAs per
// SM, every SM taking the same share of entries; the persistent kernels sum
// on the integer pipes.
constexpr int kCgBlock = 256;      // vector kernels
constexpr int kVecCtasPerSm = 4;   // vector kernels: CTAs per SM (grid-stride loops)
constexpr int kSlicesPerCta = 4;   // matvec: one warp per 32-row slice, one thread per row
constexpr int kSpmvBlock = 32 * kSlicesPerCta;

// fixed-order sum over the NT threads of a block of K values each; the
// result is valid in thread 0.  Called by every thread of the block; sm
// holds K * NT doubles of shared memory.
template <int K, int NT>
__device__ __forceinline__ void block_sum(double (&v)[K], double *sm)
{
	const int lane = threadIdx.x & 31;
	for (int k = 0; k < K; ++k) sm[k * NT + threadIdx.x] = v[k];
	__syncthreads();
	if (threadIdx.x < 32)
		for (int k = 0; k < K; ++k) {
			double s = sm[k * NT + lane];
#pragma unroll
			for (int q = 1; q < NT / 32; ++q) s += sm[k * NT + lane + 32 * q];
			for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
			v[k] = s;
		}
}

// u = M^-1 r for one row with the row's B x B block-Jacobi inverse bv (row-major)
template <int B, typename TV>
__device__ __forceinline__ void prec_block(const TV *bv, const TV (&r)[B], TV (&u)[B])
{
	for (int a = 0; a < B; ++a) {
		TV t = bv[a * B] * r[0];
		for (int c = 1; c < B; ++c) t += bv[a * B + c] * r[c];
		u[a] = t;
	}
}

// the same with the inverse read from global memory through the read-only path
template <int B, typename TV>
__device__ __forceinline__ void prec_block_ldg(const TV *__restrict__ bv, const TV (&r)[B], TV (&u)[B])
{
	TV m[B * B];
	for (int t = 0; t < B * B; ++t) m[t] = __ldg(bv + t);
	prec_block<B, TV>(m, r, u);
}

// The preconditioner is chosen at compile time.  Velocity solves (B = D node blocks) are block-Jacobi
// preconditioned in both precisions, with the inverses of the operator's diagonal D x D blocks; FP32
// reaction-diffusion inner solves (B = 1) take their 1 x 1 "blocks" from the same inverse pointer; FP64
// reaction-diffusion solves use the inverse diagonal (point Jacobi, the same preconditioner for B = 1).
template <int B, typename TV> constexpr bool block_prec() { return B > 1 || sizeof(TV) == sizeof(float); }

// block partials part[k * nb + blockIdx.x]; returns true in the block that
// arrives last (the one that finishes the reduction)
template <int K, int NT>
__device__ __forceinline__ bool reduce_partials(double (&v)[K], double *part, unsigned int *counter)
{
	__shared__ double sm[K * NT];
	__shared__ bool last;
	block_sum<K, NT>(v, sm);
	if (threadIdx.x == 0) {
		for (int k = 0; k < K; ++k) part[k * gridDim.x + blockIdx.x] = v[k];
		__threadfence();
		last = (atomicAdd(counter, 1u) == gridDim.x - 1);
	}
	__syncthreads();
	return last;
}

// fixed-order sum of the partials by every thread of the last block
// (thread t adds partials t, t + NT, ...; then block_sum); valid in thread 0
template <int K, int NT>
__device__ __forceinline__ void finish_partials(double (&out)[K], const double *part)
{
	__shared__ double sm[K * NT];
	const int G = gridDim.x;
	for (int k = 0; k < K; ++k) {
		double s = 0.0;
#pragma unroll 8
		for (int b = threadIdx.x; b < G; b += NT) s += __ldcg(part + (long) k * G + b);
		out[k] = s;
	}
	block_sum<K, NT>(out, sm);
}

// one block slot of a row: acc += A_slot * u[col]
template <int B, typename TM, typename TV>
__device__ __forceinline__ void spmv_slot(const SellOp &A, const TM *__restrict__ blk, const TV *__restrict__ u,
                                          long idx, TV (&acc)[B])
{
	int j = __ldg(A.col + idx);
	TV xj[B];
	for (int c = 0; c < B; ++c) xj[c] = u[(long) j * B + c];
	TM a[B * B];
	load_block<B, TM>(blk, A.total, idx, a);
	for (int r = 0; r < B; ++r)
		for (int c = 0; c < B; ++c) acc[r] += (TV) a[r * B + c] * xj[c];
}

// ---------------------------------------------------------------------------
// matvec kernel: w = A u and the partial (w, u).  One warp per 32-row slice,
// one thread per row, kSlicesPerCta slices per CTA; every load instruction
// of a warp reads 32 consecutive slots.  Even and odd slots go to separate
// accumulators (two independent load and FMA streams per thread).  The last
// CTA to finish forms alpha and beta.
// ---------------------------------------------------------------------------
template <int B, typename TM, typename TV>
__global__ void __launch_bounds__(kSpmvBlock) k_cg_spmv(SellOp A, const TM *__restrict__ blk,
                                                        const TV *__restrict__ u, TV *__restrict__ w,
                                                        double *part, CgScal *sc)
{
	if (sc->done) return;
	__shared__ double wsum[kSlicesPerCta];
	__shared__ bool last;
	const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
	const int sl = blockIdx.x * kSlicesPerCta + wp;
	const int nsl = (A.N + 31) >> 5;
	double v = 0.0;
	if (sl < nsl) {
		const int i = sl * 32 + lane;
		const int wdt = __ldg(A.width + sl);
		const long base = __ldg(A.off + sl) + lane;
		TV acc0[B], acc1[B];
		for (int r = 0; r < B; ++r) { acc0[r] = (TV) 0; acc1[r] = (TV) 0; }
		int k = 0;
		for (; k + 2 <= wdt; k += 2) {
			spmv_slot<B, TM, TV>(A, blk, u, base + ((long) k << 5), acc0);
			spmv_slot<B, TM, TV>(A, blk, u, base + ((long) (k + 1) << 5), acc1);
		}
		if (k < wdt) spmv_slot<B, TM, TV>(A, blk, u, base + ((long) k << 5), acc0);
		if (i < A.N)
			for (int r = 0; r < B; ++r) {
				TV o = acc0[r] + acc1[r];
				w[(long) i * B + r] = o;
				v += (double) o * (double) u[(long) i * B + r];
			}
		for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
	}
	if (lane == 0) wsum[wp] = v;
	__syncthreads();
	if (threadIdx.x == 0) {
		double s = wsum[0];
		for (int q = 1; q < kSlicesPerCta; ++q) s += wsum[q];
		part[blockIdx.x] = s;
		__threadfence();
		last = (atomicAdd(&sc->counter, 1u) == gridDim.x - 1);
	}
	__syncthreads();
	if (!last) return;
	double d[1];
	finish_partials<1, kSpmvBlock>(d, part);
	if (threadIdx.x == 0) {
		double delta = d[0], gam = sc->gam, alpha, beta;
		if (sc->first) { beta = 0.0; alpha = gam / delta; }
		else {
			beta = gam / sc->gamPrev;
			alpha = gam / (delta - beta * gam / sc->alpha);
		}
		if (!(alpha > 0.0) || !isfinite(alpha) || !isfinite(beta)) {
			sc->code = isfinite(delta) ? SA_ERR_BREAKDOWN : SA_ERR_NONFINITE;
			sc->done = 1;
		}
		sc->delta = delta; sc->alpha = alpha; sc->beta = beta; sc->first = 0;
		sc->counter = 0;
	}
}

// ---------------------------------------------------------------------------
// vector kernel (grid-stride over entries):
// p = u + beta p; s = w + beta s; x += alpha p; r -= alpha s; u = D^{-1} r
// and the dots (r, u), (r, r)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cg_update_finish(double (&v)[2], double *part, CgScal *sc)
{
	if (!reduce_partials<2, kCgBlock>(v, part, &sc->counter)) return;
	double d[2];
	finish_partials<2, kCgBlock>(d, part);
	if (threadIdx.x == 0) {
		sc->gamPrev = sc->gam;
		sc->gam = d[0];
		sc->rr = d[1];
		sc->iters += 1;
		if (!isfinite(d[0]) || !isfinite(d[1])) { sc->code = SA_ERR_NONFINITE; sc->done = 1; }
		else if (d[1] < sc->tolSqu * sc->bb) { sc->code = SA_OK; sc->done = 1; }
		else if (sc->iters >= sc->itrMax) { sc->code = SA_ERR_NOT_CONVERGED; sc->done = 1; }
		sc->counter = 0;
	}
}

template <typename TV, typename TX>
__global__ void __launch_bounds__(kCgBlock) k_cg_update(long n, TX *__restrict__ x, TV *__restrict__ r,
                                                        TV *__restrict__ u, const TV *__restrict__ w,
                                                        TV *__restrict__ p, TV *__restrict__ s,
                                                        const TV *__restrict__ dinv, double *part, CgScal *sc)
{
	if (sc->done) return;
	const long stride = (long) gridDim.x * blockDim.x;
	double v[2] = {0.0, 0.0};
	const TV al = (TV) sc->alpha, be = (TV) sc->beta;
#pragma unroll 2
	for (long k = blockIdx.x * (long) blockDim.x + threadIdx.x; k < n; k += stride) {
		TV pk = u[k] + be * p[k];
		TV sk = w[k] + be * s[k];
		p[k] = pk; s[k] = sk;
		x[k] = x[k] + (TX) al * (TX) pk;
		TV rk = r[k] - al * sk;
		r[k] = rk;
		TV uk = dinv[k] * rk;
		u[k] = uk;
		v[0] += (double) rk * (double) uk;
		v[1] += (double) rk * (double) rk;
	}
	cg_update_finish(v, part, sc);
}

// the same with the block-Jacobi preconditioner: grid-stride over rows (B entries each), u = Binv r
template <int B, typename TV, typename TX>
__global__ void __launch_bounds__(kCgBlock) k_cg_update_blk(int N, TX *__restrict__ x, TV *__restrict__ r,
                                                            TV *__restrict__ u, const TV *__restrict__ w,
                                                            TV *__restrict__ p, TV *__restrict__ s,
                                                            const TV *__restrict__ binv, double *part, CgScal *sc)
{
	if (sc->done) return;
	const int stride = gridDim.x * blockDim.x;
	double v[2] = {0.0, 0.0};
	const TV al = (TV) sc->alpha, be = (TV) sc->beta;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
		TV rk[B], uk[B];
		for (int c = 0; c < B; ++c) {
			const long k = (long) i * B + c;
			TV pk = u[k] + be * p[k];
			TV sk = w[k] + be * s[k];
			p[k] = pk; s[k] = sk;
			x[k] = x[k] + (TX) al * (TX) pk;
			rk[c] = r[k] - al * sk;
			r[k] = rk[c];
		}
		prec_block_ldg<B, TV>(binv + (long) i * B * B, rk, uk);
		for (int c = 0; c < B; ++c) {
			u[(long) i * B + c] = uk[c];
			v[0] += (double) rk[c] * (double) uk[c];
			v[1] += (double) rk[c] * (double) rk[c];
		}
	}
	cg_update_finish(v, part, sc);
}

// r = b - q, u = D^{-1} r, partials (b, b), (r, r), (r, u)
template <typename TV>
__global__ void __launch_bounds__(kCgBlock) k_cg_init(long n, const double *__restrict__ b, const double *__restrict__ q,
                                                      const TV *__restrict__ dinv, TV *__restrict__ r,
                                                      TV *__restrict__ u, double *part, CgScal *sc)
{
	const long stride = (long) gridDim.x * blockDim.x;
	double v[3] = {0.0, 0.0, 0.0};
	for (long k = blockIdx.x * (long) blockDim.x + threadIdx.x; k < n; k += stride) {
		double rk = b[k] - q[k];
		TV rt = (TV) rk;
		TV uk = dinv[k] * rt;
		r[k] = rt; u[k] = uk;
		v[0] += b[k] * b[k];
		v[1] += rk * rk;
		v[2] += (double) rt * (double) uk;
	}
	if (!reduce_partials<3, kCgBlock>(v, part, &sc->counter)) return;
	double d[3];
	finish_partials<3, kCgBlock>(d, part);
	if (threadIdx.x == 0) {
		if (sc->bb < 0.0) sc->bb = d[0];       // bb < 0: take |b|^2 from this rhs
		sc->rr = d[1]; sc->gam = d[2];
		sc->first = 1; sc->done = 0; sc->code = SA_OK;
		if (!isfinite(d[0]) || !isfinite(d[1])) { sc->code = SA_ERR_NONFINITE; sc->done = 1; }
		else if (sc->bb == 0.0) { sc->zero = 1; sc->done = 1; }
		else if (d[1] < sc->tolSqu * sc->bb) sc->done = 1;
		else if (sc->itrMax <= 0) { sc->code = SA_ERR_NOT_CONVERGED; sc->done = 1; }
		sc->counter = 0;
	}
}

// k_cg_init for the block-Jacobi preconditioner: one row (B entries) per thread, r = b - q, u = Binv r,
// partials (b, b), (r, r), (r, u)
template <int B, typename TV>
__global__ void __launch_bounds__(kCgBlock) k_cg_init_blk(int N, const double *__restrict__ b,
                                                          const double *__restrict__ q,
                                                          const TV *__restrict__ binv, TV *__restrict__ r,
                                                          TV *__restrict__ u, double *part, CgScal *sc)
{
	const int stride = gridDim.x * blockDim.x;
	double v[3] = {0.0, 0.0, 0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
		TV rt[B], ut[B];
		for (int c = 0; c < B; ++c) {
			const long k = (long) i * B + c;
			double rk = b[k] - q[k];
			rt[c] = (TV) rk;
			r[k] = rt[c];
			v[0] += b[k] * b[k];
			v[1] += rk * rk;
		}
		prec_block_ldg<B, TV>(binv + (long) i * B * B, rt, ut);
		for (int c = 0; c < B; ++c) {
			u[(long) i * B + c] = ut[c];
			v[2] += (double) rt[c] * (double) ut[c];
		}
	}
	if (!reduce_partials<3, kCgBlock>(v, part, &sc->counter)) return;
	double d[3];
	finish_partials<3, kCgBlock>(d, part);
	if (threadIdx.x == 0) {
		if (sc->bb < 0.0) sc->bb = d[0];
		sc->rr = d[1]; sc->gam = d[2];
		sc->first = 1; sc->done = 0; sc->code = SA_OK;
		if (!isfinite(d[0]) || !isfinite(d[1])) { sc->code = SA_ERR_NONFINITE; sc->done = 1; }
		else if (sc->bb == 0.0) { sc->zero = 1; sc->done = 1; }
		else if (d[1] < sc->tolSqu * sc->bb) sc->done = 1;
		else if (sc->itrMax <= 0) { sc->code = SA_ERR_NOT_CONVERGED; sc->done = 1; }
		sc->counter = 0;
	}
}

template <typename TX>
__global__ void k_cg_zero(long n, TX *x, const CgScal *sc)
{
	if (!sc->zero) return;
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) x[k] = (TX) 0;
}

template <typename TA, typename TB>
__global__ void k_convert(long n, const TA *a, TB *b)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) b[k] = (TB) a[k];
}

__global__ void k_axpy_f32(long n, double *x, const float *d)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) x[k] += (double) d[k];
}

// q = A x in FP64 (for the initial / true residual)
template <int B>
__global__ void k_spmv64(SellOp A, const double *__restrict__ blk, const double *__restrict__ x,
                         double *__restrict__ q)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= A.N) return;
	double acc[B];
	sell_row<B, double, double>(A, blk, i, x, acc);
	for (int r = 0; r < B; ++r) q[(long) i * B + r] = acc[r];
}

// ---------------------------------------------------------------------------
// Persistent CG: one cooperative launch runs the whole solve.  Each thread
// owns one row (3 entries for the velocity, 1 for reaction-diffusion) and
// keeps x, r, u, p, s and D^{-1} of that row in registers; only u goes
// through global memory, because the matvec gathers the neighbours' u.
// One CTA per SM (up to kPersistMaxWarps warps: one 32-row slice per row
// warp plus one reducer warp that does the grid-wide work, see below).
// Per iteration two grid-wide reductions (delta = (w, u); gamma = (r, u)
// and (r, r)) double as the grid barriers that order the u reads and
// writes: every CTA publishes its partial sums, counts itself in, waits for
// the count of the whole grid and then adds all partials exactly in 128-bit
// fixed point (sa_fixsum.cuh: order-independent, rounded once), so every CTA
// forms the same alpha, beta and stopping decision.
// Waits are bounded: a CTA that waits longer than kBarWaitNs (or sees
// another CTA give up) stops with SA_ERR_TIMEOUT.
// ---------------------------------------------------------------------------
constexpr int kPersistMaxWarps = 20;                       // CTA size limit (96 registers per thread)

// Chronopoulos-Gear step lengths from delta = (w, u) (thread 0 of each CTA; the same in every CTA)
__device__ __forceinline__ void cg_step_lengths(double delta, double gam, double gamPrev, double alphaPrev,
                                                bool first, double *out)
{
	double alpha, beta;
	if (first) { beta = 0.0; alpha = gam / delta; }
	else {
		beta = gam / gamPrev;
		alpha = gam / (delta - beta * gam / alphaPrev);
	}
	out[0] = alpha;
	out[1] = beta;
}

// the (at most 3-term) dot product of one row, in the vector type
template <int B, typename TV>
__device__ __forceinline__ TV row_dot(const TV (&a)[B], const TV (&b)[B])
{
	TV s = a[0] * b[0];
	for (int c = 1; c < B; ++c) s += a[c] * b[c];
	return s;
}

// a row's contribution to a dot product: FP64 operands fold each product into the FP64 sum; FP32
// operands form the row's (at most 3-term) FP32 sum first and add it to the FP64 sum once
template <int B, typename TV>
__device__ __forceinline__ void dot_row(double &acc, const TV (&a)[B], const TV (&b)[B])
{
	if (sizeof(TV) == sizeof(double)) {
		for (int c = 0; c < B; ++c) acc += (double) a[c] * (double) b[c];
	} else {
		TV s = a[0] * b[0];
		for (int c = 1; c < B; ++c) s += a[c] * b[c];
		acc += (double) s;
	}
}

template <int B, typename TM, typename TV>
__device__ __forceinline__ void spmv_slot_cg(const SellOp &A, const TM *__restrict__ blk, const TV *u, long idx,
                                             TV (&acc)[B])
{
	int j = __ldg(A.col + idx);
	TV xj[B];
	for (int c = 0; c < B; ++c) xj[c] = __ldcg(u + (long) j * B + c);   // written during the launch
	TM a[B * B];
	load_block<B, TM>(blk, A.total, idx, a);
	for (int r = 0; r < B; ++r)
		for (int c = 0; c < B; ++c) acc[r] += (TV) a[r * B + c] * xj[c];
}

// One reducer warp per CTA (the last warp, no rows) takes the grid-wide parts of the iteration off the
// rows' critical path: while the row warps run the matvec it adds up the (r, u), (r, r) partials of the
// previous update and forms beta and the constant part of alpha; while they update p and s it publishes
// the CTA's (w, u), waits for the grid and forms alpha.  The row warps wait only for the barrier that makes
// u complete (before the matvec) and for alpha (before x, r, u).  The convergence test of an update runs
// after the next matvec (that matvec is discarded), so iterates and iteration counts are those of the
// plain Chronopoulos-Gear loop.

// Stride of the persistent CG's gather copy of u: 3-component node blocks padded to 4, so a gathered node
// is one 16-byte load (FP32) or two (FP64) instead of three scalar loads, each of which is its own L2
// request for a random node; 2-component blocks load as one vector.
template <int B> constexpr int gather_stride() { return B == 3 ? 4 : B; }

// node j of u (stride S; read through L2: written during the launch)
template <int B, int S, typename TV>
__device__ __forceinline__ void load_node_u(const TV *u, int j, TV (&x)[B])
{
	if constexpr (B == 3 && S == 4 && sizeof(TV) == 4) {
		const float4 v = __ldcg(reinterpret_cast<const float4 *>(u) + j);
		x[0] = v.x; x[1] = v.y; x[2] = v.z;
	} else if constexpr (B == 3 && S == 4 && sizeof(TV) == 8) {
		const double2 a = __ldcg(reinterpret_cast<const double2 *>(u) + 2 * (long) j);
		const double2 b = __ldcg(reinterpret_cast<const double2 *>(u) + 2 * (long) j + 1);
		x[0] = a.x; x[1] = a.y; x[2] = b.x;
	} else if constexpr (B == 2 && S == 2 && sizeof(TV) == 4) {
		const float2 v = __ldcg(reinterpret_cast<const float2 *>(u) + j);
		x[0] = v.x; x[1] = v.y;
	} else if constexpr (B == 2 && S == 2 && sizeof(TV) == 8) {
		const double2 v = __ldcg(reinterpret_cast<const double2 *>(u) + j);
		x[0] = v.x; x[1] = v.y;
	} else {
		for (int c = 0; c < B; ++c) x[c] = __ldcg(u + (long) j * S + c);
	}
}

template <int B, int S, typename TV>
__device__ __forceinline__ void store_node_u(TV *u, int i, const TV (&x)[B])
{
	if constexpr (B == 3 && S == 4 && sizeof(TV) == 4) {
		reinterpret_cast<float4 *>(u)[i] = make_float4(x[0], x[1], x[2], 0.f);
	} else if constexpr (B == 3 && S == 4 && sizeof(TV) == 8) {
		reinterpret_cast<double2 *>(u)[2 * (long) i] = make_double2(x[0], x[1]);
		reinterpret_cast<double2 *>(u)[2 * (long) i + 1] = make_double2(x[2], 0.0);
	} else {
		for (int c = 0; c < B; ++c) u[(long) i * S + c] = x[c];
	}
}

// u (stride B) -> its gather copy (stride gather_stride<B>())
template <int B, typename TV>
__global__ void k_pad_u(int N, const TV *__restrict__ u, TV *__restrict__ ug)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	TV x[B];
	for (int c = 0; c < B; ++c) x[c] = u[(long) i * B + c];
	store_node_u<B, gather_stride<B>(), TV>(ug, i, x);
}

// a slot whose column is already known (the persistent CG keeps its CTA's columns in shared memory); u has
// stride S
template <int B, typename TM, typename TV, int S = B>
__device__ __forceinline__ void spmv_slot_col(const SellOp &A, const TM *__restrict__ blk, const TV *u, long idx, int j,
                                              TV (&acc)[B])
{
	TV xj[B];
	load_node_u<B, S, TV>(u, j, xj);
	TM a[B * B];
	load_block<B, TM>(blk, A.total, idx, a);
	for (int r = 0; r < B; ++r)
		for (int c = 0; c < B; ++c) acc[r] += (TV) a[r * B + c] * xj[c];
}

// a slot whose operator block sits in shared memory ([entry][lane] with stride 32; cs points at lane's entry 0)
template <int B, typename TM, typename TV, int S>
__device__ __forceinline__ void spmv_slot_smem(const TM *cs, const TV *u, int j, TV (&acc)[B])
{
	TV xj[B];
	load_node_u<B, S, TV>(u, j, xj);
	for (int r = 0; r < B; ++r)
		for (int c = 0; c < B; ++c) acc[r] += (TV) cs[32 * (r * B + c)] * xj[c];
}

constexpr int kColSmemMax = 160 * 1024;    // shared memory for a CTA's column indices (else two-kernel CG)

template <int B, typename TM, typename TV, typename TX>
__global__ void __launch_bounds__(32 * kPersistMaxWarps, 1)
k_cg_persist(SellOp A, const TM *__restrict__ blk, const TV *__restrict__ dinv, const TV *__restrict__ binv, TX *x,
             const TV *r0, const TV *u, TV *ug, double *part, CgScal *sc, GridBar *bar, const int *__restrict__ ctaTab,
             int colInts, int kc)
{
	__shared__ FxScratch fs;                     // block sums; fs.tot = gamma, rr of the last update
	__shared__ double nx[4];                     // next gamma, rr, beta, beta * gamma / alphaPrev
	__shared__ double al[2];                     // alpha, delta of the iteration
	__shared__ int gaveUp;
	extern __shared__ __align__(16) int scol[];  // the column of every slot of the CTA's slices
	if (sc->done) return;                        // set by k_cg_init: the same for every CTA
	const int nctas = gridDim.x, lc = blockIdx.x;
	const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
	const int H = (blockDim.x >> 5) - 1;         // the reducer warp; warps 0 .. H-1 own one slice each
	const bool reducer = wp == H;
	// the slice of each row warp (-1: none) and its place in the CTA's column cache: slices are dealt to
	// CTAs by slot count, so every CTA's matvec takes about as long (ctaTab, built on the host)
	const int sl = reducer ? -1 : __ldg(ctaTab + lc * H + wp);
	const int i = sl * 32 + lane;
	const bool rowWarp = sl >= 0;
	const bool own = rowWarp && i < A.N;
	const int wdt = rowWarp ? __ldg(A.width + sl) : 0;
	const long base = rowWarp ? __ldg(A.off + sl) + lane : 0;
	// the columns do not change during the solve: each row warp copies its slice's into the CTA's cache
	// once, then no slot waits for a column load
	const int coff = rowWarp ? __ldg(ctaTab + (long) gridDim.x * H + lc * H + wp) : 0;
	if (rowWarp)
		for (int t = lane; t < 32 * wdt; t += 32) scol[coff + t] = __ldg(A.col + (base - lane) + t);
	const int lbase = coff + lane;               // local slot of lane's slot 0 (row warps)
	// FP32 operators (mixed precision): the first kc slots of each row warp's slice also stay in shared
	// memory, [warp][slot][entry][lane], so the matvec reads only the rest of the operator from L2
	constexpr int BB = B * B;
	constexpr int S = gather_stride<B>();                   // ug: u in the gather layout (the matvec's reads)
	constexpr bool kCache = sizeof(TM) == sizeof(float);    // FP64 operators never use it (kc = 0)
	TM *scache = reinterpret_cast<TM *>(scol + colInts);
	if (kCache && kc > 0 && rowWarp)
		for (int k = 0; k < min(kc, wdt); ++k)
			for (int e = 0; e < BB; ++e)
				scache[((wp * kc + k) * BB + e) * 32 + lane] = __ldg(blk + (base - lane + ((long) k << 5)) * BB + 32 * e + lane);
	__syncthreads();                             // scol, the block cache and gaveUp before their first use
	const double bb = sc->bb, tolSqu = sc->tolSqu;
	const int itrMax = sc->itrMax;
	double gam = sc->gam, rr = sc->rr, alpha = 1.0, beta = 0.0;
	double *partD = part, *partG = part + nctas;  // (w, u) partials; (r, u) then (r, r) partials
	unsigned int target = 0;                     // bar->count is zeroed before the launch
	if (threadIdx.x == 0) gaveUp = 0;
	TX xv[B];
	// block-Jacobi (binv): FP32 inverses stay in registers, FP64 ones (twice the registers: they would
	// spill) in shared memory; FP64 B = 1 solves: point Jacobi, the inverse diagonal in registers
	constexpr bool kBlk = block_prec<B, TV>();
	constexpr bool kBlkReg = kBlk && sizeof(TV) == sizeof(float);
	constexpr int kBV = kBlkReg ? B * B : 1;
	TV rv[B], uv[B], pv[B], sv[B], dv[B], bv[kBV];
	for (int c = 0; c < B; ++c) {
		xv[c] = (TX) 0; rv[c] = uv[c] = pv[c] = sv[c] = dv[c] = (TV) 0;
		if (own) {
			long k = (long) i * B + c;
			xv[c] = x[k]; rv[c] = r0[k]; uv[c] = u[k];
			if constexpr (!kBlk) dv[c] = dinv[k];
		}
	}
	if constexpr (kBlkReg)
		for (int t = 0; t < kBV; ++t) bv[t] = own ? binv[(long) i * B * B + t] : (TV) 0;
	// FP64 block inverses: in shared memory after the column cache (8-byte aligned), [warp][entry][lane],
	// copied once per solve like the columns; sbinv points at this thread's entry 0
	TV *sbinv = reinterpret_cast<TV *>(scol + ((colInts + 1) & ~1)) + wp * B * B * 32 + lane;
	if constexpr (kBlk && !kBlkReg)
		if (rowWarp)
			for (int t = 0; t < B * B; ++t) sbinv[t * 32] = own ? __ldg(binv + (long) i * B * B + t) : (TV) 0;
	int it = 0, code = SA_OK;
	bool first = true, pending = false;
	for (;;) {
		// (1) rows: w = A u and (w, u).  Reducer: the sums of the last update, beta, beta * gamma / alpha
		TV wv[B];
		TV d1[1] = {(TV) 0};
		for (int c = 0; c < B; ++c) wv[c] = (TV) 0;
		if (rowWarp) {
			TV acc0[B], acc1[B];
			for (int c = 0; c < B; ++c) { acc0[c] = (TV) 0; acc1[c] = (TV) 0; }
			int k = 0;
			// cached slots first, in pairs (kc is even), then the rest: slot k always goes to acc[k & 1]
			const int kcw = kCache ? min(kc, wdt) & ~1 : 0;
			const TM *cs = scache + (wp * kc * BB) * 32 + lane;
			for (; kCache && k + 2 <= kcw; k += 2) {
				const int j0 = scol[lbase + (k << 5)], j1 = scol[lbase + ((k + 1) << 5)];
				spmv_slot_smem<B, TM, TV, S>(cs + k * BB * 32, ug, j0, acc0);
				spmv_slot_smem<B, TM, TV, S>(cs + (k + 1) * BB * 32, ug, j1, acc1);
			}
			for (; k + 2 <= wdt; k += 2) {
				const int j0 = scol[lbase + (k << 5)], j1 = scol[lbase + ((k + 1) << 5)];
				spmv_slot_col<B, TM, TV, S>(A, blk, ug, base + ((long) k << 5), j0, acc0);
				spmv_slot_col<B, TM, TV, S>(A, blk, ug, base + ((long) (k + 1) << 5), j1, acc1);
			}
			if (k < wdt)
				spmv_slot_col<B, TM, TV, S>(A, blk, ug, base + ((long) k << 5), scol[lbase + (k << 5)], acc0);
			for (int c = 0; c < B; ++c) wv[c] = acc0[c] + acc1[c];
			if (own) d1[0] = row_dot<B, TV>(wv, uv);
		} else if (pending) {
			// one set after the other: the loads are hidden behind the rows' matvec, registers are not spare
			const double g = warp_fx_partials(partG, nctas);
			const double q = warp_fx_partials(partG + nctas, nctas);
			if (lane == 0) {
				nx[0] = g;
				nx[1] = q;
				nx[2] = g / gam;                     // beta
				nx[3] = nx[2] * g / alpha;           // the part of alpha's denominator known before delta
			}
		}
		double cta1[1];
		block_fx_sum<1, TV>(d1, fs, cta1, H);     // its barriers also publish nx
		if (pending) {
			gam = nx[0];
			rr = nx[1];
			first = false;
			++it;
			if (!isfinite(gam) || !isfinite(rr)) { code = SA_ERR_NONFINITE; break; }
			if (rr < tolSqu * bb) { code = SA_OK; break; }
			if (it >= itrMax) { code = SA_ERR_NOT_CONVERGED; break; }
		}
		beta = first ? 0.0 : nx[2];
		// (2) reducer: publish (w, u), wait for the grid, alpha.  Rows meanwhile: p and s
		target += (unsigned int) nctas;
		if (reducer) {
			int ok = 1;
			if (lane == 0) {
				partD[lc] = cta1[0];
				__threadfence();
				atomicAdd(&bar->count, 1u);
				ok = wait_grid(bar, target) ? 1 : 0;      // its acquire load orders the reads below
			}
			ok = __shfl_sync(0xffffffffu, ok, 0);
			__syncwarp();                        // orders lane 0's acquire before the other lanes' loads
			if (ok) {
				const double delta = warp_fx_partials(partD, nctas);
				if (lane == 0) {
					al[0] = first ? gam / delta : gam / (delta - nx[3]);
					al[1] = delta;
				}
			} else if (lane == 0) {
				gaveUp = 1;
			}
		} else if (own) {
			const TV be = (TV) beta;
			for (int c = 0; c < B; ++c) {
				pv[c] = uv[c] + be * pv[c];
				sv[c] = wv[c] + be * sv[c];
			}
		}
		__syncthreads();
		if (gaveUp) { code = SA_ERR_TIMEOUT; break; }
		alpha = al[0];
		if (!(alpha > 0.0) || !isfinite(alpha) || !isfinite(beta)) {
			code = isfinite(al[1]) ? SA_ERR_BREAKDOWN : SA_ERR_NONFINITE;
			break;
		}
		// (3) rows: x, r, u and (r, u), (r, r); the reducer publishes them and waits for the grid (u complete)
		TV d2[2] = {(TV) 0, (TV) 0};
		const TV al_ = (TV) alpha;
		if (own) {
			for (int c = 0; c < B; ++c) rv[c] = rv[c] - al_ * sv[c];
			if constexpr (kBlkReg) prec_block<B, TV>(bv, rv, uv);
			else if constexpr (kBlk) {
				TV m[B * B];
				for (int t = 0; t < B * B; ++t) m[t] = sbinv[t * 32];
				prec_block<B, TV>(m, rv, uv);
			}
			else for (int c = 0; c < B; ++c) uv[c] = dv[c] * rv[c];
			store_node_u<B, S, TV>(ug, i, uv);
			d2[0] = row_dot<B, TV>(rv, uv);
			d2[1] = row_dot<B, TV>(rv, rv);
		}
		double cta2[2];
		block_fx_sum<2, TV>(d2, fs, cta2, H);
		target += (unsigned int) nctas;
		if (reducer && lane == 0) {
			partG[lc] = cta2[0];
			partG[nctas + lc] = cta2[1];
			__threadfence();
			atomicAdd(&bar->count, 1u);
			if (!wait_grid(bar, target)) gaveUp = 1;   // its acquire load orders the reads below
		} else if (own) {
			for (int c = 0; c < B; ++c) xv[c] = xv[c] + (TX) al_ * (TX) pv[c];   // while the reducer waits
		}
		__syncthreads();
		if (gaveUp) { code = SA_ERR_TIMEOUT; break; }
		pending = true;
	}
	if (own)
		for (int c = 0; c < B; ++c) x[(long) i * B + c] = xv[c];
	if (lc == 0 && threadIdx.x == 0) {
		sc->iters = it; sc->code = code; sc->rr = rr; sc->gam = gam; sc->done = 1;
	}
}

// ---------------------------------------------------------------------------
// Persistent CG for operators too large for row state in registers (more than
// one slice per row warp at one CTA per SM): the same iteration, reducer warp
// and fixed-point grid sums as k_cg_persist, but x, r, u, w, p, s live in
// global memory (mostly L2) and CTA c owns the contiguous slices
// [c nsl / nctas, (c + 1) nsl / nctas), which its row warps stride over.  The
// CTA's column indices are cached in shared memory when they fit.
// ---------------------------------------------------------------------------
template <int B, typename TM, typename TV, typename TX>
__global__ void __launch_bounds__(32 * kPersistMaxWarps, 1)
k_cg_persist_g(SellOp A, const TM *__restrict__ blk, const TV *__restrict__ dinv, const TV *__restrict__ binv, TX *x,
               TV *r, TV *u, TV *w, TV *p, TV *sv, int colsCached, double *part, CgScal *sc, GridBar *bar)
{
	__shared__ FxScratch fs;
	__shared__ double nx[4];                     // next gamma, rr, beta, beta * gamma / alphaPrev
	__shared__ double al[2];                     // alpha, delta of the iteration
	__shared__ int gaveUp;
	extern __shared__ int scol[];
	if (sc->done) return;
	const int nctas = gridDim.x, lc = blockIdx.x;
	const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
	const int H = (blockDim.x >> 5) - 1;         // reducer warp; row warps 0 .. H-1
	const bool reducer = wp == H;
	const int nsl = (A.N + 31) >> 5;
	const int s0 = (int) ((long) lc * nsl / nctas), s1 = (int) ((long) (lc + 1) * nsl / nctas);
	const long c0 = s0 < nsl ? (long) __ldg(A.off + s0) : A.total;
	const long c1 = s1 < nsl ? (long) __ldg(A.off + s1) : A.total;
	if (colsCached)
		for (long t = threadIdx.x; t < c1 - c0; t += blockDim.x) scol[t] = __ldg(A.col + c0 + t);
	if (threadIdx.x == 0) gaveUp = 0;
	__syncthreads();
	const double bb = sc->bb, tolSqu = sc->tolSqu;
	const int itrMax = sc->itrMax;
	double gam = sc->gam, rr = sc->rr, alpha = 1.0, beta = 0.0;
	double *partD = part, *partG = part + nctas;
	unsigned int target = 0;
	constexpr bool kBlk = block_prec<B, TV>();
	int it = 0, code = SA_OK;
	bool first = true, pending = false;
	for (;;) {
		// (1) rows: w = A u and (w, u) over the warp's slices.  Reducer: sums of the last update
		double d1[1] = {0.0};
		if (!reducer) {
			for (int sl = s0 + wp; sl < s1; sl += H) {
				const int i = sl * 32 + lane, wdt = __ldg(A.width + sl);
				const long base = __ldg(A.off + sl) + lane;
				TV acc0[B], acc1[B];
				for (int c = 0; c < B; ++c) { acc0[c] = (TV) 0; acc1[c] = (TV) 0; }
				int k = 0;
				for (; k + 2 <= wdt; k += 2) {
					const long i0 = base + ((long) k << 5), i1 = i0 + 32;
					const int j0 = colsCached ? scol[i0 - c0] : __ldg(A.col + i0);
					const int j1 = colsCached ? scol[i1 - c0] : __ldg(A.col + i1);
					spmv_slot_col<B, TM, TV>(A, blk, u, i0, j0, acc0);
					spmv_slot_col<B, TM, TV>(A, blk, u, i1, j1, acc1);
				}
				if (k < wdt) {
					const long i0 = base + ((long) k << 5);
					spmv_slot_col<B, TM, TV>(A, blk, u, i0, colsCached ? scol[i0 - c0] : __ldg(A.col + i0), acc0);
				}
				if (i < A.N) {
					TV wv[B], uv[B];
					for (int c = 0; c < B; ++c) {
						wv[c] = acc0[c] + acc1[c];
						w[(long) i * B + c] = wv[c];
						uv[c] = __ldcg(u + (long) i * B + c);
					}
					d1[0] += (double) row_dot<B, TV>(wv, uv);
				}
			}
		} else if (pending) {
			const double g = warp_fx_partials(partG, nctas);
			const double q = warp_fx_partials(partG + nctas, nctas);
			if (lane == 0) {
				nx[0] = g;
				nx[1] = q;
				nx[2] = g / gam;
				nx[3] = nx[2] * g / alpha;
			}
		}
		double cta1[1];
		block_fx_sum<1, double>(d1, fs, cta1, H);
		if (pending) {
			gam = nx[0];
			rr = nx[1];
			first = false;
			++it;
			if (!isfinite(gam) || !isfinite(rr)) { code = SA_ERR_NONFINITE; break; }
			if (rr < tolSqu * bb) { code = SA_OK; break; }
			if (it >= itrMax) { code = SA_ERR_NOT_CONVERGED; break; }
		}
		beta = first ? 0.0 : nx[2];
		// (2) reducer: publish (w, u), wait, alpha.  Rows: p and s
		target += (unsigned int) nctas;
		if (reducer) {
			int ok = 1;
			if (lane == 0) {
				partD[lc] = cta1[0];
				__threadfence();
				atomicAdd(&bar->count, 1u);
				ok = wait_grid(bar, target) ? 1 : 0;      // its acquire load orders the reads below
			}
			ok = __shfl_sync(0xffffffffu, ok, 0);
			__syncwarp();
			if (ok) {
				const double delta = warp_fx_partials(partD, nctas);
				if (lane == 0) {
					al[0] = first ? gam / delta : gam / (delta - nx[3]);
					al[1] = delta;
				}
			} else if (lane == 0) {
				gaveUp = 1;
			}
		} else {
			const TV be = (TV) beta;
			for (int sl = s0 + wp; sl < s1; sl += H) {
				const int i = sl * 32 + lane;
				if (i >= A.N) continue;
				for (int c = 0; c < B; ++c) {
					const long k = (long) i * B + c;
					p[k] = __ldcg(u + k) + be * p[k];
					sv[k] = w[k] + be * sv[k];
				}
			}
		}
		__syncthreads();
		if (gaveUp) { code = SA_ERR_TIMEOUT; break; }
		alpha = al[0];
		if (!(alpha > 0.0) || !isfinite(alpha) || !isfinite(beta)) {
			code = isfinite(al[1]) ? SA_ERR_BREAKDOWN : SA_ERR_NONFINITE;
			break;
		}
		// (3) rows: r, u and (r, u), (r, r); x while the reducer waits for the grid (u complete)
		double d2[2] = {0.0, 0.0};
		const TV al_ = (TV) alpha;
		if (!reducer) {
			for (int sl = s0 + wp; sl < s1; sl += H) {
				const int i = sl * 32 + lane;
				if (i >= A.N) continue;
				TV rk[B], uk[B];
				for (int c = 0; c < B; ++c) {
					const long k = (long) i * B + c;
					rk[c] = r[k] - al_ * sv[k];
					r[k] = rk[c];
				}
				if constexpr (kBlk) prec_block<B, TV>(binv + (long) i * B * B, rk, uk);
				else for (int c = 0; c < B; ++c) uk[c] = dinv[(long) i * B + c] * rk[c];
				for (int c = 0; c < B; ++c) u[(long) i * B + c] = uk[c];
				d2[0] += (double) row_dot<B, TV>(rk, uk);
				d2[1] += (double) row_dot<B, TV>(rk, rk);
			}
		}
		double cta2[2];
		block_fx_sum<2, double>(d2, fs, cta2, H);
		target += (unsigned int) nctas;
		if (reducer) {
			if (lane == 0) {
				partG[lc] = cta2[0];
				partG[nctas + lc] = cta2[1];
				__threadfence();
				atomicAdd(&bar->count, 1u);
				if (!wait_grid(bar, target)) gaveUp = 1;   // its acquire load orders the reads below
			}
		} else {
			for (int sl = s0 + wp; sl < s1; sl += H) {
				const int i = sl * 32 + lane;
				if (i >= A.N) continue;
				for (int c = 0; c < B; ++c) {
					const long k = (long) i * B + c;
					x[k] = x[k] + (TX) al_ * (TX) p[k];
				}
			}
		}
		__syncthreads();
		if (gaveUp) { code = SA_ERR_TIMEOUT; break; }
		pending = true;
	}
	if (lc == 0 && threadIdx.x == 0) {
		sc->iters = it; sc->code = code; sc->rr = rr; sc->gam = gam; sc->done = 1;
	}
}

// ---------------------------------------------------------------------------
// Batched persistent CG: one cooperative launch advances many independent
// solves (the instances of a serving batch).  Job j owns the CTAs
// [cta0, cta0 + nctas) of the launch; its warps stride over its slices, its
// CTAs reduce and synchronise only among themselves (own partials, own
// barrier, own scalars), and they stop when their solve stops.  Vectors live
// in global memory (a job may have more slices than warps); each row is
// updated by the thread that computed its matvec entry, so only u is read
// across threads.
// ---------------------------------------------------------------------------
constexpr int kBatchBlock = 256;           // largest CTA of the batched CG (the tuned size is at most this)
constexpr int kBatchMinCtas = 4;

template <int B, typename TM, typename TV, typename TX>
__global__ void __launch_bounds__(kBatchBlock, kBatchMinCtas) k_cg_batch(const CgJob *__restrict__ jobs, int njobs)
{
	__shared__ FxScratch fs;                      // grid-reduction scratch
	__shared__ double ab[2];                      // alpha, beta of the iteration
	__shared__ int jS;
	if (threadIdx.x == 0) {                      // last job with cta0 <= blockIdx.x
		int lo = 0, hi = njobs - 1;
		while (lo < hi) {
			int mid = (lo + hi + 1) >> 1;
			if (jobs[mid].cta0 <= (int) blockIdx.x) lo = mid;
			else hi = mid - 1;
		}
		jS = lo;
	}
	__syncthreads();
	const CgJob &J = jobs[jS];
	const int lc = (int) blockIdx.x - J.cta0, nctas = J.nctas;
	if (lc < 0 || lc >= nctas) return;           // no job owns this CTA (launch padding)
	CgScal *sc = (CgScal *) J.sc;
	if (sc->done) return;
	const SellOp A = J.A;
	const TM *blk = (const TM *) J.blk;
	const TV *dinv = (const TV *) J.dinv;
	const TV *binv = (const TV *) J.binv;          // block-Jacobi inverses (read only when block_prec)
	TX *x = (TX *) J.x;
	TV *r = (TV *) J.r, *u = (TV *) J.u, *w = (TV *) J.w, *p = (TV *) J.p, *sv = (TV *) J.s;
	GridBar *bar = (GridBar *) J.bar;
	double *part = J.part;
	const int lane = threadIdx.x & 31, W = blockDim.x >> 5;
	const int wj = lc * W + (threadIdx.x >> 5), WJ = nctas * W;
	const int nsl = (A.N + 31) >> 5;
	const double bb = sc->bb, tolSqu = sc->tolSqu;
	const int itrMax = sc->itrMax;
	double gam = sc->gam, rr = sc->rr, gamPrev = 0.0, alphaPrev = 1.0;
	unsigned int target = 0;
	int it = 0, code = SA_OK;
	bool first = true;
	for (;;) {
		double d1[1] = {0.0};
		for (int sl = wj; sl < nsl; sl += WJ) {
			const int i = sl * 32 + lane;
			const int wdt = __ldg(A.width + sl);
			const long base = __ldg(A.off + sl) + lane;
			TV acc0[B], acc1[B];
			for (int c = 0; c < B; ++c) { acc0[c] = (TV) 0; acc1[c] = (TV) 0; }
			int k = 0;
			for (; k + 2 <= wdt; k += 2) {
				spmv_slot_cg<B, TM, TV>(A, blk, u, base + ((long) k << 5), acc0);
				spmv_slot_cg<B, TM, TV>(A, blk, u, base + ((long) (k + 1) << 5), acc1);
			}
			if (k < wdt) spmv_slot_cg<B, TM, TV>(A, blk, u, base + ((long) k << 5), acc0);
			if (i < A.N) {
				TV o[B], ui[B];
				for (int c = 0; c < B; ++c) {
					o[c] = acc0[c] + acc1[c];
					w[(long) i * B + c] = o[c];
					ui[c] = __ldcg(u + (long) i * B + c);
				}
				dot_row<B, TV>(d1[0], o, ui);
			}
		}
		double g1[1];
		if (!grid_reduce<1, double>(d1, g1, part, lc, nctas, bar, target, fs, [&](const double *t) {
			    cg_step_lengths(t[0], gam, gamPrev, alphaPrev, first, ab);
		    })) {
			code = SA_ERR_TIMEOUT;
			break;
		}
		const double delta = g1[0], alpha = ab[0], beta = ab[1];
		if (!(alpha > 0.0) || !isfinite(alpha) || !isfinite(beta)) {
			code = isfinite(delta) ? SA_ERR_BREAKDOWN : SA_ERR_NONFINITE;
			break;
		}
		double d2[2] = {0.0, 0.0};
		const TV al = (TV) alpha, be = (TV) beta;
		for (int sl = wj; sl < nsl; sl += WJ) {
			const int i = sl * 32 + lane;
			if (i >= A.N) continue;
			TV rk[B], uk[B];
			for (int c = 0; c < B; ++c) {
				const long k = (long) i * B + c;
				TV pk = __ldcg(u + k) + be * p[k];
				TV sk = w[k] + be * sv[k];
				p[k] = pk; sv[k] = sk;
				x[k] = x[k] + (TX) al * (TX) pk;
				rk[c] = r[k] - al * sk;
				r[k] = rk[c];
			}
			if constexpr (block_prec<B, TV>()) prec_block_ldg<B, TV>(binv + (long) i * B * B, rk, uk);
			else for (int c = 0; c < B; ++c) uk[c] = dinv[(long) i * B + c] * rk[c];
			for (int c = 0; c < B; ++c) u[(long) i * B + c] = uk[c];
			dot_row<B, TV>(d2[0], rk, uk);
			dot_row<B, TV>(d2[1], rk, rk);
		}
		double g2[2];
		if (!grid_reduce<2, double>(d2, g2, part + nctas, lc, nctas, bar, target, fs)) { code = SA_ERR_TIMEOUT; break; }
		gamPrev = gam;
		gam = g2[0];
		rr = g2[1];
		alphaPrev = alpha;
		first = false;
		++it;
		if (!isfinite(gam) || !isfinite(rr)) { code = SA_ERR_NONFINITE; break; }
		if (rr < tolSqu * bb) { code = SA_OK; break; }
		if (it >= itrMax) { code = SA_ERR_NOT_CONVERGED; break; }
	}
	if (lc == 0 && threadIdx.x == 0) {
		sc->iters = it; sc->code = code; sc->rr = rr; sc->gam = gam; sc->done = 1;
	}
}

// ---------------------------------------------------------------------------
// Self-test of the bounded grid wait: a cooperative launch whose barrier
// count starts 2^31 away from its target, so the arrivals never reach it (a
// flag that nothing sets).  Every CTA must give up after kBarWaitNs and report it;
// no fault, no hang, the context stays usable.
// ---------------------------------------------------------------------------
__global__ void k_barrier_probe(double *part, GridBar *bar, int *gaveUp)
{
	__shared__ FxScratch fs;
	unsigned int target = 0;
	double v[1] = {1.0}, t[1];
	bool ok = grid_reduce<1, double>(v, t, part, blockIdx.x, gridDim.x, bar, target, fs);
	if (threadIdx.x == 0 && !ok) atomicAdd(gaveUp, 1);
}

int barrier_selftest(cudaStream_t s, int *ctasGaveUp, int *abortFlag)
{
	const int nctas = 2, nt = 64;
	int per = 0;
	SA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_barrier_probe, nt, 0));
	if (per < 1) return SA_ERR_UNSUPPORTED;
	char *mem = nullptr;
	SA_CHECK(cudaMalloc(&mem, kGridBarBytes + 256));
	GridBar *bar = (GridBar *) mem;
	double *part = (double *) (mem + kGridBarBytes);
	int *gave = (int *) (mem + kGridBarBytes + 128);
	GridBar h{};
	// count - target stays in [2^31, 2^32) for every number of arrivals, i.e. "not yet" as a signed
	// difference: the wait can only end by its time limit
	h.count = 0x80000000u + (unsigned int) nctas;
	SA_CHECK(cudaMemcpyAsync(bar, &h, sizeof(GridBar), cudaMemcpyHostToDevice, s));
	SA_CHECK(cudaMemsetAsync(gave, 0, sizeof(int), s));
	void *args[] = {(void *) &part, (void *) &bar, (void *) &gave};
	cudaError_t e = cudaLaunchCooperativeKernel((const void *) k_barrier_probe, dim3(nctas), dim3(nt), args, 0, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	GridBar out{};
	int g = 0;
	if (e == cudaSuccess) e = cudaMemcpy(&out, bar, sizeof(GridBar), cudaMemcpyDeviceToHost);
	if (e == cudaSuccess) e = cudaMemcpy(&g, gave, sizeof(int), cudaMemcpyDeviceToHost);
	cudaFree(mem);
	SA_CHECK(e);
	*ctasGaveUp = g;
	*abortFlag = (int) out.abort;
	return SA_OK;
}

// ---------------------------------------------------------------------------
// FMA throughput of the FP64 or FP32 pipe: CH independent FMA chains per
// thread, 256-thread CTAs, a few chain counts and CTAs per SM (the best is
// kept).  The denominators of the pipe fractions the benchmark reports
// (measured on the same GPU in the same run).  Each CTA also records its SM
// clock cycles and nanoseconds, which give the SM clock of the launch; the
// rate per SM clock is the event-timed rate over SMs x that clock.
// ---------------------------------------------------------------------------
template <typename T, int CH>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T a, T b, long long *stamps)
{
	const long long c0 = clock64();
	const unsigned long long t0 = global_ns();
	T x[CH];
	for (int k = 0; k < CH; ++k) x[k] = (T) (threadIdx.x + k) * (T) 1e-3;
	for (int i = 0; i < iters; ++i) {
#pragma unroll
		for (int k = 0; k < CH; ++k) x[k] = fma(x[k], a, b);
	}
	T t = x[0];
	for (int k = 1; k < CH; ++k) t += x[k];
	if (threadIdx.x == 0) {
		stamps[2 * blockIdx.x] = clock64() - c0;
		stamps[2 * blockIdx.x + 1] = (long long) (global_ns() - t0);
	}
	if (t == (T) -1) stamps[0] = 0;              // never true (x stays in (0, 1]); keeps the chains live
}

template <typename T, int CH>
static void fma_peak_variant(cudaStream_t s, int sms, int ctasPerSm, long long *stamps, cudaEvent_t e0,
                             cudaEvent_t e1, double &best, double &bestMhz)
{
	const int nt = 256, nb = ctasPerSm * sms;
	// ~50 ms per launch on GB300 (FP64 ~1.1 TFLOP/s, FP32 ~70 TFLOP/s)
	const double target = sizeof(T) == 8 ? 5.5e10 : 3.5e12;
	const int iters = (int) std::max(1.0, target / (2.0 * CH * nt * (double) nb));
	const T a = sizeof(T) == 8 ? (T) 0.9999999 : (T) 0.9999f, b = sizeof(T) == 8 ? (T) 1e-7 : (T) 1e-4f;
	for (int rep = 0; rep < 3; ++rep) {                   // first launch is a warm-up
		SA_CHECK(cudaEventRecord(e0, s));
		k_fma_peak<T, CH><<<nb, nt, 0, s>>>(iters, a, b, stamps);
		SA_CHECK(cudaEventRecord(e1, s));
		SA_CHECK(cudaEventSynchronize(e1));
		float ms = 0.f;
		SA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
		long long h[2];
		SA_CHECK(cudaMemcpy(h, stamps, sizeof(h), cudaMemcpyDeviceToHost));
		const double fl = 2.0 * CH * (double) iters * (double) nt * nb;
		const double tf = fl / (ms * 1e-3) / 1e12;
		if (rep > 0 && tf > best) {
			best = tf;
			bestMhz = h[1] > 0 ? (double) h[0] / (double) h[1] * 1e3 : 0.0;
		}
	}
}

int fma_peak_selftest(cudaStream_t s, int fp64, double *tflops, double *flopsPerClockSm, double *mhz)
{
	int dev = 0, sms = 0;
	SA_CHECK(cudaGetDevice(&dev));
	SA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	long long *stamps = nullptr;
	SA_CHECK(cudaMallocAsync(&stamps, sizeof(long long) * 2 * 8 * sms, s));
	cudaEvent_t e0, e1;
	SA_CHECK(cudaEventCreate(&e0));
	SA_CHECK(cudaEventCreate(&e1));
	double best = 0.0, bestMhz = 0.0;
	for (int cps : {2, 4, 8}) {
		if (fp64) {
			fma_peak_variant<double, 4>(s, sms, cps, stamps, e0, e1, best, bestMhz);
			fma_peak_variant<double, 8>(s, sms, cps, stamps, e0, e1, best, bestMhz);
		} else {
			fma_peak_variant<float, 8>(s, sms, cps, stamps, e0, e1, best, bestMhz);
			fma_peak_variant<float, 16>(s, sms, cps, stamps, e0, e1, best, bestMhz);
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	SA_CHECK(cudaFreeAsync(stamps, s));
	SA_CHECK(cudaStreamSynchronize(s));
	*tflops = best;
	if (mhz) *mhz = bestMhz;
	if (flopsPerClockSm) *flopsPerClockSm = bestMhz > 0.0 ? best * 1e12 / ((double) sms * bestMhz * 1e6) : 0.0;
	return SA_OK;
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
// CTAs of the vector kernels: kVecCtasPerSm per SM, fewer for short vectors
static int vec_grid(long n, int smCount)
{
	int need = grid_for(n, kCgBlock);
	return std::max(1, std::min(need, kVecCtasPerSm * std::max(1, smCount)));
}

static void set_scal(CgScal *d, double tolSqu, int itrMax, double bb, cudaStream_t s)
{
	CgScal h{};
	h.tolSqu = tolSqu;
	h.itrMax = itrMax;
	h.bb = bb;
	h.first = 1;
	SA_CHECK(cudaMemcpyAsync(d, &h, sizeof(CgScal), cudaMemcpyHostToDevice, s));
}

// CTAs of k_cg_persist with `warps` warps each that can be resident at once (0: it cannot run)
// largest dynamic shared memory of one k_cg_persist CTA (the device's opt-in limit less the kernel's static
// shared memory), set as the kernel's limit on first use; 0 if that fails
template <int B, typename TM, typename TV, typename TX>
static size_t persist_smem_max()
{
	static std::mutex mu;                    // sessions and servers may size launches from several threads
	static size_t lim = (size_t) -1;
	std::lock_guard<std::mutex> lock(mu);
	if (lim == (size_t) -1) {
		lim = 0;
		int dev = 0, optin = 0;
		cudaFuncAttributes fa;
		if (cudaGetDevice(&dev) == cudaSuccess &&
		    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess &&
		    cudaFuncGetAttributes(&fa, k_cg_persist<B, TM, TV, TX>) == cudaSuccess && (size_t) optin > fa.sharedSizeBytes) {
			const size_t want = (size_t) optin - fa.sharedSizeBytes;
			if (cudaFuncSetAttribute(k_cg_persist<B, TM, TV, TX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                         (int) want) == cudaSuccess)
				lim = want;
		}
		cudaGetLastError();
	}
	return lim;
}

template <int B, typename TM, typename TV, typename TX>
static int persist_capacity(int smCount, int warps, size_t smemBytes)
{
	if (warps < 1 || warps > kPersistMaxWarps || smemBytes > persist_smem_max<B, TM, TV, TX>()) return 0;
	int v = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_cg_persist<B, TM, TV, TX>, 32 * warps, smemBytes) !=
	    cudaSuccess) {
		cudaGetLastError();
		v = 0;
	}
	return v * smCount;
}

// CTAs of k_cg_persist_g (warps per CTA, dynamic shared memory) that can be resident at once
template <int B, typename TM, typename TV, typename TX>
static int persist_g_capacity(int smCount, int warps, size_t smemBytes)
{
	static std::mutex mu;
	static bool attr = false;
	if (warps < 2 || warps > kPersistMaxWarps || smemBytes > (size_t) kColSmemMax) return 0;
	std::lock_guard<std::mutex> lock(mu);
	if (!attr) {
		if (cudaFuncSetAttribute(k_cg_persist_g<B, TM, TV, TX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         kColSmemMax) != cudaSuccess) {
			cudaGetLastError();
			return 0;
		}
		attr = true;
	}
	int v = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_cg_persist_g<B, TM, TV, TX>, 32 * warps, smemBytes) !=
	    cudaSuccess) {
		cudaGetLastError();
		v = 0;
	}
	return v * smCount;
}

// largest slot range of the nctas contiguous CTA ranges [c nsl / nctas, (c + 1) nsl / nctas), in bytes
static size_t col_span_bytes_even(const Mesh &m, int nctas)
{
	const std::vector<int> &off = m.slOffHost;
	if ((int) off.size() != m.nslice + 1 || nctas < 1) return (size_t) -1;
	long span = 0;
	for (int c = 0; c < nctas; ++c) {
		const int s0 = (int) ((long) c * m.nslice / nctas), s1 = (int) ((long) (c + 1) * m.nslice / nctas);
		span = std::max(span, (long) off[s1] - off[s0]);
	}
	return (size_t) span * sizeof(int);
}

// Slices of the persistent CG's CTAs: nctas CTAs x pw row warps, one slice per warp; warp w runs on SM
// sub-partition w % 4, whose FP64 pipe serves only its own warps.  Slices are dealt by slot count, largest
// first, each to the (CTA, sub-partition) with the least work that still has a free warp, so every
// sub-partition's matvec takes about as long (on the layered shell the inner and outer node layers have
// about half the neighbours of the others: consecutive slices per CTA left the busiest sub-partition 11 %
// above the mean, this 7 %).  Rows are computed alike wherever they run, but each CTA's partial sums are
// rounded once to FP64 before the grid sum, so the grouping can move results in the last bits; it is fixed
// for a mesh and an SM count, so results are reproducible.  Layout: nctas * pw slice ids (-1: none), then nctas * pw
// offsets into the CTA's column cache.  Returns the largest column cache in bytes, or (size_t) -1 without
// the host copy of the slice offsets.
static size_t balanced_cta_table(const Mesh &m, int pw, int nctas, std::vector<int> &tab)
{
	const std::vector<int> &off = m.slOffHost;
	const int ns = m.nslice;
	if ((int) off.size() != ns + 1 || pw < 1 || (long) nctas * pw < ns) return (size_t) -1;
	auto slots = [&](int sl) { return (long) off[sl + 1] - off[sl]; };
	std::vector<int> order(ns);
	for (int k = 0; k < ns; ++k) order[k] = k;
	std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return slots(a) > slots(b); });
	int cap[4] = {0, 0, 0, 0};                          // row warps per sub-partition
	for (int w = 0; w < pw; ++w) ++cap[w % 4];
	typedef std::pair<long, int> Load;                  // (slots so far, bin = 4 CTA + sub-partition)
	std::priority_queue<Load, std::vector<Load>, std::greater<Load>> open;
	for (int c = 0; c < nctas; ++c)
		for (int q = 0; q < 4; ++q)
			if (cap[q] > 0) open.push(Load(0, 4 * c + q));
	std::vector<int> used((size_t) 4 * nctas, 0);
	tab.assign((size_t) 2 * nctas * pw, -1);
	for (int sl : order) {
		const Load l = open.top();
		open.pop();
		const int c = l.second >> 2, q = l.second & 3;
		tab[(size_t) c * pw + q + 4 * used[l.second]] = sl;
		if (++used[l.second] < cap[q]) open.push(Load(l.first + slots(sl), l.second));
	}
	long span = 0;
	for (int c = 0; c < nctas; ++c) {
		long cache = 0;
		for (int w = 0; w < pw; ++w) {
			tab[(size_t) nctas * pw + (size_t) c * pw + w] = (int) cache;
			const int sl = tab[(size_t) c * pw + w];
			if (sl >= 0) cache += slots(sl);
		}
		span = std::max(span, cache);
	}
	return (size_t) span * sizeof(int);
}

static CgScal read_scal(const CgScal *d, cudaStream_t s)
{
	CgScal h;
	SA_CHECK(cudaMemcpyAsync(&h, d, sizeof(CgScal), cudaMemcpyDeviceToHost, s));
	SA_CHECK(cudaStreamSynchronize(s));
	return h;
}

// one inner CG run: vectors of type TV, operator of type TM, solution TX
template <int B, typename TM, typename TV, typename TX>
static CgScal run_cg(const Mesh &m, const TM *blk, const TV *dinv, const double *b, TX *x, const double *q,
                     TV *r, TV *u, TV *w, TV *p, TV *sv, double *part, CgScal *sc, int itrMax, double tolSqu,
                     double bb, cudaStream_t s, CgWork *prof = nullptr)
{
	int N = m.N;
	long n = (long) N * B;
	int nb = vec_grid(n, prof->smCount);
	const int chunk = 16;
	bool timing = prof->profileEnabled && prof->profileOn;
	if (timing && !prof->ev[0])
		for (int k = 0; k < 4 * chunk; ++k) SA_CHECK(cudaEventCreate(&prof->ev[k]));
	set_scal(sc, tolSqu, itrMax, bb, s);
	// block-Jacobi inverses of this solve (FP32 copies for FP32 vectors); every CG path uses them
	const TV *binv = nullptr;
	if constexpr (block_prec<B, TV>()) {
		binv = sizeof(TV) == sizeof(float) ? (const TV *) (const void *) prof->binv32
		                                   : (const TV *) (const void *) prof->binv64;
		if (!binv) throw CudaError{cudaErrorInvalidValue, "block-Jacobi CG without block inverses"};
	}
	// persistent launch: one CTA per SM, one slice per row warp plus the reducer warp
	const int pwCap = std::max(1, std::min(kPersistMaxWarps, tuning().persistMaxWarps) - 1);
	const int pw = std::max(1, std::min(pwCap, (m.nslice + prof->smCount - 1) / prof->smCount));
	const int nctas = (m.nslice + pw - 1) / pw;
	if (prof->ctaTab && (prof->ctaTabWarps != pw || prof->ctaTabCtas != nctas) && 2L * nctas * pw <= prof->ctaTabCap) {
		prof->ctaTabSmem = balanced_cta_table(m, pw, nctas, prof->ctaTabHost);
		if (prof->ctaTabSmem != (size_t) -1) {
			SA_CHECK(cudaMemcpyAsync(prof->ctaTab, prof->ctaTabHost.data(), sizeof(int) * prof->ctaTabHost.size(),
			                         cudaMemcpyHostToDevice, s));
			prof->ctaTabWarps = pw;
			prof->ctaTabCtas = nctas;
		}
	}
	const bool tabOk = prof->ctaTab && prof->ctaTabWarps == pw && prof->ctaTabCtas == nctas &&
	                   prof->ctaTabSmem <= (size_t) kColSmemMax;
	const size_t colSmem = tabOk ? prof->ctaTabSmem : (size_t) -1;
	// FP32 operators: cache the leading slots of every slice in the shared memory left over (an even count)
	int kc = 0;
	size_t dynSmem = colSmem;
	if (sizeof(TM) == sizeof(float) && tabOk) {
		const size_t lim = persist_smem_max<B, TM, TV, TX>(), perSlot = (size_t) pw * 32 * B * B * sizeof(TM);
		int widest = 0;
		for (int sl = 0; sl < m.nslice; ++sl)
			widest = std::max(widest, (m.slOffHost[sl + 1] - m.slOffHost[sl]) / 32);
		if (lim > colSmem) kc = (int) std::min<size_t>((size_t) widest + 1, (lim - colSmem) / perSlot) & ~1;
		dynSmem = colSmem + (size_t) kc * perSlot;
	}
	// FP64 block-Jacobi: every row warp's block inverses after the columns, 8-byte aligned
	if (block_prec<B, TV>() && sizeof(TV) == sizeof(double) && tabOk)
		dynSmem = ((colSmem + 7) & ~(size_t) 7) + (size_t) pw * 32 * B * B * sizeof(TV);
	const int colInts = tabOk ? (int) (colSmem / sizeof(int)) : 0;
	const bool persist = prof->cgKernel != SA_CG_TWO_KERNEL && prof->cgKernel != SA_CG_PERSISTENT_GLOBAL && prof->bar &&
	                     tabOk && (B != 3 || prof->u4) &&
	                     nctas <= persist_capacity<B, TM, TV, TX>(prof->smCount, pw + 1, dynSmem);
	if (persist) {
		// one cooperative launch for the whole solve (k_cg_init sets r, u and the scalars first)
		if constexpr (block_prec<B, TV>())
			k_cg_init_blk<B, TV><<<vec_grid(N, prof->smCount), kCgBlock, 0, s>>>(N, b, q, binv, r, u, part, sc);
		else
			k_cg_init<TV><<<nb, kCgBlock, 0, s>>>(n, b, q, dinv, r, u, part, sc);
		// the matvec gathers u from a copy in its own layout (3-component nodes padded to 4)
		TV *ug = u;
		if (B == 3) {
			ug = reinterpret_cast<TV *>(prof->u4);
			k_pad_u<B, TV><<<grid_for(N), kBlock, 0, s>>>(N, u, ug);
			++prof->launches;
		}
		GridBar *bar = (GridBar *) prof->bar;
		SA_CHECK(cudaMemsetAsync(bar, 0, sizeof(GridBar), s));
		SellOp A = sell_of(m);
		const TV *r0 = r;
		const TV *uc = u;
		const int *tab = prof->ctaTab;
		void *args[] = {&A, (void *) &blk, (void *) &dinv, (void *) &binv, (void *) &x, (void *) &r0, (void *) &uc,
		                (void *) &ug, (void *) &part, (void *) &sc, (void *) &bar, (void *) &tab, (void *) &colInts,
		                (void *) &kc};
		if (timing) SA_CHECK(cudaEventRecord(prof->ev[0], s));
		SA_CHECK(cudaLaunchCooperativeKernel((const void *) k_cg_persist<B, TM, TV, TX>, dim3(nctas),
		                                     dim3(32 * (pw + 1)), args, dynSmem, s));
		if (timing) SA_CHECK(cudaEventRecord(prof->ev[1], s));
		k_cg_zero<TX><<<grid_for(n), kBlock, 0, s>>>(n, x, sc);
		prof->launches += 3;
		unsigned int gaveUp = 0;
		SA_CHECK(cudaMemcpyAsync(&gaveUp, &bar->abort, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
		CgScal h = read_scal(sc, s);
		if (timing && h.iters > 0) {
			float ms = 0.f;
			SA_CHECK(cudaEventElapsedTime(&ms, prof->ev[0], prof->ev[1]));
			prof->spmvMs += ms;
			prof->spmvCount += 1;
			// per iteration: operator values, column indices and slice table once, u gathered once and
			// written once (x, r, p, s, D^-1 stay in registers); per launch: x, r, u, D^-1 in, x out
			prof->profBytes += (double) h.iters * ((double) m.slTotal * (B * B * sizeof(TM) + 4.0) +
			                                       8.0 * m.nslice + 2.0 * sizeof(TV) * n) +
			                   4.0 * sizeof(TV) * n + sizeof(TX) * n;
			// FMAs per vector entry: x, r, p, s updates, three dot terms, and u = D^-1 r (1) or the
			// entry's row of the block inverse (B)
			prof->profFlops += (double) h.iters * 2.0 * ((double) B * B * m.slTotal + (block_prec<B, TV>() ? 7.0 + B : 8.0) * n);
		}
		// any CTA that gave up leaves the abort flag set, whatever CTA 0 reported
		if (gaveUp || h.code == SA_ERR_TIMEOUT) throw DeviceWaitError{"persistent CG grid barrier"};
		return h;
	}
	// too large for row state in registers: the global-state persistent kernel, one CTA per SM
	if (prof->cgKernel != SA_CG_TWO_KERNEL && prof->bar) {
		const int warpsG = pwCap + 1;
		const int nctasG = std::min(prof->smCount, m.nslice);
		const size_t span = col_span_bytes_even(m, nctasG);
		const int cached = span <= (size_t) kColSmemMax ? 1 : 0;
		const size_t smemG = cached ? span : 0;
		if (nctasG >= 1 && nctasG <= persist_g_capacity<B, TM, TV, TX>(prof->smCount, warpsG, smemG)) {
			if constexpr (block_prec<B, TV>())
				k_cg_init_blk<B, TV><<<vec_grid(N, prof->smCount), kCgBlock, 0, s>>>(N, b, q, binv, r, u, part, sc);
			else
				k_cg_init<TV><<<nb, kCgBlock, 0, s>>>(n, b, q, dinv, r, u, part, sc);
			SA_CHECK(cudaMemsetAsync(p, 0, sizeof(TV) * n, s));
			SA_CHECK(cudaMemsetAsync(sv, 0, sizeof(TV) * n, s));
			GridBar *bar = (GridBar *) prof->bar;
			SA_CHECK(cudaMemsetAsync(bar, 0, sizeof(GridBar), s));
			SellOp A = sell_of(m);
			void *args[] = {&A, (void *) &blk, (void *) &dinv, (void *) &binv, (void *) &x, (void *) &r, (void *) &u,
			                (void *) &w, (void *) &p, (void *) &sv, (void *) &cached, (void *) &part, (void *) &sc,
			                (void *) &bar};
			if (timing) SA_CHECK(cudaEventRecord(prof->ev[0], s));
			SA_CHECK(cudaLaunchCooperativeKernel((const void *) k_cg_persist_g<B, TM, TV, TX>, dim3(nctasG),
			                                     dim3(32 * warpsG), args, smemG, s));
			if (timing) SA_CHECK(cudaEventRecord(prof->ev[1], s));
			k_cg_zero<TX><<<grid_for(n), kBlock, 0, s>>>(n, x, sc);
			prof->launches += 3;
			unsigned int gaveUp = 0;
			SA_CHECK(cudaMemcpyAsync(&gaveUp, &bar->abort, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
			CgScal h = read_scal(sc, s);
			if (timing && h.iters > 0) {
				float ms = 0.f;
				SA_CHECK(cudaEventElapsedTime(&ms, prof->ev[0], prof->ev[1]));
				prof->spmvMs += ms;
				prof->spmvCount += 1;
				// per iteration: operator values (+ columns unless cached), slice table, u gathered, and the
				// vectors w, p, s, r, x read and written, u read twice and written
				prof->profBytes += (double) h.iters * ((double) m.slTotal * (B * B * sizeof(TM) + (cached ? 0.0 : 4.0)) +
				                                       8.0 * m.nslice + 14.0 * sizeof(TV) * n);
				prof->profFlops += (double) h.iters * 2.0 * ((double) B * B * m.slTotal + (block_prec<B, TV>() ? 7.0 + B : 8.0) * n);
			}
			if (gaveUp || h.code == SA_ERR_TIMEOUT) throw DeviceWaitError{"persistent CG grid barrier"};
			return h;
		}
	}
	SA_CHECK(cudaMemsetAsync(p, 0, sizeof(TV) * n, s));
	SA_CHECK(cudaMemsetAsync(sv, 0, sizeof(TV) * n, s));
	if constexpr (block_prec<B, TV>())
		k_cg_init_blk<B, TV><<<vec_grid(N, prof->smCount), kCgBlock, 0, s>>>(N, b, q, binv, r, u, part, sc);
	else
		k_cg_init<TV><<<nb, kCgBlock, 0, s>>>(n, b, q, dinv, r, u, part, sc);
	const int nbRows = vec_grid(N, prof->smCount);
	if (!prof->pinned) {
		SA_CHECK(cudaHostAlloc(&prof->pinned, 2 * sizeof(CgScal), cudaHostAllocDefault));
		for (int k = 0; k < 2; ++k) SA_CHECK(cudaEventCreateWithFlags(&prof->chunkEv[k], cudaEventDisableTiming));
	}
	CgScal *hs = (CgScal *) prof->pinned;
	// chunks of iterations are queued one ahead: while the host waits for the
	// status of chunk c - 1, chunk c is already on the GPU (its kernels return
	// at once if c - 1 converged), so the device never idles on the host
	auto launch_chunk = [&](int set) {
		for (int k = 0; k < chunk; ++k) {
			if (timing) SA_CHECK(cudaEventRecord(prof->ev[set * 2 * chunk + 2 * k], s));
			k_cg_spmv<B, TM, TV><<<(m.nslice + kSlicesPerCta - 1) / kSlicesPerCta, kSpmvBlock, 0, s>>>(
				sell_of(m), blk, u, w, part, sc);
			if (timing) SA_CHECK(cudaEventRecord(prof->ev[set * 2 * chunk + 2 * k + 1], s));
			if constexpr (block_prec<B, TV>())
				k_cg_update_blk<B, TV, TX><<<nbRows, kCgBlock, 0, s>>>(N, x, r, u, w, p, sv, binv, part, sc);
			else
				k_cg_update<TV, TX><<<nb, kCgBlock, 0, s>>>(n, x, r, u, w, p, sv, dinv, part, sc);
		}
		SA_CHECK(cudaMemcpyAsync(hs + set, sc, sizeof(CgScal), cudaMemcpyDeviceToHost, s));
		SA_CHECK(cudaEventRecord(prof->chunkEv[set], s));
		SA_CHECK(cudaGetLastError());
		prof->launches += 2 * chunk;
	};
	const int maxChunks = (itrMax + chunk - 1) / chunk + 1;
	int itersBefore = 0;
	launch_chunk(0);
	for (int c = 1; c <= maxChunks; ++c) {
		if (c < maxChunks) launch_chunk(c & 1);
		int prev = (c - 1) & 1;
		SA_CHECK(cudaEventSynchronize(prof->chunkEv[prev]));
		CgScal h = hs[prev];
		if (timing) {
			// matvec launches that did work in this chunk = iterations completed in it
			int worked = std::min(chunk, h.iters - itersBefore);
			for (int k = 0; k < worked; ++k) {
				float ms = 0.f;
				SA_CHECK(cudaEventElapsedTime(&ms, prof->ev[prev * 2 * chunk + 2 * k],
				                              prof->ev[prev * 2 * chunk + 2 * k + 1]));
				prof->spmvMs += ms;
			}
			prof->spmvCount += worked;
			// per matvec: operator values, column indices, slice table, u read and w written once
			prof->profBytes += worked * ((double) m.slTotal * (B * B * sizeof(TM) + 4.0) + 8.0 * m.nslice +
			                             2.0 * sizeof(TV) * n);
			prof->profFlops += worked * 2.0 * B * B * (double) m.slTotal;
			itersBefore = h.iters;
		}
		if (h.done) break;
	}
	k_cg_zero<TX><<<grid_for(n), kBlock, 0, s>>>(n, x, sc);
	if (prof) prof->launches += 2;          // k_cg_init + k_cg_zero
	return read_scal(sc, s);
}

__global__ void k_sub(long n, const double *a, const double *b, double *c)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) c[k] = a[k] - b[k];
}

template <int B>
int cg_jacobi(const Mesh &m, const double *blk, const double *dinv, const double *b, double *x, int itrMax,
              double tolSqu, CgWork &wk, Status *st, int *itersOut, cudaStream_t s, int precision)
{
	(void) st;
	int N = m.N;
	long n = (long) N * B;
	double *q = wk.xr;                       // A x (FP64)
	CgScal *sc = (CgScal *) wk.scal;
	if (precision == SA_PREC_FP64 || !wk.blk32) {
		k_spmv64<B><<<grid_for(N), kBlock, 0, s>>>(sell_of(m), blk, x, q);
		wk.launches += 1;
		CgScal h = run_cg<B, double, double, double>(m, blk, dinv, b, x, q, wk.r, wk.u, wk.w, wk.p, wk.sv,
		                                              wk.part, sc, itrMax, tolSqu, -1.0, s, &wk);
		if (itersOut) *itersOut = h.iters;
		return h.code;
	}
	// Mixed precision: FP64 iterative refinement.  Each outer step forms the
	// true residual rin = b - A x with the FP64 operator, solves A d = rin
	// with the FP32 operator and FP32 vectors (FP64 dot products), and
	// updates x += d in FP64.
	float *r32 = wk.f32, *u32 = r32 + n, *w32 = r32 + 2 * n, *p32 = r32 + 3 * n, *s32 = r32 + 4 * n;
	float *dinv32 = r32 + 5 * n, *d32 = r32 + 6 * n;
	double *rin = wk.xr + n, *zero = wk.xr + 2 * n;
	k_convert<double, float><<<grid_for(n), kBlock, 0, s>>>(n, dinv, dinv32);
	SA_CHECK(cudaMemsetAsync(zero, 0, sizeof(double) * n, s));
	int total = 0, code = SA_ERR_NOT_CONVERGED;
	double bb = -1.0;
	const int nb = vec_grid(n, wk.smCount);
	for (int outer = 0; outer < 64; ++outer) {
		k_spmv64<B><<<grid_for(N), kBlock, 0, s>>>(sell_of(m), blk, x, q);
		k_sub<<<grid_for(n), kBlock, 0, s>>>(n, b, q, rin);
		wk.launches += 4;                     // spmv64, sub, init, axpy of this outer step
		// outer test: |b - A x|^2 < tol^2 |b|^2 (k_cg_init with b and q gives both norms)
		set_scal(sc, tolSqu, 1, bb, s);
		k_cg_init<float><<<nb, kCgBlock, 0, s>>>(n, b, q, dinv32, r32, u32, wk.part, sc);
		CgScal h0 = read_scal(sc, s);
		if (bb < 0.0) bb = h0.bb;
		if (h0.code == SA_ERR_NONFINITE) { code = SA_ERR_NONFINITE; break; }
		if (h0.zero) { SA_CHECK(cudaMemsetAsync(x, 0, sizeof(double) * n, s)); code = SA_OK; break; }
		if (h0.rr < tolSqu * bb) { code = SA_OK; break; }
		if (total >= itrMax) { code = SA_ERR_NOT_CONVERGED; break; }
		// inner tolerance: just below what the outer test still needs, not below the FP32 floor
		double need = 0.01 * tolSqu * bb / h0.rr;
		const double floorSqu = std::pow(10.0, -(double) tuning().mixedInnerFloor);
		double innerTol = need > floorSqu ? need : floorSqu;
		SA_CHECK(cudaMemsetAsync(d32, 0, sizeof(float) * n, s));
		CgScal h = run_cg<B, float, float, float>(m, wk.blk32, dinv32, rin, d32, zero, r32, u32, w32, p32, s32,
		                                           wk.part, sc, itrMax - total, innerTol, -1.0, s, &wk);
		total += h.iters;
		if (h.code == SA_ERR_NONFINITE) { code = h.code; break; }
		k_axpy_f32<<<grid_for(n), kBlock, 0, s>>>(n, x, d32);
	}
	if (itersOut) *itersOut = total;
	return code;
}

// ---------------------------------------------------------------------------
// batched CG (serving): per-solve preparation, one launch for all solves
// ---------------------------------------------------------------------------
template <int B>
void cg_prepare_fp64(const Mesh &m, const double *blk, const double *dinv, const double *b, double *x, int itrMax,
                     double tolSqu, CgWork &w, cudaStream_t s)
{
	long n = (long) m.N * B;
	double *q = w.xr;
	k_spmv64<B><<<grid_for(m.N), kBlock, 0, s>>>(sell_of(m), blk, x, q);
	set_scal((CgScal *) w.scal, tolSqu, itrMax, -1.0, s);
	SA_CHECK(cudaMemsetAsync(w.p, 0, sizeof(double) * n, s));
	SA_CHECK(cudaMemsetAsync(w.sv, 0, sizeof(double) * n, s));
	if constexpr (block_prec<B, double>()) {
		if (!w.binv64) throw CudaError{cudaErrorInvalidValue, "block-Jacobi CG without block inverses"};
		k_cg_init_blk<B, double><<<vec_grid(m.N, w.smCount), kCgBlock, 0, s>>>(m.N, b, q, w.binv64, w.r, w.u,
		                                                                        w.part, (CgScal *) w.scal);
	} else {
		k_cg_init<double><<<vec_grid(n, w.smCount), kCgBlock, 0, s>>>(n, b, q, dinv, w.r, w.u, w.part,
		                                                                (CgScal *) w.scal);
	}
	w.launches += 2;
}

template <int B>
void cg_finish_fp64(const Mesh &m, double *x, CgWork &w, cudaStream_t s)
{
	long n = (long) m.N * B;
	k_cg_zero<double><<<grid_for(n), kBlock, 0, s>>>(n, x, (const CgScal *) w.scal);
	w.launches += 1;
}

template <int B>
void cg_mixed_outer(const Mesh &m, const double *blk, const double *dinv, const double *b, const double *x,
                    double bb, int first, CgWork &w, cudaStream_t s)
{
	long n = (long) m.N * B;
	float *r32 = w.f32, *u32 = r32 + n, *dinv32 = r32 + 5 * n;
	double *q = w.xr, *rin = w.xr + n;
	if (first) k_convert<double, float><<<grid_for(n), kBlock, 0, s>>>(n, dinv, dinv32);
	k_spmv64<B><<<grid_for(m.N), kBlock, 0, s>>>(sell_of(m), blk, x, q);
	k_sub<<<grid_for(n), kBlock, 0, s>>>(n, b, q, rin);
	set_scal((CgScal *) w.scal, 1.0, 1, bb, s);
	k_cg_init<float><<<vec_grid(n, w.smCount), kCgBlock, 0, s>>>(n, b, q, dinv32, r32, u32, w.part,
	                                                               (CgScal *) w.scal);
	w.launches += 3 + (first ? 1 : 0);
}

template <int B>
void cg_mixed_inner(const Mesh &m, int itrMax, double innerTolSqu, CgWork &w, cudaStream_t s)
{
	long n = (long) m.N * B;
	float *r32 = w.f32, *u32 = r32 + n, *p32 = r32 + 3 * n, *s32 = r32 + 4 * n;
	float *dinv32 = r32 + 5 * n, *d32 = r32 + 6 * n;
	double *rin = w.xr + n, *zero = w.xr + 2 * n;
	SA_CHECK(cudaMemsetAsync(zero, 0, sizeof(double) * n, s));
	SA_CHECK(cudaMemsetAsync(d32, 0, sizeof(float) * n, s));
	SA_CHECK(cudaMemsetAsync(p32, 0, sizeof(float) * n, s));
	SA_CHECK(cudaMemsetAsync(s32, 0, sizeof(float) * n, s));
	set_scal((CgScal *) w.scal, innerTolSqu, itrMax, -1.0, s);
	if (!w.binv32) throw CudaError{cudaErrorInvalidValue, "mixed precision without block inverses"};
	(void) dinv32;
	k_cg_init_blk<B, float><<<vec_grid(m.N, w.smCount), kCgBlock, 0, s>>>(m.N, rin, zero, w.binv32, r32, u32, w.part,
	                                                                (CgScal *) w.scal);
	w.launches += 1;
}

void cg_mixed_apply(long n, double *x, const CgWork &w, cudaStream_t s)
{
	k_axpy_f32<<<grid_for(n), kBlock, 0, s>>>(n, x, w.f32 + 6 * n);
}

// the scalars of many solves with one host synchronisation: one small copy per solve into pinned memory
// (at least ws.size() CgScal-sized slots, cg_scal_bytes() each), then one wait for the stream
size_t cg_scal_bytes() { return sizeof(CgScal); }

void cg_states(const std::vector<const CgWork *> &ws, void *pinned, cudaStream_t s, std::vector<CgState> &out)
{
	CgScal *h = (CgScal *) pinned;
	for (size_t k = 0; k < ws.size(); ++k)
		SA_CHECK(cudaMemcpyAsync(h + k, ws[k]->scal, sizeof(CgScal), cudaMemcpyDeviceToHost, s));
	SA_CHECK(cudaStreamSynchronize(s));
	out.resize(ws.size());
	for (size_t k = 0; k < ws.size(); ++k)
		out[k] = CgState{h[k].code, h[k].iters, h[k].zero, h[k].done, h[k].rr, h[k].bb};
}

CgState cg_state(const CgWork &w, cudaStream_t s)
{
	CgScal h = read_scal((const CgScal *) w.scal, s);
	return CgState{h.code, h.iters, h.zero, h.done, h.rr, h.bb};
}

// CTAs of k_cg_batch (block threads per CTA, at most kBatchBlock) resident at once
template <int B, typename TM, typename TV, typename TX>
static int batch_capacity(int smCount, int block)
{
	static std::mutex mu;
	static int perSm[kBatchBlock / 32 + 1];
	static bool known[kBatchBlock / 32 + 1] = {};
	const int w = block / 32;
	if (w < 1 || w > kBatchBlock / 32 || block % 32) return 0;
	std::lock_guard<std::mutex> lock(mu);
	if (!known[w]) {
		int v = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_cg_batch<B, TM, TV, TX>, block, 0) != cudaSuccess) {
			cudaGetLastError();
			v = 0;
		}
		perSm[w] = v;
		known[w] = true;
	}
	return perSm[w] * smCount;
}

template <int B, typename TM, typename TV, typename TX>
int cg_batch_run(const std::vector<BatchSolve> &solves, int smCount, CgJob *devJobs, int maxJobs, cudaStream_t s)
{
	int nLaunch = 0;
	const int block = std::max(32, std::min(kBatchBlock, tuning().batchBlock / 32 * 32));
	const int cap = batch_capacity<B, TM, TV, TX>(smCount, block);
	if (cap <= 0) throw CudaError{cudaErrorLaunchOutOfResources, "k_cg_batch occupancy"};
	const int W = block / 32;
	std::vector<char> taken(solves.size(), 0);
	size_t left = solves.size();
	while (left > 0) {
		// CTAs of a solve: one per batchSlicesPerWarp slices per warp, from its own size only (its partial
		// sums, and so its result, do not depend on the other solves).  First fit in the caller's order:
		// each launch takes every remaining solve that still fits its co-resident CTA capacity
		std::vector<CgJob> jobs;
		int cta = 0;
		for (size_t k1 = 0; k1 < solves.size() && (int) jobs.size() < maxJobs; ++k1) {
			if (taken[k1]) continue;
			const BatchSolve &b = solves[k1];
			const Mesh &m = *b.m;
			const int per = W * std::max(1, tuning().batchSlicesPerWarp);
			const int want = std::max(1, std::min(cap, (m.nslice + per - 1) / per));
			if (cta + want > cap) continue;
			taken[k1] = 1;
			--left;
			CgWork &w = *b.cw;
			CgJob j;
			j.A = sell_of(m);
			if (block_prec<B, TV>() && !b.binv) throw CudaError{cudaErrorInvalidValue, "batched CG without block inverses"};
			j.blk = b.blk; j.dinv = b.dinv; j.binv = b.binv; j.x = b.x;
			if (sizeof(TV) == sizeof(double)) {
				j.r = w.r; j.u = w.u; j.w = w.w; j.p = w.p; j.s = w.sv;
			} else {
				long n = (long) m.N * B;
				float *f = w.f32;
				j.r = f; j.u = f + n; j.w = f + 2 * n; j.p = f + 3 * n; j.s = f + 4 * n;
			}
			j.part = w.part; j.sc = w.scal; j.bar = w.bar;
			j.cta0 = cta; j.nctas = want;
			cta += want;
			SA_CHECK(cudaMemsetAsync(w.bar, 0, sizeof(GridBar), s));
			w.launches += 1;
			jobs.push_back(j);
		}
		SA_CHECK(cudaMemcpyAsync(devJobs, jobs.data(), sizeof(CgJob) * jobs.size(), cudaMemcpyHostToDevice, s));
		int nj = (int) jobs.size();
		const CgJob *dj = devJobs;
		void *args[] = {(void *) &dj, (void *) &nj};
		SA_CHECK(cudaLaunchCooperativeKernel((const void *) k_cg_batch<B, TM, TV, TX>, dim3(cta), dim3(block),
		                                     args, 0, s));
		++nLaunch;
		// the job table is read by the kernel: wait before the host vector goes away or is rewritten
		SA_CHECK(cudaStreamSynchronize(s));
		for (const CgJob &j : jobs) {
			unsigned int gaveUp = 0;
			SA_CHECK(cudaMemcpy(&gaveUp, &((GridBar *) j.bar)->abort, sizeof(unsigned int), cudaMemcpyDeviceToHost));
			if (gaveUp) throw DeviceWaitError{"batched CG grid barrier"};
		}
	}
	return nLaunch;
}

#define SA_BATCH_INST(B)                                                                                          \
	template void cg_prepare_fp64<B>(const Mesh &, const double *, const double *, const double *, double *, int, \
	                                 double, CgWork &, cudaStream_t);                                             \
	template void cg_finish_fp64<B>(const Mesh &, double *, CgWork &, cudaStream_t);                             \
	template void cg_mixed_outer<B>(const Mesh &, const double *, const double *, const double *, const double *, \
	                                double, int, CgWork &, cudaStream_t);                                         \
	template void cg_mixed_inner<B>(const Mesh &, int, double, CgWork &, cudaStream_t);                          \
	template int cg_batch_run<B, double, double, double>(const std::vector<BatchSolve> &, int, CgJob *, int,    \
	                                                      cudaStream_t);                                          \
	template int cg_batch_run<B, float, float, float>(const std::vector<BatchSolve> &, int, CgJob *, int,       \
	                                                   cudaStream_t);
SA_BATCH_INST(1)
SA_BATCH_INST(2)
SA_BATCH_INST(3)
#undef SA_BATCH_INST

template int cg_jacobi<1>(const Mesh &, const double *, const double *, const double *, double *, int, double,
                          CgWork &, Status *, int *, cudaStream_t, int);
template int cg_jacobi<2>(const Mesh &, const double *, const double *, const double *, double *, int, double,
                          CgWork &, Status *, int *, cudaStream_t, int);
template int cg_jacobi<3>(const Mesh &, const double *, const double *, const double *, double *, int, double,
                          CgWork &, Status *, int *, cudaStream_t, int);

}  // namespace sa
