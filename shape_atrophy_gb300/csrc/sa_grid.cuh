// sa_grid.cuh -- grid-wide barriers and exact sums for persistent cooperative kernels (one CTA per SM).
//
// A reduction is also a barrier: every CTA publishes its partial sums, counts itself in, waits for the
// count of the whole grid and then adds all partials exactly in 128-bit fixed point (sa_fixsum.cuh:
// order-independent, rounded once), so every CTA obtains the same value.  Ordering: the arriving thread
// fences its CTA's writes (after a CTA barrier) before its relaxed atomic arrival, the waiting thread reads
// the count with acquire loads, and a CTA (or warp) barrier then passes the order on to the other threads:
// a release-acquire chain at GPU scope, without a second fence after the wait.  Waits are bounded: a CTA that
// waits longer than kBarWaitNs (or sees another CTA give up) returns false and the kernel stops with a
// timeout status.
#pragma once
#include "sa_internal.cuh"
#include "sa_fixsum.cuh"

namespace sa {

struct GridBar {
	unsigned int count, pad0[31];      // arrivals, grows by nctas per reduction (zeroed per launch)
	unsigned int abort, pad1[31];      // set by a CTA that gave up
};
static_assert(sizeof(GridBar) <= kGridBarBytes, "grid barrier larger than its allocation");
constexpr unsigned long long kBarWaitNs = 1000000000ull;   // 1 s

__device__ __forceinline__ unsigned long long global_ns()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ unsigned int load_acquire(const unsigned int *p)
{
	unsigned int v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

// Per-CTA scratch of the fixed-point reductions (K <= 2 values, up to 32 warps).
struct FxScratch {
	int e[2][32];          // per-warp largest exponent
	Fx f[2][32];           // per-warp fixed-point sums
	double tot[2];         // grid sums, broadcast to the CTA
	int ok;                // the barrier wait ended normally
};

// Sum of K values over the threads of the CTA (any multiple of 32 threads, every thread calls), exact in
// 128-bit fixed point (sa_fixsum.cuh), rounded once; valid in lane 0 of warp sumWarp.  Integer pipes only: the FP64 pipe
// (2 adds per clock per SM on GB300) would make a tree of FP64 adds the longest part of a grid reduction.
template <int K, typename T>
__device__ __forceinline__ void block_fx_sum(const T (&v)[K], FxScratch &fs, double (&out)[K], int sumWarp = 0)
{
	const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, W = blockDim.x >> 5;
	int e[K];
	for (int k = 0; k < K; ++k) {
		e[k] = fx_warp_max(fx_exp(v[k]));
		if (lane == 0) fs.e[k][wp] = e[k];
	}
	__syncthreads();
	for (int k = 0; k < K; ++k) {
		e[k] = fx_warp_max(lane < W ? fs.e[k][lane] : 1);
		const Fx t = fx_warp_sum(fx_from(v[k], e[k]));
		if (lane == 0) fs.f[k][wp] = t;
	}
	__syncthreads();
	if (wp == sumWarp)
		for (int k = 0; k < K; ++k) {
			const Fx t = fx_warp_sum(lane < W ? fs.f[k][lane] : fx_zero());
			if (lane == 0) out[k] = fx_to_double(t, e[k]);
		}
}

// Sum of nctas partials of one value by one warp, in fixed point (exact, then rounded once; the same in
// every CTA because it does not depend on the order); lane 0 returns it.
constexpr int kFxRegs = 5;     // partials held in registers per lane (nctas <= 160); more take two passes
__device__ __forceinline__ double warp_fx_partials(const double *part, int nctas)
{
	const int lane = threadIdx.x & 31;
	Fx t = fx_zero();
	int em;
	if (nctas <= 32 * kFxRegs) {
		double r[kFxRegs];
		int e = 1;
#pragma unroll
		for (int q = 0; q < kFxRegs; ++q) {
			const int b = lane + 32 * q;
			r[q] = b < nctas ? __ldcg(part + b) : 0.0;
			e = max(e, fx_exp(r[q]));
		}
		em = fx_warp_max(e);
#pragma unroll
		for (int q = 0; q < kFxRegs; ++q) t = fx_add(t, fx_from(r[q], em));
	} else {
		int e = 1;
		for (int b = lane; b < nctas; b += 32) e = max(e, fx_exp(__ldcg(part + b)));
		em = fx_warp_max(e);
		for (int b = lane; b < nctas; b += 32) t = fx_add(t, fx_from(__ldcg(part + b), em));
	}
	t = fx_warp_sum(t);
	return fx_to_double(t, em);
}

// sum of K values over all threads of the nctas CTAs of one solve plus a barrier among them; lc is the
// CTA's index within the solve.  Every thread gets the sums in res.  false: the wait gave up.
// post(sums) runs once per CTA (lane 0 of warp 0) before the sums are broadcast.
struct NoPost { __device__ void operator()(const double *) const {} };

template <int K, typename T, typename Post = NoPost>
__device__ __forceinline__ bool grid_reduce(const T (&v)[K], double (&res)[K], double *part, int lc, int nctas,
                                            GridBar *bar, unsigned int &target, FxScratch &fs, Post post = Post())
{
	double cta[K];
	block_fx_sum<K, T>(v, fs, cta);
	target += (unsigned int) nctas;
	if (threadIdx.x == 0) {
		for (int k = 0; k < K; ++k) part[k * nctas + lc] = cta[k];
		__threadfence();
		atomicAdd(&bar->count, 1u);
		int ok = 1;
		const unsigned long long t0 = global_ns();
		while ((int) (load_acquire(&bar->count) - target) < 0) {
			if (load_acquire(&bar->abort)) { ok = 0; break; }
			if (global_ns() - t0 > kBarWaitNs) { atomicExch(&bar->abort, 1u); ok = 0; break; }
		}
		fs.ok = ok;            // the acquire load that saw the count orders the partial reads after the barrier
	}
	__syncthreads();
	if (!fs.ok) return false;
	const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, W = blockDim.x >> 5;
	for (int k = wp; k < K; k += W) {            // one warp per value
		const double t = warp_fx_partials(part + (long) k * nctas, nctas);
		if (lane == 0) fs.tot[k] = t;
	}
	if (threadIdx.x == 0) post(fs.tot);          // K == 1 with a post: warp 0 wrote tot[0] itself
	__syncthreads();
	for (int k = 0; k < K; ++k) res[k] = fs.tot[k];
	return true;
}

// the barrier alone (no sums): wait for the arrival count to reach target
__device__ __forceinline__ bool wait_grid(GridBar *bar, unsigned int target)
{
	const unsigned long long t0 = global_ns();
	while ((int) (load_acquire(&bar->count) - target) < 0) {
		if (load_acquire(&bar->abort)) return false;
		if (global_ns() - t0 > kBarWaitNs) { atomicExch(&bar->abort, 1u); return false; }
	}
	return true;
}

}  // namespace sa
