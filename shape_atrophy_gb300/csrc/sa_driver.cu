// sa_driver.cu -- context, mesh set-up, the forward time loop and the C-ABI.
//
// Replaces the reference's MEX gateways (2D_frame/deformation.cu:14-199,
// computeObjfcn.cu:14-212), its memory arena (assignStructMemory.cu:33-229)
// and drivers deform() / objfcn() (deform.cu:22-119, objfcn.cu:23-123).
//
// One time step (layered model):
//   activity(tau_t) -> yank rhs b (geometry t) -> elasticity blocks (geometry t,
//   + bottom penalty) -> Jacobi CG for v_t (warm start v_{t-1}) -> x_{t+1} =
//   x_t + dt v_t -> geometry t+1 -> M', L = M' + dt G' -> rhs = M_t tau_t +
//   dt R-load(geometry t) -> Jacobi CG for tau_{t+1} (warm start tau_t).
// Frame mode is the same step with the frame stress, frame diffusion, the
// reference's activity polynomials, and the velocity solved by the
// K-preconditioned CG with the dense RKHS matrix of x_t.
#include "sa_internal.cuh"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <functional>
#include <mutex>
#include <thread>
#include <type_traits>
#include <unistd.h>

struct sa_context {
	int device = 0;
	cudaStream_t stream = nullptr;
	cudaStream_t side = nullptr;                    // work that overlaps the host's set-up (target varifold rows)
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	cudaEvent_t sideIn = nullptr, sideOut = nullptr;
	std::string err;
};

namespace sa {

// ---------------------------------------------------------------------------
// pointer helpers: accept host or device memory for every array
// ---------------------------------------------------------------------------
static bool is_device_ptr(const void *p)
{
	if (!p) return false;
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
	return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

struct Pool {                 // device allocations of one call, freed at the end
	std::vector<void *> ptrs;
	cudaStream_t s;
	size_t bytes = 0;         // device bytes allocated
	// stream-ordered (cudaMallocAsync on s, freed on s): for a call whose side stream runs while the host
	// allocates -- a plain cudaMalloc between two streams' launches keeps them from running concurrently.
	// Only for pools whose memory no other stream uses after the pool's stream has moved on.
	bool ordered = false;
	explicit Pool(cudaStream_t st, bool streamOrdered = false) : s(st), ordered(streamOrdered) {}
	~Pool() { release(); }
	void release()
	{
		for (void *p : ptrs) {
			if (ordered) cudaFreeAsync(p, s);
			else cudaFree(p);
		}
		ptrs.clear();
	}
	template <typename T> T *alloc(size_t n)
	{
		void *p = nullptr;
		if (ordered) SA_CHECK(cudaMallocAsync(&p, sizeof(T) * (n ? n : 1), s));
		else SA_CHECK(cudaMalloc(&p, sizeof(T) * (n ? n : 1)));
		ptrs.push_back(p);
		bytes += sizeof(T) * (n ? n : 1);
		return (T *) p;
	}
	template <typename T> T *zeros(size_t n)
	{
		T *p = alloc<T>(n);
		SA_CHECK(cudaMemsetAsync(p, 0, sizeof(T) * (n ? n : 1), s));
		return p;
	}
	template <typename T> const T *dev(const T *p, size_t n)     // device view of a host or device array
	{
		if (!p) return nullptr;
		if (is_device_ptr(p)) return p;
		T *d = alloc<T>(n);
		SA_CHECK(cudaMemcpyAsync(d, p, sizeof(T) * n, cudaMemcpyHostToDevice, s));
		return d;
	}
};

// Host-side phase timing of the one-call entry points, printed to stderr when the environment variable
// SA_TRACE is set (each mark waits for the stream, so traced calls run slightly slower).
struct PhaseTrace {
	bool on;
	cudaStream_t s;
	std::chrono::steady_clock::time_point t0;
	explicit PhaseTrace(cudaStream_t st) : on(std::getenv("SA_TRACE") != nullptr), s(st)
	{
		if (on) t0 = std::chrono::steady_clock::now();
	}
	void mark(const char *phase)
	{
		if (!on) return;
		cudaStreamSynchronize(s);
		const auto t = std::chrono::steady_clock::now();
		std::fprintf(stderr, "[sa_trace] %-30s %9.3f ms\n", phase,
		             std::chrono::duration<double, std::milli>(t - t0).count());
		t0 = t;
	}
};

// waits for the context's side stream when a call that launched work on it leaves (normally or by an error)
struct SideJoin {
	cudaStream_t side;
	bool on = false;
	~SideJoin() { if (on) cudaStreamSynchronize(side); }
};

struct ArgError { std::string msg; };
#define SA_REQUIRE(c, m) do { if (!(c)) throw ::sa::ArgError{m}; } while (0)

// A persistent pool of host threads for the set-up loops (thread start-up would cost more than the loops).
// run(f) calls f(t) for t = 0 .. size()-1, t = 0 on the calling thread; calls from several threads are
// serialised.  The pool lives for the process (never destroyed: its workers end with the process); a
// child made by fork() has none of the parent's threads, so it gets a pool of its own.
class HostPool {
public:
	static HostPool &get()
	{
		static std::mutex m;
		static HostPool *pool = nullptr;
		std::lock_guard<std::mutex> g(m);
		if (!pool || pool->pid != getpid()) pool = new HostPool();
		return *pool;
	}
	int size() const { return T; }
	void run(const std::function<void(int)> &f)
	{
		std::lock_guard<std::mutex> one(callMu);
		{
			std::lock_guard<std::mutex> g(mu);
			job = &f;
			pending = T - 1;
			++gen;
		}
		cv.notify_all();
		f(0);
		std::unique_lock<std::mutex> lk(mu);
		doneCv.wait(lk, [this] { return pending == 0; });
		job = nullptr;
	}

private:
	HostPool() : T((int) std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency()))), pid(getpid())
	{
		for (int i = 1; i < T; ++i) th.emplace_back([this, i] { worker(i); });
	}
	void worker(int i)
	{
		long seen = 0;
		for (;;) {
			const std::function<void(int)> *f;
			{
				std::unique_lock<std::mutex> lk(mu);
				cv.wait(lk, [&] { return gen != seen; });
				seen = gen;
				f = job;
			}
			(*f)(i);
			std::lock_guard<std::mutex> g(mu);
			if (--pending == 0) doneCv.notify_one();
		}
	}
	int T;
	pid_t pid;
	std::vector<std::thread> th;
	std::mutex mu, callMu;
	std::condition_variable cv, doneCv;
	const std::function<void(int)> *job = nullptr;
	long gen = 0;
	int pending = 0;
};

// f(lo, hi) over [0, n) in contiguous chunks on the host pool (small n: the calling thread alone); an
// ArgError in any chunk is rethrown after all chunks end
template <typename F> static void parallel_chunks(long n, F &&f)
{
	HostPool &pool = HostPool::get();
	const long T = pool.size();
	if (n < 32768 || T <= 1) {
		f(0L, n);
		return;
	}
	std::vector<std::string> err((size_t) T);
	pool.run([&](int t) {
		try {
			f(n * t / T, n * (t + 1) / T);
		} catch (const ArgError &e) {
			err[(size_t) t] = e.msg;
		}
	});
	for (const std::string &e : err)
		if (!e.empty()) throw ArgError{e};
}

// the same with the chunk's index t (chunks 0 .. chunk_count(n) - 1, in order over [0, n))
static int chunk_count(long n)
{
	const int T = HostPool::get().size();
	return n < 32768 || T <= 1 ? 1 : T;
}

template <typename F> static void parallel_chunks_t(long n, F &&f)
{
	const int T = chunk_count(n);
	if (T == 1) {
		f(0, 0L, n);
		return;
	}
	HostPool::get().run([&](int t) { f(t, n * t / T, n * (t + 1) / T); });
}

template <typename T> static std::vector<T> to_host(const T *p, size_t n, cudaStream_t s)
{
	std::vector<T> h(n);
	if (n) SA_CHECK(cudaMemcpyAsync(h.data(), p, sizeof(T) * n, cudaMemcpyDefault, s));
	SA_CHECK(cudaStreamSynchronize(s));
	return h;
}

// ---------------------------------------------------------------------------
// mesh set-up: validation, CSR row pointers, ordered assembly table
// ---------------------------------------------------------------------------
__global__ void k_asm_table(int Z, int E, int V, const int *__restrict__ femVtx, const int *__restrict__ femIfo,
                            const int *__restrict__ elmVtx, int *__restrict__ tab, int *bad)
{
	int z = blockIdx.x * blockDim.x + threadIdx.x;
	if (z >= Z) return;
	int i = femVtx[z], j = femVtx[Z + z];
	int cnt = femIfo[z];
	for (int k = 0; k < cnt; ++k) {
		int e = femIfo[(2 + 2 * k) * (long) Z + z];
		if (e < 0 || e >= E) { atomicOr(bad, 1); tab[k * (long) Z + z] = 0; continue; }
		int a = -1, b = -1;
		for (int l = 0; l < V; ++l) {
			int n = elmVtx[l * (long) E + e];
			if (n == i) a = l;
			if (n == j) b = l;
		}
		if (a < 0 || b < 0) { atomicOr(bad, 2); a = 0; b = 0; }
		tab[k * (long) Z + z] = e * 16 + a * 4 + b;
	}
}

template <int D>
__global__ void k_init_sign(int E, const int *__restrict__ elmVtx, const double *__restrict__ x,
                            signed char *__restrict__ sg)
{
	int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= E) return;
	Vec<D> q0 = load_node<D>(x, elmVtx[e]);
	Vec<D> q[D];
	for (int k = 0; k < D; ++k) q[k] = vsub(load_node<D>(x, elmVtx[(k + 1) * (long) E + e]), q0);
	double det = det_edges<D>(q);
	sg[e] = det > 0.0 ? 1 : (det < 0.0 ? -1 : 0);
}

static void build_mesh(Mesh &m, const sa_element_object *o, bool needVfd, bool needGrad, bool layered, int lyrNum,
                       Pool &P, PhaseTrace *tr = nullptr)
{
	cudaStream_t s = P.s;
	int D = o->dim;
	SA_REQUIRE(D == 2 || D == 3, "dim must be 2 or 3");
	m.dim = D; m.V = D + 1; m.N = o->lmkNum; m.E = o->elmNum; m.Z = o->nzrNum;
	m.Bt = o->btmElmNum; m.Nb = o->btmLmkNum; m.Vd = needVfd ? o->vfdElmNum : 0;
	SA_REQUIRE(m.N > 0 && m.E > 0 && m.Z >= m.N, "empty mesh or femVtxMat smaller than the node count");
	SA_REQUIRE(o->elmVtxMat && o->vtxElmMat && o->femVtxMat && o->femIfoMat, "missing element-object array");
	// the frame arrays are read by the frame model only (the layered model neither uploads nor checks them)
	SA_REQUIRE(layered || (o->frmVtxMat && o->tsvVtxMat), "frame model needs tanVtxMat/nmlVtxMat and tsvVtxMat");
	const bool haveFrame = !layered && o->frmVtxMat && o->tsvVtxMat;
	SA_REQUIRE(o->vtxElmCols >= 1 && o->femIfoCols >= 2, "adjacency matrices need a count column");
	SA_REQUIRE((long) m.E * 16 < (1L << 31), "too many elements for the 32-bit assembly table");
	m.vtxElmCols = o->vtxElmCols; m.femIfoCols = o->femIfoCols;
	int frmCols = D == 2 ? 4 : 6;
	m.elmVtx = (int *) P.dev(o->elmVtxMat, (size_t) m.E * m.V);
	m.vtxElm = (int *) P.dev(o->vtxElmMat, (size_t) m.N * o->vtxElmCols);
	if (haveFrame) {
		m.frmVtx = (int *) P.dev(o->frmVtxMat, (size_t) m.E * frmCols);
		m.tsvVtx = (int *) P.dev(o->tsvVtxMat, (size_t) m.E * frmCols);
	}
	m.femVtx = (int *) P.dev(o->femVtxMat, (size_t) m.Z * 2);
	m.femIfo = (int *) P.dev(o->femIfoMat, (size_t) m.Z * o->femIfoCols);
	if (m.Bt > 0) {
		SA_REQUIRE(o->btmVtxMat && o->vtxBtmMat && o->vtxBtmCols >= 1 && m.Nb > 0 && m.Nb <= m.N,
		           "bottom arrays inconsistent");
		m.btmVtx = (int *) P.dev(o->btmVtxMat, (size_t) m.Bt * D);
		m.vtxBtm = (int *) P.dev(o->vtxBtmMat, (size_t) m.Nb * o->vtxBtmCols);
		m.vtxBtmCols = o->vtxBtmCols;
	}
	if (needVfd) {
		SA_REQUIRE(o->vfdVtxMat && m.Vd > 0, "objective needs vfdVtxMat");
		m.vfdVtx = (int *) P.dev(o->vfdVtxMat, (size_t) m.Vd * D);
	}
	if (needGrad) {
		SA_REQUIRE(o->vfdIfoMat && o->vfdIfoCols >= 1, "gradient needs vfdIfoMat");
		m.vfdIfo = (int *) P.dev(o->vfdIfoMat, (size_t) m.N * o->vfdIfoCols);
		m.vfdIfoCols = o->vfdIfoCols;
	}
	if (layered) {
		SA_REQUIRE(o->elmLyrVec, "layered model needs elmLyrVec");
		m.elmLyr = (int *) P.dev(o->elmLyrVec, (size_t) m.E);
	}

	if (tr) tr->mark("mesh: upload");
	// host-side validation of every index (one pass over each array, split over host threads); host inputs
	// are read where they are, device inputs are downloaded once
	auto host_ints = [&](const int *orig, const int *dev, size_t n, std::vector<int> &buf) -> const int * {
		if (orig && !is_device_ptr(orig)) return orig;
		buf = to_host(dev, n, s);
		return buf.data();
	};
	auto in_range = [&](const int *v, size_t n, int hi, const char *msg) {
		parallel_chunks((long) n, [&](long lo, long up) {
			for (long k = lo; k < up; ++k) SA_REQUIRE(v[k] >= 0 && v[k] < hi, msg);
		});
	};
	std::vector<int> evBuf, fvBuf, fiBuf, veBuf;
	const int *ev = host_ints(o->elmVtxMat, m.elmVtx, (size_t) m.E * m.V, evBuf);
	in_range(ev, (size_t) m.E * m.V, m.N, "elmVtxMat index out of range");
	const int *fv = host_ints(o->femVtxMat, m.femVtx, (size_t) m.Z * 2, fvBuf);
	parallel_chunks(m.Z, [&](long lo, long up) {
		for (long z = lo; z < up; ++z) {
			int r = fv[z], c = fv[m.Z + z];
			SA_REQUIRE(r >= 0 && r < m.N && c >= 0 && c < m.N, "femVtxMat index out of range");
			if (z > 0) SA_REQUIRE(r > fv[z - 1] || (r == fv[z - 1] && c > fv[m.Z + z - 1]),
			                      "femVtxMat rows must be sorted by (row, col) (generateElementObject sortrows)");
		}
	});
	std::vector<int> rp(m.N + 1, -1);
	parallel_chunks(m.Z, [&](long lo, long up) {        // sorted: each row starts at exactly one slot
		for (long z = lo; z < up; ++z)
			if (z == 0 || fv[z] != fv[z - 1]) rp[fv[z]] = (int) z;
	});
	rp[m.N] = m.Z;
	parallel_chunks(m.N, [&](long lo, long up) {
		for (long i = lo; i < up; ++i) SA_REQUIRE(rp[i] >= 0, "femVtxMat misses a node row");
	});
	const int *fi = host_ints(o->femIfoMat, m.femIfo, (size_t) m.Z * 2, fiBuf);   // count row first
	int maxAdj = 0;
	{
		std::mutex mx;
		parallel_chunks(m.Z, [&](long lo, long up) {
			int mloc = 0;
			for (long z = lo; z < up; ++z) {
				SA_REQUIRE(fi[z] >= 0 && 2 + 2 * fi[z] <= o->femIfoCols, "femIfoMat count exceeds its columns");
				mloc = std::max(mloc, fi[z]);
			}
			std::lock_guard<std::mutex> g(mx);
			maxAdj = std::max(maxAdj, mloc);
		});
	}
	const int *ve = host_ints(o->vtxElmMat, m.vtxElm, (size_t) m.N * o->vtxElmCols, veBuf);
	parallel_chunks(m.N, [&](long lo, long up) {
		for (long i = lo; i < up; ++i) {
			int c = ve[i];
			SA_REQUIRE(c >= 0 && 1 + 2 * c <= o->vtxElmCols, "vtxElmMat count exceeds its columns");
			for (int a = 0; a < c; ++a) {
				int e = ve[(1 + 2 * a) * (long) m.N + i], l = ve[(2 + 2 * a) * (long) m.N + i];
				SA_REQUIRE(e >= 0 && e < m.E && l >= 0 && l < m.V && ev[(long) l * m.E + e] == i,
				           "vtxElmMat entry does not match elmVtxMat");
			}
		}
	});
	if (haveFrame) {
		std::vector<int> b1, b2;
		in_range(host_ints(o->frmVtxMat, m.frmVtx, (size_t) m.E * frmCols, b1), (size_t) m.E * frmCols, m.N,
		         "tan/nmlVtxMat index out of range");
		in_range(host_ints(o->tsvVtxMat, m.tsvVtx, (size_t) m.E * frmCols, b2), (size_t) m.E * frmCols, m.N,
		         "tsvVtxMat index out of range");
	}
	if (m.Bt > 0) {
		std::vector<int> b1, b2;
		const int *bv = host_ints(o->btmVtxMat, m.btmVtx, (size_t) m.Bt * D, b1);
		in_range(bv, (size_t) m.Bt * D, m.N, "btmVtxMat index out of range");
		const int *vb = host_ints(o->vtxBtmMat, m.vtxBtm, (size_t) m.Nb * o->vtxBtmCols, b2);
		parallel_chunks(m.Nb, [&](long lo, long up) {
			for (long i = lo; i < up; ++i) {
				int c = vb[i];
				SA_REQUIRE(c >= 0 && 1 + 2 * c <= o->vtxBtmCols, "vtxBtmMat count exceeds its columns");
				for (int a = 0; a < c; ++a) {
					int f = vb[(1 + 2 * a) * (long) m.Nb + i], l = vb[(2 + 2 * a) * (long) m.Nb + i];
					SA_REQUIRE(f >= 0 && f < m.Bt && l >= 0 && l < D && bv[(long) l * m.Bt + f] == i,
					           "vtxBtmMat entry must name its own node (bottom nodes numbered first)");
				}
			}
		});
	}
	if (needVfd) {
		std::vector<int> b1;
		in_range(host_ints(o->vfdVtxMat, m.vfdVtx, (size_t) m.Vd * D, b1), (size_t) m.Vd * D, m.N,
		         "vfdVtxMat index out of range");
	}
	if (needGrad) {
		std::vector<int> b1;
		const int *gi = host_ints(o->vfdIfoMat, m.vfdIfo, (size_t) m.N * o->vfdIfoCols, b1);
		int w = D == 2 ? 2 : 3;
		parallel_chunks(m.N, [&](long lo, long up) {
			for (long i = lo; i < up; ++i) {
				int c = gi[i];
				SA_REQUIRE(c >= 0 && 1 + w * c <= o->vfdIfoCols, "vfdIfoMat count exceeds its columns");
				for (int a = 0; a < c; ++a) {
					int e = gi[(1 + w * a) * (long) m.N + i];
					SA_REQUIRE(e >= 0 && e < m.Vd, "vfdIfoMat element out of range");
					if (D == 3)
						for (int t = 2; t <= 3; ++t) {
							int q = gi[(t + w * a) * (long) m.N + i];
							SA_REQUIRE(q >= 0 && q < m.N, "vfdIfoMat node out of range");
						}
				}
			}
		});
	}
	if (layered) {
		std::vector<int> b1;
		in_range(host_ints(o->elmLyrVec, m.elmLyr, (size_t) m.E, b1), (size_t) m.E, lyrNum,
		         "elmLyrVec entry outside the layer tables");
	}
	if (tr) tr->mark("mesh: validate");
	m.rowPtr = P.alloc<int>(m.N + 1);
	SA_CHECK(cudaMemcpyAsync(m.rowPtr, rp.data(), sizeof(int) * (m.N + 1), cudaMemcpyHostToDevice, s));
	{   // sliced layout: 32-row slices, slot k of row 32 s + lane at off[s] + 32 k + lane
		int nsl = (m.N + 31) / 32;
		std::vector<int> wid(nsl), off(nsl);
		parallel_chunks(nsl, [&](long lo, long up) {
			for (long sl = lo; sl < up; ++sl) {
				int w = 0;
				for (int i = (int) sl * 32; i < std::min(m.N, (int) sl * 32 + 32); ++i) w = std::max(w, rp[i + 1] - rp[i]);
				wid[sl] = w;
			}
		});
		long total = 0;
		for (int sl = 0; sl < nsl; ++sl) {
			off[sl] = (int) std::min(total, (long) INT32_MAX);
			total += 32L * wid[sl];
		}
		SA_REQUIRE(total < (1L << 31) / 8, "operator too large for 32-bit slot offsets");
		if (tr) tr->mark("mesh: slice widths");
		// every entry of col and dest is written below: no zero fill (the pages are touched by the threads)
		std::unique_ptr<int[]> col(new int[total > 0 ? total : 1]), dest(new int[m.Z]);
		parallel_chunks(nsl, [&](long lo, long up) {
			for (long sl = lo; sl < up; ++sl)
				for (int lane = 0; lane < 32; ++lane) {
					int i = (int) sl * 32 + lane;
					int len = i < m.N ? rp[i + 1] - rp[i] : 0;
					for (int k = 0; k < wid[sl]; ++k) {
						long idx = off[sl] + 32L * k + lane;
						if (k < len) {
							col[idx] = fv[m.Z + rp[i] + k];
							dest[rp[i] + k] = (int) idx;
						} else col[idx] = i < m.N ? i : 0;     // padding: zero block on the row's own node
					}
				}
		});
		if (tr) tr->mark("mesh: slot columns");
		m.nslice = nsl;
		m.slTotal = total;
		m.slWidth = P.alloc<int>(nsl);
		m.slOff = P.alloc<int>(nsl);
		m.slCol = P.alloc<int>(total);
		m.slDest = P.alloc<int>(m.Z);
		// slot of the transposed entry: row j of femVtxMat is sorted by column
		// (checked above), so (j, i) is found by bisection
		std::unique_ptr<int[]> tz(new int[m.Z]);
		parallel_chunks(m.Z, [&](long lo, long up) {
			for (long z = lo; z < up; ++z) {
				int i = fv[z], j = fv[m.Z + z];
				const int *b = fv + m.Z + rp[j], *e = fv + m.Z + rp[j + 1];
				const int *q = std::lower_bound(b, e, i);
				SA_REQUIRE(q != e && *q == i, "femVtxMat pattern is not symmetric");
				tz[z] = rp[j] + (int) (q - b);
				SA_REQUIRE(fi[z] == fi[tz[z]], "femIfoMat lists differ between (i, j) and (j, i)");
			}
		});
		if (tr) tr->mark("mesh: transposes");
		m.transZ = P.alloc<int>(m.Z);
		SA_CHECK(cudaMemcpyAsync(m.transZ, tz.get(), sizeof(int) * m.Z, cudaMemcpyHostToDevice, s));
		// assembly order: the N diagonal slots (many elements each) first, then
		// the strictly upper slots (few elements each), so a warp's threads
		// loop over similar element counts; per host chunk counts, then each chunk writes at its offsets
		const int nch = chunk_count(m.Z);
		std::vector<long> nDiag(nch + 1, 0), nUp(nch + 1, 0);
		parallel_chunks_t(m.Z, [&](int t, long lo, long up) {
			long a = 0, b = 0;
			for (long z = lo; z < up; ++z) {
				a += fv[z] == fv[m.Z + z];
				b += fv[z] < fv[m.Z + z];
			}
			nDiag[t + 1] = a;
			nUp[t + 1] = b;
		});
		for (int t = 0; t < nch; ++t) { nDiag[t + 1] += nDiag[t]; nUp[t + 1] += nUp[t]; }
		std::vector<int> ord((size_t) (nDiag[nch] + nUp[nch]));
		parallel_chunks_t(m.Z, [&](int t, long lo, long up) {
			long a = nDiag[t], b = nDiag[nch] + nUp[t];
			for (long z = lo; z < up; ++z) {
				if (fv[z] == fv[m.Z + z]) ord[a++] = (int) z;
				else if (fv[z] < fv[m.Z + z]) ord[b++] = (int) z;
			}
		});
		if (tr) tr->mark("mesh: assembly order");
		m.nAsm = (int) ord.size();
		m.asmOrder = P.alloc<int>(ord.size());
		SA_CHECK(cudaMemcpyAsync(m.asmOrder, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice, s));
		SA_CHECK(cudaMemcpyAsync(m.slWidth, wid.data(), sizeof(int) * nsl, cudaMemcpyHostToDevice, s));
		SA_CHECK(cudaMemcpyAsync(m.slOff, off.data(), sizeof(int) * nsl, cudaMemcpyHostToDevice, s));
		m.slOffHost = off;
		m.slOffHost.push_back((int) total);
		SA_CHECK(cudaMemcpyAsync(m.slCol, col.get(), sizeof(int) * total, cudaMemcpyHostToDevice, s));
		SA_CHECK(cudaMemcpyAsync(m.slDest, dest.get(), sizeof(int) * m.Z, cudaMemcpyHostToDevice, s));
		SA_CHECK(cudaStreamSynchronize(s));      // host vectors go out of scope
	}
	if (tr) tr->mark("mesh: layout upload");
	m.asmCols = maxAdj;
	m.asmTab = P.alloc<int>((size_t) std::max(1, maxAdj) * m.Z);
	int *bad = P.zeros<int>(1);
	if (tr) tr->mark("mesh: assembly table memory");
	k_asm_table<<<grid_for(m.Z), kBlock, 0, s>>>(m.Z, m.E, m.V, m.femVtx, m.femIfo, m.elmVtx, m.asmTab, bad);
	int hbad = 0;
	SA_CHECK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
	SA_CHECK(cudaStreamSynchronize(s));
	SA_REQUIRE(hbad == 0, "femIfoMat lists an element that does not contain both nodes of the slot");
	m.sign0 = P.alloc<signed char>(m.E);
	if (tr) tr->mark("mesh: assembly table");
}

// ---------------------------------------------------------------------------
// one forward solve
// ---------------------------------------------------------------------------
struct Work {
	double *xa, *xb;            // node positions t, t+1 (interleaved)
	double *v, *b, *pd, *blk, *dinv, *fy, *fr;
	double *vHist = nullptr;    // velocities of earlier steps (extrapolated CG start), velocityGuess x n
	double *Mnow, *Mnxt, *L, *dinvRd, *rhs;
	float *L32 = nullptr, *rdInv32 = nullptr;   // mixed precision: FP32 copy of L and of its inverse diagonal
	Geom g0, g1;
	CgWork cw;
	KpcgWork kw;
	double *K = nullptr;
	double *trajX = nullptr, *trajT = nullptr;   // device trajectory (SoA per step), tau
};

template <int D>
static void alloc_work(Work &w, const Mesh &m, const Model &md, bool wantTraj, Pool &P)
{
	long N = m.N, E = m.E, Z = m.Z, n = N * D;
	w.xa = P.alloc<double>(n); w.xb = P.alloc<double>(n);
	w.v = P.alloc<double>(n); w.b = P.alloc<double>(n); w.pd = P.zeros<double>(N);
	if (md.velocityGuess > 0) w.vHist = P.zeros<double>((size_t) md.velocityGuess * n);
	long T = m.slTotal;                    // sliced slots, padding included (padding stays zero)
	w.blk = P.zeros<double>((size_t) T * sell_vals<D>()); w.dinv = P.alloc<double>(n);
	w.fy = P.alloc<double>(N); w.fr = P.alloc<double>(N);
	w.Mnow = P.alloc<double>(Z); w.Mnxt = P.alloc<double>(Z); w.L = P.zeros<double>(T);
	w.dinvRd = P.alloc<double>(N); w.rhs = P.alloc<double>(N);
	for (Geom *g : {&w.g0, &w.g1}) {
		g->rec = P.alloc<double>((size_t) rec_len<D>() * E);
		if (md.frame) { g->frm = P.alloc<double>((size_t) D * E); g->tsv = P.alloc<double>((size_t) D * E); }
	}
	int nb = grid_for(N, 256);
	CgWork &c = w.cw;
	c.r = P.alloc<double>(n); c.u = P.alloc<double>(n); c.w = P.alloc<double>(n);
	c.p = P.alloc<double>(n); c.sv = P.alloc<double>(n);
	// partial sums: up to 3 per CTA of the widest CG kernel grid (entries / 256, or one CTA per slice)
	int nbCg = std::max(grid_for(n, 256), std::max(m.nslice, nb));
	c.part = P.alloc<double>((size_t) 3 * nbCg + 64); c.scal = P.zeros<double>(32); c.maxBlocks = nbCg;
	c.bar = P.zeros<char>(kGridBarBytes);
	c.u4 = P.alloc<double>((size_t) 4 * N);
	c.ctaTabCap = 2L * (m.nslice + 64);
	c.ctaTab = P.alloc<int>((size_t) c.ctaTabCap);
	c.cgKernel = md.cgKernel;
	{
		int dev = 0;
		SA_CHECK(cudaGetDevice(&dev));
		SA_CHECK(cudaDeviceGetAttribute(&c.smCount, cudaDevAttrMultiProcessorCount, dev));
	}
	c.xr = P.alloc<double>((size_t) 3 * n);
	bool useK = md.frame || md.ldmWgt != 0.0;
	// the velocity solves' block-Jacobi inverses: FP64 for FP64 Jacobi-PCG, FP32 for the mixed inner solves
	if (md.precision == SA_PREC_FP64 && !useK) c.binv64 = P.alloc<double>((size_t) N * D * D);
	if (md.precision == SA_PREC_MIXED) {
		c.blk32 = P.alloc<float>((size_t) T * sell_vals<D>());
		c.binv32 = P.alloc<float>((size_t) N * D * D);
		c.f32 = P.alloc<float>((size_t) 7 * n);
		if (!md.frame) { w.L32 = P.zeros<float>(T); w.rdInv32 = P.alloc<float>(N); }
	}
	if (useK) {
		KpcgWork &k = w.kw;
		k.Ad = P.alloc<double>(n); k.Kid = P.alloc<double>(n); k.r = P.alloc<double>(n);
		k.Kr = P.alloc<double>(n); k.dv = P.alloc<double>(n); k.wK = P.zeros<double>(n);
		k.partLen = (long) 4 * nb + 16 * n + 64;
		k.part = P.alloc<double>((size_t) k.partLen); k.scal = P.zeros<double>(32);
		k.maxBlocks = nb;
		k.dv2 = P.alloc<double>(n); k.bar = P.zeros<char>(kGridBarBytes);
		if (!md.kernelFree) w.K = P.alloc<double>((size_t) N * N);
	}
	if (wantTraj) {
		w.trajX = P.zeros<double>((size_t) n * md.timeNum);
	}
	w.trajT = P.zeros<double>((size_t) N * md.timeNum);
}

__global__ void k_to_f32(long n, const double *a, float *b)
{
	long k = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (k < n) b[k] = (float) a[k];
}

struct SolveOut { int status; int cgTotal, rdTotal, cgMax; int inverted; };

// time stepper of one parameter column: start() sets up t = 0, step(n)
// advances up to n steps, finish() leaves the final positions in w.xa
template <int D>
struct Stepper {
	const Mesh &m;
	const Model &md;
	Work &w;
	cudaStream_t s;
	Status *st = nullptr;
	Geom *gn = nullptr, *gx = nullptr;
	double *xn = nullptr, *xx = nullptr;
	int t = 0;
	bool useK = false;
	SolveOut out{SA_OK, 0, 0, 0, 0};

	Stepper(const Mesh &m_, const Model &md_, Work &w_, cudaStream_t s_) : m(m_), md(md_), w(w_), s(s_) {}

	void start(const double *x0soa, const double *tauVar)
	{
		int N = m.N;
		long n = (long) N * D;
		useK = md.frame || md.ldmWgt != 0.0;
		out = SolveOut{SA_OK, 0, 0, 0, 0};
		t = 0;
		st = reinterpret_cast<Status *>(w.cw.scal + 24);   // inverted-element counter
		SA_CHECK(cudaMemsetAsync(st, 0, sizeof(Status), s));
		launch_soa_to_aos(N, D, x0soa, w.xa, s);
		if (w.trajX) SA_CHECK(cudaMemcpyAsync(w.trajX, x0soa, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
		launch_tau_initial<D>(m, md, tauVar, w.xa, w.trajT, s);
		launch_elem_geom<D>(m, md, w.xa, w.g0, st, false, s);
		launch_assemble_rd<D>(m, md, w.g0, md.timeStp, w.Mnow, w.L, w.dinvRd, s);
		SA_CHECK(cudaMemsetAsync(w.v, 0, sizeof(double) * n, s));
		if (useK) SA_CHECK(cudaMemsetAsync(w.kw.wK, 0, sizeof(double) * n, s));
		gn = &w.g0; gx = &w.g1;
		xn = w.xa; xx = w.xb;
	}

	double *tau_now() const { return w.trajT + (long) t * m.N; }
	double *tau_next() const { return w.trajT + (long) (t + 1) * m.N; }

	// step part 1: loads and the velocity operator at the current shape
	void pre_velocity()
	{
		// CG start: the previous velocity (the reference's choice), or (layered model, velocityGuess
		// SA_GUESS_EXTRAPOLATE) its linear extrapolation 2 v_t-1 - v_t-2 from the third step on: the same
		// converged answer to the CG tolerance, about a third fewer iterations when the motion is smooth
		if (md.velocityGuess > 0 && !useK) launch_extrap_poly(m.N * (long) D, md.velocityGuess, t, w.v, w.vHist, s);
		launch_activity<D>(m, md, tau_now(), w.fy, w.fr, s);
		if (m.Bt > 0 && md.btmWgt != 0.0) launch_penalty_diag<D>(m, md, xn, w.pd, s);
		launch_assemble_elastic<D>(m, md, *gn, w.pd, w.blk, w.dinv, w.cw.binv64, w.cw.binv32, s);
		launch_yank_rhs<D>(m, *gn, w.fy, w.b, s);
		if (useK) {
			if (!md.kernelFree) launch_kernel_matrix<D>(md, m.N, xn, w.K, s);
		} else if (md.precision == SA_PREC_MIXED)
			k_to_f32<<<grid_for(m.slTotal * sell_vals<D>()), kBlock, 0, s>>>(m.slTotal * sell_vals<D>(), w.blk,
			                                                                  w.cw.blk32);
		// activity, (penalty), elastic assembly, yank, (kernel matrix or FP32 copy)
		w.cw.launches += 3 + (m.Bt > 0 && md.btmWgt != 0.0) + ((useK && !md.kernelFree) || md.precision == SA_PREC_MIXED);
	}

	// step part 2 (after the velocity solve): new shape, reaction-diffusion operator and right-hand side
	void post_velocity()
	{
		long n = (long) m.N * D;
		double dt = md.timeStp;
		launch_advance<D>(m.N, xn, w.v, dt, xx, w.trajX ? w.trajX + (long) (t + 1) * n : nullptr, s);
		launch_elem_geom<D>(m, md, xx, *gx, st, true, s);
		launch_assemble_rd<D>(m, md, *gx, dt, w.Mnxt, w.L, w.dinvRd, s);
		launch_rd_rhs<D>(m, *gn, w.Mnow, tau_now(), w.fr, dt, w.rhs, s);
		// reaction-diffusion CG start: tau_t, or its linear extrapolation 2 tau_t - tau_t-1 when the velocity
		// starts are extrapolated (layered model; the trajectory holds tau_t-1)
		if (md.velocityGuess != SA_GUESS_PREVIOUS && !md.frame && t >= 1)
			launch_lin_extrap(m.N, tau_now(), tau_now() - m.N, tau_next(), s);
		else
			SA_CHECK(cudaMemcpyAsync(tau_next(), tau_now(), sizeof(double) * m.N, cudaMemcpyDeviceToDevice, s));
		w.cw.launches += 4;                 // advance, geometry, rd assembly, rd rhs
	}

	// step part 3 (after the reaction-diffusion solve)
	void end_step()
	{
		std::swap(gn, gx);
		std::swap(xn, xx);
		std::swap(w.Mnow, w.Mnxt);
		++t;
	}

	// Mixed precision (layered model): the reaction-diffusion solve as the velocity solve, FP32 operator and
	// FP32 inner CG with FP64 dot products inside FP64 iterative refinement whose residual b - L tau uses the
	// FP64 operator.  The FP32 copies of L and of its inverse diagonal (the 1 x 1 block inverses of the inner
	// solve) replace the velocity's FP32 operator in the CG work for this solve only.
	int rd_mixed(int *rits)
	{
		k_to_f32<<<grid_for(m.slTotal), kBlock, 0, s>>>(m.slTotal, w.L, w.L32);
		k_to_f32<<<grid_for(m.N), kBlock, 0, s>>>(m.N, w.dinvRd, w.rdInv32);
		w.cw.launches += 2;
		float *blk32 = w.cw.blk32, *binv32 = w.cw.binv32;
		w.cw.blk32 = w.L32;
		w.cw.binv32 = w.rdInv32;
		int code;
		try {
			code = cg_jacobi<1>(m, w.L, w.dinvRd, w.rhs, tau_next(), md.rdItrMax, md.rdTolSqu, w.cw, st, rits, s,
			                    SA_PREC_MIXED);
		} catch (...) {
			w.cw.blk32 = blk32;
			w.cw.binv32 = binv32;
			throw;
		}
		w.cw.blk32 = blk32;
		w.cw.binv32 = binv32;
		return code;
	}

	// returns the number of steps taken; stops early at timeNum - 1 or on a failed solve
	int step(int nsteps)
	{
		int T = md.timeNum, done = 0;
		while (done < nsteps && t < T - 1 && out.status == SA_OK) {
			pre_velocity();
			int its = 0, code;
			if (useK) {
				code = kpcg<D>(m, md, w.blk, w.K, xn, w.b, w.v, w.kw, st, &its, s);
			} else {
				w.cw.profileOn = 1;
				code = cg_jacobi<D>(m, w.blk, w.dinv, w.b, w.v, md.cgItrMax, md.cgTolSqu, w.cw, st, &its, s,
				                    md.precision);
				w.cw.profileOn = 0;
			}
			out.cgTotal += its;
			out.cgMax = std::max(out.cgMax, its);
			if (code != SA_OK) { out.status = code; break; }
			post_velocity();
			int rits = 0;
			code = w.L32 ? rd_mixed(&rits)
			             : cg_jacobi<1>(m, w.L, w.dinvRd, w.rhs, tau_next(), md.rdItrMax, md.rdTolSqu, w.cw, st,
			                            &rits, s, SA_PREC_FP64);
			out.rdTotal += rits;
			if (code != SA_OK) { out.status = code; break; }
			end_step();
			++done;
		}
		return done;
	}

	void finish()
	{
		Status hs;
		SA_CHECK(cudaMemcpyAsync(&hs, st, sizeof(Status), cudaMemcpyDeviceToHost, s));
		SA_CHECK(cudaStreamSynchronize(s));
		out.inverted = hs.inverted;
		long n = (long) m.N * D;
		if (xn != w.xa) {   // the objective reads the final positions from w.xa
			SA_CHECK(cudaMemcpyAsync(w.xa, xn, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
			xx = w.xb;
			xn = w.xa;
		}
	}
};

template <int D>
static SolveOut forward_one(const Mesh &m, const Model &md, Work &w, const double *x0soa, const double *tauVar,
                            cudaStream_t s)
{
	Stepper<D> st(m, md, w, s);
	st.start(x0soa, tauVar);
	st.step(md.timeNum);
	st.finish();
	return st.out;
}

static void fill_model(Model &md, int dim, const sa_params *p, const sa_target *tgt, Pool &P)
{
	memset(&md, 0, sizeof(md));
	md.dim = dim;
	SA_REQUIRE(p->elaType == SA_ELA_FRAME || p->elaType == SA_ELA_ISOTROPIC, "unknown elaType");
	md.frame = p->elaType == SA_ELA_FRAME;
	md.precision = p->precision;
	SA_REQUIRE(md.precision == SA_PREC_FP64 || md.precision == SA_PREC_MIXED, "unknown precision");
	SA_REQUIRE(!(md.frame && md.precision == SA_PREC_MIXED), "mixed precision is available for the layered model");
	SA_REQUIRE(p->modVec && p->ynkActPrmVec && p->reaActPrmVec, "missing parameter vectors");
	std::vector<double> mod = to_host(p->modVec, (size_t) p->modNum, P.s);
	std::vector<double> ynk = to_host(p->ynkActPrmVec, md.frame ? 4 : 1, P.s);
	std::vector<double> rea = to_host(p->reaActPrmVec, md.frame ? 5 : 1, P.s);
	for (size_t k = 0; k < ynk.size(); ++k) md.ynk[k] = ynk[k];
	for (size_t k = 0; k < rea.size(); ++k) md.rea[k] = rea[k];
	if (p->tauPrmVec && p->tauPrmNum > 0) {
		std::vector<double> tp = to_host(p->tauPrmVec, (size_t) std::min(p->tauPrmNum, 2), P.s);
		for (size_t k = 0; k < tp.size(); ++k) md.tauPrm[k] = tp[k];
	}
	if (md.frame) {
		SA_REQUIRE(p->modNum >= (dim == 2 ? 3 : 4), "frame modVec needs 3 (2D) / 4 (3D) values");
		for (int k = 0; k < (dim == 2 ? 3 : 4); ++k) md.mod[k] = mod[k];
		SA_REQUIRE(p->tauPrmNum >= (dim == 2 ? 1 : 2), "tauPrmVec too short");
	} else {
		SA_REQUIRE(p->lyrNum > 0 && p->modNum == 2 * p->lyrNum && p->spdLyrVec, "layer tables inconsistent");
		md.lyrNum = p->lyrNum;
		md.lyrMod = P.dev(p->modVec, (size_t) p->modNum);
		md.lyrSpd = P.dev(p->spdLyrVec, (size_t) p->lyrNum);
	}
	md.spdTan = p->spdTanVal; md.spdTsv = p->spdTsvVal;
	md.ldmWgt = p->ldmWgt; md.knlOrder = p->knlOrder; md.knlWidth = p->knlWidth; md.knlEps = p->knlEps;
	SA_REQUIRE(md.knlOrder >= -1 && md.knlOrder <= 4, "knlOrder must be -1..4");
	md.btmWgt = p->btmWgt; md.timeStp = p->timeStp; md.timeNum = p->timeNum;
	md.cgItrMax = p->cgItrMax; md.cgTolSqu = p->cgTolSqu;
	SA_REQUIRE(md.timeNum >= 1, "timeNum must be >= 1");
	md.rdItrMax = p->rdItrMax > 0 ? p->rdItrMax : std::max(p->cgItrMax, 1000);
	md.rdTolSqu = p->rdTolSqu > 0.0 ? p->rdTolSqu : (md.frame ? 1e-26 : p->cgTolSqu);
	SA_REQUIRE(p->cgKernel >= SA_CG_AUTO && p->cgKernel <= SA_CG_PERSISTENT_GLOBAL, "cgKernel must be 0, 1, 2 or 3");
	md.cgKernel = p->cgKernel;
	SA_REQUIRE(p->velocityGuess >= 0 && p->velocityGuess <= SA_GUESS_MAX_ORDER,
	           "velocityGuess must be a polynomial order 0 .. 5");
	md.velocityGuess = md.frame ? SA_GUESS_PREVIOUS : p->velocityGuess;
	if (tgt) {
		md.cenKnl = tgt->cenKnlType; md.dirKnl = tgt->dirKnlType;
		md.cenWidth = tgt->cenKnlWidth; md.dirWidth = tgt->dirKnlWidth;
		SA_REQUIRE(md.cenKnl == 'G' || md.cenKnl == 'C' || md.cenKnl == 'M', "cenKnlType must be G, C or M");
		SA_REQUIRE(md.dirKnl == 'B' || md.dirKnl == 'L' || md.dirKnl == 'O' || md.dirKnl == 'U',
		           "dirKnlType must be B, L, O or U");
		SA_REQUIRE(kernel_widths_ok(md.cenWidth, md.dirKnl, md.dirWidth),
		           "cenKnlWidth (and dirKnlWidth for 'O'/'U') must be finite and > 0");
	}
}

static const size_t kDenseCapBytes = (size_t) 96 << 30;   // stored RKHS matrix cap: N <= 113 511

// The RKHS term's N x N kernel matrix (frame model, or ldmWgt != 0) is stored when it fits: up to 96 GiB of
// the 288 GB part and three quarters of the device memory free now.  A K x product then streams 8 bytes per
// entry.  Beyond that (or with the kernelMatrixFree tuning switch) the products evaluate each entry from the
// node positions instead, with the same instructions in the same order, so the choice changes the speed and
// never the bits.  The evaluation costs a square root and an exponential (2D Matern: Bessel rational
// approximations too) per entry, ~15x the stored matrix's product time on this part.
static void choose_kernel_storage(Model &md, int N)
{
	md.kernelFree = 0;
	if (!md.frame && md.ldmWgt == 0.0) return;
	size_t freeBytes = 0, totalBytes = 0;
	SA_CHECK(cudaMemGetInfo(&freeBytes, &totalBytes));
	const size_t need = (size_t) N * N * sizeof(double);
	md.kernelFree = tuning().kernelMatrixFree != 0 || need > kDenseCapBytes || need > freeBytes / 4 * 3;
}

template <int D>
static int forward_impl(sa_context *ctx, const sa_element_object *obj, const double *lmkIni, const sa_params *prm,
                        const sa_target *tgt, const double *tauVarMat, int tauVarNum, int objNum, double *lmkStk,
                        double *tauMat, double *objVec, sa_solve_info *info)
{
	cudaStream_t s = ctx->stream;
	PhaseTrace tr(s);
	Pool P(s, true);                          // stream-ordered: the host's set-up overlaps the side stream
	SideJoin join{ctx->side};                 // before P's destructor frees what the side stream reads
	Mesh m;
	Model md;
	fill_model(md, D, prm, tgt, P);
	tr.mark("model");
	const double *tc = nullptr, *tu = nullptr, *tvl = nullptr;
	VfdTargetCache vcache;                    // target-target varifold rows, shared by the columns
	if (tgt) {
		SA_REQUIRE(tgt->tgtElmNum > 0 && tgt->cenPosMat && tgt->uniDirMat && tgt->elmVolVec, "empty target");
		SA_REQUIRE(obj && obj->vfdElmNum >= 0, "vfdElmNum");
		const int Vt = tgt->tgtElmNum, Vd = obj->vfdElmNum;
		tc = P.dev(tgt->cenPosMat, (size_t) Vt * D);
		tu = P.dev(tgt->uniDirMat, (size_t) Vt * D);
		tvl = P.dev(tgt->elmVolVec, (size_t) Vt);
		vcache.rows = P.alloc<double>((size_t) Vt);
		vcache.capacity = Vt;
		if (Vd >= Vt) {
			// the objective's target-target rows depend on the target only: the side stream computes them
			// while the host validates and lays out the mesh (the objective finds them in the cache)
			double *part = P.alloc<double>(varifold_target_rows_scratch(D, Vd, Vt, md.precision));
			SA_CHECK(cudaEventRecord(ctx->sideIn, s));
			SA_CHECK(cudaStreamWaitEvent(ctx->side, ctx->sideIn, 0));
			join.on = true;
			varifold_target_rows<D>(md, Vd, tc, tu, tvl, Vt, md.precision, part, vcache, ctx->side);
			SA_CHECK(cudaEventRecord(ctx->sideOut, ctx->side));
		}
	}
	build_mesh(m, obj, tgt != nullptr, false, !md.frame, md.lyrNum, P, &tr);
	choose_kernel_storage(md, m.N);
	SA_REQUIRE(tauVarMat && tauVarNum >= (md.frame ? (D == 2 ? 4 : 4) : D + 2) && objNum >= 1,
	           "tauVarMat too small");
	const double *x0 = P.dev(lmkIni, (size_t) m.N * D);
	std::vector<double> tv = to_host(tauVarMat, (size_t) tauVarNum * objNum, s);
	Work w;
	alloc_work<D>(w, m, md, lmkStk != nullptr, P);
	{   // initial element orientation for the Jacobian sign check
		double *xa = P.alloc<double>((size_t) m.N * D);
		launch_soa_to_aos(m.N, D, x0, xa, s);
		k_init_sign<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, xa, m.sign0);
	}
	std::vector<double> objs(objNum, 0.0);
	SolveOut last{};
	tr.mark("inputs, work buffers");
	if (join.on) SA_CHECK(cudaStreamWaitEvent(s, ctx->sideOut, 0));
	SA_CHECK(cudaEventRecord(ctx->e0, s));
	for (int k = 0; k < objNum; ++k) {
		const double *tvk = tv.data() + (size_t) k * tauVarNum;
		SolveOut o = forward_one<D>(m, md, w, x0, tvk, s);
		last = o;
		if (o.status == SA_ERR_NOT_CONVERGED || o.status == SA_ERR_BREAKDOWN || o.status == SA_ERR_NONFINITE) {
			objs[k] = DBL_MAX;            // 2D_frame/deform.cu:68-73
			continue;
		}
		if (tgt) {
			int err = SA_OK;
			// the interleaved final positions sit in w.xa after forward_one
			objs[k] = varifold<D>(m, md, w.xa, tc, tu, tvl, tgt->tgtElmNum, nullptr, s, md.precision, &err,
			                      &vcache);
			SA_REQUIRE(err == SA_OK, "varifold arguments");
		}
	}
	SA_CHECK(cudaEventRecord(ctx->e1, s));
	SA_CHECK(cudaEventSynchronize(ctx->e1));
	float ms = 0.f;
	cudaEventElapsedTime(&ms, ctx->e0, ctx->e1);
	tr.mark("solve, objective");
	long n = (long) m.N * D;
	if (lmkStk) SA_CHECK(cudaMemcpyAsync(lmkStk, w.trajX, sizeof(double) * n * md.timeNum, cudaMemcpyDefault, s));
	if (tauMat) SA_CHECK(cudaMemcpyAsync(tauMat, w.trajT, sizeof(double) * m.N * md.timeNum, cudaMemcpyDefault, s));
	if (objVec) SA_CHECK(cudaMemcpyAsync(objVec, objs.data(), sizeof(double) * objNum, cudaMemcpyDefault, s));
	SA_CHECK(cudaStreamSynchronize(s));
	tr.mark("download");
	if (info) {
		info->status = last.status;
		info->cgIterTotal = last.cgTotal;
		info->rdIterTotal = last.rdTotal;
		info->cgIterMax = last.cgMax;
		info->invertedElements = last.inverted;
		info->elapsedMs = ms;
	}
	if (tr.on) {
		P.release();
		tr.mark("free");
	}
	return SA_OK;
}

template <int D>
static int varifold_impl(sa_context *ctx, const sa_element_object *obj, const double *lmk, const sa_target *tgt,
                         int precision, double *objOut, double *grad)
{
	cudaStream_t s = ctx->stream;
	Pool P(s);
	Mesh m;
	Model md;
	memset(&md, 0, sizeof(md));
	md.dim = D;
	SA_REQUIRE(tgt && tgt->tgtElmNum > 0, "missing target");
	md.cenKnl = tgt->cenKnlType; md.dirKnl = tgt->dirKnlType;
	md.cenWidth = tgt->cenKnlWidth; md.dirWidth = tgt->dirKnlWidth;
	SA_REQUIRE(md.cenKnl == 'G' || md.cenKnl == 'C' || md.cenKnl == 'M', "cenKnlType must be G, C or M");
	SA_REQUIRE(md.dirKnl == 'B' || md.dirKnl == 'L' || md.dirKnl == 'O' || md.dirKnl == 'U',
	           "dirKnlType must be B, L, O or U");
	SA_REQUIRE(kernel_widths_ok(md.cenWidth, md.dirKnl, md.dirWidth),
	           "cenKnlWidth (and dirKnlWidth for 'O'/'U') must be finite and > 0");
	build_mesh(m, obj, true, grad != nullptr, false, 0, P);
	const double *x = P.dev(lmk, (size_t) m.N * D);
	double *xa = P.alloc<double>((size_t) m.N * D);
	launch_soa_to_aos(m.N, D, x, xa, s);
	const double *tc = P.dev(tgt->cenPosMat, (size_t) tgt->tgtElmNum * D);
	const double *tu = P.dev(tgt->uniDirMat, (size_t) tgt->tgtElmNum * D);
	const double *tvl = P.dev(tgt->elmVolVec, (size_t) tgt->tgtElmNum);
	double *ga = grad ? P.alloc<double>((size_t) m.N * D) : nullptr;
	int err = SA_OK;
	double v = varifold<D>(m, md, xa, tc, tu, tvl, tgt->tgtElmNum, ga, s, precision, &err);
	SA_REQUIRE(err == SA_OK, "varifold gradient needs vfdIfoMat");
	*objOut = v;
	if (grad) {
		// back to the reference's column-major N x D layout
		std::vector<double> h = to_host(ga, (size_t) m.N * D, s), o((size_t) m.N * D);
		for (int i = 0; i < m.N; ++i)
			for (int d = 0; d < D; ++d) o[(size_t) d * m.N + i] = h[(size_t) i * D + d];
		SA_CHECK(cudaMemcpyAsync(grad, o.data(), sizeof(double) * o.size(), cudaMemcpyDefault, s));
		SA_CHECK(cudaStreamSynchronize(s));
	}
	return SA_OK;
}

// ---------------------------------------------------------------------------
// objective gradient with respect to the bump parameters [c, h, sigma]
// (layered model): the forward steps with the tangent-linear model of every
// step carried along for each of the dim + 2 parameters (sa_tangent.cu), then
// dJ/dp_k = grad_x J(x_T) . dx_T,k.  One extra velocity and one extra
// reaction-diffusion solve per parameter and step, on the operators the
// forward step assembled; no trajectory is stored.
// ---------------------------------------------------------------------------
template <int D>
static int gradient_impl(sa_context *ctx, const sa_element_object *obj, const double *lmkIni, const sa_params *prm,
                         const sa_target *tgt, const double *tauVar, int tauVarNum, double *objOut, double *gradOut,
                         sa_solve_info *info)
{
	cudaStream_t s = ctx->stream;
	PhaseTrace tr(s);
	Pool P(s);
	Mesh m;
	Model md;
	fill_model(md, D, prm, tgt, P);
	SA_REQUIRE(!md.frame && md.ldmWgt == 0.0, "gradients: layered model (elaType isotropic, ldmWgt 0) only");
	SA_REQUIRE(tgt && tgt->tgtElmNum > 0 && tgt->cenPosMat && tgt->uniDirMat && tgt->elmVolVec, "gradients need a target");
	const int K = D + 2;
	SA_REQUIRE(tauVar && tauVarNum >= K, "tauVarVec needs [c (dim), h, sigma]");
	build_mesh(m, obj, true, true, true, md.lyrNum, P, &tr);
	const double *x0 = P.dev(lmkIni, (size_t) m.N * D);
	std::vector<double> tv = to_host(tauVar, (size_t) tauVarNum, s);
	const double *tc = P.dev(tgt->cenPosMat, (size_t) tgt->tgtElmNum * D);
	const double *tu = P.dev(tgt->uniDirMat, (size_t) tgt->tgtElmNum * D);
	const double *tvl = P.dev(tgt->elmVolVec, (size_t) tgt->tgtElmNum);
	Work w;
	alloc_work<D>(w, m, md, false, P);
	{
		double *xa = P.alloc<double>((size_t) m.N * D);
		launch_soa_to_aos(m.N, D, x0, xa, s);
		k_init_sign<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, xa, m.sign0);
	}
	const long n = (long) m.N * D, N = m.N;
	// tangent state per parameter: positions (two copies: t, t+1), concentration (t, t+1), velocity
	std::vector<double *> dx[2], dtau[2], dv, dvHist;
	for (int k = 0; k < K; ++k) {
		for (int c = 0; c < 2; ++c) { dx[c].push_back(P.zeros<double>(n)); dtau[c].push_back(P.zeros<double>(N)); }
		dv.push_back(P.zeros<double>(n));
		dvHist.push_back(md.velocityGuess > 0 ? P.zeros<double>((size_t) md.velocityGuess * n) : nullptr);
	}
	double *drecA = P.alloc<double>((size_t) rec_len<D>() * m.E), *drecB = P.alloc<double>((size_t) rec_len<D>() * m.E);
	double *rhsV = P.alloc<double>(n), *rhsT = P.alloc<double>(N), *dpd = P.zeros<double>(N), *dfy = P.alloc<double>(N);
	double *gx = P.alloc<double>(n);
	Stepper<D> st(m, md, w, s);
	st.start(x0, tv.data());
	for (int k = 0; k < K; ++k) launch_tau0_tan<D>(m, st.xn, st.tau_now(), tv.data(), k, dtau[0][k], s);
	tr.mark("inputs, work buffers");
	SA_CHECK(cudaEventRecord(ctx->e0, s));
	int cur = 0, status = SA_OK, tanIts = 0;
	const int T = md.timeNum;
	const double dt = md.timeStp, y0 = md.ynk[0];
	// velocity solves in the model's precision (mixed: FP32 inner CG with FP64 refinement, as the forward
	// step); reaction-diffusion solves in FP64, as the forward step
	auto solve = [&](auto B_, const double *A, const double *dinvA, const double *rhs, double *xs, int itrMax,
	                 double tolSqu) {
		constexpr int B = decltype(B_)::value;
		int its = 0;
		int code = cg_jacobi<B>(m, A, dinvA, rhs, xs, itrMax, tolSqu, w.cw, st.st, &its, s,
		                        B == D ? md.precision : SA_PREC_FP64);
		tanIts += its;
		return code;
	};
	while (st.t < T - 1 && status == SA_OK) {
		st.pre_velocity();
		int its = 0;
		int code = cg_jacobi<D>(m, w.blk, w.dinv, w.b, w.v, md.cgItrMax, md.cgTolSqu, w.cw, st.st, &its, s,
		                        md.precision);
		st.out.cgTotal += its;
		st.out.cgMax = std::max(st.out.cgMax, its);
		if (code != SA_OK) { status = code; break; }
		// velocity tangents: K dv = db - dK v - btmWgt dpd v at x_t
		for (int k = 0; k < K && status == SA_OK; ++k) {
			launch_geom_tan<D>(m, st.gn->rec, dx[cur][k], drecA, s);
			if (m.Bt > 0 && md.btmWgt != 0.0) launch_penalty_tan<D>(m, st.xn, dx[cur][k], dpd, s);
			launch_axpy64(N, dtau[cur][k], y0 - 1.0, dtau[cur][k], dfy, s);     // dfy = y0 dtau
			launch_vel_tan_rhs<D>(m, md, st.gn->rec, drecA, w.fy, dfy, w.v, dpd, rhsV, s);
			// start as the forward solve does: previous tangent velocity, or its extrapolation
			if (md.velocityGuess > 0) launch_extrap_poly(n, md.velocityGuess, st.t, dv[k], dvHist[k], s);
			code = solve(std::integral_constant<int, D>(), w.blk, w.dinv, rhsV, dv[k], md.cgItrMax, md.cgTolSqu);
			if (code != SA_OK) { status = code; break; }
			launch_axpy64(n, dx[cur][k], dt, dv[k], dx[1 - cur][k], s);
		}
		if (status != SA_OK) break;
		st.post_velocity();
		int rits = 0;
		code = cg_jacobi<1>(m, w.L, w.dinvRd, w.rhs, st.tau_next(), md.rdItrMax, md.rdTolSqu, w.cw, st.st, &rits, s,
		                    SA_PREC_FP64);
		st.out.rdTotal += rits;
		if (code != SA_OK) { status = code; break; }
		// concentration tangents: L dtau' = dM_t (tau + dt R) + M_t (dtau + dt R' dtau) - (dM' + dt dG') tau'
		for (int k = 0; k < K && status == SA_OK; ++k) {
			launch_geom_tan<D>(m, st.gn->rec, dx[cur][k], drecA, s);
			launch_geom_tan<D>(m, st.gx->rec, dx[1 - cur][k], drecB, s);
			launch_rd_tan_rhs<D>(m, md, w.Mnow, st.gn->rec, drecA, st.gx->rec, drecB, st.tau_now(), w.fr,
			                     dtau[cur][k], st.tau_next(), rhsT, s);
			// start as the forward concentration solve does (dtau[1 - cur] still holds the step before)
			if (md.velocityGuess != SA_GUESS_PREVIOUS && st.t >= 1)
				launch_lin_extrap(N, dtau[cur][k], dtau[1 - cur][k], dtau[1 - cur][k], s);
			else
				SA_CHECK(cudaMemcpyAsync(dtau[1 - cur][k], dtau[cur][k], sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
			code = solve(std::integral_constant<int, 1>(), w.L, w.dinvRd, rhsT, dtau[1 - cur][k], md.rdItrMax,
			             md.rdTolSqu);
			if (code != SA_OK) { status = code; break; }
		}
		if (status != SA_OK) break;
		st.end_step();
		cur = 1 - cur;
	}
	st.finish();
	double J = DBL_MAX;
	std::vector<double> grad((size_t) K, std::nan(""));
	if (status == SA_OK) {
		int err = SA_OK;
		J = varifold<D>(m, md, w.xa, tc, tu, tvl, tgt->tgtElmNum, gx, s, md.precision, &err, nullptr);
		SA_REQUIRE(err == SA_OK, "varifold gradient needs vfdIfoMat");
		std::vector<double> hg = to_host(gx, (size_t) n, s);
		for (int k = 0; k < K; ++k) {
			std::vector<double> hd = to_host(dx[cur][k], (size_t) n, s);
			double acc = 0.0;
			for (long q = 0; q < n; ++q) acc += hg[q] * hd[q];
			grad[k] = acc;
		}
	}
	SA_CHECK(cudaEventRecord(ctx->e1, s));
	SA_CHECK(cudaEventSynchronize(ctx->e1));
	float ms = 0.f;
	cudaEventElapsedTime(&ms, ctx->e0, ctx->e1);
	tr.mark("forward + tangent steps, objective, gradient");
	if (objOut) SA_CHECK(cudaMemcpyAsync(objOut, &J, sizeof(double), cudaMemcpyDefault, s));
	if (gradOut) SA_CHECK(cudaMemcpyAsync(gradOut, grad.data(), sizeof(double) * K, cudaMemcpyDefault, s));
	SA_CHECK(cudaStreamSynchronize(s));
	if (info) {
		info->status = status;
		info->cgIterTotal = st.out.cgTotal;
		info->rdIterTotal = st.out.rdTotal;
		info->cgIterMax = tanIts;            // iterations of all tangent solves
		info->invertedElements = st.out.inverted;
		info->elapsedMs = ms;
		info->kernelLaunches = w.cw.launches;
	}
	return SA_OK;
}

// ---------------------------------------------------------------------------
// discrete adjoint of the frame model (the reference's own): the same sweep as the layered one below, with
// the frame operators (frame stress, anisotropic diffusion, frames built from other nodes, projected 3D
// penalty), the activity templates, the dense RKHS term ldm K^{-1} of the velocity operator and the
// polynomial bump.  The forward solve keeps v_t and K_t^{-1} v_t (tracked by the K-preconditioned CG); the
// velocity adjoint solve is the same K-preconditioned CG and leaves K_t^{-1} n in its tracked vector.
// Returns dJ/d tauVar (2D [cx, cy, h, R], 3D [cx, cy, cz, h]), dJ/dtau_0 and dJ/d(initial positions).
// ---------------------------------------------------------------------------
template <int D>
static int adjoint_frame_impl(sa_context *ctx, Pool &P, Mesh &m, Model &md, const double *x0,
                              const std::vector<double> &tv, const double *tc, const double *tu, const double *tvl,
                              int Vt, double *objOut, double *gradBump, double *gradTau0, double *gradX0,
                              sa_solve_info *info, PhaseTrace &tr)
{
	cudaStream_t s = ctx->stream;
	Work w;
	alloc_work<D>(w, m, md, true, P);
	const long n = (long) m.N * D, N = m.N;
	const int T = md.timeNum;
	const double dt = md.timeStp;
	{
		double *xa = P.alloc<double>((size_t) n);
		launch_soa_to_aos(m.N, D, x0, xa, s);
		k_init_sign<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, xa, m.sign0);
	}
	// inverse maps node -> (element, role) of the frame-building node lists
	int *fRow = nullptr, *fEnt = nullptr;
	{
		const int cols = D == 2 ? 4 : 6;
		std::vector<int> hf = to_host(m.frmVtx, (size_t) m.E * cols, s), ht = to_host(m.tsvVtx, (size_t) m.E * cols, s);
		std::vector<int> cnt((size_t) N + 1, 0);
		for (int which = 0; which < 2; ++which)
			for (int k = 0; k < cols; ++k)
				for (long e = 0; e < m.E; ++e) ++cnt[(size_t) (which ? ht : hf)[(size_t) k * m.E + e] + 1];
		for (long i = 0; i < N; ++i) cnt[i + 1] += cnt[i];
		std::vector<int> ent((size_t) cnt[N]), pos(cnt.begin(), cnt.end() - 1);
		for (long e = 0; e < m.E; ++e)
			for (int which = 0; which < 2; ++which)
				for (int k = 0; k < cols; ++k) {
					const int node = (which ? ht : hf)[(size_t) k * m.E + e];
					ent[(size_t) pos[node]++] = (int) (e * 16 + which * 8 + k);
				}
		fRow = (int *) P.dev(cnt.data(), cnt.size());
		fEnt = (int *) P.dev(ent.data(), ent.size());
		SA_CHECK(cudaStreamSynchronize(s));
	}
	double *vAll = P.alloc<double>((size_t) n * std::max(T - 1, 1));
	double *bAll = P.alloc<double>((size_t) n * std::max(T - 1, 1));       // K_t^{-1} v_t
	Stepper<D> st(m, md, w, s);
	st.start(x0, tv.data());
	tr.mark("inputs, work buffers");
	SA_CHECK(cudaEventRecord(ctx->e0, s));
	int status = SA_OK, adjIts = 0;
	while (st.t < T - 1 && status == SA_OK) {
		st.pre_velocity();
		int its = 0;
		int code = kpcg<D>(m, md, w.blk, w.K, st.xn, w.b, w.v, w.kw, st.st, &its, s);
		st.out.cgTotal += its;
		st.out.cgMax = std::max(st.out.cgMax, its);
		if (code != SA_OK) { status = code; break; }
		SA_CHECK(cudaMemcpyAsync(vAll + (long) st.t * n, w.v, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
		SA_CHECK(cudaMemcpyAsync(bAll + (long) st.t * n, w.kw.wK, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
		st.post_velocity();
		int rits = 0;
		code = cg_jacobi<1>(m, w.L, w.dinvRd, w.rhs, st.tau_next(), md.rdItrMax, md.rdTolSqu, w.cw, st.st, &rits, s,
		                    SA_PREC_FP64);
		st.out.rdTotal += rits;
		if (code != SA_OK) { status = code; break; }
		st.end_step();
	}
	const int steps = st.t;
	st.finish();
	double J = DBL_MAX;
	std::vector<double> gb((size_t) 4, std::nan(""));
	double *aX = P.zeros<double>(n), *aXn = P.zeros<double>(n);
	double *aT = P.zeros<double>(N), *aTn = P.zeros<double>(N);
	if (status == SA_OK) {
		int err = SA_OK;
		J = varifold<D>(m, md, w.xa, tc, tu, tvl, Vt, aXn, s, SA_PREC_FP64, &err, nullptr);
		SA_REQUIRE(err == SA_OK, "the adjoint needs vfdIfoMat (varifold gradient)");
		double *xt = P.alloc<double>((size_t) n), *xt1 = P.alloc<double>((size_t) n);
		double *nu = P.zeros<double>(n), *mu = P.zeros<double>(N), *rhsV = P.alloc<double>((size_t) n);
		double *wv = P.alloc<double>((size_t) N), *fyd = P.alloc<double>((size_t) N), *frd = P.alloc<double>((size_t) N);
		double *gF = P.alloc<double>((size_t) D * m.E), *gS = P.alloc<double>((size_t) D * m.E);
		Status *stt = st.st;
		SA_CHECK(cudaMemsetAsync(w.kw.wK, 0, sizeof(double) * n, s));      // the first adjoint solve starts at 0
		launch_soa_to_aos(m.N, D, w.trajX + (long) steps * n, xt1, s);
		for (int t = steps - 1; t >= 0 && status == SA_OK; --t) {
			const double *tauT = w.trajT + (long) t * N, *tauT1 = w.trajT + (long) (t + 1) * N;
			launch_soa_to_aos(m.N, D, w.trajX + (long) t * n, xt, s);
			launch_elem_geom<D>(m, md, xt, w.g0, stt, false, s);
			launch_elem_geom<D>(m, md, xt1, w.g1, stt, false, s);
			launch_assemble_rd<D>(m, md, w.g0, dt, w.Mnow, w.L, w.dinvRd, s);
			launch_assemble_rd<D>(m, md, w.g1, dt, w.Mnxt, w.L, w.dinvRd, s);
			int its = 0;
			int code = cg_jacobi<1>(m, w.L, w.dinvRd, aTn, mu, md.rdItrMax, md.rdTolSqu, w.cw, stt, &its, s,
			                        SA_PREC_FP64);
			adjIts += its;
			if (code != SA_OK) { status = code; break; }
			// -(d(L tau_t+1)/dx_t+1)^T m: mass and anisotropic diffusion at fixed frames, then the frames
			SA_CHECK(cudaMemsetAsync(gF, 0, sizeof(double) * D * m.E, s));
			SA_CHECK(cudaMemsetAsync(gS, 0, sizeof(double) * D * m.E, s));
			launch_adj_rd_frame<D>(m, md, w.g1, mu, tauT1, -1.0, -1.0, aXn, gF, gS, s);
			launch_adj_frame_scatter<D>(m, fRow, fEnt, xt1, gF, gS, aXn, s);
			launch_activity<D>(m, md, tauT, w.fy, w.fr, s);
			launch_act_deriv(m, md, tauT, fyd, frd, s);
			launch_adj_axpy(N, tauT, dt, w.fr, wv, s);
			SA_CHECK(cudaMemsetAsync(aX, 0, sizeof(double) * n, s));
			launch_adj_rd_frame<D>(m, md, w.g0, mu, wv, 1.0, 0.0, aX, nullptr, nullptr, s);   // mass only
			launch_adj_tau_d(m, md, w.Mnow, mu, frd, aT, s);
			launch_adj_axpy(n, aX, 1.0, aXn, aX, s);
			launch_adj_axpy(n, aXn, dt - 1.0, aXn, rhsV, s);
			// velocity adjoint: (ldm K_t^{-1} + E_t) n = a_v, K-preconditioned CG started from K_t times the
			// previous step's K^{-1} n
			if (!md.kernelFree) launch_kernel_matrix<D>(md, m.N, xt, w.K, s);
			if (m.Bt > 0 && md.btmWgt != 0.0) launch_penalty_diag<D>(m, md, xt, w.pd, s);
			launch_assemble_elastic<D>(m, md, w.g0, w.pd, w.blk, w.dinv, w.cw.binv64, nullptr, s);
			code = kpcg<D>(m, md, w.blk, w.K, xt, rhsV, nu, w.kw, stt, &its, s);
			adjIts += its;
			if (code != SA_OK) { status = code; break; }
			const double *vt = vAll + (long) t * n, *bt = bAll + (long) t * n;
			SA_CHECK(cudaMemsetAsync(gF, 0, sizeof(double) * D * m.E, s));
			SA_CHECK(cudaMemsetAsync(gS, 0, sizeof(double) * D * m.E, s));
			launch_adj_velocity_frame<D>(m, md, w.g0, w.fy, fyd, xt, vt, nu, aX, aT, gF, gS, s);
			launch_adj_frame_scatter<D>(m, fRow, fEnt, xt, gF, gS, aX, s);
			if (md.ldmWgt != 0.0) launch_adj_kernel_term<D>(md, m.N, xt, w.kw.wK, bt, aX, s);
			w.cw.launches += 24;
			std::swap(aX, aXn);
			std::swap(aT, aTn);
			std::swap(xt, xt1);
		}
		if (status == SA_OK) {
			// aXn, aTn: a_x^0, a_tau^0; the polynomial bump's parameters and its dependence on x_0
			double *x0a = xt1, *tmp = P.alloc<double>((size_t) 4 * N);
			launch_adj_bump_poly<D>(m, md, x0a, aTn, tv.data(), tmp, aXn, s);
			std::vector<double> ht = to_host(tmp, (size_t) 4 * N, s);
			for (int k = 0; k < 4; ++k) {
				double acc = 0.0;
				for (long q = 0; q < N; ++q) acc += ht[(size_t) k * N + q];
				gb[k] = acc;
			}
			if (gradTau0) SA_CHECK(cudaMemcpyAsync(gradTau0, aTn, sizeof(double) * N, cudaMemcpyDefault, s));
			if (gradX0) {
				launch_aos_to_soa(m.N, D, aXn, rhsV, s);
				SA_CHECK(cudaMemcpyAsync(gradX0, rhsV, sizeof(double) * n, cudaMemcpyDefault, s));
			}
		} else {
			J = DBL_MAX;
		}
	}
	SA_CHECK(cudaEventRecord(ctx->e1, s));
	SA_CHECK(cudaEventSynchronize(ctx->e1));
	float ms = 0.f;
	cudaEventElapsedTime(&ms, ctx->e0, ctx->e1);
	tr.mark("forward, adjoint sweep, gradients");
	if (objOut) SA_CHECK(cudaMemcpyAsync(objOut, &J, sizeof(double), cudaMemcpyDefault, s));
	if (gradBump) SA_CHECK(cudaMemcpyAsync(gradBump, gb.data(), sizeof(double) * 4, cudaMemcpyDefault, s));
	SA_CHECK(cudaStreamSynchronize(s));
	if (info) {
		info->status = status;
		info->cgIterTotal = st.out.cgTotal;
		info->rdIterTotal = st.out.rdTotal;
		info->cgIterMax = adjIts;
		info->invertedElements = st.out.inverted;
		info->elapsedMs = ms;
		info->kernelLaunches = w.cw.launches;
	}
	return SA_OK;
}

// ---------------------------------------------------------------------------
// discrete adjoint (layered model): forward pass keeping the trajectory and the velocities, then one
// backward sweep (two symmetric solves per step, sa_adjoint.cu) for the gradient of the objective with
// respect to every parameter at once: the bump [c, h, sigma], the per-layer (lambda, mu, D), the initial
// concentration of every node and the initial node positions
// ---------------------------------------------------------------------------
template <int D>
static int adjoint_impl(sa_context *ctx, const sa_element_object *obj, const double *lmkIni, const sa_params *prm,
                        const sa_target *tgt, const double *tauVar, int tauVarNum, double *objOut, double *gradBump,
                        double *gradLayer, double *gradTau0, double *gradX0, sa_solve_info *info)
{
	cudaStream_t s = ctx->stream;
	PhaseTrace tr(s);
	Pool P(s);
	Mesh m;
	Model md;
	fill_model(md, D, prm, tgt, P);
	SA_REQUIRE(md.frame || md.ldmWgt == 0.0, "adjoint: layered model with ldmWgt 0, or the frame model");
	SA_REQUIRE(tgt && tgt->tgtElmNum > 0 && tgt->cenPosMat && tgt->uniDirMat && tgt->elmVolVec, "the adjoint needs a target");
	md.precision = SA_PREC_FP64;             // forward and adjoint solves in FP64
	if (md.frame) {
		SA_REQUIRE(tauVar && tauVarNum >= 4, "tauVarVec needs 4 values (2D [cx, cy, h, R], 3D [cx, cy, cz, h])");
		build_mesh(m, obj, true, true, false, 0, P, &tr);
		const double *x0 = P.dev(lmkIni, (size_t) m.N * D);
		std::vector<double> tv = to_host(tauVar, (size_t) tauVarNum, s);
		const double *tc = P.dev(tgt->cenPosMat, (size_t) tgt->tgtElmNum * D);
		const double *tu = P.dev(tgt->uniDirMat, (size_t) tgt->tgtElmNum * D);
		const double *tvl = P.dev(tgt->elmVolVec, (size_t) tgt->tgtElmNum);
		choose_kernel_storage(md, m.N);
		return adjoint_frame_impl<D>(ctx, P, m, md, x0, tv, tc, tu, tvl, tgt->tgtElmNum, objOut, gradBump, gradTau0,
		                             gradX0, info, tr);
	}
	SA_REQUIRE(tauVar && tauVarNum >= D + 2, "tauVarVec needs [c (dim), h, sigma]");
	build_mesh(m, obj, true, true, true, md.lyrNum, P, &tr);
	const double *x0 = P.dev(lmkIni, (size_t) m.N * D);
	std::vector<double> tv = to_host(tauVar, (size_t) tauVarNum, s);
	const double *tc = P.dev(tgt->cenPosMat, (size_t) tgt->tgtElmNum * D);
	const double *tu = P.dev(tgt->uniDirMat, (size_t) tgt->tgtElmNum * D);
	const double *tvl = P.dev(tgt->elmVolVec, (size_t) tgt->tgtElmNum);
	Work w;
	alloc_work<D>(w, m, md, true, P);
	const long n = (long) m.N * D, N = m.N;
	const int T = md.timeNum;
	const double dt = md.timeStp;
	{
		double *xa = P.alloc<double>((size_t) n);
		launch_soa_to_aos(m.N, D, x0, xa, s);
		k_init_sign<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, xa, m.sign0);
	}
	double *vAll = P.alloc<double>((size_t) n * std::max(T - 1, 1));
	Stepper<D> st(m, md, w, s);
	st.start(x0, tv.data());
	tr.mark("inputs, work buffers");
	SA_CHECK(cudaEventRecord(ctx->e0, s));
	// forward: the one-call solve, keeping v_t
	int status = SA_OK, adjIts = 0;
	while (st.t < T - 1 && status == SA_OK) {
		st.pre_velocity();
		int its = 0;
		int code = cg_jacobi<D>(m, w.blk, w.dinv, w.b, w.v, md.cgItrMax, md.cgTolSqu, w.cw, st.st, &its, s,
		                        SA_PREC_FP64);
		st.out.cgTotal += its;
		st.out.cgMax = std::max(st.out.cgMax, its);
		if (code != SA_OK) { status = code; break; }
		SA_CHECK(cudaMemcpyAsync(vAll + (long) st.t * n, w.v, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
		st.post_velocity();
		int rits = 0;
		code = cg_jacobi<1>(m, w.L, w.dinvRd, w.rhs, st.tau_next(), md.rdItrMax, md.rdTolSqu, w.cw, st.st, &rits, s,
		                    SA_PREC_FP64);
		st.out.rdTotal += rits;
		if (code != SA_OK) { status = code; break; }
		st.end_step();
	}
	const int steps = st.t;
	st.finish();
	double J = DBL_MAX;
	std::vector<double> gb((size_t) D + 2, std::nan("")), gl((size_t) 3 * md.lyrNum, std::nan(""));
	double *aX = P.zeros<double>(n), *aXn = P.zeros<double>(n);       // a_x^t, a_x^t+1
	double *aT = P.zeros<double>(N), *aTn = P.zeros<double>(N);       // a_tau^t, a_tau^t+1
	if (status == SA_OK) {
		int err = SA_OK;
		J = varifold<D>(m, md, w.xa, tc, tu, tvl, tgt->tgtElmNum, aXn, s, SA_PREC_FP64, &err, nullptr);
		SA_REQUIRE(err == SA_OK, "the adjoint needs vfdIfoMat (varifold gradient)");
		double *xt = P.alloc<double>((size_t) n), *xt1 = P.alloc<double>((size_t) n);
		double *nu = P.zeros<double>(n), *mu = P.zeros<double>(N), *rhsV = P.alloc<double>((size_t) n);
		double *wv = P.alloc<double>((size_t) N);
		double *accLam = P.zeros<double>((size_t) m.E), *accMu = P.zeros<double>((size_t) m.E);
		double *accD = P.zeros<double>((size_t) m.E);
		Status *stt = st.st;
		launch_soa_to_aos(m.N, D, w.trajX + (long) steps * n, xt1, s);
		for (int t = steps - 1; t >= 0 && status == SA_OK; --t) {
			const double *tauT = w.trajT + (long) t * N, *tauT1 = w.trajT + (long) (t + 1) * N;
			launch_soa_to_aos(m.N, D, w.trajX + (long) t * n, xt, s);
			launch_elem_geom<D>(m, md, xt, w.g0, stt, false, s);
			launch_elem_geom<D>(m, md, xt1, w.g1, stt, false, s);
			launch_assemble_rd<D>(m, md, w.g0, dt, w.Mnow, w.L, w.dinvRd, s);     // M_t (L is overwritten next)
			launch_assemble_rd<D>(m, md, w.g1, dt, w.Mnxt, w.L, w.dinvRd, s);     // L_t+1
			// reaction-diffusion adjoint: L_t+1 m = a_tau^t+1 (the previous step's m starts the CG)
			int its = 0;
			int code = cg_jacobi<1>(m, w.L, w.dinvRd, aTn, mu, md.rdItrMax, md.rdTolSqu, w.cw, stt, &its, s,
			                        SA_PREC_FP64);
			adjIts += its;
			if (code != SA_OK) { status = code; break; }
			launch_adj_rd<D>(m, md, w.g1.rec, mu, tauT1, -1.0, -1.0, aXn, s);     // -(d(L tau_t+1)/dx_t+1)^T m
			launch_adj_diffusivity<D>(m, md, w.g1.rec, mu, tauT1, accD, s);
			launch_activity<D>(m, md, tauT, w.fy, w.fr, s);
			launch_adj_axpy(N, tauT, dt, w.fr, wv, s);                             // w = tau_t + dt R(tau_t)
			SA_CHECK(cudaMemsetAsync(aX, 0, sizeof(double) * n, s));
			launch_adj_rd<D>(m, md, w.g0.rec, mu, wv, 1.0, 0.0, aX, s);             // (d(M w)/dx_t)^T m
			launch_adj_tau(m, md, w.Mnow, mu, tauT, aT, s);                         // (I + dt R') M_t m
			// node update: a_x^t += a_x^t+1, a_v = dt a_x^t+1
			launch_adj_axpy(n, aX, 1.0, aXn, aX, s);
			launch_adj_axpy(n, aXn, dt - 1.0, aXn, rhsV, s);
			// velocity adjoint: K(x_t) n = a_v
			if (m.Bt > 0 && md.btmWgt != 0.0) launch_penalty_diag<D>(m, md, xt, w.pd, s);
			launch_assemble_elastic<D>(m, md, w.g0, w.pd, w.blk, w.dinv, w.cw.binv64, nullptr, s);
			code = cg_jacobi<D>(m, w.blk, w.dinv, rhsV, nu, md.cgItrMax, md.cgTolSqu, w.cw, stt, &its, s,
			                    SA_PREC_FP64);
			adjIts += its;
			if (code != SA_OK) { status = code; break; }
			const double *vt = vAll + (long) t * n;
			launch_adj_velocity<D>(m, md, w.g0.rec, w.fy, xt, vt, nu, aX, aT, s);
			launch_adj_moduli<D>(m, w.g0.rec, vt, nu, accLam, accMu, s);
			w.cw.launches += 14;
			std::swap(aX, aXn);
			std::swap(aT, aTn);
			std::swap(xt, xt1);
		}
		if (status == SA_OK) {
			// aXn, aTn: a_x^0, a_tau^0.  The bump's parameters, and its dependence on the initial shape
			double *x0a = xt1, *tmp = rhsV;
			const double *tau0 = w.trajT;
			for (int k = 0; k < D + 2; ++k) {
				launch_tau0_tan<D>(m, x0a, tau0, tv.data(), k, tmp, s);
				std::vector<double> hd = to_host(tmp, (size_t) N, s), ha = to_host(aTn, (size_t) N, s);
				double acc = 0.0;
				for (long q = 0; q < N; ++q) acc += ha[q] * hd[q];
				gb[k] = acc;
			}
			launch_adj_tau0_x<D>(m, x0a, tau0, aTn, tv.data(), aXn, s);
			if (gradLayer) {
				std::vector<double> hl = to_host(accLam, (size_t) m.E, s), hm = to_host(accMu, (size_t) m.E, s);
				std::vector<double> hD = to_host(accD, (size_t) m.E, s);
				std::vector<int> ly = to_host(m.elmLyr, (size_t) m.E, s);
				for (int l = 0; l < 3 * md.lyrNum; ++l) gl[l] = 0.0;
				for (long e = 0; e < m.E; ++e) {
					gl[3 * ly[e]] += hl[e];
					gl[3 * ly[e] + 1] += hm[e];
					gl[3 * ly[e] + 2] += hD[e];
				}
			}
			if (gradTau0) SA_CHECK(cudaMemcpyAsync(gradTau0, aTn, sizeof(double) * N, cudaMemcpyDefault, s));
			if (gradX0) {
				launch_aos_to_soa(m.N, D, aXn, tmp, s);
				SA_CHECK(cudaMemcpyAsync(gradX0, tmp, sizeof(double) * n, cudaMemcpyDefault, s));
			}
		}
		if (status != SA_OK) J = DBL_MAX;
	}
	SA_CHECK(cudaEventRecord(ctx->e1, s));
	SA_CHECK(cudaEventSynchronize(ctx->e1));
	float ms = 0.f;
	cudaEventElapsedTime(&ms, ctx->e0, ctx->e1);
	tr.mark("forward, adjoint sweep, gradients");
	if (objOut) SA_CHECK(cudaMemcpyAsync(objOut, &J, sizeof(double), cudaMemcpyDefault, s));
	if (gradBump) SA_CHECK(cudaMemcpyAsync(gradBump, gb.data(), sizeof(double) * gb.size(), cudaMemcpyDefault, s));
	if (gradLayer) SA_CHECK(cudaMemcpyAsync(gradLayer, gl.data(), sizeof(double) * gl.size(), cudaMemcpyDefault, s));
	SA_CHECK(cudaStreamSynchronize(s));
	if (info) {
		info->status = status;
		info->cgIterTotal = st.out.cgTotal;
		info->rdIterTotal = st.out.rdTotal;
		info->cgIterMax = adjIts;            // iterations of all adjoint solves
		info->invertedElements = st.out.inverted;
		info->elapsedMs = ms;
		info->kernelLaunches = w.cw.launches;
	}
	return SA_OK;
}

// ---------------------------------------------------------------------------
// sessions: one parameter vector, stepped on demand, state device-resident
// ---------------------------------------------------------------------------
struct SessionBase {
	sa_context *ctx;
	explicit SessionBase(sa_context *c) : ctx(c) {}
	virtual ~SessionBase() {}
	virtual int step(int n) = 0;
	virtual void state(double *lmk, double *tau, int *t) = 0;
	virtual double objective() = 0;
	virtual void info(sa_solve_info *i) = 0;
	virtual void profile(int enable, double *ms, long long *cnt, double *bytes, double *flops) = 0;
	virtual int stream(int nsteps, int stride, double *lmkOut, double *tauOut, int maxSnap, int *written) = 0;
};

template <int D>
struct Session : SessionBase {
	Pool P;
	Mesh m;
	Model md;
	Work w;
	Stepper<D> st;
	const double *tc = nullptr, *tu = nullptr, *tvl = nullptr;
	int Vt = 0;
	std::vector<double> tauVar;
	VfdTargetCache vcache;                    // target-target varifold rows, kept across objective() calls

	Session(sa_context *c, const sa_element_object *obj, const double *lmkIni, const sa_params *prm,
	        const sa_target *tgt, const double *tv, int tvNum)
		: SessionBase(c), P(c->stream), st(m, md, w, c->stream)
	{
		cudaStream_t s = c->stream;
		fill_model(md, D, prm, tgt, P);
		build_mesh(m, obj, tgt != nullptr, false, !md.frame, md.lyrNum, P);
		choose_kernel_storage(md, m.N);
		SA_REQUIRE(tv && tvNum >= (md.frame ? 4 : D + 2), "tauVarVec too small");
		tauVar = to_host(tv, (size_t) tvNum, s);
		const double *x0 = P.dev(lmkIni, (size_t) m.N * D);
		if (tgt) {
			SA_REQUIRE(tgt->tgtElmNum > 0 && tgt->cenPosMat && tgt->uniDirMat && tgt->elmVolVec, "empty target");
			Vt = tgt->tgtElmNum;
			tc = P.dev(tgt->cenPosMat, (size_t) Vt * D);
			tu = P.dev(tgt->uniDirMat, (size_t) Vt * D);
			tvl = P.dev(tgt->elmVolVec, (size_t) Vt);
		}
		alloc_work<D>(w, m, md, false, P);
		double *xa = P.alloc<double>((size_t) m.N * D);
		launch_soa_to_aos(m.N, D, x0, xa, s);
		k_init_sign<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, xa, m.sign0);
		// the stepper keeps x0 in SoA for the trajectory; keep our own device copy alive
		double *x0d = P.alloc<double>((size_t) m.N * D);
		SA_CHECK(cudaMemcpyAsync(x0d, x0, sizeof(double) * m.N * D, cudaMemcpyDeviceToDevice, s));
		st.start(x0d, tauVar.data());
		SA_CHECK(cudaStreamSynchronize(s));
	}
	double lastStepMs = 0.0;
	int step(int n) override
	{
		SA_CHECK(cudaEventRecord(ctx->e0, ctx->stream));
		int k = st.step(n);
		SA_CHECK(cudaEventRecord(ctx->e1, ctx->stream));
		SA_CHECK(cudaEventSynchronize(ctx->e1));
		float ms = 0.f;
		SA_CHECK(cudaEventElapsedTime(&ms, ctx->e0, ctx->e1));
		lastStepMs = ms;
		SA_CHECK(cudaGetLastError());
		return k;
	}
	void state(double *lmk, double *tau, int *t) override
	{
		cudaStream_t s = ctx->stream;
		if (t) *t = st.t;
		if (lmk) {
			std::vector<double> h = to_host(st.xn, (size_t) m.N * D, s), o((size_t) m.N * D);
			for (int i = 0; i < m.N; ++i)
				for (int d = 0; d < D; ++d) o[(size_t) d * m.N + i] = h[(size_t) i * D + d];
			SA_CHECK(cudaMemcpyAsync(lmk, o.data(), sizeof(double) * o.size(), cudaMemcpyDefault, s));
		}
		if (tau) SA_CHECK(cudaMemcpyAsync(tau, w.trajT + (long) st.t * m.N, sizeof(double) * m.N,
		                                  cudaMemcpyDefault, s));
		SA_CHECK(cudaStreamSynchronize(s));
	}
	double objective() override
	{
		SA_REQUIRE(tc, "session has no target");
		if (st.out.status != SA_OK) return DBL_MAX;
		int err = SA_OK;
		if (!vcache.rows) { vcache.rows = P.alloc<double>((size_t) Vt); vcache.capacity = Vt; }
		double v = varifold<D>(m, md, st.xn, tc, tu, tvl, Vt, nullptr, ctx->stream, md.precision, &err, &vcache);
		SA_REQUIRE(err == SA_OK, "varifold arguments");
		return v;
	}
	void info(sa_solve_info *i) override
	{
		Status hs;
		SA_CHECK(cudaMemcpyAsync(&hs, st.st, sizeof(Status), cudaMemcpyDeviceToHost, ctx->stream));
		SA_CHECK(cudaStreamSynchronize(ctx->stream));
		i->status = st.out.status;
		i->cgIterTotal = st.out.cgTotal;
		i->rdIterTotal = st.out.rdTotal;
		i->cgIterMax = st.out.cgMax;
		i->invertedElements = hs.inverted;
		i->elapsedMs = lastStepMs;             // device time of the last sa_session_step call
		i->kernelLaunches = w.cw.launches;
	}
	// streamed snapshots: a ring of device and pinned host buffers; each snapshot is converted to the
	// lmkStk layout on the compute stream, copied to pinned memory on a copy stream while the next steps
	// run, and moved into the caller's buffer when its ring slot is needed again (or at the end)
	struct Slot {
		double *dev = nullptr, *host = nullptr;
		cudaEvent_t ready = nullptr, copied = nullptr;
		long snap = -1;                    // snapshot index held, -1: free
	};
	static constexpr int kRing = 3;
	Slot ring[kRing];
	cudaStream_t copyStream = nullptr;
	~Session() override
	{
		if (copyStream) cudaStreamSynchronize(copyStream);
		for (Slot &r : ring) {
			if (r.host) cudaFreeHost(r.host);
			if (r.ready) cudaEventDestroy(r.ready);
			if (r.copied) cudaEventDestroy(r.copied);
		}
		if (copyStream) cudaStreamDestroy(copyStream);
	}
	int stream(int nsteps, int stride, double *lmkOut, double *tauOut, int maxSnap, int *written) override
	{
		SA_REQUIRE(nsteps >= 0 && stride >= 1 && maxSnap >= 0, "stream: nsteps >= 0, stride >= 1, maxSnapshots >= 0");
		SA_REQUIRE(!is_device_ptr(lmkOut) && !is_device_ptr(tauOut), "stream: output buffers must be host memory");
		cudaStream_t s = ctx->stream;
		const size_t nx = (size_t) m.N * D, per = nx + (size_t) m.N;
		if (!copyStream) {
			SA_CHECK(cudaStreamCreateWithFlags(&copyStream, cudaStreamNonBlocking));
			for (Slot &r : ring) {
				r.dev = P.alloc<double>(per);
				SA_CHECK(cudaHostAlloc((void **) &r.host, sizeof(double) * per, cudaHostAllocDefault));
				SA_CHECK(cudaEventCreateWithFlags(&r.ready, cudaEventDisableTiming));
				SA_CHECK(cudaEventCreateWithFlags(&r.copied, cudaEventDisableTiming));
			}
		}
		auto drain = [&](Slot &r) {
			if (r.snap < 0) return;
			SA_CHECK(cudaEventSynchronize(r.copied));
			if (lmkOut) std::memcpy(lmkOut + (size_t) r.snap * nx, r.host, sizeof(double) * nx);
			if (tauOut) std::memcpy(tauOut + (size_t) r.snap * m.N, r.host + nx, sizeof(double) * m.N);
			r.snap = -1;
		};
		int snaps = 0, done = 0;
		SA_CHECK(cudaEventRecord(ctx->e0, s));
		while (done < nsteps) {
			if (st.step(1) == 0) break;
			++done;
			if (st.t % stride != 0 || snaps >= maxSnap) continue;
			Slot &r = ring[snaps % kRing];
			drain(r);                          // the snapshot kRing back, copied long since
			launch_aos_to_soa(m.N, D, st.xn, r.dev, s);
			SA_CHECK(cudaMemcpyAsync(r.dev + nx, st.tau_now(), sizeof(double) * m.N, cudaMemcpyDeviceToDevice, s));
			SA_CHECK(cudaEventRecord(r.ready, s));
			SA_CHECK(cudaStreamWaitEvent(copyStream, r.ready, 0));
			SA_CHECK(cudaMemcpyAsync(r.host, r.dev, sizeof(double) * per, cudaMemcpyDeviceToHost, copyStream));
			SA_CHECK(cudaEventRecord(r.copied, copyStream));
			r.snap = snaps++;
			w.cw.launches += 1;
		}
		SA_CHECK(cudaEventRecord(ctx->e1, s));
		for (int k = std::max(0, snaps - kRing); k < snaps; ++k) drain(ring[k % kRing]);
		SA_CHECK(cudaEventSynchronize(ctx->e1));
		float ms = 0.f;
		SA_CHECK(cudaEventElapsedTime(&ms, ctx->e0, ctx->e1));
		lastStepMs = ms;
		SA_CHECK(cudaGetLastError());
		if (written) *written = snaps;
		return done;
	}
	void profile(int enable, double *ms, long long *cnt, double *bytes, double *flops) override
	{
		if (ms) *ms = w.cw.spmvMs;
		if (cnt) *cnt = w.cw.spmvCount;
		if (bytes) *bytes = w.cw.profBytes;
		if (flops) *flops = w.cw.profFlops;
		if (enable >= 0) {
			w.cw.profileEnabled = enable;
			w.cw.spmvMs = 0.0;
			w.cw.spmvCount = 0;
			w.cw.profBytes = 0.0;
			w.cw.profFlops = 0.0;
		}
	}
};

template <typename F>
static int guarded(sa_context *ctx, F &&f)
{
	if (!ctx) return SA_ERR_ARG;
	try {
		SA_CHECK(cudaSetDevice(ctx->device));
		int rc = f();
		ctx->err.clear();
		return rc;
	} catch (const ArgError &e) {
		ctx->err = e.msg;
		return SA_ERR_ARG;
	} catch (const CudaError &e) {
		ctx->err = std::string(e.where) + ": " + cudaGetErrorString(e.e);
		cudaGetLastError();
		return SA_ERR_CUDA;
	} catch (const DeviceWaitError &e) {
		ctx->err = std::string(e.where) + ": a device-side wait gave up after its time limit";
		return SA_ERR_TIMEOUT;
	} catch (const std::bad_alloc &) {
		ctx->err = "host allocation failed";
		return SA_ERR_CUDA;
	}
}


// ---------------------------------------------------------------------------
// serving: continuous batching of forward solves (layered model)
//
// A request is copied at submission.  The loop thread admits queued
// requests in arrival order while their device footprint fits the budget
// (and fewer than maxInstances run), keeps each admitted instance's mesh,
// state and solver vectors device-resident, and advances all running
// instances one time step per tick: element kernels per instance, then ONE
// batched persistent CG launch for all velocity solves of a precision and
// dimension, then one batched launch for all reaction-diffusion solves.
// Instances that finish (or fail) leave at the end of a tick and free their
// memory; queued requests enter at the start of the next one.  The CTAs a
// solve gets depend only on its own size, so its result does not depend on
// what else runs in the batch.
// ---------------------------------------------------------------------------
struct Request {
	long long id = 0;
	int dim = 0;
	sa_element_object obj{};
	sa_params prm{};
	sa_target tgt{};
	bool hasTgt = false;
	std::vector<int> elmVtx, vtxElm, btmVtx, vtxBtm, femVtx, femIfo, vfdVtx, elmLyr;
	std::vector<double> lmk, tauPrm, mod, spdLyr, ynk, rea, tauVar, cen, dir, vol;
	int state = SA_REQ_QUEUED;
	int status = SA_OK;
	std::string err;
	std::vector<double> lmkOut, tauOut;
	double objOut = 0.0;
	sa_solve_info info{};
	size_t estBytes = 0;
	std::chrono::steady_clock::time_point tSubmit, tStart, tDone;
};

template <typename T> static void copy_in(std::vector<T> &dst, const T *src, size_t n)
{
	dst.resize(n);
	if (n) {
		SA_REQUIRE(src, "missing input array");
		SA_CHECK(cudaMemcpy(dst.data(), src, sizeof(T) * n, cudaMemcpyDefault));
	}
}

// device bytes an instance will hold, from the request's sizes (before the sliced layout exists)
static size_t estimate_bytes(const Request &r)
{
	const sa_element_object &o = r.obj;
	size_t D = r.dim, N = o.lmkNum, E = o.elmNum, Z = o.nzrNum, T = r.prm.timeNum;
	size_t slots = Z + Z / 8 + 32 * (N / 32 + 1);                 // sliced slots incl. padding (bound)
	size_t ints = E * (D + 1) + N * o.vtxElmCols + Z * (2 + o.femIfoCols) + Z * 4 + slots + 2 * E +
	              (size_t) o.btmElmNum * D + (size_t) o.btmLmkNum * o.vtxBtmCols + (size_t) o.vfdElmNum * D;
	size_t dbl = slots * (D * D + 1) + 2 * Z + 2 * E * (D == 3 ? 16 : 8) + 20 * N * D + 8 * N + T * N;
	if (r.prm.precision == SA_PREC_MIXED) dbl += (slots * D * D + 7 * N * D + N * D * D) / 2;
	else dbl += N * D * D;                                         // FP64 block-Jacobi inverses
	if (r.hasTgt) dbl += (size_t) r.tgt.tgtElmNum * (2 * D + 1) + (size_t) o.vfdElmNum * (3 * D + 2);
	return 4 * ints + 8 * dbl + (1 << 20);
}

enum { kMixedVelocity = 0, kMixedRd = 1 };

struct InstBase {
	Request *req = nullptr;
	size_t bytes = 0;
	int failed = 0;
	int its = 0, rits = 0;
	double bb = -1.0, innerTol = 0.0;
	int mixedTotal = 0, mixedDone = 0;
	int lastVelIts = 0;                      // velocity iterations of the previous step (launch packing order)
	virtual ~InstBase() {}
	virtual int nodes() const = 0;
	// expected length of the next solve, for packing batched launches: the previous step's iterations,
	// or 1.5 sqrt(N) before the first step.  Only the order of solves in launches depends on it.
	double vel_key() const { return lastVelIts > 0 ? lastVelIts : 1.5 * std::sqrt((double) nodes()); }
	virtual int dim() const = 0;
	virtual int precision() const = 0;
	virtual bool finished() const = 0;
	virtual void pre_velocity() = 0;
	virtual void prepare_velocity_fp64() = 0;
	virtual void finish_velocity_fp64() = 0;
	virtual BatchSolve velocity_fp64() = 0;
	// mixed precision, for the solve `kind` of the step (kMixedVelocity: B = dim, kMixedRd: B = 1): FP64
	// residual and outer test, FP32 inner solve (batched), FP64 update
	virtual void mixed_outer(int kind, int first) = 0;
	virtual void mixed_inner(int kind) = 0;
	virtual BatchSolve mixed_solve(int kind) = 0;
	virtual void mixed_apply(int kind) = 0;
	virtual void mixed_zero(int kind) = 0;
	virtual void post_velocity() = 0;
	virtual void prepare_rd() = 0;
	virtual BatchSolve rd_solve() = 0;
	virtual void finish_rd() = 0;
	virtual void end_step() = 0;
	virtual CgWork &cg() = 0;
	virtual const Model &model() const = 0;
	virtual void results() = 0;              // final state, objective and diagnostics into the request
	virtual void account(int velIts, int rdIts) = 0;
	virtual void set_status(int code) = 0;
};

template <int D>
struct Inst : InstBase {
	Pool P;
	Mesh m;
	Model md;
	Work w;
	Stepper<D> st;
	cudaStream_t s;
	const double *tc = nullptr, *tu = nullptr, *tvl = nullptr;
	int Vt = 0;

	Inst(Request *r, cudaStream_t s_) : P(s_), st(m, md, w, s_), s(s_)
	{
		req = r;
		fill_model(md, D, &r->prm, r->hasTgt ? &r->tgt : nullptr, P);
		SA_REQUIRE(!md.frame && md.ldmWgt == 0.0, "the server runs the layered model (elaType isotropic, ldmWgt 0)");
		build_mesh(m, &r->obj, r->hasTgt, false, true, md.lyrNum, P);
		SA_REQUIRE(r->tauVar.size() >= (size_t) D + 2, "tauVarVec too small");
		const double *x0 = P.dev(r->lmk.data(), (size_t) m.N * D);
		if (r->hasTgt) {
			Vt = r->tgt.tgtElmNum;
			tc = P.dev(r->cen.data(), (size_t) Vt * D);
			tu = P.dev(r->dir.data(), (size_t) Vt * D);
			tvl = P.dev(r->vol.data(), (size_t) Vt);
		}
		alloc_work<D>(w, m, md, false, P);
		double *xa = P.alloc<double>((size_t) m.N * D);
		launch_soa_to_aos(m.N, D, x0, xa, s);
		k_init_sign<D><<<grid_for(m.E), kBlock, 0, s>>>(m.E, m.elmVtx, xa, m.sign0);
		st.start(x0, r->tauVar.data());
		SA_CHECK(cudaStreamSynchronize(s));
		bytes = P.bytes;
	}
	int dim() const override { return D; }
	int precision() const override { return md.precision; }
	bool finished() const override { return failed || st.t >= md.timeNum - 1; }
	void pre_velocity() override { st.pre_velocity(); }
	void prepare_velocity_fp64() override
	{
		cg_prepare_fp64<D>(m, w.blk, w.dinv, w.b, w.v, md.cgItrMax, md.cgTolSqu, w.cw, s);
	}
	void finish_velocity_fp64() override { cg_finish_fp64<D>(m, w.v, w.cw, s); }
	BatchSolve velocity_fp64() override { return BatchSolve{&m, &w.cw, w.blk, w.dinv, w.v, w.cw.binv64}; }
	void mixed_outer(int kind, int first) override
	{
		if (kind == kMixedVelocity) {
			cg_mixed_outer<D>(m, w.blk, w.dinv, w.b, w.v, bb, first, w.cw, s);
			return;
		}
		if (first) {                         // FP32 copies of L and of its inverse diagonal
			k_to_f32<<<grid_for(m.slTotal), kBlock, 0, s>>>(m.slTotal, w.L, w.L32);
			k_to_f32<<<grid_for(m.N), kBlock, 0, s>>>(m.N, w.dinvRd, w.rdInv32);
			w.cw.launches += 2;
		}
		cg_mixed_outer<1>(m, w.L, w.dinvRd, w.rhs, st.tau_next(), bb, first, w.cw, s);
	}
	void mixed_inner(int kind) override
	{
		if (kind == kMixedVelocity) {
			cg_mixed_inner<D>(m, md.cgItrMax - mixedTotal, innerTol, w.cw, s);
			return;
		}
		float *binv32 = w.cw.binv32;          // the inner solve's 1 x 1 block inverses: L's inverse diagonal
		w.cw.binv32 = w.rdInv32;
		try {
			cg_mixed_inner<1>(m, md.rdItrMax - mixedTotal, innerTol, w.cw, s);
		} catch (...) {
			w.cw.binv32 = binv32;
			throw;
		}
		w.cw.binv32 = binv32;
	}
	BatchSolve mixed_solve(int kind) override
	{
		if (kind == kMixedVelocity) {
			long n = (long) m.N * D;
			return BatchSolve{&m, &w.cw, w.cw.blk32, w.cw.f32 + 5 * n, w.cw.f32 + 6 * n, w.cw.binv32};
		}
		long n = m.N;
		return BatchSolve{&m, &w.cw, w.L32, w.cw.f32 + 5 * n, w.cw.f32 + 6 * n, w.rdInv32};
	}
	void mixed_apply(int kind) override
	{
		if (kind == kMixedVelocity) cg_mixed_apply((long) m.N * D, w.v, w.cw, s);
		else cg_mixed_apply((long) m.N, st.tau_next(), w.cw, s);
	}
	void mixed_zero(int kind) override
	{
		if (kind == kMixedVelocity) SA_CHECK(cudaMemsetAsync(w.v, 0, sizeof(double) * m.N * D, s));
		else SA_CHECK(cudaMemsetAsync(st.tau_next(), 0, sizeof(double) * m.N, s));
	}
	void post_velocity() override { st.post_velocity(); }
	void prepare_rd() override
	{
		cg_prepare_fp64<1>(m, w.L, w.dinvRd, w.rhs, st.tau_next(), md.rdItrMax, md.rdTolSqu, w.cw, s);
	}
	BatchSolve rd_solve() override { return BatchSolve{&m, &w.cw, w.L, w.dinvRd, st.tau_next(), nullptr}; }
	void finish_rd() override { cg_finish_fp64<1>(m, st.tau_next(), w.cw, s); }
	void end_step() override { st.end_step(); }
	CgWork &cg() override { return w.cw; }
	const Model &model() const override { return md; }
	void set_status(int code) override { st.out.status = code; }
	int nodes() const override { return m.N; }
	void account(int velIts, int rdIts) override
	{
		lastVelIts = velIts;
		st.out.cgTotal += velIts;
		st.out.cgMax = std::max(st.out.cgMax, velIts);
		st.out.rdTotal += rdIts;
	}
	void results() override
	{
		Request &r = *req;
		Status hs;
		SA_CHECK(cudaMemcpyAsync(&hs, st.st, sizeof(Status), cudaMemcpyDeviceToHost, s));
		std::vector<double> h = to_host(st.xn, (size_t) m.N * D, s);
		r.lmkOut.assign((size_t) m.N * D, 0.0);
		for (int i = 0; i < m.N; ++i)
			for (int d = 0; d < D; ++d) r.lmkOut[(size_t) d * m.N + i] = h[(size_t) i * D + d];
		r.tauOut = to_host(w.trajT + (long) st.t * m.N, (size_t) m.N, s);
		r.status = st.out.status;
		r.objOut = 0.0;
		if (r.hasTgt) {
			if (st.out.status != SA_OK) r.objOut = DBL_MAX;
			else {
				int err = SA_OK;
				r.objOut = varifold<D>(m, md, st.xn, tc, tu, tvl, Vt, nullptr, s, md.precision, &err);
				SA_REQUIRE(err == SA_OK, "varifold arguments");
			}
		}
		r.info.status = st.out.status;
		r.info.cgIterTotal = st.out.cgTotal;
		r.info.rdIterTotal = st.out.rdTotal;
		r.info.cgIterMax = st.out.cgMax;
		r.info.invertedElements = hs.inverted;
		r.info.kernelLaunches = w.cw.launches;
	}
};

struct Server {
	sa_context *ctx;
	cudaStream_t s = nullptr;
	size_t budget;
	int maxInst;
	std::mutex mu;
	std::condition_variable cv;
	std::deque<Request *> queue;
	std::map<long long, std::unique_ptr<Request>> reqs;
	std::vector<std::unique_ptr<InstBase>> active;
	long long nextId = 1, submitted = 0, completed = 0, failedCount = 0, ticks = 0;
	size_t inUse = 0, peak = 0;
	double busyMs = 0.0;
	bool stop = false;
	std::string loopErr;
	CgJob *devJobs = nullptr;
	int smCount = 1;
	std::thread th;
	// SA_TRACE: time per tick phase (element kernels, FP64 velocity, mixed velocity, reaction-diffusion,
	// bookkeeping) and batched CG launches, printed when the server is destroyed
	bool trace = std::getenv("SA_TRACE") != nullptr;
	double phaseMs[5] = {0, 0, 0, 0, 0};
	long long batchLaunches[4] = {0, 0, 0, 0};   // FP64 velocity, FP32 velocity, FP64 RD, FP32 RD
	std::chrono::steady_clock::time_point tMark;
	// The instances' own work (element kernels, per-instance solve set-up and updates) runs on
	// kInstStreams streams, instance k on stream k mod kInstStreams, so that the many small kernels of
	// different instances overlap on the GPU; the batched solves run on s.  join() makes s wait for all
	// instance streams (before a batched launch or a read of the instances' CG scalars), fork() makes the
	// instance streams wait for s (after a batched launch).  Each instance's work stays in order on its own
	// stream, so results do not depend on the streams.
	static constexpr int kInstStreams = 8;
	cudaStream_t pool[kInstStreams] = {};
	cudaEvent_t poolEv[kInstStreams] = {}, mainEv = nullptr;
	int nextStream = 0;
	void join()
	{
		for (int k = 0; k < kInstStreams; ++k) {
			SA_CHECK(cudaEventRecord(poolEv[k], pool[k]));
			SA_CHECK(cudaStreamWaitEvent(s, poolEv[k], 0));
		}
	}
	void fork()
	{
		SA_CHECK(cudaEventRecord(mainEv, s));
		for (int k = 0; k < kInstStreams; ++k) SA_CHECK(cudaStreamWaitEvent(pool[k], mainEv, 0));
	}
	void mark(int phase)
	{
		if (!trace) return;
		join();
		cudaStreamSynchronize(s);
		const auto t = std::chrono::steady_clock::now();
		if (phase >= 0) phaseMs[phase] += std::chrono::duration<double, std::milli>(t - tMark).count();
		tMark = t;
	}

	static constexpr int kMaxJobs = 4096;

	Server(sa_context *c, size_t budgetBytes, int maxInstances) : ctx(c), budget(budgetBytes), maxInst(maxInstances)
	{
		SA_CHECK(cudaSetDevice(ctx->device));
		SA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
		for (int k = 0; k < kInstStreams; ++k) {
			SA_CHECK(cudaStreamCreateWithFlags(&pool[k], cudaStreamNonBlocking));
			SA_CHECK(cudaEventCreateWithFlags(&poolEv[k], cudaEventDisableTiming));
		}
		SA_CHECK(cudaEventCreateWithFlags(&mainEv, cudaEventDisableTiming));
		SA_CHECK(cudaMalloc(&devJobs, sizeof(CgJob) * kMaxJobs));
		SA_CHECK(cudaDeviceGetAttribute(&smCount, cudaDevAttrMultiProcessorCount, ctx->device));
		th = std::thread([this] { loop(); });
	}
	~Server()
	{
		{
			std::lock_guard<std::mutex> g(mu);
			stop = true;
		}
		cv.notify_all();
		if (th.joinable()) th.join();
		active.clear();
		if (trace)
			std::fprintf(stderr,
			             "[sa_trace] server: %lld ticks; ms in element kernels %.1f, FP64 velocity %.1f, mixed "
			             "velocity %.1f, reaction-diffusion %.1f, bookkeeping %.1f; batched CG launches FP64 %lld, "
			             "FP32 %lld, RD FP64 %lld, RD FP32 %lld\n",
			             ticks, phaseMs[0], phaseMs[1], phaseMs[2], phaseMs[3], phaseMs[4], batchLaunches[0],
			             batchLaunches[1], batchLaunches[2], batchLaunches[3]);
		cudaSetDevice(ctx->device);
		for (int k = 0; k < kInstStreams; ++k) {
			if (pool[k]) { cudaStreamSynchronize(pool[k]); cudaStreamDestroy(pool[k]); }
			if (poolEv[k]) cudaEventDestroy(poolEv[k]);
		}
		if (mainEv) cudaEventDestroy(mainEv);
		if (devJobs) cudaFree(devJobs);
		if (statPinned) cudaFreeHost(statPinned);
		if (s) cudaStreamDestroy(s);
	}

	// a solve that did not converge (or broke down): the instance stops, the request completes with that
	// per-solve status and objective DBL_MAX, as sa_forward reports it
	void fail(InstBase &in, int code)
	{
		in.failed = 1;
		in.set_status(code);
	}

	// one time step of every running instance.  When the solves of a batched CG do not fit one cooperative
	// launch they run in several (first fit), each as long as its slowest solve.  The FP32 inner solves of
	// mixed precision are latency bound, so their length follows their iteration count: they are ordered
	// longest first, so that long solves share launches.  The FP64 solves are FP64-pipe bound and keep
	// arrival order (measured faster on the served stream).  Results do not depend on the order.
	// CG scalars of every instance in g with one host synchronisation (pinned staging grows as needed)
	void *statPinned = nullptr;
	size_t statCap = 0;
	std::vector<CgState> states(const std::vector<InstBase *> &g)
	{
		if (g.size() > statCap) {
			if (statPinned) SA_CHECK(cudaFreeHost(statPinned));
			statPinned = nullptr;
			statCap = std::max(g.size(), (size_t) 256);
			SA_CHECK(cudaHostAlloc(&statPinned, statCap * cg_scal_bytes(), cudaHostAllocDefault));
		}
		std::vector<const CgWork *> ws;
		for (InstBase *in : g) ws.push_back(&in->cg());
		std::vector<CgState> out;
		join();                              // the scalars may come from the instances' own streams
		cg_states(ws, statPinned, s, out);
		return out;
	}

	// Mixed precision: FP64 iterative refinement of one solve of every instance in g (all of dimension B's
	// kind), each refinement round one batched FP32 launch over the instances still refining.  Leaves each
	// instance's FP32 iterations in mixedTotal; failed instances are marked.
	void refine_mixed(std::vector<InstBase *> g, int kind, int B)
	{
		for (InstBase *in : g) { in->bb = -1.0; in->mixedTotal = 0; in->mixedDone = 0; }
		for (int outer = 0; outer < 64 && !g.empty(); ++outer) {
			for (InstBase *in : g) in->mixed_outer(kind, outer == 0);
			std::vector<InstBase *> inner;
			const std::vector<CgState> cs = states(g);
			for (size_t q = 0; q < g.size(); ++q) {
				InstBase *in = g[q];
				const CgState &c = cs[q];
				const Model &md = in->model();
				const double tolSqu = kind == kMixedVelocity ? md.cgTolSqu : md.rdTolSqu;
				const int itrMax = kind == kMixedVelocity ? md.cgItrMax : md.rdItrMax;
				if (in->bb < 0.0) in->bb = c.bb;
				if (c.code == SA_ERR_NONFINITE) { fail(*in, SA_ERR_NONFINITE); continue; }
				if (c.zero) { in->mixed_zero(kind); continue; }
				if (c.rr < tolSqu * in->bb) continue;
				if (in->mixedTotal >= itrMax) { fail(*in, SA_ERR_NOT_CONVERGED); continue; }
				double need = 0.01 * tolSqu * in->bb / c.rr;
				const double floorSqu = std::pow(10.0, -(double) tuning().mixedInnerFloor);
				in->innerTol = need > floorSqu ? need : floorSqu;
				inner.push_back(in);
			}
			if (inner.empty()) break;
			std::vector<BatchSolve> bs;
			for (InstBase *in : inner) { in->mixed_inner(kind); bs.push_back(in->mixed_solve(kind)); }
			const int li = kind == kMixedVelocity ? 1 : 3;
			join();
			batchLaunches[li] += B == 1 ? cg_batch_run<1, float, float, float>(bs, smCount, devJobs, kMaxJobs, s)
			                   : B == 2 ? cg_batch_run<2, float, float, float>(bs, smCount, devJobs, kMaxJobs, s)
			                            : cg_batch_run<3, float, float, float>(bs, smCount, devJobs, kMaxJobs, s);
			fork();
			std::vector<InstBase *> next;
			const std::vector<CgState> ci = states(inner);
			for (size_t q = 0; q < inner.size(); ++q) {
				InstBase *in = inner[q];
				const CgState &c = ci[q];
				in->mixedTotal += c.iters;
				if (c.code == SA_ERR_NONFINITE) { fail(*in, SA_ERR_NONFINITE); continue; }
				in->mixed_apply(kind);
				next.push_back(in);
			}
			g.swap(next);
			if (outer == 63)
				for (InstBase *in : g) fail(*in, SA_ERR_NOT_CONVERGED);
		}
	}

	void tick()
	{
		std::vector<InstBase *> run;
		for (auto &u : active) if (!u->finished()) run.push_back(u.get());
		mark(-1);
		for (InstBase *in : run) { in->its = 0; in->rits = 0; in->pre_velocity(); }
		mark(0);
		// velocity: FP64 instances, one batched launch per dimension
		for (int D = 2; D <= 3; ++D) {
			std::vector<InstBase *> g;
			for (InstBase *in : run) if (in->dim() == D && in->precision() == SA_PREC_FP64) g.push_back(in);
			if (g.empty()) continue;
			std::vector<BatchSolve> bs;
			for (InstBase *in : g) { in->prepare_velocity_fp64(); bs.push_back(in->velocity_fp64()); }
			join();
			batchLaunches[0] += D == 2 ? cg_batch_run<2, double, double, double>(bs, smCount, devJobs, kMaxJobs, s)
			                           : cg_batch_run<3, double, double, double>(bs, smCount, devJobs, kMaxJobs, s);
			fork();
			for (InstBase *in : g) in->finish_velocity_fp64();
			const std::vector<CgState> cs = states(g);
			for (size_t q = 0; q < g.size(); ++q) {
				g[q]->its = cs[q].iters;
				if (cs[q].code != SA_OK) fail(*g[q], cs[q].code);
			}
		}
		mark(1);
		// velocity: mixed precision, FP64 iterative refinement around batched FP32 solves
		for (int D = 2; D <= 3; ++D) {
			std::vector<InstBase *> g;
			for (InstBase *in : run) if (in->dim() == D && in->precision() == SA_PREC_MIXED) g.push_back(in);
			if (g.empty()) continue;
			std::stable_sort(g.begin(), g.end(), [](const InstBase *a, const InstBase *b) {
				return a->vel_key() > b->vel_key();
			});
			refine_mixed(g, kMixedVelocity, D);
			for (InstBase *in : g) in->its = in->mixedTotal;
		}
		mark(2);
		for (InstBase *in : run) if (!in->failed) in->post_velocity();
		// reaction-diffusion: one batched launch for the FP64 instances still running, the same FP64
		// refinement around batched FP32 solves for the mixed-precision ones
		std::vector<InstBase *> rd, rdMixed;
		for (InstBase *in : run)
			if (!in->failed) (in->precision() == SA_PREC_MIXED ? rdMixed : rd).push_back(in);
		if (!rd.empty()) {
			std::vector<BatchSolve> bs;
			for (InstBase *in : rd) { in->prepare_rd(); bs.push_back(in->rd_solve()); }
			join();
			batchLaunches[2] += cg_batch_run<1, double, double, double>(bs, smCount, devJobs, kMaxJobs, s);
			fork();
			for (InstBase *in : rd) in->finish_rd();
			const std::vector<CgState> cs = states(rd);
			for (size_t q = 0; q < rd.size(); ++q) {
				rd[q]->rits = cs[q].iters;
				if (cs[q].code != SA_OK) fail(*rd[q], cs[q].code);
			}
		}
		if (!rdMixed.empty()) {
			refine_mixed(rdMixed, kMixedRd, 1);
			for (InstBase *in : rdMixed) in->rits = in->mixedTotal;
		}
		mark(3);
		for (InstBase *in : run) {
			in->account(in->its, in->rits);
			if (!in->failed) in->end_step();
		}
		mark(4);
		++ticks;
	}

	void admit(std::unique_lock<std::mutex> &lk)
	{
		while (!queue.empty() && (int) active.size() < maxInst) {
			Request *r = queue.front();
			if (!active.empty() && inUse + r->estBytes > budget) break;     // wait for memory
			queue.pop_front();
			r->state = SA_REQ_RUNNING;
			r->tStart = std::chrono::steady_clock::now();
			lk.unlock();
			std::unique_ptr<InstBase> in;
			std::string err;
			int code = SA_OK;
			try {
				cudaStream_t is = pool[nextStream];
				nextStream = (nextStream + 1) % kInstStreams;
				if (r->dim == 2) in.reset(new Inst<2>(r, is));
				else in.reset(new Inst<3>(r, is));
			} catch (const ArgError &e) { code = SA_ERR_ARG; err = e.msg; }
			catch (const CudaError &e) { code = SA_ERR_CUDA; err = std::string(e.where) + ": " + cudaGetErrorString(e.e); cudaGetLastError(); }
			catch (const std::bad_alloc &) { code = SA_ERR_CUDA; err = "host allocation failed"; }
			lk.lock();
			if (!in) {
				r->status = code; r->err = err; r->state = SA_REQ_FAILED;
				r->tDone = std::chrono::steady_clock::now();
				++failedCount;
				cv.notify_all();
				continue;
			}
			inUse += in->bytes;
			peak = std::max(peak, inUse);
			active.push_back(std::move(in));
		}
	}

	void retire(std::unique_lock<std::mutex> &lk)
	{
		for (size_t k = 0; k < active.size();) {
			InstBase *in = active[k].get();
			if (!in->finished()) { ++k; continue; }
			Request *r = in->req;
			lk.unlock();
			std::string err;
			try { in->results(); }
			catch (const ArgError &e) { err = e.msg; }
			catch (const CudaError &e) { err = std::string(e.where) + ": " + cudaGetErrorString(e.e); cudaGetLastError(); }
			lk.lock();
			if (!err.empty() && r->err.empty()) { r->status = SA_ERR_CUDA; r->err = err; }
			bool ok = r->err.empty();
			r->state = ok ? SA_REQ_DONE : SA_REQ_FAILED;
			r->tDone = std::chrono::steady_clock::now();
			if (ok) ++completed; else ++failedCount;
			inUse -= in->bytes;
			active.erase(active.begin() + k);
			cv.notify_all();
		}
	}

	void loop()
	{
		cudaSetDevice(ctx->device);
		std::unique_lock<std::mutex> lk(mu);
		while (true) {
			if (stop && queue.empty() && active.empty()) break;
			admit(lk);
			if (active.empty()) {
				if (stop) break;
				cv.wait(lk, [this] { return stop || !queue.empty(); });
				continue;
			}
			lk.unlock();
			auto t0 = std::chrono::steady_clock::now();
			std::string err;
			int code = SA_OK;
			try { tick(); }
			catch (const CudaError &e) { code = SA_ERR_CUDA; err = std::string(e.where) + ": " + cudaGetErrorString(e.e); cudaGetLastError(); }
			catch (const DeviceWaitError &e) { code = SA_ERR_TIMEOUT; err = std::string(e.where) + ": a device-side wait gave up"; }
			catch (const ArgError &e) { code = SA_ERR_ARG; err = e.msg; }
			busyMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
			lk.lock();
			if (code != SA_OK) {             // an error, not a solve status: the running requests fail
				loopErr = err;
				for (auto &u : active)
					if (!u->finished()) { u->failed = 1; u->set_status(code); u->req->status = code; u->req->err = err; }
			}
			retire(lk);
		}
	}

	long long submit(int dim, const sa_element_object *o, const double *lmkIni, const sa_params *p,
	                 const sa_target *t, const double *tauVar, int tauVarNum)
	{
		SA_REQUIRE(o && lmkIni && p && tauVar, "missing argument");
		SA_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
		SA_REQUIRE(o->dim == dim, "element object dimension");
		SA_REQUIRE(p->elaType == SA_ELA_ISOTROPIC, "the server runs the layered model (elaType isotropic)");
		SA_REQUIRE(o->lmkNum > 0 && o->elmNum > 0 && o->nzrNum > 0 && p->timeNum >= 1, "empty problem");
		std::unique_ptr<Request> r(new Request);
		r->dim = dim;
		size_t N = o->lmkNum, E = o->elmNum, Z = o->nzrNum;
		copy_in(r->elmVtx, o->elmVtxMat, E * (dim + 1));
		copy_in(r->vtxElm, o->vtxElmMat, N * o->vtxElmCols);
		copy_in(r->btmVtx, o->btmVtxMat, (size_t) o->btmElmNum * dim);
		copy_in(r->vtxBtm, o->vtxBtmMat, (size_t) o->btmLmkNum * o->vtxBtmCols);
		copy_in(r->femVtx, o->femVtxMat, Z * 2);
		copy_in(r->femIfo, o->femIfoMat, Z * o->femIfoCols);
		copy_in(r->elmLyr, o->elmLyrVec, E);
		r->obj = *o;
		r->obj.elmVtxMat = r->elmVtx.data(); r->obj.vtxElmMat = r->vtxElm.data();
		r->obj.frmVtxMat = nullptr; r->obj.tsvVtxMat = nullptr; r->obj.bdrVtxMat = nullptr;
		r->obj.vtxBdrMat = nullptr; r->obj.vfdIfoMat = nullptr;
		r->obj.btmVtxMat = r->btmVtx.empty() ? nullptr : r->btmVtx.data();
		r->obj.vtxBtmMat = r->vtxBtm.empty() ? nullptr : r->vtxBtm.data();
		r->obj.femVtxMat = r->femVtx.data(); r->obj.femIfoMat = r->femIfo.data();
		r->obj.elmLyrVec = r->elmLyr.data();
		copy_in(r->lmk, lmkIni, N * dim);
		copy_in(r->tauVar, tauVar, (size_t) tauVarNum);
		r->prm = *p;
		copy_in(r->tauPrm, p->tauPrmVec, p->tauPrmVec ? (size_t) p->tauPrmNum : 0);
		copy_in(r->mod, p->modVec, (size_t) p->modNum);
		copy_in(r->spdLyr, p->spdLyrVec, (size_t) p->lyrNum);
		copy_in(r->ynk, p->ynkActPrmVec, 1);
		copy_in(r->rea, p->reaActPrmVec, 1);
		r->prm.tauPrmVec = r->tauPrm.empty() ? nullptr : r->tauPrm.data();
		r->prm.modVec = r->mod.data(); r->prm.spdLyrVec = r->spdLyr.data();
		r->prm.ynkActPrmVec = r->ynk.data(); r->prm.reaActPrmVec = r->rea.data();
		if (t) {
			r->hasTgt = true;
			size_t Vt = t->tgtElmNum, Vd = o->vfdElmNum;
			copy_in(r->vfdVtx, o->vfdVtxMat, Vd * dim);
			r->obj.vfdVtxMat = r->vfdVtx.data();
			copy_in(r->cen, t->cenPosMat, Vt * dim);
			copy_in(r->dir, t->uniDirMat, Vt * dim);
			copy_in(r->vol, t->elmVolVec, Vt);
			r->tgt = *t;
			r->tgt.cenPosMat = r->cen.data(); r->tgt.uniDirMat = r->dir.data(); r->tgt.elmVolVec = r->vol.data();
		} else {
			r->obj.vfdVtxMat = nullptr;
		}
		r->estBytes = estimate_bytes(*r);
		SA_REQUIRE(r->estBytes <= budget, "request larger than the server's device memory budget");
		r->tSubmit = std::chrono::steady_clock::now();
		std::lock_guard<std::mutex> g(mu);
		SA_REQUIRE(!stop, "server is stopping");
		long long id = nextId++;
		r->id = id;
		queue.push_back(r.get());
		reqs[id] = std::move(r);
		++submitted;
		cv.notify_all();
		return id;
	}
};

Tuning &tuning()
{
	static Tuning t;
	return t;
}

}  // namespace sa

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

int sa_create(sa_context **out, int device)
{
	if (!out) return SA_ERR_ARG;
	*out = nullptr;
	int count = 0;
	if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
		cudaGetLastError();
		return SA_ERR_CUDA;
	}
	sa_context *c = new sa_context();
	c->device = device;
	if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaEventCreate(&c->e0) != cudaSuccess || cudaEventCreate(&c->e1) != cudaSuccess ||
	    cudaEventCreateWithFlags(&c->sideIn, cudaEventDisableTiming) != cudaSuccess ||
	    cudaEventCreateWithFlags(&c->sideOut, cudaEventDisableTiming) != cudaSuccess) {
		cudaGetLastError();
		delete c;
		return SA_ERR_CUDA;
	}
	// the one-call entry points allocate their work buffers stream-ordered from the device's default
	// memory pool; by default the pool hands freed memory back to the driver at every synchronisation, so
	// each call mapped its ~0.5 GB again (tens of ms, varying from call to call).  Keep up to 4 GiB of
	// freed memory in the pool between calls.
	cudaMemPool_t mp;
	if (cudaDeviceGetDefaultMemPool(&mp, device) == cudaSuccess) {
		unsigned long long keep = 4ull << 30;
		cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep);
	}
	cudaGetLastError();
	*out = c;
	return SA_OK;
}

int sa_destroy(sa_context *c)
{
	if (!c) return SA_OK;
	cudaSetDevice(c->device);
	if (c->stream) cudaStreamSynchronize(c->stream);
	if (c->side) cudaStreamSynchronize(c->side);
	if (c->e0) cudaEventDestroy(c->e0);
	if (c->e1) cudaEventDestroy(c->e1);
	if (c->sideIn) cudaEventDestroy(c->sideIn);
	if (c->sideOut) cudaEventDestroy(c->sideOut);
	if (c->stream) cudaStreamDestroy(c->stream);
	if (c->side) cudaStreamDestroy(c->side);
	delete c;
	return SA_OK;
}

const char *sa_error_message(const sa_context *c) { return c ? c->err.c_str() : "no context"; }

int sa_forward(sa_context *ctx, const sa_element_object *obj, const double *lmkIniMat, const sa_params *prm,
               const sa_target *tgt, const double *tauVarMat, int tauVarNum, int objNum, double *lmkStk,
               double *tauMat, double *objVec, sa_solve_info *info)
{
	return sa::guarded(ctx, [&]() {
		SA_REQUIRE(obj && prm && lmkIniMat, "null argument");
		if (obj->dim == 2)
			return sa::forward_impl<2>(ctx, obj, lmkIniMat, prm, tgt, tauVarMat, tauVarNum, objNum, lmkStk, tauMat,
			                           objVec, info);
		SA_REQUIRE(obj->dim == 3, "dim must be 2 or 3");
		return sa::forward_impl<3>(ctx, obj, lmkIniMat, prm, tgt, tauVarMat, tauVarNum, objNum, lmkStk, tauMat,
		                           objVec, info);
	});
}

int sa_varifold(sa_context *ctx, const sa_element_object *obj, const double *lmkMat, const sa_target *tgt,
                int precision, double *objOut, double *gradMat)
{
	return sa::guarded(ctx, [&]() {
		SA_REQUIRE(obj && lmkMat && objOut, "null argument");
		if (obj->dim == 2) return sa::varifold_impl<2>(ctx, obj, lmkMat, tgt, precision, objOut, gradMat);
		SA_REQUIRE(obj->dim == 3, "dim must be 2 or 3");
		return sa::varifold_impl<3>(ctx, obj, lmkMat, tgt, precision, objOut, gradMat);
	});
}

struct sa_session {
	sa::SessionBase *impl;
};

int sa_session_create(sa_context *ctx, const sa_element_object *obj, const double *lmkIniMat, const sa_params *prm,
                      const sa_target *tgt, const double *tauVarVec, int tauVarNum, sa_session **out)
{
	if (!out) return SA_ERR_ARG;
	*out = nullptr;
	return sa::guarded(ctx, [&]() {
		SA_REQUIRE(obj && prm && lmkIniMat, "null argument");
		sa::SessionBase *impl;
		if (obj->dim == 2) impl = new sa::Session<2>(ctx, obj, lmkIniMat, prm, tgt, tauVarVec, tauVarNum);
		else {
			SA_REQUIRE(obj->dim == 3, "dim must be 2 or 3");
			impl = new sa::Session<3>(ctx, obj, lmkIniMat, prm, tgt, tauVarVec, tauVarNum);
		}
		*out = new sa_session{impl};
		return SA_OK;
	});
}

int sa_session_step(sa_session *s, int nsteps, int *stepsDone)
{
	if (!s) return SA_ERR_ARG;
	return sa::guarded(s->impl->ctx, [&]() {
		int k = s->impl->step(nsteps);
		if (stepsDone) *stepsDone = k;
		return SA_OK;
	});
}

int sa_objective_gradient(sa_context *ctx, const sa_element_object *obj, const double *lmkIniMat,
                          const sa_params *prm, const sa_target *tgt, const double *tauVarVec, int tauVarNum,
                          double *objOut, double *gradOut, sa_solve_info *info)
{
	if (!ctx || !obj || !prm) return SA_ERR_ARG;
	return sa::guarded(ctx, [&]() {
		if (obj->dim == 2)
			return sa::gradient_impl<2>(ctx, obj, lmkIniMat, prm, tgt, tauVarVec, tauVarNum, objOut, gradOut, info);
		SA_REQUIRE(obj->dim == 3, "dim must be 2 or 3");
		return sa::gradient_impl<3>(ctx, obj, lmkIniMat, prm, tgt, tauVarVec, tauVarNum, objOut, gradOut, info);
	});
}

int sa_objective_adjoint(sa_context *ctx, const sa_element_object *obj, const double *lmkIniMat, const sa_params *prm,
                         const sa_target *tgt, const double *tauVarVec, int tauVarNum, double *objOut,
                         double *gradBump, double *gradLayer, double *gradTau0, double *gradX0, sa_solve_info *info)
{
	if (!obj || !lmkIniMat || !prm || !tgt || !tauVarVec) return SA_ERR_ARG;
	return sa::guarded(ctx, [&]() {
		if (obj->dim == 2)
			return sa::adjoint_impl<2>(ctx, obj, lmkIniMat, prm, tgt, tauVarVec, tauVarNum, objOut, gradBump,
			                           gradLayer, gradTau0, gradX0, info);
		SA_REQUIRE(obj->dim == 3, "dim must be 2 or 3");
		return sa::adjoint_impl<3>(ctx, obj, lmkIniMat, prm, tgt, tauVarVec, tauVarNum, objOut, gradBump, gradLayer,
		                           gradTau0, gradX0, info);
	});
}

int sa_session_stream(sa_session *s, int nsteps, int stride, double *lmkOut, double *tauOut, int maxSnapshots,
                      int *snapshotsWritten, int *stepsDone)
{
	if (!s) return SA_ERR_ARG;
	return sa::guarded(s->impl->ctx, [&]() {
		int k = s->impl->stream(nsteps, stride, lmkOut, tauOut, maxSnapshots, snapshotsWritten);
		if (stepsDone) *stepsDone = k;
		return SA_OK;
	});
}

int sa_session_state(sa_session *s, double *lmkMat, double *tauVec, int *step)
{
	if (!s) return SA_ERR_ARG;
	return sa::guarded(s->impl->ctx, [&]() { s->impl->state(lmkMat, tauVec, step); return SA_OK; });
}

int sa_session_objective(sa_session *s, double *obj)
{
	if (!s || !obj) return SA_ERR_ARG;
	return sa::guarded(s->impl->ctx, [&]() { *obj = s->impl->objective(); return SA_OK; });
}

int sa_session_info(sa_session *s, sa_solve_info *info)
{
	if (!s || !info) return SA_ERR_ARG;
	return sa::guarded(s->impl->ctx, [&]() { s->impl->info(info); return SA_OK; });
}

int sa_session_profile(sa_session *s, int enable, double *kernelMs, long long *launches, double *bytes,
                       double *flops)
{
	if (!s || !s->impl) return SA_ERR_ARG;
	return sa::guarded(s->impl->ctx, [&]() { s->impl->profile(enable, kernelMs, launches, bytes, flops); return SA_OK; });
}

int sa_session_destroy(sa_session *s)
{
	if (!s) return SA_OK;
	cudaSetDevice(s->impl->ctx->device);
	cudaStreamSynchronize(s->impl->ctx->stream);
	delete s->impl;
	delete s;
	return SA_OK;
}

static void frame_object(sa_element_object &o, int dim, int lmkNum, const int *elmVtxMat, int elmNum,
                         const int *vtxElmMat, int vtxElmCols, const int *frmVtxMat, const int *tsvVtxMat,
                         const int *bdrVtxMat, int bdrElmNum, const int *vtxBdrMat, int vtxBdrCols,
                         const int *btmVtxMat, int btmElmNum, const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols,
                         const int *femVtxMat, int nzrNum, const int *femIfoMat, int femIfoCols)
{
	memset(&o, 0, sizeof(o));
	o.dim = dim; o.lmkNum = lmkNum; o.elmNum = elmNum;
	o.elmVtxMat = elmVtxMat; o.vtxElmMat = vtxElmMat; o.vtxElmCols = vtxElmCols;
	o.frmVtxMat = frmVtxMat; o.tsvVtxMat = tsvVtxMat;
	o.bdrVtxMat = bdrVtxMat; o.bdrElmNum = bdrElmNum; o.vtxBdrMat = vtxBdrMat; o.vtxBdrCols = vtxBdrCols;
	o.btmVtxMat = btmVtxMat; o.btmElmNum = btmElmNum; o.vtxBtmMat = vtxBtmMat; o.btmLmkNum = btmLmkNum;
	o.vtxBtmCols = vtxBtmCols; o.femVtxMat = femVtxMat; o.nzrNum = nzrNum; o.femIfoMat = femIfoMat;
	o.femIfoCols = femIfoCols;
}

static void frame_params(sa_params &p, int dim, const double *tauPrmVec, int tauPrmNum, double ldmWgt, int knlOrder,
                         double knlWidth, double knlEps, const double *modVec, double spdTanVal, double spdTsvVal,
                         const double *ynk, const double *rea, double btmWgt, double timeStp, int timeNum,
                         int cgItrMax, double cgTolSqu)
{
	memset(&p, 0, sizeof(p));
	p.elaType = SA_ELA_FRAME; p.precision = SA_PREC_FP64;
	p.tauPrmVec = tauPrmVec; p.tauPrmNum = tauPrmNum;
	p.ldmWgt = ldmWgt; p.knlOrder = knlOrder; p.knlWidth = knlWidth; p.knlEps = knlEps;
	p.modVec = modVec; p.modNum = dim == 2 ? 3 : 4;
	p.spdTanVal = spdTanVal; p.spdTsvVal = spdTsvVal;
	p.ynkActPrmVec = ynk; p.reaActPrmVec = rea;
	p.btmWgt = btmWgt; p.timeStp = timeStp; p.timeNum = timeNum; p.cgItrMax = cgItrMax; p.cgTolSqu = cgTolSqu;
}

int sa_deformation_frame(sa_context *ctx, int dim, const double *tauVarMat, int tauVarNum, int objTotNum,
                         const double *tauPrmVec, int tauPrmNum, const double *lmkIniMat, int lmkNum,
                         const int *elmVtxMat, int elmNum, const int *vtxElmMat, int vtxElmCols,
                         const int *frmVtxMat, const int *tsvVtxMat, const int *bdrVtxMat, int bdrElmNum,
                         const int *vtxBdrMat, int vtxBdrCols, const int *btmVtxMat, int btmElmNum,
                         const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols, const int *femVtxMat, int nzrNum,
                         const int *femIfoMat, int femIfoCols, double ldmWgt, int knlOrder, double knlWidth,
                         double knlEps, const double *modVec, double spdTanVal, double spdTsvVal,
                         const double *ynkActPrmVec, const double *reaActPrmVec, double btmWgt, double timeStp,
                         int timeNum, int cgItrMax, double cgTolSqu, double *lmkStk, double *tauMat, double *objVec)
{
	sa_element_object o;
	frame_object(o, dim, lmkNum, elmVtxMat, elmNum, vtxElmMat, vtxElmCols, frmVtxMat, tsvVtxMat, bdrVtxMat,
	             bdrElmNum, vtxBdrMat, vtxBdrCols, btmVtxMat, btmElmNum, vtxBtmMat, btmLmkNum, vtxBtmCols,
	             femVtxMat, nzrNum, femIfoMat, femIfoCols);
	sa_params p;
	frame_params(p, dim, tauPrmVec, tauPrmNum, ldmWgt, knlOrder, knlWidth, knlEps, modVec, spdTanVal, spdTsvVal,
	             ynkActPrmVec, reaActPrmVec, btmWgt, timeStp, timeNum, cgItrMax, cgTolSqu);
	return sa_forward(ctx, &o, lmkIniMat, &p, nullptr, tauVarMat, tauVarNum, objTotNum, lmkStk, tauMat, objVec,
	                  nullptr);
}

int sa_computeObjfcn_frame(sa_context *ctx, int dim, const double *tauVarMat, int tauVarNum, int objTotNum,
                           const double *tauPrmVec, int tauPrmNum, const double *lmkIniMat, int lmkNum,
                           const int *elmVtxMat, int elmNum, const int *vtxElmMat, int vtxElmCols,
                           const int *frmVtxMat, const int *tsvVtxMat, const int *bdrVtxMat, int bdrElmNum,
                           const int *vtxBdrMat, int vtxBdrCols, const int *btmVtxMat, int btmElmNum,
                           const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols, const int *femVtxMat, int nzrNum,
                           const int *femIfoMat, int femIfoCols, const int *vfdVtxMat, int vfdElmNum,
                           const double *tgtCenPosMat, const double *tgtUniDirMat, const double *tgtElmVolVec,
                           int tgtElmNum, double cenKnlType, double cenKnlWidth, double dirKnlType,
                           double dirKnlWidth, double ldmWgt, int knlOrder, double knlWidth, double knlEps,
                           const double *modVec, double spdTanVal, double spdTsvVal, const double *ynkActPrmVec,
                           const double *reaActPrmVec, double btmWgt, double timeStp, int timeNum, int cgItrMax,
                           double cgTolSqu, double *objVec)
{
	sa_element_object o;
	frame_object(o, dim, lmkNum, elmVtxMat, elmNum, vtxElmMat, vtxElmCols, frmVtxMat, tsvVtxMat, bdrVtxMat,
	             bdrElmNum, vtxBdrMat, vtxBdrCols, btmVtxMat, btmElmNum, vtxBtmMat, btmLmkNum, vtxBtmCols,
	             femVtxMat, nzrNum, femIfoMat, femIfoCols);
	o.vfdVtxMat = vfdVtxMat;
	o.vfdElmNum = vfdElmNum;
	sa_params p;
	frame_params(p, dim, tauPrmVec, tauPrmNum, ldmWgt, knlOrder, knlWidth, knlEps, modVec, spdTanVal, spdTsvVal,
	             ynkActPrmVec, reaActPrmVec, btmWgt, timeStp, timeNum, cgItrMax, cgTolSqu);
	sa_target t;
	memset(&t, 0, sizeof(t));
	t.cenPosMat = tgtCenPosMat; t.uniDirMat = tgtUniDirMat; t.elmVolVec = tgtElmVolVec; t.tgtElmNum = tgtElmNum;
	t.cenKnlType = (char) cenKnlType; t.cenKnlWidth = cenKnlWidth;
	t.dirKnlType = (char) dirKnlType; t.dirKnlWidth = dirKnlWidth;
	return sa_forward(ctx, &o, lmkIniMat, &p, &t, tauVarMat, tauVarNum, objTotNum, nullptr, nullptr, objVec,
	                  nullptr);
}


// The layered (isotropic) model behind the positional surface of the frame entry points: the branch
// CUDA/deformation.m:12-13,22-24 and CUDA/computeObjfcn.m:12-13,22-24 leave empty.  modMat is the wrapper's
// d_modMat = reshape(h_modVec, 2, [])' (lyrNum x 2, column-major: lambda in column 0, mu in column 1, host or
// device memory); the library's parameter table interleaves (lambda, mu) per layer.
static int isotropic_params(sa_params &p, std::vector<double> &mod, const double *tauPrmVec, int tauPrmNum,
                            double ldmWgt, int knlOrder, double knlWidth, double knlEps, const double *modMat,
                            int lyrNum, const double *spdLyrVec, const double *ynk, const double *rea,
                            double btmWgt, double timeStp, int timeNum, int cgItrMax, double cgTolSqu)
{
	if (lyrNum <= 0 || !modMat || !spdLyrVec) return SA_ERR_ARG;
	std::vector<double> cm((size_t) 2 * lyrNum);
	if (cudaMemcpy(cm.data(), modMat, sizeof(double) * cm.size(), cudaMemcpyDefault) != cudaSuccess) {
		cudaGetLastError();
		return SA_ERR_ARG;
	}
	mod.resize(cm.size());
	for (int l = 0; l < lyrNum; ++l) { mod[2 * l] = cm[l]; mod[2 * l + 1] = cm[lyrNum + l]; }
	memset(&p, 0, sizeof(p));
	p.elaType = SA_ELA_ISOTROPIC; p.precision = SA_PREC_FP64;
	p.tauPrmVec = tauPrmVec; p.tauPrmNum = tauPrmNum;
	p.ldmWgt = ldmWgt; p.knlOrder = knlOrder; p.knlWidth = knlWidth; p.knlEps = knlEps;
	p.modVec = mod.data(); p.modNum = 2 * lyrNum;
	p.spdLyrVec = spdLyrVec; p.lyrNum = lyrNum;
	p.ynkActPrmVec = ynk; p.reaActPrmVec = rea;
	p.btmWgt = btmWgt; p.timeStp = timeStp; p.timeNum = timeNum; p.cgItrMax = cgItrMax; p.cgTolSqu = cgTolSqu;
	p.cgKernel = SA_CG_AUTO;
	p.velocityGuess = SA_GUESS_DEFAULT;
	return SA_OK;
}

int sa_deformation_isotropic(sa_context *ctx, int dim, const double *tauVarMat, int tauVarNum, int objTotNum,
                             const double *tauPrmVec, int tauPrmNum, const double *lmkIniMat, int lmkNum,
                             const int *elmVtxMat, int elmNum, const int *vtxElmMat, int vtxElmCols,
                             const int *frmVtxMat, const int *tsvVtxMat, const int *bdrVtxMat, int bdrElmNum,
                             const int *vtxBdrMat, int vtxBdrCols, const int *btmVtxMat, int btmElmNum,
                             const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols, const int *femVtxMat,
                             int nzrNum, const int *femIfoMat, int femIfoCols, const int *elmLyrVec,
                             double ldmWgt, int knlOrder, double knlWidth, double knlEps, const double *modMat,
                             int lyrNum, const double *spdLyrVec, const double *ynkActPrmVec,
                             const double *reaActPrmVec, double btmWgt, double timeStp, int timeNum, int cgItrMax,
                             double cgTolSqu, double *lmkStk, double *tauMat, double *objVec)
{
	sa_element_object o;
	frame_object(o, dim, lmkNum, elmVtxMat, elmNum, vtxElmMat, vtxElmCols, frmVtxMat, tsvVtxMat, bdrVtxMat,
	             bdrElmNum, vtxBdrMat, vtxBdrCols, btmVtxMat, btmElmNum, vtxBtmMat, btmLmkNum, vtxBtmCols,
	             femVtxMat, nzrNum, femIfoMat, femIfoCols);
	o.elmLyrVec = elmLyrVec;
	sa_params p;
	std::vector<double> mod;
	int rc = isotropic_params(p, mod, tauPrmVec, tauPrmNum, ldmWgt, knlOrder, knlWidth, knlEps, modMat, lyrNum,
	                          spdLyrVec, ynkActPrmVec, reaActPrmVec, btmWgt, timeStp, timeNum, cgItrMax, cgTolSqu);
	if (rc != SA_OK) return rc;
	return sa_forward(ctx, &o, lmkIniMat, &p, nullptr, tauVarMat, tauVarNum, objTotNum, lmkStk, tauMat, objVec,
	                  nullptr);
}

int sa_computeObjfcn_isotropic(sa_context *ctx, int dim, const double *tauVarMat, int tauVarNum, int objTotNum,
                               const double *tauPrmVec, int tauPrmNum, const double *lmkIniMat, int lmkNum,
                               const int *elmVtxMat, int elmNum, const int *vtxElmMat, int vtxElmCols,
                               const int *frmVtxMat, const int *tsvVtxMat, const int *bdrVtxMat, int bdrElmNum,
                               const int *vtxBdrMat, int vtxBdrCols, const int *btmVtxMat, int btmElmNum,
                               const int *vtxBtmMat, int btmLmkNum, int vtxBtmCols, const int *femVtxMat,
                               int nzrNum, const int *femIfoMat, int femIfoCols, const int *elmLyrVec,
                               const int *vfdVtxMat, int vfdElmNum, const double *tgtCenPosMat,
                               const double *tgtUniDirMat, const double *tgtElmVolVec, int tgtElmNum,
                               double cenKnlType, double cenKnlWidth, double dirKnlType, double dirKnlWidth,
                               double ldmWgt, int knlOrder, double knlWidth, double knlEps, const double *modMat,
                               int lyrNum, const double *spdLyrVec, const double *ynkActPrmVec,
                               const double *reaActPrmVec, double btmWgt, double timeStp, int timeNum,
                               int cgItrMax, double cgTolSqu, double *objVec)
{
	sa_element_object o;
	frame_object(o, dim, lmkNum, elmVtxMat, elmNum, vtxElmMat, vtxElmCols, frmVtxMat, tsvVtxMat, bdrVtxMat,
	             bdrElmNum, vtxBdrMat, vtxBdrCols, btmVtxMat, btmElmNum, vtxBtmMat, btmLmkNum, vtxBtmCols,
	             femVtxMat, nzrNum, femIfoMat, femIfoCols);
	o.elmLyrVec = elmLyrVec;
	o.vfdVtxMat = vfdVtxMat;
	o.vfdElmNum = vfdElmNum;
	sa_params p;
	std::vector<double> mod;
	int rc = isotropic_params(p, mod, tauPrmVec, tauPrmNum, ldmWgt, knlOrder, knlWidth, knlEps, modMat, lyrNum,
	                          spdLyrVec, ynkActPrmVec, reaActPrmVec, btmWgt, timeStp, timeNum, cgItrMax, cgTolSqu);
	if (rc != SA_OK) return rc;
	sa_target t;
	memset(&t, 0, sizeof(t));
	t.cenPosMat = tgtCenPosMat; t.uniDirMat = tgtUniDirMat; t.elmVolVec = tgtElmVolVec; t.tgtElmNum = tgtElmNum;
	t.cenKnlType = (char) cenKnlType; t.cenKnlWidth = cenKnlWidth;
	t.dirKnlType = (char) dirKnlType; t.dirKnlWidth = dirKnlWidth;
	return sa_forward(ctx, &o, lmkIniMat, &p, &t, tauVarMat, tauVarNum, objTotNum, nullptr, nullptr, objVec,
	                  nullptr);
}

// ---------------------------------------------------------------------------
// serving
// ---------------------------------------------------------------------------
struct sa_server {
	sa_context *ctx;
	sa::Server *impl;
	std::string err;
};

int sa_server_create(sa_context *ctx, double hbmBudgetBytes, int maxInstances, sa_server **out)
{
	if (!out) return SA_ERR_ARG;
	*out = nullptr;
	return sa::guarded(ctx, [&]() {
		SA_REQUIRE(hbmBudgetBytes > 0.0 && maxInstances > 0, "budget and instance limit must be positive");
		std::unique_ptr<sa_server> sv(new sa_server{ctx, nullptr, std::string()});
		sv->impl = new sa::Server(ctx, (size_t) hbmBudgetBytes, maxInstances);
		*out = sv.release();
		return SA_OK;
	});
}

int sa_server_submit(sa_server *sv, const sa_element_object *obj, const double *lmkIniMat, const sa_params *prm,
                     const sa_target *tgt, const double *tauVarVec, int tauVarNum, long long *requestId)
{
	if (!sv || !requestId || !obj) return SA_ERR_ARG;
	return sa::guarded(sv->ctx, [&]() {
		*requestId = sv->impl->submit(obj->dim, obj, lmkIniMat, prm, tgt, tauVarVec, tauVarNum);
		return SA_OK;
	});
}

int sa_server_poll(sa_server *sv, long long requestId, int *state)
{
	if (!sv || !state) return SA_ERR_ARG;
	std::lock_guard<std::mutex> g(sv->impl->mu);
	auto it = sv->impl->reqs.find(requestId);
	if (it == sv->impl->reqs.end()) return SA_ERR_ARG;
	*state = it->second->state;
	return SA_OK;
}

int sa_server_wait(sa_server *sv, long long requestId, double timeoutMs, int *state)
{
	if (!sv || !state) return SA_ERR_ARG;
	sa::Server &S = *sv->impl;
	std::unique_lock<std::mutex> lk(S.mu);
	auto it = S.reqs.find(requestId);
	if (it == S.reqs.end()) return SA_ERR_ARG;
	sa::Request *r = it->second.get();
	auto done = [r] { return r->state == SA_REQ_DONE || r->state == SA_REQ_FAILED; };
	if (timeoutMs < 0) S.cv.wait(lk, done);
	else S.cv.wait_for(lk, std::chrono::duration<double, std::milli>(timeoutMs), done);
	*state = r->state;
	return SA_OK;
}

int sa_server_result(sa_server *sv, long long requestId, double *lmkMat, double *tauVec, double *objOut,
                     sa_solve_info *info, double *latencyMs)
{
	if (!sv) return SA_ERR_ARG;
	sa::Server &S = *sv->impl;
	std::unique_ptr<sa::Request> r;
	{
		std::lock_guard<std::mutex> g(S.mu);
		auto it = S.reqs.find(requestId);
		if (it == S.reqs.end()) return SA_ERR_ARG;
		if (it->second->state != SA_REQ_DONE && it->second->state != SA_REQ_FAILED) return SA_ERR_ARG;
		r = std::move(it->second);
		S.reqs.erase(it);
	}
	if (r->state == SA_REQ_FAILED) {
		sv->ctx->err = r->err;
		if (latencyMs) *latencyMs = std::chrono::duration<double, std::milli>(r->tDone - r->tSubmit).count();
		return r->status != SA_OK ? r->status : SA_ERR_CUDA;
	}
	if (lmkMat && !r->lmkOut.empty()) memcpy(lmkMat, r->lmkOut.data(), sizeof(double) * r->lmkOut.size());
	if (tauVec && !r->tauOut.empty()) memcpy(tauVec, r->tauOut.data(), sizeof(double) * r->tauOut.size());
	if (objOut) *objOut = r->objOut;
	if (info) {
		*info = r->info;
		info->elapsedMs = std::chrono::duration<double, std::milli>(r->tDone - r->tStart).count();
	}
	if (latencyMs) *latencyMs = std::chrono::duration<double, std::milli>(r->tDone - r->tSubmit).count();
	return SA_OK;
}

int sa_server_stats(sa_server *sv, sa_server_counters *st)
{
	if (!sv || !st) return SA_ERR_ARG;
	sa::Server &S = *sv->impl;
	std::lock_guard<std::mutex> g(S.mu);
	st->submitted = S.submitted;
	st->completed = S.completed;
	st->failed = S.failedCount;
	st->queued = (int) S.queue.size();
	st->running = (int) S.active.size();
	st->bytesInUse = (double) S.inUse;
	st->peakBytes = (double) S.peak;
	st->ticks = S.ticks;
	st->busyMs = S.busyMs;
	return SA_OK;
}

int sa_server_destroy(sa_server *sv)
{
	if (!sv) return SA_OK;
	delete sv->impl;
	delete sv;
	return SA_OK;
}


int sa_selftest_wait_timeout(sa_context *ctx, int *ctasGaveUp, double *elapsedMs)
{
	if (!ctasGaveUp) return SA_ERR_ARG;
	return sa::guarded(ctx, [&]() {
		int gave = 0, abortFlag = 0;
		auto t0 = std::chrono::steady_clock::now();
		int rc = sa::barrier_selftest(ctx->stream, &gave, &abortFlag);
		if (elapsedMs) *elapsedMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
		*ctasGaveUp = gave;
		if (rc != SA_OK) return rc;
		SA_REQUIRE(abortFlag == 1, "the poisoned barrier did not record an abort");
		return SA_OK;
	});
}

int sa_selftest_fma_peak(sa_context *ctx, int fp64, double *tflops, double *flopsPerClockSm, double *smMhz)
{
	if (!tflops) return SA_ERR_ARG;
	return sa::guarded(ctx, [&]() {
		return sa::fma_peak_selftest(ctx->stream, fp64 ? 1 : 0, tflops, flopsPerClockSm, smMhz);
	});
}

int sa_selftest_math(sa_context *ctx, int fn, long n, const double *x, double *y, double *yref)
{
	if (fn < 0 || fn > 1 || n < 0 || (n > 0 && (!x || !y || !yref))) return SA_ERR_ARG;
	return sa::guarded(ctx, [&]() {
		if (n == 0) return SA_OK;
		double *d = nullptr;
		cudaStream_t s = ctx->stream;
		SA_CHECK(cudaMallocAsync(&d, sizeof(double) * 3 * n, s));
		SA_CHECK(cudaMemcpyAsync(d, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
		sa::math_check(fn, n, d, d + n, d + 2 * n, s);
		SA_CHECK(cudaMemcpyAsync(y, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
		SA_CHECK(cudaMemcpyAsync(yref, d + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
		SA_CHECK(cudaFreeAsync(d, s));
		SA_CHECK(cudaStreamSynchronize(s));
		return SA_OK;
	});
}


int sa_set_tuning(const char *name, int value)
{
	if (!name) return SA_ERR_ARG;
	sa::Tuning &t = sa::tuning();
	std::string n(name);
	if (n == "persistMaxWarps" && value >= 1 && value <= 20) t.persistMaxWarps = value;
	else if (n == "batchBlock" && (value == 128 || value == 256)) t.batchBlock = value;
	else if (n == "batchSlicesPerWarp" && value >= 1 && value <= 16) t.batchSlicesPerWarp = value;
	else if (n == "vfdCtasPerSm" && value >= 1 && value <= 32) t.vfdCtasPerSm = value;
	else if (n == "mixedInnerFloor" && value >= 4 && value <= 16) t.mixedInnerFloor = value;
	else if (n == "kernelMatrixFree" && (value == 0 || value == 1)) t.kernelMatrixFree = value;
	else return SA_ERR_ARG;
	return SA_OK;
}

int sa_device_name(int device, char *buf, int len, int *smCount)
{
	if (!buf || len < 1) return SA_ERR_ARG;
	cudaDeviceProp prop;
	if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
		cudaGetLastError();
		return SA_ERR_CUDA;
	}
	std::snprintf(buf, (size_t) len, "%s", prop.name);
	if (smCount) *smCount = prop.multiProcessorCount;
	return SA_OK;
}

int sa_get_tuning(const char *name, int *value)
{
	if (!name || !value) return SA_ERR_ARG;
	const sa::Tuning &t = sa::tuning();
	std::string n(name);
	if (n == "persistMaxWarps") *value = t.persistMaxWarps;
	else if (n == "batchBlock") *value = t.batchBlock;
	else if (n == "batchSlicesPerWarp") *value = t.batchSlicesPerWarp;
	else if (n == "vfdCtasPerSm") *value = t.vfdCtasPerSm;
	else if (n == "mixedInnerFloor") *value = t.mixedInnerFloor;
	else if (n == "kernelMatrixFree") *value = t.kernelMatrixFree;
	else return SA_ERR_ARG;
	return SA_OK;
}

}  // extern "C"
