// sa_builder.cu -- element-object builders in C++ (host code).
//
// The reference builds element objects in MATLAB (CUDA/generateElementObject2D.m,
// CUDA/generateElementObject3D.m, CUDA/tri2tetra.m) with find-per-node loops
// that are O(E * nzr).  These builders produce the same arrays in O(E log E):
//
//   tri2tetra                   tri2tetra.m:1-69 (3 tets per prism, the
//                               circshift label cases, nml/tsv vertex lists)
//   element object 2D           generateElementObject2D.m:1-150 (plus a
//                               periodic ring option for annuli)
//   element object 3D           generateElementObject3D.m:1-127
//
// Orders kept: adjacency lists in MATLAB's column-major find order (entity
// ascending, then local index); femVtxMat sorted by (row, col) (sortrows);
// femIfoMat per nonzero lists the contributing elements in ascending order
// with the packed element-matrix index pair * E + e of glbIdxMat (upper-
// triangle pair enumeration (1,1),(1,2),...); freeBoundary faces in the order
// (dropped local vertex, element).  Arrays are column-major "R x C" int32,
// 0-based, exactly as the reference's gateways receive them.
#include "sa_internal.cuh"
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

struct sa_elmobj {
	int dim = 0, N = 0, E = 0, V = 0;
	int lyrLmkNum = 0, lyrCntNum = 0, elmPerLayer = 0;
	std::vector<int> elmVtx, vtxElm, frmVtx, tsvVtx, bdrVtx, vtxBdr, btmVtx, vtxBtm, femVtx, femIfo, vfdVtx, vfdIfo;
	int vtxElmCols = 0, vtxBdrCols = 0, vtxBtmCols = 0, femIfoCols = 0, vfdIfoCols = 0;
	int bdrNum = 0, btmNum = 0, btmLmkNum = 0, nzr = 0, vfdNum = 0;
};

namespace sa {
namespace {

struct BuildError { std::string msg; };
#define SB_REQUIRE(c, m) do { if (!(c)) throw ::sa::BuildError{m}; } while (0)

// [lcl, ent] = find(idx == n) for every node n: idx is k x m (entry (l, e) at l * m + e);
// returns the (num) x (1 + 2 maxCnt) column-major matrix and its column count
std::vector<int> adjacency(const std::vector<int> &idx, int k, int m, int num, int *cols)
{
	std::vector<int> cnt(num, 0);
	for (int e = 0; e < m; ++e)
		for (int l = 0; l < k; ++l) {
			int n = idx[(size_t) l * m + e];
			SB_REQUIRE(n >= 0 && n < num, "index out of range");
			++cnt[n];
		}
	int maxc = 0;
	for (int c : cnt) maxc = std::max(maxc, c);
	*cols = 1 + 2 * maxc;
	std::vector<int> out((size_t) num * *cols, 0), fill(num, 0);
	for (int n = 0; n < num; ++n) out[n] = cnt[n];
	for (int e = 0; e < m; ++e)                 // entity ascending, then local index: find's order
		for (int l = 0; l < k; ++l) {
			int n = idx[(size_t) l * m + e], r = fill[n]++;
			out[(size_t) (1 + 2 * r) * num + n] = e;
			out[(size_t) (2 + 2 * r) * num + n] = l;
		}
	return out;
}

// faces used by exactly one element (freeBoundary), in (dropped local vertex, element) order
std::vector<int> free_boundary(const std::vector<int> &elm, int V, int E, int N, int *F)
{
	const int k = V - 1;
	auto key_of = [&](int drop, int e) {
		int v[3];
		int j = 0;
		for (int l = 0; l < V; ++l)
			if (l != drop) v[j++] = elm[(size_t) l * E + e];
		std::sort(v, v + k);
		unsigned long long key = 0;
		for (int t = 0; t < k; ++t) key = key * (unsigned long long) N + (unsigned long long) v[t];
		return key;
	};
	// occurrence count per face: open-addressing table (linear probing), keys + 1 so that 0 marks empty
	size_t cap = 1;
	while (cap < (size_t) 2 * V * E) cap <<= 1;
	std::vector<unsigned long long> tk(cap, 0);
	std::vector<unsigned char> tc(cap, 0);
	auto slot_of = [&](unsigned long long key) {
		size_t h = (size_t) ((key + 1) * 0x9E3779B97F4A7C15ull) & (cap - 1);
		while (tk[h] != 0 && tk[h] != key + 1) h = (h + 1) & (cap - 1);
		return h;
	};
	for (int d = 0; d < V; ++d)
		for (int e = 0; e < E; ++e) {
			unsigned long long key = key_of(d, e);
			size_t h = slot_of(key);
			tk[h] = key + 1;
			if (tc[h] < 255) ++tc[h];
		}
	std::vector<int> faces;
	int nf = 0;
	for (int d = 0; d < V; ++d)
		for (int e = 0; e < E; ++e)
			if (tc[slot_of(key_of(d, e))] == 1) {
				for (int l = 0; l < V; ++l)
					if (l != d) faces.push_back(elm[(size_t) l * E + e]);
				++nf;
			}
	*F = nf;
	std::vector<int> out((size_t) k * nf);          // k x F (entry (l, f) at l * F + f)
	for (int f = 0; f < nf; ++f)
		for (int l = 0; l < k; ++l) out[(size_t) l * nf + f] = faces[(size_t) f * k + l];
	return out;
}

// femVtxMat and femIfoMat (generateElementObject2D.m:98-126, 3D :62-104)
void fem_pattern(sa_elmobj &o)
{
	const int V = o.V, E = o.E, N = o.N;
	// pattern: every node with itself and with the nodes it shares an element with, columns sorted
	std::vector<int> cnt(N, 0);
	for (size_t t = 0; t < o.elmVtx.size(); ++t) ++cnt[o.elmVtx[t]];
	int maxAdj = 0;
	for (int c : cnt) maxAdj = std::max(maxAdj, c);
	std::vector<long> rowPtr(N + 1, 0);
	std::vector<int> cols;
	// elements of each node, ascending (column-major find order)
	std::vector<int> start(N + 1, 0), list((size_t) E * V);
	for (int n = 0; n < N; ++n) start[n + 1] = start[n] + cnt[n];
	{
		std::vector<int> fill(start.begin(), start.end() - 1);
		for (int e = 0; e < E; ++e)
			for (int l = 0; l < V; ++l) list[fill[o.elmVtx[(size_t) l * E + e]]++] = e;
	}
	{
		std::vector<int> nb;
		for (int n = 0; n < N; ++n) {
			nb.clear();
			for (int t = start[n]; t < start[n + 1]; ++t)
				for (int l = 0; l < V; ++l) nb.push_back(o.elmVtx[(size_t) l * E + list[t]]);
			if (start[n] == start[n + 1]) nb.push_back(n);
			std::sort(nb.begin(), nb.end());
			nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
			rowPtr[n + 1] = rowPtr[n] + (long) nb.size();
			cols.insert(cols.end(), nb.begin(), nb.end());
		}
	}
	SB_REQUIRE(rowPtr[N] < (1L << 31), "too many nonzeros");
	const int nzr = (int) rowPtr[N];
	o.nzr = nzr;
	o.femVtx.assign((size_t) nzr * 2, 0);
	for (int n = 0; n < N; ++n)
		for (long z = rowPtr[n]; z < rowPtr[n + 1]; ++z) {
			o.femVtx[z] = n;
			o.femVtx[(size_t) nzr + z] = cols[z];
		}
	// glbIdxMat pair index: upper-triangle enumeration of local pairs
	int pidx[4][4];
	{
		int k = 0;
		for (int a = 0; a < V; ++a)
			for (int b = a; b < V; ++b) pidx[a][b] = pidx[b][a] = k++;
	}
	SB_REQUIRE((long) 10 * E < (1L << 31), "too many elements for the packed index");
	o.femIfoCols = 2 + 2 * maxAdj;
	o.femIfo.assign((size_t) nzr * o.femIfoCols, 0);
	std::vector<int> fill(nzr, 0);
	for (int z = 0; z < nzr; ++z) o.femIfo[(size_t) nzr + z] = o.femVtx[z] == o.femVtx[(size_t) nzr + z] ? 2 : 1;
	// row by row (the writes stay within the row's slots), each node's elements ascending, so every slot
	// lists its elements in ascending order
	for (int n1 = 0; n1 < N; ++n1) {
		const int *c0 = cols.data() + rowPtr[n1], *c1 = cols.data() + rowPtr[n1 + 1];
		for (int t = start[n1]; t < start[n1 + 1]; ++t) {
			const int e = list[t];
			int a = 0;
			while (o.elmVtx[(size_t) a * E + e] != n1) ++a;
			for (int b = 0; b < V; ++b) {
				int n2 = o.elmVtx[(size_t) b * E + e];
				int z = (int) (rowPtr[n1] + (std::lower_bound(c0, c1, n2) - c0));
				int r = fill[z]++;
				o.femIfo[(size_t) (2 + 2 * r) * nzr + z] = e;
				o.femIfo[(size_t) (3 + 2 * r) * nzr + z] = pidx[a][b] * E + e;
			}
		}
	}
	for (int z = 0; z < nzr; ++z) o.femIfo[z] = fill[z];
}

// varifold node-gradient gather table (count, then (element, sign) in 2D or (element, qa, qb) in 3D)
void vfd_gradient_table(sa_elmobj &o)
{
	const int k = o.dim, m = o.vfdNum, N = o.N, w = k == 2 ? 2 : 3;
	std::vector<int> cnt(N, 0);
	for (int t = 0; t < k * m; ++t) ++cnt[o.vfdVtx[t]];
	int maxc = 0;
	for (int c : cnt) maxc = std::max(maxc, c);
	o.vfdIfoCols = 1 + w * maxc;
	o.vfdIfo.assign((size_t) N * o.vfdIfoCols, 0);
	std::vector<int> fill(N, 0);
	for (int n = 0; n < N; ++n) o.vfdIfo[n] = cnt[n];
	static const int pa[3] = {2, 0, 1}, pb[3] = {1, 2, 0};
	for (int e = 0; e < m; ++e)
		for (int l = 0; l < k; ++l) {
			int n = o.vfdVtx[(size_t) l * m + e], r = fill[n]++;
			o.vfdIfo[(size_t) (1 + w * r) * N + n] = e;
			if (k == 2) o.vfdIfo[(size_t) (2 + 2 * r) * N + n] = l == 0 ? -1 : 1;
			else {
				o.vfdIfo[(size_t) (2 + 3 * r) * N + n] = o.vfdVtx[(size_t) pa[l] * m + e];
				o.vfdIfo[(size_t) (3 + 3 * r) * N + n] = o.vfdVtx[(size_t) pb[l] * m + e];
			}
		}
}

void finish_common(sa_elmobj &o)
{
	o.vtxElm = adjacency(o.elmVtx, o.V, o.E, o.N, &o.vtxElmCols);
	o.bdrVtx = free_boundary(o.elmVtx, o.V, o.E, o.N, &o.bdrNum);
	o.vtxBdr = adjacency(o.bdrVtx, o.V - 1, o.bdrNum, o.N, &o.vtxBdrCols);
	o.vtxBtm = adjacency(o.btmVtx, o.dim, o.btmNum, o.btmLmkNum, &o.vtxBtmCols);
	fem_pattern(o);
	vfd_gradient_table(o);
}

template <typename F>
int guarded_build(F &&f)
{
	try {
		return f();
	} catch (const BuildError &) {
		return SA_ERR_ARG;
	} catch (const std::bad_alloc &) {
		return SA_ERR_CUDA;
	}
}

}  // namespace
}  // namespace sa

extern "C" {

int sa_tri2tetra(const int *triVtxMat, int triNum, int lyrCntNum, int *tetVtxMat, int *nmlVtxMat, int *tsvVtxMat)
{
	if (!triVtxMat || triNum <= 0 || lyrCntNum < 2 || !tetVtxMat || !nmlVtxMat || !tsvVtxMat) return SA_ERR_ARG;
	const int T = triNum, nl = lyrCntNum - 1;
	int Ln = 0;
	for (int t = 0; t < 3 * T; ++t) {
		if (triVtxMat[t] < 0) return SA_ERR_ARG;
		Ln = std::max(Ln, triVtxMat[t] + 1);
	}
	if ((long) Ln * lyrCntNum >= (1L << 31) || (long) 3 * T * nl >= (1L << 31)) return SA_ERR_ARG;
	const long E = 3L * T * nl;
	for (int t = 0; t < T; ++t) {
		const int L1 = triVtxMat[t], L2 = triVtxMat[T + t], L3 = triVtxMat[2 * T + t];
		const int U1 = L1 + Ln, U2 = L2 + Ln, U3 = L3 + Ln;
		// label = circshift(tri, -1) - tri > 0, read as a 3-bit pattern
		const int pat = (L2 - L1 > 0) * 4 + (L3 - L2 > 0) * 2 + (L1 - L3 > 0);
		int te[3][4];
		switch (pat) {
		case 1: { int a[3][4] = {{L1, L2, L3, U1}, {L2, L3, U1, U2}, {L3, U1, U2, U3}}; memcpy(te, a, sizeof te); break; }
		case 2: { int a[3][4] = {{L1, L2, L3, U3}, {U3, L1, L2, U1}, {L2, U1, U2, U3}}; memcpy(te, a, sizeof te); break; }
		case 3: { int a[3][4] = {{L1, L2, L3, U1}, {L2, L3, U1, U3}, {U3, U1, L2, U2}}; memcpy(te, a, sizeof te); break; }
		case 4: { int a[3][4] = {{L1, L2, L3, U2}, {L1, L3, U3, U2}, {U2, U3, L1, U1}}; memcpy(te, a, sizeof te); break; }
		case 5: { int a[3][4] = {{L1, L2, L3, U2}, {L3, U1, L1, U2}, {U1, L3, U3, U2}}; memcpy(te, a, sizeof te); break; }
		case 6: { int a[3][4] = {{L1, L2, L3, U3}, {U3, L1, L2, U2}, {U2, U3, L1, U1}}; memcpy(te, a, sizeof te); break; }
		default: return SA_ERR_ARG;                  // repeated vertex: degenerate triangle
		}
		const int nml[6] = {L1, L2, L3, U1, U2, U3}, tsv[6] = {L1, U1, L2, U2, L3, U3};
		for (int k = 0; k < nl; ++k)
			for (int j = 0; j < 3; ++j) {
				const long e = (long) k * 3 * T + 3L * t + j;
				for (int v = 0; v < 4; ++v) tetVtxMat[(size_t) v * E + e] = te[j][v] + k * Ln;
				for (int v = 0; v < 6; ++v) {
					nmlVtxMat[(size_t) v * E + e] = nml[v] + k * Ln;
					tsvVtxMat[(size_t) v * E + e] = tsv[v] + k * Ln;
				}
			}
	}
	return SA_OK;
}

int sa_build_element_object_3d(const int *tetVtxMat, int elmNum, const int *btmVtxMat, int btmElmNum,
                               const int *nmlVtxMat, const int *tsvVtxMat, const int *vfdLyrVec, int vfdLyrNum,
                               sa_elmobj **out)
{
	if (!out || !tetVtxMat || elmNum <= 0 || !btmVtxMat || btmElmNum <= 0 || !nmlVtxMat || !tsvVtxMat ||
	    !vfdLyrVec || vfdLyrNum <= 0)
		return SA_ERR_ARG;
	*out = nullptr;
	return sa::guarded_build([&]() {
		std::unique_ptr<sa_elmobj> o(new sa_elmobj);
		o->dim = 3; o->V = 4; o->E = elmNum;
		o->elmVtx.assign(tetVtxMat, tetVtxMat + (size_t) 4 * elmNum);
		int N = 0, Ln = 0;
		for (int v : o->elmVtx) { SB_REQUIRE(v >= 0, "negative index"); N = std::max(N, v + 1); }
		o->btmNum = btmElmNum;
		o->btmVtx.assign(btmVtxMat, btmVtxMat + (size_t) 3 * btmElmNum);
		for (int v : o->btmVtx) { SB_REQUIRE(v >= 0 && v < N, "btmVtxMat index out of range"); Ln = std::max(Ln, v + 1); }
		o->N = N; o->btmLmkNum = Ln;
		o->lyrLmkNum = Ln; o->lyrCntNum = N / Ln; o->elmPerLayer = 3 * btmElmNum;
		o->frmVtx.assign(nmlVtxMat, nmlVtxMat + (size_t) 6 * elmNum);
		o->tsvVtx.assign(tsvVtxMat, tsvVtxMat + (size_t) 6 * elmNum);
		o->vfdNum = btmElmNum * vfdLyrNum;
		o->vfdVtx.assign((size_t) 3 * o->vfdNum, 0);
		for (int q = 0; q < vfdLyrNum; ++q) {
			int l = vfdLyrVec[q];
			SB_REQUIRE(l >= 1 && (long) (l - 1) * Ln < N, "vfdLyrVec layer out of range");
			for (int k = 0; k < 3; ++k)
				for (int f = 0; f < btmElmNum; ++f)
					o->vfdVtx[(size_t) k * o->vfdNum + (size_t) q * btmElmNum + f] =
						o->btmVtx[(size_t) k * btmElmNum + f] + (l - 1) * Ln;
		}
		sa::finish_common(*o);
		*out = o.release();
		return SA_OK;
	});
}

int sa_build_element_object_2d(int lyrLmkNum, int lyrCntNum, const int *vfdLyrVec, int vfdLyrNum, int periodic,
                               sa_elmobj **out)
{
	if (!out || lyrLmkNum < 2 || lyrCntNum < 2 || !vfdLyrVec || vfdLyrNum <= 0) return SA_ERR_ARG;
	*out = nullptr;
	return sa::guarded_build([&]() {
		const int L = lyrLmkNum, C = lyrCntNum, N = L * C, nq = periodic ? L : L - 1;
		SB_REQUIRE((long) L * C < (1L << 31) / 4, "mesh too large");
		std::unique_ptr<sa_elmobj> o(new sa_elmobj);
		o->dim = 2; o->V = 3; o->N = N; o->E = 2 * (C - 1) * nq;
		o->lyrLmkNum = L; o->lyrCntNum = C; o->elmPerLayer = 2 * nq;
		const int E = o->E;
		o->elmVtx.assign((size_t) 3 * E, 0);
		o->frmVtx.assign((size_t) 4 * E, 0);
		o->tsvVtx.assign((size_t) 4 * E, 0);
		for (int c = 0; c < C - 1; ++c)
			for (int l = 0; l < nq; ++l) {
				const int q = c * nq + l, lmk = c * L + l, nxt = c * L + (l + 1) % L, up = lmk + L, upn = nxt + L;
				const int e0 = 2 * q, e1 = 2 * q + 1;
				const int a0[3] = {lmk, nxt, up}, a1[3] = {nxt, upn, up};
				for (int v = 0; v < 3; ++v) { o->elmVtx[(size_t) v * E + e0] = a0[v]; o->elmVtx[(size_t) v * E + e1] = a1[v]; }
				const int tn[4] = {lmk, nxt, up, upn}, ts[4] = {lmk, up, nxt, upn};
				for (int v = 0; v < 4; ++v)
					for (int e : {e0, e1}) {
						o->frmVtx[(size_t) v * E + e] = tn[v];
						o->tsvVtx[(size_t) v * E + e] = ts[v];
					}
			}
		o->btmNum = nq; o->btmLmkNum = L;
		o->btmVtx.assign((size_t) 2 * nq, 0);
		for (int f = 0; f < nq; ++f) { o->btmVtx[f] = f; o->btmVtx[(size_t) nq + f] = (f + 1) % L; }
		o->vfdNum = nq * vfdLyrNum;
		o->vfdVtx.assign((size_t) 2 * o->vfdNum, 0);
		for (int q = 0; q < vfdLyrNum; ++q) {
			int lyr = vfdLyrVec[q];
			SB_REQUIRE(lyr >= 1 && lyr <= C, "vfdLyrVec layer out of range");
			for (int f = 0; f < nq; ++f) {
				o->vfdVtx[(size_t) q * nq + f] = (lyr - 1) * L + f;
				o->vfdVtx[(size_t) o->vfdNum + (size_t) q * nq + f] = (lyr - 1) * L + (f + 1) % L;
			}
		}
		sa::finish_common(*o);
		*out = o.release();
		return SA_OK;
	});
}

int sa_elmobj_view(const sa_elmobj *o, sa_element_object *v)
{
	if (!o || !v) return SA_ERR_ARG;
	memset(v, 0, sizeof *v);
	v->dim = o->dim; v->lmkNum = o->N; v->elmNum = o->E;
	v->elmVtxMat = o->elmVtx.data();
	v->vtxElmMat = o->vtxElm.data(); v->vtxElmCols = o->vtxElmCols;
	v->frmVtxMat = o->frmVtx.data(); v->tsvVtxMat = o->tsvVtx.data();
	v->bdrVtxMat = o->bdrVtx.data(); v->bdrElmNum = o->bdrNum;
	v->vtxBdrMat = o->vtxBdr.data(); v->vtxBdrCols = o->vtxBdrCols;
	v->btmVtxMat = o->btmVtx.data(); v->btmElmNum = o->btmNum;
	v->vtxBtmMat = o->vtxBtm.data(); v->btmLmkNum = o->btmLmkNum; v->vtxBtmCols = o->vtxBtmCols;
	v->femVtxMat = o->femVtx.data(); v->nzrNum = o->nzr;
	v->femIfoMat = o->femIfo.data(); v->femIfoCols = o->femIfoCols;
	v->vfdVtxMat = o->vfdVtx.data(); v->vfdElmNum = o->vfdNum;
	v->vfdIfoMat = o->vfdIfo.data(); v->vfdIfoCols = o->vfdIfoCols;
	v->elmLyrVec = nullptr;
	return SA_OK;
}

int sa_elmobj_layers(const sa_elmobj *o, int *lyrLmkNum, int *lyrCntNum, int *elmPerLayer)
{
	if (!o) return SA_ERR_ARG;
	if (lyrLmkNum) *lyrLmkNum = o->lyrLmkNum;
	if (lyrCntNum) *lyrCntNum = o->lyrCntNum;
	if (elmPerLayer) *elmPerLayer = o->elmPerLayer;
	return SA_OK;
}

int sa_elmobj_free(sa_elmobj *o)
{
	delete o;
	return SA_OK;
}

}  // extern "C"
