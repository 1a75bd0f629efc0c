"""Element-object builders: the reference's mesh layout contract.

Every array is returned exactly as the reference's MATLAB builders hand it
to the MEX gateways, i.e. ``int32(Mat' - 1)`` for index matrices and
``int32(Mat')`` for count/adjacency matrices.  A MATLAB ``Mat`` of size
``k x n`` transposed to ``n x k`` and stored column-major has the same
memory as the C-contiguous numpy array of shape ``(k, n)``; that is the
shape used here (``elmVtxMat.shape == (V, E)``), so ``arr.ctypes.data`` is
byte-for-byte the int32 gpuArray the reference passes.

Builders restated (file:line in the reference's CUDA/ folder):

* ``generate_element_object_2d``  -- generateElementObject2D.m:1-150
* ``tri2tetra``                   -- tri2tetra.m:1-69
* ``generate_element_object_3d``  -- generateElementObject3D.m:1-127

``find``-based adjacency lists follow MATLAB's column-major ``find``
order (ascending element, then local index); ``femVtxMat`` is the
``sortrows`` (row, col)-lexicographic CSR pattern and ``femIfoMat`` lists,
per nonzero, the contributing elements in ascending order with the packed
element-matrix index ``pair * E + e`` of ``glbIdxMat`` -- all bit-exact.
``bdrVtxMat``/``vtxBdrMat`` come from MATLAB's ``freeBoundary``, which
feeds only the reference's commented-out boundary-traction code; they are
built with the right shapes and contents but their row order is not
MATLAB's.

New generators (not in the reference): periodic annulus, icosphere and
spherical shell, element layer ids, varifold gradient gather tables and
varifold targets.
"""
from __future__ import annotations

import numpy as np

I32 = np.int32


# --------------------------------------------------------------------------
# generic helpers
# --------------------------------------------------------------------------
def _adjacency(idx: np.ndarray, num: int) -> np.ndarray:
    """MATLAB block ``[lcl, elm] = find(idxMat == n)`` for every node n.

    ``idx`` is the 0-based (k x m) index matrix.  Returns the
    (1 + 2*maxCnt, num) matrix: count row, then (entity, local) pairs in
    column-major find order (entity ascending, then local index).
    """
    k, m = idx.shape
    flat = idx.T.reshape(-1)                    # column-major order: entity-major
    ent = np.repeat(np.arange(m, dtype=np.int64), k)
    lcl = np.tile(np.arange(k, dtype=np.int64), m)
    order = np.argsort(flat, kind="stable")     # stable keeps (entity, local) order per node
    node = flat[order]
    cnt = np.bincount(node, minlength=num)
    maxc = int(cnt.max()) if cnt.size else 0
    out = np.zeros((1 + 2 * maxc, num), dtype=I32)
    out[0] = cnt
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    rank = np.arange(order.size) - np.repeat(start, cnt)
    out[1 + 2 * rank, node] = ent[order]
    out[2 + 2 * rank, node] = lcl[order]
    return out


def _pair_index(V: int) -> np.ndarray:
    """glbIdxMat column for a local pair (a, b): upper-triangle enumeration
    (1,1),(1,2),...,(1,V),(2,2),... of generateElementObject2D.m:82-116."""
    pidx = np.zeros((V, V), dtype=np.int64)
    k = 0
    for a in range(V):
        for b in range(a, V):
            pidx[a, b] = pidx[b, a] = k
            k += 1
    return pidx


def _fem_pattern(elm: np.ndarray, num: int, elm_cnt_max: int):
    """femVtxMat and femIfoMat (generateElementObject2D.m:98-126)."""
    V, E = elm.shape
    # unique undirected edges (triangulation.edges) -> full sorted pattern
    a_idx, b_idx = np.triu_indices(V, 1)
    ea = elm[a_idx].reshape(-1).astype(np.int64)
    eb = elm[b_idx].reshape(-1).astype(np.int64)
    lo, hi = np.minimum(ea, eb), np.maximum(ea, eb)
    ekey = np.unique(lo * num + hi)
    edges = np.stack([ekey // num, ekey % num], axis=1)
    rows = np.concatenate([np.arange(num), edges[:, 0], edges[:, 1]])
    cols = np.concatenate([np.arange(num), edges[:, 1], edges[:, 0]])
    mul = np.concatenate([np.full(num, 2), np.ones(2 * len(edges), dtype=np.int64)])
    key = rows * num + cols
    srt = np.argsort(key, kind="stable")        # sortrows: (row, col) lexicographic
    key = key[srt]
    rows, cols, mul = rows[srt], cols[srt], mul[srt]
    nzr = key.size
    # contributions: element e, local (l1, l2) -> slot of (node l1, node l2)
    pidx = _pair_index(V)
    L1, L2 = np.meshgrid(np.arange(V), np.arange(V), indexing="ij")
    L1, L2 = L1.reshape(-1), L2.reshape(-1)
    ce = np.repeat(np.arange(E, dtype=np.int64), V * V)
    n1 = elm[L1][:, :].T.reshape(-1).astype(np.int64)   # (E, V*V) element-major
    n2 = elm[L2][:, :].T.reshape(-1).astype(np.int64)
    slot = np.searchsorted(key, n1 * num + n2)
    packed = np.tile(pidx[L1, L2], E) * E + ce
    order = np.argsort(slot, kind="stable")     # per slot: ascending element
    slot, ce, packed = slot[order], ce[order], packed[order]
    cnt = np.bincount(slot, minlength=nzr)
    ifo = np.zeros((2 + 2 * elm_cnt_max, nzr), dtype=I32)
    ifo[0] = cnt
    ifo[1] = mul
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    rank = np.arange(slot.size) - np.repeat(start, cnt)
    ifo[2 + 2 * rank, slot] = ce
    ifo[3 + 2 * rank, slot] = packed
    fvtx = np.stack([rows, cols]).astype(I32)
    return fvtx, ifo, edges


def _free_boundary(elm: np.ndarray, num: int) -> np.ndarray:
    """Faces used by exactly one element (MATLAB freeBoundary), 0-based (V-1, F)."""
    V, E = elm.shape
    faces = []
    for drop in range(V):
        keep = [k for k in range(V) if k != drop]
        faces.append(elm[keep].T)
    f = np.concatenate(faces, axis=0).astype(np.int64)
    srt = np.sort(f, axis=1)
    _, inv, cnt = np.unique(srt, axis=0, return_inverse=True, return_counts=True)
    once = cnt[inv.reshape(-1)] == 1
    return f[once].T.astype(I32)


def element_layers(elm_num: int, elm_per_layer: int, layer_of_prism) -> np.ndarray:
    """Per-element material layer id: element index // elm_per_layer gives the
    prism (or quad-strip) layer, mapped through ``layer_of_prism``."""
    prism = np.arange(elm_num) // elm_per_layer
    return np.asarray(layer_of_prism, dtype=I32)[prism]


# --------------------------------------------------------------------------
# 2D
# --------------------------------------------------------------------------
def generate_element_object_2d(lyrLmkNum: int, lyrCntNum: int, vfdLyrVec, periodic: bool = False) -> dict:
    """generateElementObject2D(lyrLmkNum, lyrCntNum, vfdLyrVec).

    ``vfdLyrVec`` uses MATLAB's 1-based layer numbers.  ``periodic=True``
    closes each layer into a ring (node lyrLmkNum-1 joins node 0), giving the
    annulus layout of the layered model: (L * (C-1) * 2) triangles.
    """
    L, C = int(lyrLmkNum), int(lyrCntNum)
    N = L * C
    nq = L if periodic else L - 1
    c, l = np.meshgrid(np.arange(C - 1), np.arange(nq), indexing="ij")
    c, l = c.reshape(-1), l.reshape(-1)
    lmk = c * L + l                            # 0-based lmkIdx
    nxt = c * L + (l + 1) % L
    up, upn = lmk + L, nxt + L
    E = 2 * lmk.size
    elm = np.zeros((3, E), dtype=np.int64)
    elm[:, 0::2] = np.stack([lmk, nxt, up])
    elm[:, 1::2] = np.stack([nxt, upn, up])
    tan = np.zeros((4, E), dtype=np.int64)
    tsv = np.zeros((4, E), dtype=np.int64)
    tan[:, 0::2] = tan[:, 1::2] = np.stack([lmk, nxt, up, upn])
    tsv[:, 0::2] = tsv[:, 1::2] = np.stack([lmk, up, nxt, upn])
    elm_cnt = np.bincount(elm.reshape(-1), minlength=N)
    obj = {}
    obj["elmVtxMat"] = elm.astype(I32)
    obj["vtxElmMat"] = _adjacency(elm, N)
    obj["tanVtxMat"] = tan.astype(I32)
    obj["tsvVtxMat"] = tsv.astype(I32)
    bdr = _free_boundary(elm, N)
    obj["bdrVtxMat"] = bdr
    obj["vtxBdrMat"] = _adjacency(bdr.astype(np.int64), N)
    nb = L if periodic else L - 1
    btm = np.stack([np.arange(nb), (np.arange(nb) + 1) % L]).astype(np.int64)
    obj["btmVtxMat"] = btm.astype(I32)
    obj["vtxBtmMat"] = _adjacency(btm, L)
    fvtx, ifo, _ = _fem_pattern(elm, N, int(elm_cnt.max()))
    obj["femVtxMat"] = fvtx
    obj["femIfoMat"] = ifo
    glb = np.arange(N).reshape(C, L)           # glbIdxMat(l, c) = c*L + l
    blocks = []
    for lyr in vfdLyrVec:
        row = glb[int(lyr) - 1]
        blocks.append(np.stack([row[:nb], row[(np.arange(nb) + 1) % L]]))
    obj["vfdVtxMat"] = np.concatenate(blocks, axis=1).astype(I32)
    obj["dim"] = 2
    obj["lyrLmkNum"], obj["lyrCntNum"] = L, C
    obj["elmPerLayer"] = 2 * nq
    return obj


def strip_nodes(lyrNdeNum: int, lyrCntNum: int, x=(-3.0, 3.0), y=(-1.0, 1.0)) -> np.ndarray:
    """demo/getInitialShape.m: (2, N) grid, layer-major node order."""
    xv = np.linspace(x[0], x[1], lyrNdeNum)
    yv = np.linspace(y[0], y[1], lyrCntNum)
    nde = np.zeros((2, lyrCntNum, lyrNdeNum))
    nde[0] = xv[None, :]
    nde[1] = yv[:, None]
    return nde.reshape(2, -1)


def annulus_nodes(angNum: int, radNum: int, r0: float, r1: float) -> np.ndarray:
    """(2, N) periodic annulus nodes: layer c (radius) major, angle minor."""
    th = 2.0 * np.pi * np.arange(angNum) / angNum
    r = np.linspace(r0, r1, radNum)
    x = r[:, None] * np.cos(th)[None, :]
    y = r[:, None] * np.sin(th)[None, :]
    return np.stack([x.reshape(-1), y.reshape(-1)])


# --------------------------------------------------------------------------
# 3D
# --------------------------------------------------------------------------
def tri2tetra(triVtxMat: np.ndarray, lyrCntNum: int):
    """tri2tetra(triVtxMat, lyrCntNum) with 0-based input/outputs.

    ``triVtxMat``: (3, T) surface triangles.  Returns (tetVtxMat (4, E),
    nmlVtxMat (6, E), tsvVtxMat (6, E)), E = 3 T (lyrCntNum - 1).
    """
    tri = np.asarray(triVtxMat, dtype=np.int64)
    T = tri.shape[1]
    Ln = int(tri.max()) + 1
    lbl = (np.roll(tri, -1, axis=0) - tri) > 0          # circshift(tri, -1) - tri > 0
    low, upp = tri, tri + Ln
    L1, L2, L3 = low
    U1, U2, U3 = upp
    tets = np.zeros((T, 3, 4), dtype=np.int64)
    pat = lbl[0] * 4 + lbl[1] * 2 + lbl[2] * 1
    cases = {
        1: lambda s: [[L1, L2, L3, U1], [L2, L3, U1, U2], [L3, U1, U2, U3]],   # [0;0;1]
        2: lambda s: [[L1, L2, L3, U3], [U3, L1, L2, U1], [L2, U1, U2, U3]],   # [0;1;0]
        3: lambda s: [[L1, L2, L3, U1], [L2, L3, U1, U3], [U3, U1, L2, U2]],   # [0;1;1]
        4: lambda s: [[L1, L2, L3, U2], [L1, L3, U3, U2], [U2, U3, L1, U1]],   # [1;0;0]
        5: lambda s: [[L1, L2, L3, U2], [L3, U1, L1, U2], [U1, L3, U3, U2]],   # [1;0;1]
        6: lambda s: [[L1, L2, L3, U3], [U3, L1, L2, U2], [U2, U3, L1, U1]],   # [1;1;0] (else)
    }
    for p, f in cases.items():
        sel = pat == p
        if not sel.any():
            continue
        arr = np.array(f(None))                         # (3 tets, 4, T)
        tets[sel] = np.transpose(arr[:, :, sel], (2, 0, 1))
    bad = ~np.isin(pat, list(cases))
    if bad.any():
        raise ValueError("degenerate surface triangle (repeated vertex)")
    tet1 = tets.reshape(T * 3, 4).T                      # columns 3(t-1)+(1:3)
    nml1 = np.repeat(np.concatenate([low, upp]), 3, axis=1)
    tsv1 = np.repeat(np.stack([L1, U1, L2, U2, L3, U3]), 3, axis=1)
    nl = lyrCntNum - 1
    tet = np.concatenate([tet1 + k * Ln for k in range(nl)], axis=1)
    nml = np.concatenate([nml1 + k * Ln for k in range(nl)], axis=1)
    tsv = np.concatenate([tsv1 + k * Ln for k in range(nl)], axis=1)
    return tet.astype(I32), nml.astype(I32), tsv.astype(I32)


def generate_element_object_3d(tetVtxMat, btmVtxMat, nmlVtxMat, tsvVtxMat, vfdLyrVec) -> dict:
    """generateElementObject3D(tetObj, btmVtxMat, nmlVtxMat, tsvVtxMat, vfdLyrVec), 0-based."""
    elm = np.asarray(tetVtxMat, dtype=np.int64)
    btm = np.asarray(btmVtxMat, dtype=np.int64)
    N = int(elm.max()) + 1
    Ln = int(btm.max()) + 1
    elm_cnt = np.bincount(elm.reshape(-1), minlength=N)
    obj = {}
    obj["elmVtxMat"] = elm.astype(I32)
    obj["vtxElmMat"] = _adjacency(elm, N)
    obj["nmlVtxMat"] = np.asarray(nmlVtxMat, dtype=I32)
    obj["tsvVtxMat"] = np.asarray(tsvVtxMat, dtype=I32)
    bdr = _free_boundary(elm, N)
    obj["bdrVtxMat"] = bdr
    obj["vtxBdrMat"] = _adjacency(bdr.astype(np.int64), N)
    obj["btmVtxMat"] = btm.astype(I32)
    obj["vtxBtmMat"] = _adjacency(btm, Ln)
    fvtx, ifo, _ = _fem_pattern(elm, N, int(elm_cnt.max()))
    obj["femVtxMat"] = fvtx
    obj["femIfoMat"] = ifo
    obj["vfdVtxMat"] = np.concatenate([btm + (int(l) - 1) * Ln for l in vfdLyrVec], axis=1).astype(I32)
    obj["dim"] = 3
    obj["lyrLmkNum"], obj["lyrCntNum"] = Ln, N // Ln
    obj["elmPerLayer"] = 3 * btm.shape[1]
    return obj


def icosphere(level: int):
    """Unit icosphere: (3, V) vertices, (3, F) triangles (0-based, outward CCW).

    Level 0 is the icosahedron (12, 20); each level splits every triangle in
    four with normalised edge midpoints: level 5 has 10242 vertices and
    20480 faces.  Vertex order: parents first, then midpoints in order of
    first appearance.
    """
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
         [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
         [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
         [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    V = np.array(v, dtype=np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array(f, dtype=np.int64)
    for _ in range(level):
        a, b, c = F[:, 0], F[:, 1], F[:, 2]
        e = np.stack([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)], 1).reshape(-1, 2)
        key = np.minimum(e[:, 0], e[:, 1]) * len(V) + np.maximum(e[:, 0], e[:, 1])
        uk, first, inv = np.unique(key, return_index=True, return_inverse=True)
        order = np.argsort(first, kind="stable")          # order of first appearance
        rank = np.empty_like(order)
        rank[order] = np.arange(order.size)
        mid_id = len(V) + rank[inv.reshape(-1)]
        ue = e[first[order]]
        M = 0.5 * (V[ue[:, 0]] + V[ue[:, 1]])
        M /= np.linalg.norm(M, axis=1, keepdims=True)
        V = np.concatenate([V, M])
        m = mid_id.reshape(-1, 3)                          # ab, bc, ca midpoints
        F = np.concatenate([np.stack([a, m[:, 0], m[:, 2]], 1), np.stack([b, m[:, 1], m[:, 0]], 1),
                            np.stack([c, m[:, 2], m[:, 1]], 1), np.stack([m[:, 0], m[:, 1], m[:, 2]], 1)])
    return V.T.copy(), F.T.astype(I32)


def shell_nodes(surf: np.ndarray, lyrCntNum: int, r0: float, r1: float) -> np.ndarray:
    """(3, Ln * lyrCntNum) nodes: surface copies at radii linspace(r0, r1), inner first."""
    r = np.linspace(r0, r1, lyrCntNum)
    return np.concatenate([surf * rk for rk in r], axis=1)


def shell_element_object(level: int, lyrCntNum: int, vfdLyrVec=None, native: bool = False):
    """Icosphere-level shell: (nodes (3, N), elmObj) with bottom = inner surface.

    native=True builds tri2tetra and the element object with the C library's
    builders (the same arrays, bit for bit, much faster for large meshes)."""
    surf, tri = icosphere(level)
    if vfdLyrVec is None:
        vfdLyrVec = [lyrCntNum]
    if native:
        from . import api
        tet, nml, tsv = api.tri2tetra(tri, lyrCntNum)
        return surf, tri, tet, nml, tsv, api.build_element_object_3d(tet, tri, nml, tsv, vfdLyrVec)
    tet, nml, tsv = tri2tetra(tri, lyrCntNum)
    return surf, tri, tet, nml, tsv, generate_element_object_3d(tet, tri, nml, tsv, vfdLyrVec)


# --------------------------------------------------------------------------
# varifold helpers
# --------------------------------------------------------------------------
def vfd_gradient_table(vfdVtxMat: np.ndarray, lmkNum: int) -> np.ndarray:
    """Gather table for the varifold node gradient (d_dfmElmIfoMat of the
    reference's gradient kernels, 2D/varifold.cu:435-466, 3D :492-528).

    2D rows: count, then (element, sign) pairs with sign -1 for the first and
    +1 for the second segment end.  3D rows: count, then (element, qa, qb)
    triples with the cross-product partners of the vertex
    (q2,q1), (q0,q2), (q1,q0) for local vertex 0, 1, 2.
    """
    vfd = np.asarray(vfdVtxMat, dtype=np.int64)
    k, m = vfd.shape
    flat = vfd.T.reshape(-1)
    ent = np.repeat(np.arange(m), k)
    lcl = np.tile(np.arange(k), m)
    order = np.argsort(flat, kind="stable")
    node, ent, lcl = flat[order], ent[order], lcl[order]
    cnt = np.bincount(node, minlength=lmkNum)
    maxc = int(cnt.max()) if cnt.size else 0
    width = 2 if k == 2 else 3
    out = np.zeros((1 + width * maxc, lmkNum), dtype=I32)
    out[0] = cnt
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    rank = np.arange(order.size) - np.repeat(start, cnt)
    out[1 + width * rank, node] = ent
    if k == 2:
        out[2 + 2 * rank, node] = np.where(lcl == 0, -1, 1)
    else:
        pa = np.array([2, 0, 1])[lcl]
        pb = np.array([1, 2, 0])[lcl]
        out[2 + 3 * rank, node] = vfd[pa, ent]
        out[3 + 3 * rank, node] = vfd[pb, ent]
    return out


def varifold_target(lmk: np.ndarray, vfdVtxMat: np.ndarray):
    """Target (cenPosMat, uniDirMat, elmVolVec) of a shape, by the formula of
    landmarksToVarifoldKernel (2D/varifold.cu:9-36, 3D/varifold.cu:9-43).
    Returned as C-contiguous (D, Vt) / (Vt,) arrays (column-major Vt x D)."""
    D = lmk.shape[0]
    q = [lmk[:, vfdVtxMat[k]] for k in range(vfdVtxMat.shape[0])]
    if D == 2:
        cen = 0.5 * (q[0] + q[1])
        d = q[1] - q[0]
        vol = np.sqrt(d[0] * d[0] + d[1] * d[1])
        return cen.copy(), (d / vol).copy(), vol.copy()
    cen = (q[0] + q[1] + q[2]) / 3.0
    a, b = q[1] - q[0], q[2] - q[0]
    c = np.stack([a[1] * b[2] - a[2] * b[1], -a[0] * b[2] + a[2] * b[0], a[0] * b[1] - a[1] * b[0]])
    n = np.sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])
    return cen.copy(), (c / n).copy(), (0.5 * n).copy()


def smooth_displacement(lmk: np.ndarray, amplitude: float, seed: int, modes: int = 8) -> np.ndarray:
    """Seeded smooth random displacement: a sum of ``modes`` low-frequency
    Fourier modes in angle (2D) or low-order spherical waves (3D), scaled so
    that the largest node displacement equals ``amplitude``."""
    rng = np.random.default_rng(seed)
    D, N = lmk.shape
    disp = np.zeros_like(lmk)
    if D == 2:
        th = np.arctan2(lmk[1], lmk[0])
        for _ in range(modes):
            k = rng.integers(1, 5)
            ph = rng.uniform(0, 2 * np.pi, size=2)
            amp = rng.normal(size=2)
            disp[0] += amp[0] * np.cos(k * th + ph[0])
            disp[1] += amp[1] * np.cos(k * th + ph[1])
    else:
        for _ in range(modes):
            kv = rng.normal(size=3)
            kv *= rng.uniform(1.0, 3.0) / np.linalg.norm(kv)
            ph = rng.uniform(0, 2 * np.pi)
            amp = rng.normal(size=3)
            s = np.cos(kv @ lmk + ph)
            disp += amp[:, None] * s[None, :]
    disp *= amplitude / np.abs(disp).max()
    return lmk + disp
