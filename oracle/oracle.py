"""Python face of the CPU oracle (test infrastructure only).

The oracle restates the reference's algorithm on the CPU in FP64:

* :func:`kantorovich` -- ``MA::kantorovich`` (include/MA/kantorovich.hpp:35-141)
  plus the moments of ``first_moment`` / ``second_moment`` (include/MA/lloyd.hpp:30-123),
  computed by ``ma_oracle.c``;
* :func:`ot_solve` -- ``MA::ot_solve`` (include/MA/optimal_transport.hpp:89-193) with
  ``solve_laplacian_matrix`` (optimal_transport.hpp:41-87) done by a direct sparse
  factorisation of the Hessian with its last row and column removed;
* :func:`lloyd` -- ``MA::lloyd`` (lloyd.hpp:126-144);
* :func:`polygon_cells` -- ``MA::voronoi_polygon_intersection``
  (include/MA/voronoi_polygon_intersection.hpp:27-188) for every site.

Parity unpinned against reference outputs (the reference cannot be built here and
its tests hold no golden vectors).  Only the test-suite, the smoke check and the
CPU-baseline leg of the benchmark import this module.  Its results are pinned by the exact-arithmetic fixtures in
``tests/golden`` and by the invariants the reference's own drivers print
(total area, mass conservation, finite-difference consistency).
"""
from __future__ import annotations

import ctypes
import os
import sys
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import build as _build  # noqa: E402

_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.ora_kantorovich.restype = ctypes.c_void_p
        L.ora_kantorovich.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip, ctypes.c_int,
                                      _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, _ip, _ip]
        for name in ("ora_value", "ora_total_mass", "ora_total_area"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [ctypes.c_void_p]
        for name in ("ora_nnz", "ora_npieces", "ora_neighbor_count"):
            getattr(L, name).restype = ctypes.c_long
            getattr(L, name).argtypes = [ctypes.c_void_p]
        L.ora_masses.argtypes = [ctypes.c_void_p, _dp]
        L.ora_moments.argtypes = [ctypes.c_void_p, _dp]
        L.ora_hessian.argtypes = [ctypes.c_void_p, _ip, _ip, _dp]
        L.ora_pieces.argtypes = [ctypes.c_void_p, _ip, _ip, _ip]
        L.ora_piece_vertices.restype = ctypes.c_long
        L.ora_piece_vertices.argtypes = [ctypes.c_void_p, _dp, _ip]
        L.ora_neighbors.argtypes = [ctypes.c_void_p, _ip, _ip]
        L.ora_pred_stats.argtypes = [ctypes.c_void_p, _lp]
        L.ora_free.argtypes = [ctypes.c_void_p]
        L.ora_set_threads.argtypes = [ctypes.c_int]
        L.ora_max_threads.restype = ctypes.c_int
        L.ora_set_precision.argtypes = [ctypes.c_int]
        L.ora_albrecht_collatz.argtypes = [ctypes.c_double] * 5 + [_dp, _dp]
        L.ora_side1.restype = ctypes.c_int
        L.ora_side1.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_double]
        L.ora_side2.restype = ctypes.c_int
        L.ora_side2.argtypes = [_dp, _dp, _dp, _dp]
        L.ora_side3.restype = ctypes.c_int
        L.ora_side3.argtypes = [_dp, _dp, _dp, _dp, _dp]
        L.ora_polygon_cell.restype = ctypes.c_int
        L.ora_polygon_cell.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_int,
                                       _dp, _dp, ctypes.c_int, _dp, _ip]
        _lib = L
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_ip)


@dataclass
class Pieces:
    face: np.ndarray
    site: np.ndarray
    nvert: np.ndarray
    offsets: np.ndarray
    xy: np.ndarray       # (sum nvert, 2) polygon vertices, kantorovich.hpp:95-102 order
    label: np.ndarray    # edge label: site index of an EDGE_DT edge, -1 for a mesh edge


@dataclass
class KResult:
    value: float
    g: np.ndarray          # cell masses (the gradient of kantorovich.hpp)
    moments: np.ndarray    # (N, 6): rho, rho x, rho y, rho x^2, rho y^2, rho xy
    rows: np.ndarray
    cols: np.ndarray
    vals: np.ndarray
    total_mass: float
    total_area: float
    neighbors: list
    filter_calls: int
    exact_calls: int
    pieces: Pieces | None = None

    @property
    def n(self):
        return self.g.shape[0]

    def hessian(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.vals, (self.rows, self.cols)), shape=(self.n, self.n))


def set_threads(n: int) -> None:
    lib().ora_set_threads(int(n))


def max_threads() -> int:
    return int(lib().ora_max_threads())


def candidates(x, y, w, ring: int = 2):
    """Candidate neighbour lists (CSR) for every site: its regular-triangulation
    neighbours, the lower convex hull of the lifted sites (x, y, x^2 + y^2 - w)
    (the reference builds the same triangulation with CGAL, kantorovich.hpp:65-72).

    ``ring=2`` adds the neighbours' neighbours, so that a near-degenerate quad that
    qhull triangulated along the other diagonal cannot hide a true neighbour.  A site
    that is not a hull vertex (hidden, or dropped by qhull's merging) gets the
    vertices of the hull facet below it and their neighbours.  Extra candidates never
    change a cell: the clipping is exact."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    w = np.asarray(w, np.float64)
    n = x.shape[0]
    if n <= 64:
        lists = [np.array([j for j in range(n) if j != i], np.int32) for i in range(n)]
    else:
        import scipy.sparse as sp
        from scipy.spatial import ConvexHull
        cx, cy = x.mean(), y.mean()
        pts = np.c_[x - cx, y - cy, (x - cx) ** 2 + (y - cy) ** 2 - w]
        hull = ConvexHull(pts)
        low = hull.equations[:, 2] < 0
        simp = hull.simplices[low]
        eqs = hull.equations[low]
        r = np.r_[simp[:, 0], simp[:, 1], simp[:, 2], simp[:, 1], simp[:, 2], simp[:, 0]]
        c = np.r_[simp[:, 1], simp[:, 2], simp[:, 0], simp[:, 0], simp[:, 1], simp[:, 2]]
        A = sp.csr_matrix((np.ones(r.size, np.int8), (r, c)), shape=(n, n))
        on = np.zeros(n, bool)
        on[np.unique(simp)] = True
        extra_r, extra_c = [], []
        for i in np.nonzero(~on)[0]:
            # the lower-hull surface is the max of its facet planes
            z = -(eqs[:, 0] * pts[i, 0] + eqs[:, 1] * pts[i, 1] + eqs[:, 3]) / eqs[:, 2]
            f = simp[int(np.argmax(z))]
            s = set(int(v) for v in f)
            for v in f:
                s |= set(A.indices[A.indptr[v]:A.indptr[v + 1]].tolist())
            extra_r += [i] * len(s)
            extra_c += list(s)
        if extra_r:
            A = A + sp.csr_matrix((np.ones(len(extra_r), np.int8), (extra_r, extra_c)), shape=(n, n))
        A = (A != 0).astype(np.int8).tocsr()
        if ring >= 2:
            A = ((A + A @ A) != 0).astype(np.int8).tocsr()
        A.setdiag(0)
        A.eliminate_zeros()
        A.sort_indices()
        return A.indptr.astype(np.int32), A.indices.astype(np.int32)
    start = np.zeros(n + 1, np.int32)
    start[1:] = np.cumsum([len(l) for l in lists])
    flat = np.concatenate(lists).astype(np.int32) if n else np.zeros(0, np.int32)
    return start, flat


def kantorovich(mesh, x, y, w, mode: int = 1, keep_pieces: bool = False, arith: str = "dd",
                ring: int = 2) -> KResult:
    """One evaluation of ``MA::kantorovich`` (+ moments) on the CPU.

    ``mode=0`` runs the reference's global flood fill on one thread
    (voronoi_triangulation_intersection.hpp:219-313); ``mode=1`` finds the same
    pieces triangle by triangle on all OpenMP threads.  Both give identical bits.

    ``arith="fp64"`` builds vertices and integrals in FP64 from absolute coordinates,
    as the reference does; ``arith="dd"`` uses the same formulas in double-double,
    which removes that rounding (the parity anchor).  The pieces are the same.
    """
    L = lib()
    L.ora_set_precision(1 if arith == "dd" else 0)
    m = mesh.explicit()
    vx, pvx = _d(m.vx)
    vy, pvy = _d(m.vy)
    vv, pvv = _d(m.values)
    tri, ptri = _i(m.tri)
    x, px = _d(x)
    y, py = _d(y)
    w, pw = _d(w)
    n = x.shape[0]
    cs, cl = candidates(x, y, w, ring)
    cs, pcs = _i(cs)
    cl, pcl = _i(cl if cl.size else np.zeros(1, np.int32))
    h = L.ora_kantorovich(m.nv, pvx, pvy, pvv, m.nt, ptri, n, px, py, pw, int(mode), int(keep_pieces), pcs, pcl)
    if not h:
        raise RuntimeError("oracle failed")
    try:
        g = np.zeros(n)
        L.ora_masses(h, g.ctypes.data_as(_dp))
        mom = np.zeros((n, 6))
        L.ora_moments(h, mom.ctypes.data_as(_dp))
        nnz = L.ora_nnz(h)
        rows = np.zeros(nnz, np.int32)
        cols = np.zeros(nnz, np.int32)
        vals = np.zeros(nnz)
        L.ora_hessian(h, rows.ctypes.data_as(_ip), cols.ctypes.data_as(_ip), vals.ctypes.data_as(_dp))
        nc = L.ora_neighbor_count(h)
        start = np.zeros(n + 1, np.int32)
        lst = np.zeros(max(nc, 1), np.int32)
        L.ora_neighbors(h, start.ctypes.data_as(_ip), lst.ctypes.data_as(_ip))
        nbrs = [lst[start[i]:start[i + 1]].copy() for i in range(n)]
        st = np.zeros(2, np.int64)
        L.ora_pred_stats(h, st.ctypes.data_as(_lp))
        pieces = None
        np_ = L.ora_npieces(h)
        if keep_pieces:
            face = np.zeros(np_, np.int32)
            site = np.zeros(np_, np.int32)
            nvert = np.zeros(np_, np.int32)
            L.ora_pieces(h, face.ctypes.data_as(_ip), site.ctypes.data_as(_ip), nvert.ctypes.data_as(_ip))
            tot = int(nvert.sum())
            xy = np.zeros((max(tot, 1), 2))
            lab = np.zeros(max(tot, 1), np.int32)
            L.ora_piece_vertices(h, xy.ctypes.data_as(_dp), lab.ctypes.data_as(_ip))
            off = np.zeros(np_ + 1, np.int64)
            off[1:] = np.cumsum(nvert)
            pieces = Pieces(face, site, nvert, off, xy[:tot], lab[:tot])
        return KResult(L.ora_value(h), g, mom, rows, cols, vals, L.ora_total_mass(h),
                       L.ora_total_area(h), nbrs, int(st[0]), int(st[1]), pieces)
    finally:
        L.ora_free(h)


def polygon_cells(x, y, w, qx, qy):
    """``MA::voronoi_polygon_intersection`` (voronoi_polygon_intersection.hpp:153-188)
    for every site: ``(off, xy, lab)`` with site i's polygon at ``xy[off[i]:off[i+1]]``;
    ``lab[j]`` is the edge starting at vertex j (a neighbour's index, or -1-e for edge e
    of the polygon).  Candidates: the regular triangulation's neighbours and theirs."""
    L = lib()
    x, px = _d(x)
    y, py = _d(y)
    w, pw = _d(w)
    qx, pqx = _d(qx)
    qy, pqy = _d(qy)
    n, k = x.shape[0], qx.shape[0]
    cs, cl = candidates(x, y, w, 2)
    cap = 512
    out_xy = np.zeros((cap, 2))
    out_lab = np.zeros(cap, np.int32)
    xs, labs, off = [], [], [0]
    for i in range(n):
        c = np.ascontiguousarray(cl[cs[i]:cs[i + 1]], dtype=np.int32)
        if c.size == 0:
            c = np.zeros(1, np.int32) + i
        m = L.ora_polygon_cell(n, px, py, pw, i, c.ctypes.data_as(_ip), int(cs[i + 1] - cs[i]), k, pqx, pqy, cap,
                               out_xy.ctypes.data_as(_dp), out_lab.ctypes.data_as(_ip))
        if m < 0:
            raise RuntimeError("oracle polygon capacity")
        xs.append(out_xy[:m].copy())
        labs.append(out_lab[:m].copy())
        off.append(off[-1] + m)
    return (np.array(off, np.int64), np.concatenate(xs) if xs else np.zeros((0, 2)),
            np.concatenate(labs) if labs else np.zeros(0, np.int32))


def albrecht_collatz(lin, site, tri):
    """quadrature.hpp:24-42 (integrate_albrecht_collatz) over one triangle
    ``tri`` (3 x 2) for the linear function ``lin`` = (a, b, c), rho = a x + b y + c:
    the integrals of rho |x - site|^2, rho, rho x, rho y, rho x^2, rho y^2, rho x y."""
    L = lib()
    t, tp = _d(np.asarray(tri, dtype=np.float64).reshape(6))
    out = np.zeros(7)
    L.ora_albrecht_collatz(float(lin[0]), float(lin[1]), float(lin[2]), float(site[0]), float(site[1]), tp,
                           out.ctypes.data_as(_dp))
    return out


def side1(v, w, e):
    L = lib()
    return bool(L.ora_side1(_d(v)[1], _d(w)[1], float(e[0]), float(e[1])))


def side2(v, a, b, w):
    L = lib()
    arrs = [np.ascontiguousarray(t, dtype=np.float64) for t in (v, a, b, w)]
    return bool(L.ora_side2(*[t.ctypes.data_as(_dp) for t in arrs]))


def side3(v, u, p, q, w):
    L = lib()
    arrs = [np.ascontiguousarray(t, dtype=np.float64) for t in (v, u, p, q, w)]
    return bool(L.ora_side3(*[t.ctypes.data_as(_dp) for t in arrs]))


# --------------------------------------------------------------------------- #
# the damped Newton solve (optimal_transport.hpp:41-193)                      #
# --------------------------------------------------------------------------- #

class EmptyCellError(RuntimeError):
    pass


@dataclass
class SolveResult:
    w: np.ndarray
    m: np.ndarray
    niter: int
    neval: int
    value: float
    grad_norm: float
    max_rel_err: float
    history: list


def solve_laplacian_matrix(h, g):
    """optimal_transport.hpp:41-87: drop the last row and column, factorise, set
    d[N-1] = 0.  The reference factorises with Eigen's SimplicialLLT; a sparse LU
    of the same symmetric positive-definite block gives the same direction."""
    import scipy.sparse.linalg as spla
    n = g.shape[0]
    d = np.zeros(n)
    if n == 1:
        return d
    hs = h[: n - 1, : n - 1].tocsc()
    d[: n - 1] = spla.splu(hs).solve(g[: n - 1])
    return d


def ot_solve(mesh, x, y, nu, w=None, eps_g: float = 1e-7, maxiter: int = 100,
             tol_rel: float | None = None, mode: int = 1, verbose: bool = False, arith: str = "dd",
             ring: int = 2, keep_iterates: bool = False) -> SolveResult:
    """``MA::ot_solve`` restated.  The stop rule is the reference's
    ``|m - nu|_2 < eps_g`` unless ``tol_rel`` is given, in which case it is
    ``max_i |m_i - nu_i| / nu_i <= tol_rel``.  ``keep_iterates`` adds each accepted
    Newton iterate's weights to the history entries."""
    nu = np.asarray(nu, dtype=np.float64)
    n = nu.shape[0]
    w = np.zeros(n) if w is None or len(w) != n else np.array(w, dtype=np.float64)
    stats = {"neval": 0}
    history = []

    def f(wv):
        stats["neval"] += 1
        r = kantorovich(mesh, x, y, wv, mode=mode, arith=arith, ring=ring)
        m = r.g
        g = m - nu
        return r.value - nu @ wv, m, g, r.hessian()

    def converged(g):
        if tol_rel is not None:
            return np.max(np.abs(g) / nu) <= tol_rel
        return np.linalg.norm(g) < eps_g

    fx, m, g, h = f(w)
    eps0 = min(m.min(), nu.min()) / 2.0
    if eps0 <= 0:
        raise EmptyCellError(f"cell {int(np.argmin(m))} is empty")
    niter = 0
    while not converged(g):
        if niter > maxiter:
            break
        niter += 1
        d = -solve_laplacian_matrix(h, g)
        alpha = 1.0
        w0 = w.copy()
        n0 = np.linalg.norm(g)
        while True:
            w = w0 + alpha * d
            fx, m, g, h = f(w)
            if m.min() >= eps0 and np.linalg.norm(g) <= (1.0 - alpha / 2.0) * n0:
                break
            alpha *= 0.5
            if alpha < 2.0 ** -40:
                raise RuntimeError("line search failed")
        history.append((niter, fx, float(np.linalg.norm(g)), alpha, stats["neval"]) +
                       ((w.copy(),) if keep_iterates else ()))
        if verbose:
            print(f"it {niter}: f={fx} |df|={np.linalg.norm(g)} tau={alpha} eval={stats['neval']}")
    return SolveResult(w, m, niter, stats["neval"], fx, float(np.linalg.norm(g)),
                       float(np.max(np.abs(m - nu) / nu)), history)


def lloyd(mesh, x, y, w, mode: int = 1):
    """lloyd.hpp:126-144: masses and centroids (first moments / mass)."""
    r = kantorovich(mesh, x, y, w, mode=mode)
    m = r.moments[:, 0]
    c = np.full((m.shape[0], 2), np.nan)  # an empty cell has no centroid
    np.divide(r.moments[:, 1:3], m[:, None], out=c, where=m[:, None] > 0)
    return m, c


def _pixel_cover(poly, i, j):
    """Area of the convex polygon ``poly`` (pixel units) inside [i, i+1] x [j, j+1],
    clipped and summed relative to the pixel's corner."""
    pts = [(p[0] - i, p[1] - j) for p in poly]
    for axis, sgn, c in ((0, 1.0, 0.0), (0, -1.0, -1.0), (1, 1.0, 0.0), (1, -1.0, -1.0)):
        out = []
        m = len(pts)
        for k in range(m):
            a, b = pts[k], pts[(k + 1) % m]
            da, db = sgn * a[axis] - c, sgn * b[axis] - c
            if da >= 0:
                out.append(a)
            if (da >= 0) != (db >= 0):
                t = da / (da - db)
                out.append((a[0] + t * (b[0] - a[0]), a[1] + t * (b[1] - a[1])))
        pts = out
        if not pts:
            return 0.0
    x = np.array([p[0] for p in pts])
    y = np.array([p[1] for p in pts])
    return 0.5 * float(np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y))


def draw_laguerre_diagram(mesh, x, y, w, colors, bbox, width, height):
    """``MA::draw_laguerre_diagram`` (include/MA/rasterization.hpp:516-547) restated:
    every piece of the oracle's evaluation, its colour ``colors[site]`` times the mean of
    the triangle's linear density at the piece's vertices (:530-540), rasterised with
    exact pixel coverage (rasterize_convex_polygon, :403-480, computes the covered
    area of each pixel; its 1e-6 nudge off integer coordinates is not reproduced).
    Returns an ``(height, width, channels)`` image."""
    colors = np.asarray(colors, dtype=np.float64)
    if colors.ndim == 1:
        colors = colors[:, None]
    r = kantorovich(mesh, x, y, w, keep_pieces=True, arith="dd")
    P = r.pieces
    m = mesh.explicit()
    x0, y0, x1, y1 = bbox
    sx, sy = width / (x1 - x0), height / (y1 - y0)
    img = np.zeros((height, width, colors.shape[1]))
    for k in range(len(P.site)):
        xy = P.xy[P.offsets[k]:P.offsets[k + 1]]
        t = m.tri[P.face[k]]
        a, b, c = t
        ax, ay, bx, by, cx, cy = m.vx[a], m.vy[a], m.vx[b], m.vy[b], m.vx[c], m.vy[c]
        det = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax)
        f1, f2 = m.values[b] - m.values[a], m.values[c] - m.values[a]
        gx = (f1 * (cy - ay) - f2 * (by - ay)) / det
        gy = ((bx - ax) * f2 - (cx - ax) * f1) / det
        ff = np.mean(m.values[a] + gx * (xy[:, 0] - ax) + gy * (xy[:, 1] - ay))
        pp = np.c_[(xy[:, 0] - x0) * sx, (xy[:, 1] - y0) * sy]
        i0, i1 = max(0, int(np.floor(pp[:, 0].min()))), min(width - 1, int(np.floor(pp[:, 0].max())))
        j0, j1 = max(0, int(np.floor(pp[:, 1].min()))), min(height - 1, int(np.floor(pp[:, 1].max())))
        for j in range(j0, j1 + 1):
            for i in range(i0, i1 + 1):
                cov = _pixel_cover(pp, i, j)
                if cov > 0:
                    img[j, i] += cov * ff * colors[P.site[k]]
    return img
