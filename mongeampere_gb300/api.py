"""Python mirror of the reference's C++ API over the C ABI.

Names and argument meaning follow MongeAmpere++:

* :func:`kantorovich` -- ``MA::kantorovich(densityT, densityF, X, weights, g, h)``
  (include/MA/kantorovich.hpp:35-141): returns the value, fills ``g`` (cell masses)
  and returns the Hessian ``h`` as a CSR matrix;
* :func:`ot_solve` -- ``MA::ot_solve(t, functions, X, masses, x, eps_g, maxiter,
  verbose, stats)`` (include/MA/optimal_transport.hpp:89-193);
* :func:`first_moment`, :func:`second_moment`, :func:`lloyd` --
  include/MA/lloyd.hpp:30-144;
* :func:`solve_laplacian_matrix` -- include/MA/optimal_transport.hpp:41-87, for the
  Hessian of the last evaluation on the context;
* :func:`kantorovich_vjp` -- the adjoint (no counterpart in the reference), wrapped for
  torch by :mod:`mongeampere_gb300.autograd`.

``X`` is an ``(N, 2)`` array (or a pair ``(x, y)``).  Arrays may be numpy arrays
(host memory) or CUDA torch tensors (device memory, used in place).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .mesh import GridMesh, TriMesh


def _is_device(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def _check(lib, ctx, st: int, what: str):
    if st != L.MA_OK:
        msg = lib.ma_status_string(st).decode()
        if ctx:
            extra = lib.ma_ctx_last_error(ctx).decode()
            if extra:
                msg += ": " + extra
        raise L.MaError(st, f"{what}: {msg}")


def _host(a, dtype=np.float64):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


class Context:
    """One CUDA stream plus the scratch memory of the engine (``ma_ctx``)."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        h = ctypes.c_void_p()
        st = self.lib.ma_ctx_create(int(device), ctypes.byref(h))
        _check(self.lib, None, st, "ma_ctx_create")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.ma_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def use_stream(self, stream_handle: int):
        _check(self.lib, self.h, self.lib.ma_ctx_set_stream(self.h, ctypes.c_void_p(int(stream_handle))),
               "ma_ctx_set_stream")

    def use_torch_stream(self):
        import torch
        self.use_stream(torch.cuda.current_stream(self.device).cuda_stream)

    @property
    def launch_count(self) -> int:
        return int(self.lib.ma_ctx_launch_count(self.h))

    def profile(self, enable: bool = True):
        _check(self.lib, self.h, self.lib.ma_ctx_profile(self.h, 1 if enable else 0), "ma_ctx_profile")

    def profile_read(self) -> dict:
        p = L.MaProfile()
        _check(self.lib, self.h, self.lib.ma_ctx_profile_read(self.h, ctypes.byref(p)), "ma_ctx_profile_read")
        out = {f: getattr(p, f) for f, _ in L.MaProfile._fields_}
        out["search"] = list(out["search"])
        out["mixed"] = list(out["mixed"])
        return out

    def mesh(self, mesh) -> "DeviceMesh":
        return DeviceMesh(self, mesh)


class DeviceMesh:
    """A density uploaded to the device (``ma_mesh``)."""

    def __init__(self, ctx: Context, mesh):
        self.ctx = ctx
        self.src = mesh
        lib = ctx.lib
        h = ctypes.c_void_p()
        if isinstance(mesh, GridMesh):
            gx, gy, v = _host(mesh.gx), _host(mesh.gy), _host(mesh.values.ravel())
            st = lib.ma_mesh_create_grid(ctx.h, mesh.nx, mesh.ny, gx.ctypes.data_as(L._dp),
                                         gy.ctypes.data_as(L._dp), v.ctypes.data_as(L._dp), ctypes.byref(h))
        elif isinstance(mesh, TriMesh):
            vx, vy, v = _host(mesh.vx), _host(mesh.vy), _host(mesh.values)
            tri = _host(mesh.tri.ravel(), np.int32)
            st = lib.ma_mesh_create_triangles(ctx.h, mesh.nv, vx.ctypes.data_as(L._dp), vy.ctypes.data_as(L._dp),
                                              v.ctypes.data_as(L._dp), mesh.nt, tri.ctypes.data_as(L._ip),
                                              ctypes.byref(h))
        else:
            raise TypeError("mesh must be a GridMesh or a TriMesh")
        _check(lib, ctx.h, st, "ma_mesh_create")
        self.h = h

    def set_values(self, values):
        """New vertex values for the same geometry (``ma_mesh_set_values``)."""
        a = _Args(values.reshape(-1) if hasattr(values, "reshape") else values)
        _check(self.ctx.lib, self.ctx.h, self.ctx.lib.ma_mesh_set_values(self.ctx.h, self.h, a.ptrs[0], a.mem),
               "ma_mesh_set_values")

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.ma_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def total_mass(self) -> float:
        out = ctypes.c_double()
        _check(self.ctx.lib, self.ctx.h, self.ctx.lib.ma_mesh_total_mass(self.h, ctypes.byref(out)), "total_mass")
        return out.value


_default_ctx = None
_mesh_cache = {}


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _dmesh(ctx: Context, mesh):
    if isinstance(mesh, DeviceMesh):
        return mesh
    key = (id(ctx), id(mesh))
    dm = _mesh_cache.get(key)
    if dm is None or dm.src is not mesh:
        dm = DeviceMesh(ctx, mesh)
        _mesh_cache[key] = dm
    return dm


def _split_xy(X, y=None):
    if y is not None:
        return X, y
    if _is_device(X):
        return X[:, 0].contiguous(), X[:, 1].contiguous()
    X = np.asarray(X, dtype=np.float64)
    return np.ascontiguousarray(X[:, 0]), np.ascontiguousarray(X[:, 1])


class _Args:
    """Hold pointers of a call's array arguments (all host or all device)."""

    def __init__(self, *arrays):
        self.device = any(_is_device(a) for a in arrays if a is not None)
        self.keep = []
        self.ptrs = []
        for a in arrays:
            if a is None:
                self.ptrs.append(None)
                continue
            if self.device:
                import torch
                t = a if _is_device(a) else torch.as_tensor(np.asarray(a, dtype=np.float64), device="cuda")
                t = t.to(torch.float64).contiguous()
                self.keep.append(t)
                self.ptrs.append(ctypes.c_void_p(t.data_ptr()))
            else:
                h = _host(a)
                self.keep.append(h)
                self.ptrs.append(ctypes.c_void_p(h.ctypes.data))
        self.mem = L.MA_MEM_DEVICE if self.device else L.MA_MEM_HOST

    def out(self, n, like=None):
        if self.device:
            import torch
            t = torch.empty(n, dtype=torch.float64, device=self.keep[0].device)
            return t, ctypes.c_void_p(t.data_ptr())
        h = np.empty(n, dtype=np.float64)
        return h, ctypes.c_void_p(h.ctypes.data)


@dataclass
class Hessian:
    rowptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    n: int

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.rowptr), shape=(self.n, self.n))


def kantorovich(mesh, X, weights, y=None, *, precision: str = "fp64", hessian: bool = True,
                ctx: Context | None = None):
    """``MA::kantorovich``: returns ``(value, g, h)`` with ``g`` the cell masses and
    ``h`` a :class:`Hessian` (``None`` when ``hessian=False``)."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    x, yy = _split_xy(X, y)
    a = _Args(x, yy, weights)
    n = int(a.keep[0].shape[0])
    g, gp = a.out(n)
    val = ctypes.c_double()
    nnz = ctypes.c_int64()
    prec = L.MA_MIXED if precision == "mixed" else L.MA_FP64
    st = ctx.lib.ma_kantorovich(ctx.h, dm.h, n, a.ptrs[0], a.ptrs[1], a.ptrs[2], a.mem, prec, ctypes.byref(val),
                                gp, ctypes.byref(nnz))
    _check(ctx.lib, ctx.h, st, "ma_kantorovich")
    h = None
    if hessian:
        h = hessian_copy(ctx, n, int(nnz.value))
    return val.value, g, h


@dataclass
class Pieces:
    """Every non-empty cell-triangle intersection (``MA::voronoi_triangulation_intersection``):
    piece ``k`` is cell ``site[k]`` on triangle ``tri[k]`` with vertices
    ``xy[off[k]:off[k+1]]`` (counter-clockwise); ``edge[v]`` labels the edge from vertex
    ``v`` to the next: the neighbouring site, or ``-1-e`` for triangle edge ``e``."""
    site: np.ndarray
    tri: np.ndarray
    off: np.ndarray
    xy: np.ndarray
    edge: np.ndarray

    def polygon(self, k):
        return self.xy[self.off[k]:self.off[k + 1]], self.edge[self.off[k]:self.off[k + 1]]


def pieces(mesh, X, weights, y=None, ctx: Context | None = None) -> Pieces:
    """``MA::voronoi_triangulation_intersection`` (``ma_pieces`` + ``ma_pieces_copy``)."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    x, yy = _split_xy(X, y)
    a = _Args(x, yy, weights)
    n = int(a.keep[0].shape[0])
    npc, nvt = ctypes.c_int64(), ctypes.c_int64()
    st = ctx.lib.ma_pieces(ctx.h, dm.h, n, a.ptrs[0], a.ptrs[1], a.ptrs[2], a.mem, ctypes.byref(npc),
                           ctypes.byref(nvt))
    _check(ctx.lib, ctx.h, st, "ma_pieces")
    np_, nv = int(npc.value), int(nvt.value)
    site = np.empty(np_, np.int32)
    tri = np.empty(np_, np.int32)
    off = np.empty(np_ + 1, np.int64)
    xy = np.empty((nv, 2), np.float64)
    edge = np.empty(nv, np.int32)
    vp = lambda arr: ctypes.c_void_p(arr.ctypes.data)
    st = ctx.lib.ma_pieces_copy(ctx.h, vp(site), vp(tri), vp(off), vp(xy), vp(edge), L.MA_MEM_HOST)
    _check(ctx.lib, ctx.h, st, "ma_pieces_copy")
    return Pieces(site, tri, off, xy, edge)


@dataclass
class PolygonCells:
    """Every cell clipped to one polygon (``MA::voronoi_polygon_intersection`` for each
    site): site ``i``'s polygon is ``xy[off[i]:off[i+1]]`` (empty when the cell misses
    the polygon); ``edge[v]`` labels the edge from vertex ``v`` to the next: the
    neighbouring site, or ``-1-e`` for edge ``e`` of the clipping polygon."""
    off: np.ndarray
    xy: np.ndarray
    edge: np.ndarray

    def polygon(self, i):
        return self.xy[self.off[i]:self.off[i + 1]], self.edge[self.off[i]:self.off[i + 1]]

    def areas(self):
        """Signed shoelace area of every site's polygon."""
        x, y = self.xy[:, 0], self.xy[:, 1]
        nxt = np.arange(x.shape[0]) + 1
        n = self.off.shape[0] - 1
        a = np.zeros(n)
        nz = self.off[1:] > self.off[:-1]
        nxt[self.off[1:][nz] - 1] = self.off[:-1][nz]
        cr = x * y[nxt] - x[nxt] * y
        a[nz] = 0.5 * np.add.reduceat(cr, self.off[:-1][nz]) if cr.size else 0.0
        return a


def voronoi_polygon_intersection(polygon, X, weights=None, y=None, ctx: Context | None = None) -> PolygonCells:
    """``MA::voronoi_polygon_intersection`` (voronoi_polygon_intersection.hpp:153-188)
    for every site at once (``ma_polygon_cells`` + ``ma_polygon_cells_copy``):
    ``polygon`` is ``(k, 2)`` corners, 3 <= k <= 64; ``weights`` None gives the Voronoi
    cells."""
    ctx = ctx or default_context()
    P = np.ascontiguousarray(polygon, dtype=np.float64).reshape(-1, 2)
    qx, qy = np.ascontiguousarray(P[:, 0]), np.ascontiguousarray(P[:, 1])
    x, yy = _split_xy(X, y)
    if weights is None:
        a = _Args(x, yy)
        wp = ctypes.c_void_p(None)
    else:
        a = _Args(x, yy, weights)
        wp = a.ptrs[2]
    n = int(a.keep[0].shape[0])
    nvt = ctypes.c_int64()
    st = ctx.lib.ma_polygon_cells(ctx.h, n, a.ptrs[0], a.ptrs[1], wp, ctypes.c_void_p(qx.ctypes.data),
                                  ctypes.c_void_p(qy.ctypes.data), int(P.shape[0]), a.mem, ctypes.byref(nvt))
    _check(ctx.lib, ctx.h, st, "ma_polygon_cells")
    nv = int(nvt.value)
    off = np.empty(n + 1, np.int64)
    xy = np.empty((nv, 2), np.float64)
    edge = np.empty(nv, np.int32)
    vp = lambda arr: ctypes.c_void_p(arr.ctypes.data)
    st = ctx.lib.ma_polygon_cells_copy(ctx.h, vp(off), vp(xy), vp(edge), L.MA_MEM_HOST)
    _check(ctx.lib, ctx.h, st, "ma_polygon_cells_copy")
    return PolygonCells(off, xy, edge)


def draw_laguerre_diagram(mesh, X, weights, colors, bbox, width: int, height: int, image=None, y=None,
                          ctx: Context | None = None):
    """``MA::draw_laguerre_diagram`` (``ma_draw_laguerre``): every cell-triangle piece
    rasterised with exact pixel coverage, ``cover * (mean density at the piece's
    vertices) * colors[site]`` added to ``image`` (``(height, width, channels)``, zeros
    when not given); ``colors`` is ``(N,)`` or ``(N, channels)``; ``bbox`` =
    ``(x0, y0, x1, y1)``.  Returns the image."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    x, yy = _split_xy(X, y)
    col = colors
    nc = 1 if len(col.shape) == 1 else int(col.shape[1])
    col = col.reshape(-1)
    a = _Args(x, yy, weights, col)
    n = int(a.keep[0].shape[0])
    if image is None:
        if a.device:
            import torch
            image = torch.zeros((height, width, nc), dtype=torch.float64, device=a.keep[0].device)
        else:
            image = np.zeros((height, width, nc))
    img = image if a.device else np.ascontiguousarray(image, dtype=np.float64)
    ip = ctypes.c_void_p(img.data_ptr()) if a.device else ctypes.c_void_p(img.ctypes.data)
    x0, y0, x1, y1 = (float(v) for v in bbox)
    st = ctx.lib.ma_draw_laguerre(ctx.h, dm.h, n, a.ptrs[0], a.ptrs[1], a.ptrs[2], a.ptrs[3], nc, x0, y0, x1, y1,
                                  int(width), int(height), ip, a.mem)
    _check(ctx.lib, ctx.h, st, "ma_draw_laguerre")
    return img


def kantorovich_vjp(mesh, X, weights, cot_value: float = 0.0, cot_mass=None, cot_first=None, y=None, *,
                    grad_rho: bool = True, precision: str = "fp64", ctx: Context | None = None):
    """Adjoint of ``(value, masses, first moments)`` (``ma_kantorovich_vjp``; no
    counterpart in the reference).  ``cot_first`` is ``(N, 2)``.  Returns
    ``(grad_X (N, 2), grad_w (N,), grad_rho (V,) or None)`` where ``grad_rho`` is per
    mesh vertex (row-major ``ny x nx`` for a grid).  ``precision="mixed"`` integrates
    the pieces in FP32."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    x, yy = _split_xy(X, y)
    cf = None
    if cot_first is not None:
        cf = cot_first.reshape(-1) if hasattr(cot_first, "reshape") else np.asarray(cot_first).reshape(-1)
    a = _Args(x, yy, weights, cot_mass, cf)
    n = int(a.keep[0].shape[0])
    gx, gxp = a.out(n)
    gy, gyp = a.out(n)
    gw, gwp = a.out(n)
    src = dm.src
    nv = src.nx * src.ny if isinstance(src, GridMesh) else src.nv
    gr, grp = a.out(nv) if grad_rho else (None, None)
    if precision not in ("fp64", "mixed"):
        raise ValueError("precision must be 'fp64' or 'mixed'")
    prec = L.MA_MIXED if precision == "mixed" else L.MA_FP64
    st = ctx.lib.ma_kantorovich_vjp(ctx.h, dm.h, n, a.ptrs[0], a.ptrs[1], a.ptrs[2], a.mem, prec, float(cot_value),
                                    a.ptrs[3], a.ptrs[4], gxp, gyp, gwp, grp)
    _check(ctx.lib, ctx.h, st, "ma_kantorovich_vjp")
    if a.device:
        import torch
        gX = torch.stack([gx, gy], 1)
    else:
        gX = np.stack([gx, gy], 1)
    return gX, gw, gr


def hessian_copy(ctx: Context, n: int, nnz: int) -> Hessian:
    rowptr = np.empty(n + 1, np.int32)
    col = np.empty(nnz, np.int32)
    val = np.empty(nnz, np.float64)
    st = ctx.lib.ma_hessian_copy(ctx.h, ctypes.c_void_p(rowptr.ctypes.data), ctypes.c_void_p(col.ctypes.data),
                                 ctypes.c_void_p(val.ctypes.data), L.MA_MEM_HOST)
    _check(ctx.lib, ctx.h, st, "ma_hessian_copy")
    return Hessian(rowptr, col, val, n)


@dataclass
class Statistics:
    """``MA::Statistics`` (optimal_transport.hpp:35-39) plus the engine's counters."""

    niter: int = 0
    neval: int = 0
    cg_iters: int = 0
    linesearch_halvings: int = 0
    grad_norm: float = 0.0
    max_rel_err: float = 0.0
    value: float = 0.0
    t_eval_ms: float = 0.0
    t_linsolve_ms: float = 0.0
    neval_fp64: int = 0
    cg_noconv: int = 0
    status: int = 0


def ot_solve(mesh, X, masses, x=None, eps_g: float = 1e-7, maxiter: int = 100, verbose: bool = False,
             stats: Statistics | None = None, *, y=None, stop: str = "grad", precision: str = "fp64",
             cg_rtol: float = 0.0, cg_maxiter: int = 0, precond: str = "multigrid", init: str = "given",
             ctx: Context | None = None, raise_on_error: bool = True):
    """``MA::ot_solve``.  Returns the weights (``x`` is the initial guess; ``None``
    or a wrong-sized array starts from zero like the reference).  ``stop="rel"``
    uses ``max_i |m_i - nu_i| / nu_i <= eps_g`` instead of ``|m - nu|_2 < eps_g``.
    ``precond`` is the CG preconditioner of the Newton step: "multigrid" or "jacobi".
    ``init="multiscale"`` replaces the initial guess by a coarse-to-fine one;
    ``init="continuation"`` reaches the targets in stages from the masses of ``x``."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    xs, ys = _split_xy(X, y)
    n = int(xs.shape[0])
    if x is None or len(x) != n:
        if _is_device(xs):
            import torch
            x = torch.zeros(n, dtype=torch.float64, device=xs.device)
        else:
            x = np.zeros(n)
    a = _Args(xs, ys, masses, x)
    w = a.keep[3] if a.device else a.keep[3].copy()
    wp = ctypes.c_void_p(w.data_ptr()) if a.device else ctypes.c_void_p(w.ctypes.data)
    o = L.MaSolveOpts()
    ctx.lib.ma_solve_opts_default(ctypes.byref(o))
    o.eps_g = eps_g
    o.maxiter = maxiter
    o.stop_rule = L.MA_STOP_MAX_REL if stop == "rel" else L.MA_STOP_GRAD_NORM
    o.precision = L.MA_MIXED if precision == "mixed" else L.MA_FP64
    o.verbose = 1 if verbose else 0
    if cg_rtol:
        o.cg_rtol = cg_rtol
    if cg_maxiter:
        o.cg_maxiter = cg_maxiter
    if precond not in ("multigrid", "jacobi"):
        raise ValueError("precond must be 'multigrid' or 'jacobi'")
    o.precond = L.MA_PRECOND_JACOBI if precond == "jacobi" else L.MA_PRECOND_MULTIGRID
    inits = {"given": L.MA_INIT_GIVEN, "multiscale": L.MA_INIT_MULTISCALE, "continuation": L.MA_INIT_CONTINUATION}
    if init not in inits:
        raise ValueError("init must be 'given', 'multiscale' or 'continuation'")
    o.init = inits[init]
    s = L.MaStats()
    st = ctx.lib.ma_ot_solve(ctx.h, dm.h, n, a.ptrs[0], a.ptrs[1], a.ptrs[2], wp, a.mem, ctypes.byref(o),
                             ctypes.byref(s))
    if stats is not None:
        for f, _ in L.MaStats._fields_:
            setattr(stats, f, getattr(s, f))
        stats.status = st
    if raise_on_error and st not in (L.MA_OK,):
        _check(ctx.lib, ctx.h, st, "ma_ot_solve")
    return w


def ot_solve_batch(problems, eps_g: float = 1e-6, stop: str = "rel", precision: str = "fp64",
                   init: str = "given", workers: int = 0, maxiter: int = 100, ctx: Context | None = None):
    """Many independent problems (``ma_ot_solve_batch``): ``problems`` is a list of
    ``(mesh, X, nu)`` or ``(mesh, X, nu, w0)``.  Returns ``(weights, stats, workers)``:
    the solved weights and a :class:`Statistics` per problem (``status`` set), and
    the number of concurrent workers used (``workers=0``: autotuned).  The workers'
    streams share the device's hardware queues: set ``CUDA_DEVICE_MAX_CONNECTIONS=32``
    in the environment before the process first uses CUDA (the default is 8)."""
    ctx = ctx or default_context()
    n = len(problems)
    arr = (L.MaProblem * n)()
    keep = []
    device = None
    for k, pr in enumerate(problems):
        mesh, X, nu = pr[0], pr[1], pr[2]
        dm = _dmesh(ctx, mesh)
        x, y = _split_xy(X)
        w0 = pr[3] if len(pr) > 3 and pr[3] is not None else None
        if w0 is None:
            w0 = np.zeros(int(np.asarray(nu).shape[0])) if not _is_device(nu) else None
            if w0 is None:
                import torch
                w0 = torch.zeros(nu.shape[0], dtype=torch.float64, device=nu.device)
        a = _Args(x, y, nu, w0)
        if device is None:
            device = a.device
        elif device != a.device:
            raise ValueError("all arrays of a batch must be host arrays or all CUDA tensors")
        w = a.keep[3] if a.device else a.keep[3].copy()
        wp = ctypes.c_void_p(w.data_ptr()) if a.device else ctypes.c_void_p(w.ctypes.data)
        keep.append((dm, a, w))
        arr[k].mesh = dm.h
        arr[k].n = int(a.keep[0].shape[0])
        arr[k].x, arr[k].y, arr[k].nu = a.ptrs[0], a.ptrs[1], a.ptrs[2]
        arr[k].w = wp
    o = L.MaSolveOpts()
    ctx.lib.ma_solve_opts_default(ctypes.byref(o))
    o.eps_g = eps_g
    o.maxiter = maxiter
    o.stop_rule = L.MA_STOP_MAX_REL if stop == "rel" else L.MA_STOP_GRAD_NORM
    o.precision = L.MA_MIXED if precision == "mixed" else L.MA_FP64
    o.init = L.MA_INIT_MULTISCALE if init == "multiscale" else L.MA_INIT_GIVEN
    used = ctypes.c_int()
    mem = L.MA_MEM_DEVICE if device else L.MA_MEM_HOST
    st = ctx.lib.ma_ot_solve_batch(ctx.h, arr, n, mem, ctypes.byref(o), int(workers), ctypes.byref(used))
    _check(ctx.lib, ctx.h, st, "ma_ot_solve_batch")
    ws, stats = [], []
    for k in range(n):
        s_ = Statistics()
        for f, _ in L.MaStats._fields_:
            setattr(s_, f, getattr(arr[k].stats, f))
        s_.status = arr[k].status
        stats.append(s_)
        ws.append(keep[k][2])
    return ws, stats, int(used.value)


def w2_flow(mesh, X, nu, steps: int, tau: float, w=None, eps_g: float = 1e-6, stop: str = "rel",
            precision: str = "fp64", ctx: Context | None = None):
    """``ma_w2_flow``: ``steps`` times an OT solve then ``x <- x + tau (x - centroid)``
    (the iteration of tests/test_zeldovich.cpp:99-119; ``tau = -1`` is Lloyd's).
    Returns ``(X, w, stats)`` after the last step."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    x, y = _split_xy(X)
    n = int(np.asarray(nu).shape[0]) if not _is_device(nu) else int(nu.shape[0])
    if w is None:
        if _is_device(nu):
            import torch
            w = torch.zeros(n, dtype=torch.float64, device=nu.device)
        else:
            w = np.zeros(n)
    a = _Args(x, y, nu, w)
    xs = a.keep[0] if a.device else a.keep[0].copy()
    ys = a.keep[1] if a.device else a.keep[1].copy()
    ws = a.keep[3] if a.device else a.keep[3].copy()
    ptr = (lambda t: ctypes.c_void_p(t.data_ptr())) if a.device else (lambda t: ctypes.c_void_p(t.ctypes.data))
    o = L.MaSolveOpts()
    ctx.lib.ma_solve_opts_default(ctypes.byref(o))
    o.eps_g = eps_g
    o.stop_rule = L.MA_STOP_MAX_REL if stop == "rel" else L.MA_STOP_GRAD_NORM
    o.precision = L.MA_MIXED if precision == "mixed" else L.MA_FP64
    s = L.MaStats()
    st = ctx.lib.ma_w2_flow(ctx.h, dm.h, n, ptr(xs), ptr(ys), a.ptrs[2], ptr(ws), a.mem, int(steps), float(tau),
                            ctypes.byref(o), ctypes.byref(s))
    _check(ctx.lib, ctx.h, st, "ma_w2_flow")
    stats = Statistics()
    for f, _ in L.MaStats._fields_:
        setattr(stats, f, getattr(s, f))
    if a.device:
        import torch
        return torch.stack([xs, ys], 1), ws, stats
    return np.c_[xs, ys], ws, stats


def solve_laplacian_matrix(g, rtol: float = 1e-10, maxiter: int = 0, ctx: Context | None = None):
    """Newton direction for the Hessian of the context's last evaluation
    (optimal_transport.hpp:41-87): ``H[:n-1,:n-1] d = g[:n-1]``, ``d[n-1] = 0``."""
    ctx = ctx or default_context()
    a = _Args(g)
    n = int(a.keep[0].shape[0])
    d, dp = a.out(n)
    it = ctypes.c_int64()
    st = ctx.lib.ma_laplacian_solve(ctx.h, a.ptrs[0], dp, a.mem, float(rtol), int(maxiter), ctypes.byref(it))
    _check(ctx.lib, ctx.h, st, "ma_laplacian_solve")
    return d, int(it.value)


def first_moment(mesh, X, weights, y=None, ctx: Context | None = None):
    """``MA::first_moment``: ``(masses, first)`` with ``first[i] = (int rho x, int rho y)``."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    x, yy = _split_xy(X, y)
    a = _Args(x, yy, weights)
    n = int(a.keep[0].shape[0])
    m, mp = a.out(n)
    f, fp = a.out(2 * n)
    st = ctx.lib.ma_moments(ctx.h, dm.h, n, a.ptrs[0], a.ptrs[1], a.ptrs[2], a.mem, mp, fp, None)
    _check(ctx.lib, ctx.h, st, "ma_moments")
    return m, f.reshape(n, 2)


def second_moment(mesh, X, weights, y=None, ctx: Context | None = None):
    """``MA::second_moment``: ``(masses, first, inertia)``, inertia = (xx, yy, xy)."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    x, yy = _split_xy(X, y)
    a = _Args(x, yy, weights)
    n = int(a.keep[0].shape[0])
    m, mp = a.out(n)
    f, fp = a.out(2 * n)
    s, sp = a.out(3 * n)
    st = ctx.lib.ma_moments(ctx.h, dm.h, n, a.ptrs[0], a.ptrs[1], a.ptrs[2], a.mem, mp, fp, sp)
    _check(ctx.lib, ctx.h, st, "ma_moments")
    return m, f.reshape(n, 2), s.reshape(n, 3)


def lloyd(mesh, X, weights, y=None, ctx: Context | None = None):
    """``MA::lloyd``: ``(masses, centroids)``."""
    ctx = ctx or default_context()
    dm = _dmesh(ctx, mesh)
    x, yy = _split_xy(X, y)
    a = _Args(x, yy, weights)
    n = int(a.keep[0].shape[0])
    m, mp = a.out(n)
    c, cp = a.out(2 * n)
    st = ctx.lib.ma_lloyd(ctx.h, dm.h, n, a.ptrs[0], a.ptrs[1], a.ptrs[2], a.mem, mp, cp)
    _check(ctx.lib, ctx.h, st, "ma_lloyd")
    return m, c.reshape(n, 2)
