"""Triangulated piecewise-linear densities.

The reference represents the source density as a CGAL triangulation plus a
``std::map<Face_handle, Linear_function>`` (include/MA/functions.hpp:55-120); the
triangulation is either built from an image (``image_to_pl_function``,
functions.hpp:82-120) or assembled from explicit vertices and faces
(include/CGAL/Triangulation_incremental_builder_2.h:27-80).  Here a density is one
of two plain-array descriptions:

* :class:`GridMesh` -- a tensor-product grid ``gx x gy`` whose every square is cut
  by the diagonal from its lower-left to its upper-right corner, with one value per
  vertex.  This is the layout of every synthetic workload, and the device keeps it
  implicit (8 bytes per vertex).
* :class:`TriMesh` -- explicit vertices, per-vertex values and counter-clockwise
  triangles, for any other triangulation.

On each triangle the density is the linear interpolant of its three vertex values,
exactly the ``Linear_function`` of functions.hpp:55-80.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class TriMesh:
    """Explicit triangulation: ``vx, vy, values`` per vertex, ``tri`` (T, 3) int32, ccw."""

    vx: np.ndarray
    vy: np.ndarray
    values: np.ndarray
    tri: np.ndarray

    def __post_init__(self):
        self.vx = np.ascontiguousarray(self.vx, dtype=np.float64)
        self.vy = np.ascontiguousarray(self.vy, dtype=np.float64)
        self.values = np.ascontiguousarray(self.values, dtype=np.float64)
        self.tri = np.ascontiguousarray(self.tri, dtype=np.int32).reshape(-1, 3)

    @property
    def nv(self) -> int:
        return int(self.vx.shape[0])

    @property
    def nt(self) -> int:
        return int(self.tri.shape[0])

    def explicit(self) -> "TriMesh":
        return self

    def total_mass(self) -> float:
        """Integral of the density over the mesh (the value ``image_to_pl_function``
        returns, functions.hpp:116-119)."""
        t = self.tri
        ax, ay = self.vx[t[:, 0]], self.vy[t[:, 0]]
        bx, by = self.vx[t[:, 1]], self.vy[t[:, 1]]
        cx, cy = self.vx[t[:, 2]], self.vy[t[:, 2]]
        area = ((bx - ax) * (cy - ay) - (cx - ax) * (by - ay)) / 2.0
        mean = (self.values[t[:, 0]] + self.values[t[:, 1]] + self.values[t[:, 2]]) / 3.0
        return float(np.sum(area * mean))

    def bbox(self):
        return (float(self.vx.min()), float(self.vy.min()), float(self.vx.max()), float(self.vy.max()))


@dataclass
class GridMesh:
    """Tensor-product grid: vertex (i, j) sits at ``(gx[i], gy[j])`` and carries
    ``values[j, i]``; square (i, j) is split into the counter-clockwise triangles
    ``(k, k+1, k+nx+1)`` and ``(k, k+nx+1, k+nx)`` with ``k = j*nx + i``."""

    gx: np.ndarray
    gy: np.ndarray
    values: np.ndarray

    def __post_init__(self):
        self.gx = np.ascontiguousarray(self.gx, dtype=np.float64)
        self.gy = np.ascontiguousarray(self.gy, dtype=np.float64)
        self.values = np.ascontiguousarray(self.values, dtype=np.float64).reshape(
            self.gy.shape[0], self.gx.shape[0])
        if self.gx.shape[0] < 2 or self.gy.shape[0] < 2:
            raise ValueError("a grid mesh needs at least 2 x 2 vertices")
        if np.any(np.diff(self.gx) <= 0) or np.any(np.diff(self.gy) <= 0):
            raise ValueError("grid coordinates must be strictly increasing")

    @property
    def nx(self) -> int:
        return int(self.gx.shape[0])

    @property
    def ny(self) -> int:
        return int(self.gy.shape[0])

    @property
    def nv(self) -> int:
        return self.nx * self.ny

    @property
    def nt(self) -> int:
        return 2 * (self.nx - 1) * (self.ny - 1)

    def explicit(self) -> TriMesh:
        nx, ny = self.nx, self.ny
        X, Y = np.meshgrid(self.gx, self.gy)
        i = np.arange(nx - 1)
        j = np.arange(ny - 1)
        J, I = np.meshgrid(j, i, indexing="ij")
        k = (J * nx + I).ravel()
        tri = np.empty((2 * k.shape[0], 3), dtype=np.int32)
        tri[0::2, 0] = k
        tri[0::2, 1] = k + 1
        tri[0::2, 2] = k + nx + 1
        tri[1::2, 0] = k
        tri[1::2, 1] = k + nx + 1
        tri[1::2, 2] = k + nx
        return TriMesh(X.ravel(), Y.ravel(), self.values.ravel(), tri)

    def total_mass(self) -> float:
        return self.explicit().total_mass()

    def bbox(self):
        return (float(self.gx[0]), float(self.gy[0]), float(self.gx[-1]), float(self.gy[-1]))


def unit_grid(n: int, values: np.ndarray) -> GridMesh:
    """``n x n`` vertices on [0, 1]^2."""
    g = np.linspace(0.0, 1.0, n)
    return GridMesh(g, g.copy(), values)


def read_pgm(path) -> np.ndarray:
    """A grey image from a PGM file (P2 text or P5 binary, 8 or 16 bit) as a
    ``(height, width)`` float array, rows top first (the CImg layout of the reference's
    image inputs, functions.hpp:82-120); 16-bit values are scaled to 0..255."""
    with open(path, "rb") as fh:
        data = fh.read()
    tokens = []
    pos = 0
    while len(tokens) < 4:
        while pos < len(data) and chr(data[pos]).isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            while pos < len(data) and data[pos:pos + 1] not in (b"\n", b"\r"):
                pos += 1
            continue
        start = pos
        while pos < len(data) and not chr(data[pos]).isspace():
            pos += 1
        tokens.append(data[start:pos].decode())
    magic, w, h, maxval = tokens[0], int(tokens[1]), int(tokens[2]), int(tokens[3])
    if magic == "P5":
        pos += 1  # the single whitespace after the header
        dt = np.uint8 if maxval < 256 else np.dtype(">u2")
        img = np.frombuffer(data, dtype=dt, count=w * h, offset=pos).astype(np.float64)
    elif magic == "P2":
        img = np.array(data[pos:].split()[: w * h], dtype=np.float64)
    else:
        raise ValueError("not a PGM file: " + magic)
    img = img.reshape(h, w)
    if maxval > 255:
        img = img * (255.0 / maxval)
    return img


def image_grid(pixels) -> GridMesh:
    """``image_to_pl_function`` (functions.hpp:82-120): the image's vertex grid on
    [-1, 1]^2 with values ``pixel / 255 + 1e-3``, row ``j`` (bottom up) from image row
    ``height - 1 - j``; each square split along its (i, j)-(i+1, j+1) diagonal."""
    p = np.asarray(pixels, dtype=np.float64)
    h, w = p.shape
    gx = np.linspace(-1.0, 1.0, w)
    gy = np.linspace(-1.0, 1.0, h)
    return GridMesh(gx, gy, p[::-1, :] / 255.0 + 1e-3)
