"""Light-weight simplicial meshes and facet markers.

The reference hands DOLFIN objects to ``MPETProblem`` (``Mesh``,
``MeshFunction("size_t", mesh, tdim-1)`` and ``CompiledSubDomain.mark``,
see src/mpet/mpet/mpetproblem.py:151-163 and
src/mpet/test/test_convergence_mpetsolver.py:125-150).  This module provides
the same vocabulary on plain arrays:

* :class:`Mesh` holds vertex coordinates ``(nv, d)`` float64 and cells
  ``(nc, d+1)`` int32 with each cell's vertices in ascending global order
  (DOLFIN's "ordered" mesh convention).
* :class:`MeshFunction` stores one marker per *boundary* facet.  Interior
  facets are not represented: every marker the reference's MPET path reads
  is used through ``ds`` (exterior-facet) measures or topological
  ``DirichletBC`` on boundary facets.
* :class:`CompiledSubDomain` marks facets whose vertices and midpoint all
  satisfy a predicate, as DOLFIN's ``SubDomain.mark`` does for facets.

Generators: :func:`UnitCubeMesh` (Kuhn 6-tet split of each hexahedron, the
DOLFIN ``UnitCubeMesh`` layout), :func:`UnitSquareMesh` ("right" diagonal)
and :func:`EllipsoidShellMesh` (jittered shell used for the brain-like
case).
"""
from __future__ import annotations

import sys

import numpy as np

INVALID_MARKER = sys.maxsize


class Mesh:
    """Simplicial mesh: coordinates (nv, d) and cells (nc, d+1)."""

    def __init__(self, coordinates, cells):
        x = np.ascontiguousarray(coordinates, dtype=np.float64)
        c = np.ascontiguousarray(cells, dtype=np.int64)
        if x.ndim != 2 or x.shape[1] not in (2, 3):
            raise ValueError("coordinates must be (nv, 2) or (nv, 3)")
        if c.ndim != 2 or c.shape[1] != x.shape[1] + 1:
            raise ValueError("cells must be (nc, d+1) simplices")
        if c.size and (c.min() < 0 or c.max() >= x.shape[0]):
            raise ValueError("cell vertex index out of range")
        c = np.sort(c, axis=1)
        self._x = x
        self._cells = c.astype(np.int32)
        self._bfacets = None
        self._bfacet_cell = None

    # --- DOLFIN-like accessors -------------------------------------------
    def coordinates(self):
        return self._x

    def cells(self):
        return self._cells

    def num_vertices(self):
        return self._x.shape[0]

    def num_cells(self):
        return self._cells.shape[0]

    @property
    def gdim(self):
        return self._x.shape[1]

    @property
    def tdim(self):
        return self._cells.shape[1] - 1

    def geometry(self):
        return _Dim(self.gdim)

    def topology(self):
        return _Dim(self.tdim)

    def hmin(self):
        """Smallest cell diameter (longest edge of a simplex)."""
        x, c = self._x, self._cells
        k = c.shape[1]
        best = None
        for a in range(k):
            for b in range(a + 1, k):
                l = np.linalg.norm(x[c[:, a]] - x[c[:, b]], axis=1)
                best = l if best is None else np.maximum(best, l)
        return float(best.min())

    # --- boundary facets ---------------------------------------------------
    def _build_boundary(self):
        c = self._cells.astype(np.int64)
        nc, k = c.shape
        # facet f of a cell is the simplex opposite local vertex f
        faces = np.concatenate([np.delete(c, f, axis=1) for f in range(k)], axis=0)
        owner = np.tile(np.arange(nc), k)
        faces = np.sort(faces, axis=1)
        nv = self.num_vertices()
        key = np.zeros(faces.shape[0], dtype=np.int64)
        for j in range(k - 1):
            key = key * nv + faces[:, j]
        order = np.argsort(key, kind="stable")
        ks = key[order]
        uniq, start, counts = np.unique(ks, return_index=True, return_counts=True)
        single = start[counts == 1]
        idx = order[single]
        self._bfacets = np.ascontiguousarray(faces[idx].astype(np.int32))
        self._bfacet_cell = np.ascontiguousarray(owner[idx].astype(np.int32))

    def boundary_facets(self):
        """Boundary facets (nf, d) int32, vertices ascending, sorted by vertex key."""
        if self._bfacets is None:
            self._build_boundary()
        return self._bfacets

    def boundary_facet_cells(self):
        """Index of the cell that owns each boundary facet."""
        if self._bfacets is None:
            self._build_boundary()
        return self._bfacet_cell

    def num_boundary_facets(self):
        return self.boundary_facets().shape[0]


class _Dim:
    def __init__(self, d):
        self._d = d

    def dim(self):
        return self._d


class MeshFunction:
    """Integer marker per boundary facet (mirrors ``MeshFunction("size_t", mesh, tdim-1)``)."""

    def __init__(self, mesh: Mesh, value=INVALID_MARKER):
        self.mesh = mesh
        self._values = np.full(mesh.num_boundary_facets(), value, dtype=np.int64)

    def set_all(self, value):
        self._values[:] = value

    def array(self):
        return self._values

    def __len__(self):
        return self._values.shape[0]

    def as_int32(self):
        """Markers for the C ABI: values outside int32 (e.g. INVALID) become -1."""
        v = self._values
        out = np.where((v >= 0) & (v < 2**31 - 1), v, -1)
        return np.ascontiguousarray(out.astype(np.int32))


class CompiledSubDomain:
    """Boundary-facet predicate ``inside(x) -> bool array`` on points ``(n, d)``.

    A facet is marked when the predicate holds at all of its vertices and at
    its midpoint (DOLFIN's facet marking rule with ``check_midpoint``).
    ``CompiledSubDomain.on_boundary()`` marks every boundary facet.
    """

    def __init__(self, inside=None):
        self.inside = inside

    @staticmethod
    def on_boundary():
        return CompiledSubDomain(None)

    def mark(self, mf: MeshFunction, value):
        if self.inside is None:
            mf.array()[:] = value
            return
        mesh = mf.mesh
        f = mesh.boundary_facets()
        x = mesh.coordinates()
        ok = np.ones(f.shape[0], dtype=bool)
        for j in range(f.shape[1]):
            ok &= np.asarray(self.inside(x[f[:, j]]), dtype=bool)
        mid = x[f].mean(axis=1)
        ok &= np.asarray(self.inside(mid), dtype=bool)
        mf.array()[ok] = value


def near(a, b, tol=3e-14 * 1e2):
    return np.abs(np.asarray(a) - b) < tol


# --- generators -------------------------------------------------------------

def UnitCubeMesh(nx, ny=None, nz=None):
    """Unit cube split into nx*ny*nz hexahedra of 6 tetrahedra each.

    Vertices are numbered x-fastest; every hexahedron is cut into the six
    tetrahedra that share its main diagonal (v0 -> v7), DOLFIN's layout.
    """
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    xs = np.linspace(0.0, 1.0, nx + 1)
    ys = np.linspace(0.0, 1.0, ny + 1)
    zs = np.linspace(0.0, 1.0, nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ix, iy, iz = ix.ravel(), iy.ravel(), iz.ravel()
    sx, sy = 1, nx + 1
    sz = (nx + 1) * (ny + 1)
    v0 = iz * sz + iy * sy + ix * sx
    v1 = v0 + sx
    v2 = v0 + sy
    v3 = v0 + sx + sy
    v4 = v0 + sz
    v5 = v4 + sx
    v6 = v4 + sy
    v7 = v4 + sx + sy
    tets = np.stack([
        np.stack([v0, v1, v3, v7], 1),
        np.stack([v0, v1, v5, v7], 1),
        np.stack([v0, v4, v5, v7], 1),
        np.stack([v0, v2, v3, v7], 1),
        np.stack([v0, v4, v6, v7], 1),
        np.stack([v0, v2, v6, v7], 1),
    ], axis=1).reshape(-1, 4)
    # order cells hexahedron by hexahedron with x fastest
    order = np.lexsort((ix, iy, iz))
    tets = tets.reshape(-1, 6, 4)[order].reshape(-1, 4)
    return Mesh(coords, tets)


def UnitSquareMesh(nx, ny=None):
    """Unit square split into nx*ny squares of two triangles ("right" diagonal)."""
    ny = nx if ny is None else ny
    xs = np.linspace(0.0, 1.0, nx + 1)
    ys = np.linspace(0.0, 1.0, ny + 1)
    Y, X = np.meshgrid(ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    iy, ix = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    ix, iy = ix.ravel(), iy.ravel()
    v0 = iy * (nx + 1) + ix
    v1 = v0 + 1
    v2 = v0 + (nx + 1)
    v3 = v2 + 1
    tris = np.stack([np.stack([v0, v1, v3], 1), np.stack([v0, v2, v3], 1)], axis=1).reshape(-1, 3)
    return Mesh(coords, tris)


def EllipsoidShellMesh(n_radial, semi_axes=(1.0, 0.8, 0.7), inner_ratio=0.3,
                       jitter=0.05, seed=0):
    """Ellipsoidal shell meshed by mapping a Kuhn-split cube-sphere.

    Six cube faces are each a (n_ang x n_ang) patch extruded radially in
    ``n_radial`` layers from ``inner_ratio`` to 1; the patches are welded
    along shared vertices and every hexahedron is cut into 6 tetrahedra.
    Interior vertices are jittered by ``jitter`` times the local edge length
    (seeded).  ``n_ang = 2 * n_radial`` keeps cells near-isotropic.
    """
    rng = np.random.default_rng(seed)
    nr = int(n_radial)
    na = 2 * nr
    # vertices of a cube surface grid [-1,1]^3, times radial layers
    g = np.linspace(-1.0, 1.0, na + 1)
    pts = []
    hexes = []

    def face_points(axis, sign):
        a, b = np.meshgrid(g, g, indexing="ij")
        p = np.zeros((na + 1, na + 1, 3))
        o = [i for i in range(3) if i != axis]
        p[..., axis] = sign
        p[..., o[0]] = a
        p[..., o[1]] = b
        return p

    rs = np.linspace(inner_ratio, 1.0, nr + 1)
    key_to_id = {}
    coords = []

    def vid(p_unit, layer):
        q = np.round(p_unit * na).astype(np.int64)
        key = (int(q[0]), int(q[1]), int(q[2]), layer)
        i = key_to_id.get(key)
        if i is None:
            i = len(coords)
            key_to_id[key] = i
            d = p_unit / np.linalg.norm(p_unit)
            coords.append(d * rs[layer])
        return i

    cells = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            P = face_points(axis, sign)
            ids = np.empty((na + 1, na + 1, nr + 1), dtype=np.int64)
            for i in range(na + 1):
                for j in range(na + 1):
                    for k in range(nr + 1):
                        ids[i, j, k] = vid(P[i, j], k)
            for i in range(na):
                for j in range(na):
                    for k in range(nr):
                        v = [ids[i, j, k], ids[i + 1, j, k], ids[i, j + 1, k], ids[i + 1, j + 1, k],
                             ids[i, j, k + 1], ids[i + 1, j, k + 1], ids[i, j + 1, k + 1], ids[i + 1, j + 1, k + 1]]
                        v0, v1, v2, v3, v4, v5, v6, v7 = v
                        cells += [(v0, v1, v3, v7), (v0, v1, v5, v7), (v0, v4, v5, v7),
                                  (v0, v2, v3, v7), (v0, v4, v6, v7), (v0, v2, v6, v7)]
    x = np.array(coords) * np.asarray(semi_axes)[None, :]
    cells = np.array(cells, dtype=np.int64)
    mesh = Mesh(x, cells)
    if jitter > 0:
        bf = mesh.boundary_facets()
        onb = np.zeros(mesh.num_vertices(), dtype=bool)
        onb[bf.ravel()] = True
        h = np.min(semi_axes) * (1 - inner_ratio) / nr
        d = rng.uniform(-1.0, 1.0, size=x.shape) * (jitter * h)
        d[onb] = 0.0
        x = x + d
        mesh = Mesh(x, cells)
    return mesh


def AnnulusMesh(r_inner, r_outer, n_radial, n_angular, center=(0.0, 0.0)):
    """Triangulated annulus (2D "donut"): a polar grid of n_radial layers from
    r_inner to r_outer and n_angular sectors, every quadrilateral cut into two
    triangles."""
    nr, na = int(n_radial), int(n_angular)
    r = np.linspace(r_inner, r_outer, nr + 1)
    th = np.linspace(0.0, 2.0 * np.pi, na, endpoint=False)
    R, T = np.meshgrid(r, th, indexing="ij")                 # (nr + 1, na)
    coords = np.stack([center[0] + R * np.cos(T), center[1] + R * np.sin(T)], -1).reshape(-1, 2)
    i, j = np.meshgrid(np.arange(nr), np.arange(na), indexing="ij")
    v0 = i * na + j
    v1 = i * na + (j + 1) % na
    v2 = (i + 1) * na + j
    v3 = (i + 1) * na + (j + 1) % na
    tris = np.stack([np.stack([v0, v1, v3], -1), np.stack([v0, v3, v2], -1)], -2).reshape(-1, 3)
    return Mesh(coords, tris)
