"""P2/P1 Lagrange on affine simplices: dofmap, exact local tensors, sparsity.

Test infrastructure (oracle).  Restates what FFC/FIAT generate for the forms
of src/mpet/mpet/mpetsolver.py:196-254 on affine triangles and tetrahedra.

Conventions (shared with the GPU library by construction, checked by tests):

* P2 nodes are the mesh vertices (ids 0..nv-1) followed by the mesh edges
  (ids nv..nv+ne-1); edges are sorted lexicographically by (low, high)
  vertex id.
* Mixed global DOF order ("block natural"): displacement DOF of node i and
  component k is ``d*i + k``; pressure DOF of network a at vertex v is
  ``Nu + a*nv + v`` with ``Nu = d * (nv + ne)``.
* Local P2 node order in a cell: vertices 0..d, then edges in UFC order
  (tet: (2,3),(1,3),(1,2),(0,3),(0,2),(0,1); triangle: (1,2),(0,2),(0,1)).

All integrals are exact: gradients of P2 functions are linear, so every
bilinear term of the MPET operator is a polynomial of degree <= 2 and is
integrated with the barycentric monomial formula
``int_T lambda^alpha = |T| d! alpha! / (|alpha| + d)!``.
"""
from __future__ import annotations

import itertools
import math

import numpy as np
import scipy.sparse as sp

TET_EDGES = ((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1))
TRI_EDGES = ((1, 2), (0, 2), (0, 1))
SEG_EDGES = ((0, 1),)


def local_edges(d):
    return {3: TET_EDGES, 2: TRI_EDGES, 1: SEG_EDGES}[d]


def monomial_integral(alpha, d):
    """int over the d-simplex of prod lambda_i^alpha_i, divided by |T|."""
    num = math.factorial(d)
    for a in alpha:
        num *= math.factorial(a)
    return num / math.factorial(sum(alpha) + d)


def _bary_moment(idx, d):
    """int lambda_idx[0] * lambda_idx[1] * ... / |T| for a tuple of barycentric indices."""
    alpha = [0] * (d + 1)
    for i in idx:
        alpha[i] += 1
    return monomial_integral(alpha, d)


def p2_quadratic_forms(d):
    """Each P2 basis function as a symmetric quadratic form in barycentrics.

    Vertex m: lambda_m (2 lambda_m - 1) = lambda_m (2 lambda_m - sum lambda).
    Edge (a, b): 4 lambda_a lambda_b.
    Returns Q (nloc2, d+1, d+1) with phi_i = lambda^T Q_i lambda.
    """
    n = d + 1
    edges = local_edges(d)
    Q = np.zeros((n + len(edges), n, n))
    for m in range(n):
        for s in range(n):
            if s == m:
                Q[m, m, m] += 1.0
            else:
                Q[m, m, s] += -0.5
                Q[m, s, m] += -0.5
    for e, (a, b) in enumerate(edges):
        Q[n + e, a, b] += 2.0
        Q[n + e, b, a] += 2.0
    return Q


def p2_mass_reference(d):
    """M_hat[i, j] = int phi_i phi_j / |T| (exact)."""
    Q = p2_quadratic_forms(d)
    n = d + 1
    m4 = np.zeros((n, n, n, n))
    for idx in itertools.product(range(n), repeat=4):
        m4[idx] = _bary_moment(idx, d)
    return np.einsum("irs,jtu,rstu->ij", Q, Q, m4)


def p1_mass_reference(d):
    n = d + 1
    W = np.full((n, n), 1.0)
    W[np.diag_indices(n)] = 2.0
    return W * (math.factorial(d) / math.factorial(d + 2))


def p1_triple_reference(d):
    """T_hat[v, i, j] = int lambda_v lambda_i lambda_j / |T|."""
    n = d + 1
    T = np.zeros((n, n, n))
    for idx in itertools.product(range(n), repeat=3):
        T[idx] = _bary_moment(idx, d)
    return T


def p2_p1_triple_reference(d):
    """int phi_i lambda_v lambda_w / |T| for P2 phi_i (used by no bilinear term; kept for sources)."""
    Q = p2_quadratic_forms(d)
    n = d + 1
    m4 = np.zeros((n, n, n, n))
    for idx in itertools.product(range(n), repeat=4):
        m4[idx] = _bary_moment(idx, d)
    return np.einsum("irs,rsvw->ivw", Q, m4)


# --- mesh topology / dofmap ---------------------------------------------------

class DofMap:
    """P2-vector + A x P1 dofmap on a simplicial mesh (block-natural order)."""

    def __init__(self, x, cells, num_networks):
        self.x = np.asarray(x, dtype=np.float64)
        self.cells = np.sort(np.asarray(cells, dtype=np.int64), axis=1)
        self.d = self.x.shape[1]
        self.A = int(num_networks)
        d = self.d
        nv = self.x.shape[0]
        nc = self.cells.shape[0]
        edges_loc = local_edges(d)
        pairs = np.stack([np.stack([self.cells[:, a], self.cells[:, b]], 1) for (a, b) in edges_loc], 1)
        lo = pairs.min(axis=2)
        hi = pairs.max(axis=2)
        key = lo * nv + hi
        ukey, inv = np.unique(key.ravel(), return_inverse=True)
        self.edges = np.stack([ukey // nv, ukey % nv], 1)
        self.cell_edges = inv.reshape(nc, len(edges_loc))
        self.nv = nv
        self.ne = self.edges.shape[0]
        self.nnodes = nv + self.ne
        self.nloc2 = d + 1 + len(edges_loc)
        self.cell_nodes = np.concatenate([self.cells, nv + self.cell_edges], axis=1)
        self.Nu = d * self.nnodes
        self.N = self.Nu + self.A * nv
        self.nloc = d * self.nloc2 + self.A * (d + 1)
        # node coordinates (vertices, edge midpoints)
        self.node_x = np.concatenate([self.x, 0.5 * (self.x[self.edges[:, 0]] + self.x[self.edges[:, 1]])], 0)

    def cell_dofs(self):
        """(nc, nloc) global DOFs: u (node-major, component-minor), then p_a (vertex)."""
        d, A = self.d, self.A
        u = (d * self.cell_nodes[:, :, None] + np.arange(d)[None, None, :]).reshape(self.cells.shape[0], -1)
        ps = [self.Nu + a * self.nv + self.cells for a in range(A)]
        return np.concatenate([u] + ps, axis=1)

    def u_dof(self, node, comp):
        return self.d * node + comp

    def p_dof(self, a, v):
        return self.Nu + a * self.nv + v


# --- geometry -------------------------------------------------------------------

def simplex_geometry(x, cells):
    """Barycentric gradients b (nc, d+1, d) and volumes |T| (nc,)."""
    X = x[cells]  # (nc, d+1, d)
    J = np.transpose(X[:, 1:, :] - X[:, :1, :], (0, 2, 1))  # columns x_i - x_0
    d = x.shape[1]
    det = np.linalg.det(J)
    Jinv = np.linalg.inv(J)  # rows: grad lambda_1..lambda_d
    b = np.empty((cells.shape[0], d + 1, d))
    b[:, 1:, :] = Jinv
    b[:, 0, :] = -Jinv.sum(axis=1)
    vol = np.abs(det) / math.factorial(d)
    return b, vol


def p2_gradient_vertex_values(b):
    """g[c, i, r, :] = grad phi_i evaluated at vertex r (gradients are linear)."""
    nc, n, d = b.shape
    edges = local_edges(d)
    nloc2 = n + len(edges)
    g = np.zeros((nc, nloc2, n, d))
    for m in range(n):
        for r in range(n):
            g[:, m, r, :] = (4.0 * (m == r) - 1.0) * b[:, m, :]
    for e, (a, bb) in enumerate(edges):
        g[:, n + e, a, :] = 4.0 * b[:, bb, :]
        g[:, n + e, bb, :] = 4.0 * b[:, a, :]
    return g


def local_gradient_products(g, vol):
    """Mg[c, i, j, k, l] = int d_k phi_i d_l phi_j (exact, degree 2)."""
    nc, nloc2, n, d = g.shape
    W = p1_mass_reference(d)
    Mg = np.einsum("rs,cirk,cjsl->cijkl", W, g, g)
    return Mg * vol[:, None, None, None, None]


def local_coupling(g, vol):
    """C[c, i, k, w] = int lambda_w d_k phi_i."""
    d = g.shape[-1]
    W = p1_mass_reference(d)
    return np.einsum("wr,cirk->cikw", W, g) * vol[:, None, None, None]


# --- global sparse assembly with the DOLFIN pattern -------------------------------

def pattern_coo(cell_dofs):
    """Rows/cols of all dense cell blocks (duplicates included)."""
    nc, nloc = cell_dofs.shape
    rows = np.repeat(cell_dofs, nloc, axis=1).ravel()
    cols = np.tile(cell_dofs, (1, nloc)).ravel()
    return rows, cols


def assemble_csr(cell_dofs, local, N):
    """Sum local (nc, nloc, nloc) blocks into CSR on the union-of-cell-blocks pattern.

    Structural zeros of the mixed block are stored, as in a DOLFIN/PETSc
    matrix assembled from the mixed form.
    """
    rows, cols = pattern_coo(cell_dofs)
    A = sp.coo_matrix((local.ravel(), (rows, cols)), shape=(N, N)).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return A


def assemble_vector(cell_dofs, local, N):
    return np.bincount(cell_dofs.ravel(), weights=local.ravel(), minlength=N)
