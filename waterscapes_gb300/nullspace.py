"""Rigid-motion basis of the displacement (restates src/mpet/mpet/rm_basis_L2.py:10-74).

L2-orthonormal rigid motions of the mesh: in 2D the two translations
e_k / sqrt(|Omega|) and the rotation (-(y - c1), x - c0) / sqrt(int |x - c|^2);
in 3D the translations along the eigenvectors v_k of the rotational Gram
matrix R_ij = int (x - c) x e_i . (x - c) x e_j and the rotations
(x - c) x v_k / sqrt(w_k) (w_k the eigenvalues), c the centroid.  Integrals
are exact (products of linear functions on simplices); the modes are linear,
so their values at the P2 nodes represent them exactly.
"""
from __future__ import annotations

import math

import numpy as np


def _simplex_moments(x, cells):
    """Volumes, first moments and second moments (int x_i x_j) of every cell."""
    d = x.shape[1]
    P = x[cells]                                            # (nc, d+1, d)
    E = P[:, 1:, :] - P[:, :1, :]
    vol = np.abs(np.linalg.det(E)) / math.factorial(d)
    first = vol[:, None] * P.mean(axis=1)
    k = 1.0 / ((d + 1) * (d + 2))
    second = k * vol[:, None, None] * (np.einsum("cri,crj->cij", P, P)
                                       + np.einsum("ci,cj->cij", P.sum(1), P.sum(1)))
    return vol, first, second


def rigid_motions(mesh, nodes):
    """(nz, n_nodes, d) values at the points ``nodes`` (n_nodes x d) of the
    L2-orthonormal rigid motions of ``mesh`` (nz = 3 in 2D, 6 in 3D)."""
    x = np.asarray(mesh.coordinates(), dtype=np.float64)
    cells = np.asarray(mesh.cells(), dtype=np.int64)
    d = x.shape[1]
    vol, first, second = _simplex_moments(x, cells)
    V = vol.sum()
    c = first.sum(0) / V
    S = second.sum(0) - V * np.outer(c, c)                   # int (x - c)_i (x - c)_j
    y = np.asarray(nodes, dtype=np.float64)[:, :d] - c[None, :]
    if d == 2:
        r = np.trace(S)
        modes = [np.tile([1.0 / math.sqrt(V), 0.0], (y.shape[0], 1)),
                 np.tile([0.0, 1.0 / math.sqrt(V)], (y.shape[0], 1)),
                 np.stack([-y[:, 1], y[:, 0]], 1) / math.sqrt(r)]
        return np.stack(modes)
    if d != 3:
        raise ValueError("rigid motions for 2D and 3D meshes")
    R = np.trace(S) * np.eye(3) - S
    w, v = np.linalg.eigh(R)
    trans = [np.tile(v[:, k] / math.sqrt(V), (y.shape[0], 1)) for k in range(3)]
    rots = [np.cross(y, v[:, k]) / math.sqrt(w[k]) for k in range(3)]
    return np.stack(trans + rots)
