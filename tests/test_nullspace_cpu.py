"""Host side of the rigid-motion modes (waterscapes_gb300/nullspace.py): the basis of
rm_basis_L2.py:10-74 interpolated at the P2 nodes is L2-orthonormal under the
oracle's P2 mass matrix and spans the kernel of the oracle's displacement block
(pure traction), in 2D and 3D."""
import numpy as np
import pytest
import scipy.sparse as sp

from helpers import make_oracle


def _vector_mass(om):
    dm = om.dm
    d = dm.d
    cn = dm.cell_nodes
    cd = (d * cn[:, :, None] + np.arange(d)[None, None, :]).reshape(cn.shape[0], -1)
    loc = np.einsum("cij,kl->cikjl", om.M2, np.eye(d)).reshape(cn.shape[0], cd.shape[1], cd.shape[1])
    rows = np.repeat(cd, cd.shape[1], axis=1).ravel()
    cols = np.tile(cd, (1, cd.shape[1])).ravel()
    return sp.csr_matrix((loc.ravel(), (rows, cols)), shape=(dm.Nu, dm.Nu))


@pytest.mark.parametrize("dim", [2, 3])
def test_rigid_motions_orthonormal_and_in_kernel(dim):
    from waterscapes_gb300 import CompiledSubDomain, Constant, MPETProblem
    from waterscapes_gb300.mesh import AnnulusMesh, EllipsoidShellMesh
    from waterscapes_gb300.nullspace import rigid_motions
    mesh = AnnulusMesh(1.0, 2.0, 3, 16) if dim == 2 else EllipsoidShellMesh(2)
    params = dict(J=1, alpha=(0.5,), K=(0.1,), S=((0.0,),), c=(0.1,), nu=0.3, E=10.0)
    problem = MPETProblem(mesh, Constant(0.0), params=params)
    CompiledSubDomain.on_boundary().mark(problem.momentum_boundary_markers, 1)
    om = make_oracle(problem, 1.0)
    Z = rigid_motions(mesh, om.dm.node_x).reshape(-1, om.dm.Nu)
    assert Z.shape[0] == (3 if dim == 2 else 6)
    M = _vector_mass(om)
    assert np.allclose(Z @ (M @ Z.T), np.eye(Z.shape[0]), atol=1e-12)
    Auu = om.assemble_matrix(0.1)[:om.dm.Nu, :om.dm.Nu]
    assert np.abs(Auu @ Z.T).max() <= 1e-10 * abs(Auu).max()
