"""Host side of batches: the union mesh keeps every instance's boundary
facets and markers in order, and per-instance data dispatch by position."""
import numpy as np
import pytest

from waterscapes_gb300 import Expression, Mesh, UnitCubeMesh

torch = pytest.importorskip("torch")


def test_union_mesh_matches_rebuilt_boundary():
    from waterscapes_gb300.batch import _union_mesh
    meshes = [UnitCubeMesh(2), UnitCubeMesh(3), UnitCubeMesh(1)]
    u, L, lo = _union_mesh(meshes)
    ref = Mesh(u.coordinates(), u.cells())
    assert np.array_equal(u.boundary_facets(), ref.boundary_facets())
    assert np.array_equal(u.boundary_facet_cells(), ref.boundary_facet_cells())
    assert u.num_cells() == sum(m.num_cells() for m in meshes)
    # instance i occupies [i L, i L + 1) in x
    x = u.coordinates()
    off = 0
    for i, m in enumerate(meshes):
        xi = x[off:off + m.num_vertices()]
        assert np.allclose(xi[:, 0] - i * L, m.coordinates()[:, 0])
        off += m.num_vertices()


def test_batch_expression_dispatch():
    from waterscapes_gb300.batch import BatchExpression
    fs = [Expression(lambda x, t, k=k: (k + 1) * x[:, 0] + t) for k in range(3)]
    e = BatchExpression(fs, 2.0, False)
    x = torch.tensor([[0.5, 0, 0], [2.25, 0, 0], [4.75, 1, 1], [0.0, 1, 0]], dtype=torch.float64)
    v = e(x, 1.0)
    assert torch.allclose(v, torch.tensor([1.5, 1.5, 3.25, 1.0], dtype=torch.float64))
    z = BatchExpression([None, 0.0, None], 2.0, True)
    assert z.is_zero()
