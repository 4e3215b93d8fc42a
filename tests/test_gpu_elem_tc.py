"""The tensor-core element kernel (tcgen05, waterscapes_gb300/csrc/elem_tc.cu)
against the FP64 CUDA-core element kernel and the oracle.

Both kernels write the same per-cell record (the 55 unique 3 x 3
displacement blocks and the u-p coupling values of mpetsolver.py:196-201),
which the row-owner gather sums into the CSR values: the assembled matrices
must agree to round-off (1e-14 of the largest entry), on a Kuhn cube whose
cell count is not a multiple of the 14-cell tile and on a jittered ellipsoidal
shell (irregular cells), and the tensor-core matrix must agree with the
oracle's to 1e-12.
"""
import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _values(s, dt, kind):
    s.ctx.call("mpet_set_element_kernel", kind)
    s.ctx.call("mpet_assemble", dt, 1)
    return s.matrix_values()


@pytest.mark.parametrize("case", ["cube", "shell"])
def test_tensor_core_elements_match_fp64_kernel_and_oracle(case):
    from waterscapes_gb300 import MPETSolver
    if case == "cube":
        problem, dt = make_problem(6, 4)
        assert problem.mesh.num_cells() % 14 != 0
    else:
        import bench
        problem, dt = bench.workload(3, 2, "ellipsoid")
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision="mixed"))
    v0 = _values(s, dt, 0)
    v1 = _values(s, dt, 1)
    scale = np.abs(v0).max()
    assert np.abs(v1 - v0).max() <= 1e-14 * scale
    if case == "cube":
        om = make_oracle(problem)
        dofs, _ = om.dirichlet_values(0.0, oracle_data(4))
        Abc = om.apply_bc_matrix(om.assemble_matrix(dt), dofs)
        assert np.abs(v1 - Abc.data).max() <= 1e-12 * np.abs(Abc.data).max()
    # a step on the tensor-core matrix is a normal step
    problem.time.assign(0.0)
    st = s.step(dt)
    assert st.status == 0
