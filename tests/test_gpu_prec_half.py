"""FP16 values for the first level of each hierarchy (SpMV variant 32).

The first-level operators of the mixed-precision preconditioner can be
stored with FP16 off-diagonal values (times a power of two) and an FP32
diagonal that keeps the row sums of the original operator.  The rounded
operator is a slightly different preconditioner: one application agrees
with the FP32 one to about the FP16 rounding (1e-2 relative is the bar
here), and a step with it is still the oracle's step (the FP64 refinement
corrects the inner solves), at the same 1e-8 bar.
"""
import ctypes

import numpy as np
import pytest

from helpers import make_oracle, make_problem, oracle_data

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _apply(s, variant):
    from waterscapes_gb300 import _lib
    s.ctx.call("mpet_set_hierarchy_spmv_variant", variant)
    r = torch.tensor(np.random.default_rng(5).standard_normal(s.N), dtype=torch.float32, device=s.device)
    z = torch.empty_like(r)
    s.ctx.call("mpet_apply_preconditioner", 1, _lib._ptr(r), _lib._ptr(z))
    torch.cuda.synchronize()
    return z.double().cpu().numpy()


def test_half_first_level_close_to_fp32_and_step_matches_oracle():
    from waterscapes_gb300 import MPETSolver, _lib
    problem, dt = make_problem(6, 2)
    s = MPETSolver(problem, dict(dt=dt, T=dt, precision="mixed", rtol=1e-11))
    s.ctx.call("mpet_assemble", dt, 1)
    s.ctx.call("mpet_setup_preconditioner", dt)
    z4 = _apply(s, 4)     # SELL-32, FP32 values
    z32 = _apply(s, 32)   # first levels with FP16 values, the others CSR
    va = np.zeros(16, np.int32)
    s.ctx.call("mpet_get_amg_variants", 0, _lib._ptr(va), None, None)
    assert va[0] == 32
    d = np.linalg.norm(z32 - z4) / np.linalg.norm(z4)
    assert 0.0 < d <= 1e-2
    # a step with the FP16 first levels (the override holds until the next set-up,
    # which this step does not make: the preconditioner for this dt exists)
    s._prec_dt = float(dt)
    problem.time.assign(0.0)
    st = s.step(dt)
    assert st.status == 0
    om = make_oracle(problem)
    x_ref = om.step(np.zeros(om.dm.N), 0.0, dt, oracle_data(2))
    x = s.up.vector().cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
