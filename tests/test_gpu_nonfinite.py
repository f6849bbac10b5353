"""Non-finite inputs through the C ABI.  The reference has no check: a NaN in h, C or A runs through its
Picard loop (update_velocities.jl:59-65 compares the NaN residual with tol_picard, which is false, until
maxiter_picard).  This library's contract: a non-finite Picard residual ends the solve with
WAVI_ERR_NONFINITE before any V-cycle runs on it, and the same context then solves clean inputs as if
nothing had happened.  The failure is made on the host (a NaN or Inf written into one input cell); no
GPU fault is involved."""
import numpy as np
import pytest

from helpers import fields_from_oracle, uv_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("field,value", [("h", np.nan), ("weertman_c", np.nan), ("glen_b", np.nan),
                                         ("glen_b", np.inf), ("gu_h", np.nan)])
def test_nonfinite_input_is_reported_and_the_context_recovers(oracle, precision, field, value):
    from wavi_gb300 import synthetic
    from wavi_gb300.abi import WaviError
    from wavi_gb300.gpu import VelocitySolver
    g, bed, p, sp, ic = synthetic.small_case(nx=40, ny=16, dx=4000.0, maxiter_picard=80, tol_picard=1e-7)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    f0 = fields_from_oracle(om, g)
    om.update_velocities()
    s = VelocitySolver(g, sp, precision=precision)
    bad = {k: np.array(v, copy=True, order="F") for k, v in f0.items()}
    a = bad[field]
    idx = tuple(n // 2 for n in a.shape)  # an interior ice cell
    a[idx] = value
    with pytest.raises(WaviError, match="WAVI_ERR_NONFINITE"):
        s.solve(p, bad)
    f = {k: np.array(v, copy=True, order="F") for k, v in f0.items()}
    st = s.solve(p, f)  # the same context, clean inputs
    s.close()
    assert st["status"] == 0, st
    assert uv_err(f, om) < (1e-9 if precision == "fp64" else 1e-6), st
