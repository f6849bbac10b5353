"""The reference's iceberg verification (test/verification_tests/iceberg_test.jl) through the device-resident
time stepping (wavi_run_device): a masked, floating domain with Dirichlet centre lines, 10 000 steps of
dt = 0.1 with one Picard iteration each, against the closed-form steady state at the reference's
tolerances (the oracle meets the same tolerances in tests/test_oracle.py).  Unlike the channel and MISMIP+
runs, this domain is masked and floating, with calving fronts and Dirichlet lines."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_iceberg_reaches_the_analytic_steady_state_on_the_device(precision):
    from wavi_gb300 import synthetic
    from wavi_gb300.config import TimesteppingParams
    from wavi_gb300.model import GPUParallelSpec, Model, Simulation, release_solver, run_simulation
    g, bed, p, sp, ic = synthetic.iceberg_case()
    m = Model(g, bed, p, sp, ic, parallel_spec=GPUParallelSpec(precision=precision, device_run=True))
    sim = Simulation(m, TimesteppingParams(dt=0.1, end_time=1000.0))
    run_simulation(sim)
    release_solver(m)
    assert sim.n_iter == 10000
    h0, u0, v0 = synthetic.iceberg_analytic(g)
    f = m.fields
    assert synthetic.relative_error(f["h"], h0, np.asarray(g.h_mask, bool)) < 1.0e-4
    assert synthetic.relative_error(f["u"], u0, m.u_mask) < 3.0e-4
    assert synthetic.relative_error(f["v"], v0, m.v_mask) < 3.0e-4
