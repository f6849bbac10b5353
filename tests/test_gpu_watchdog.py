"""The persistent kernels' bounded waits, exercised without a GPU fault (wavi_selftest_watchdog): a wait
for a tagged word that nothing writes gives up after its poll limit and reports it, the error flag is
cleared, and the same context then solves normally."""
import time

import numpy as np
import pytest

from helpers import fields_from_oracle, uv_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_bounded_wait_gives_up_and_context_stays_usable(oracle):
    from wavi_gb300 import synthetic
    from wavi_gb300.gpu import VelocitySolver
    g, bed, p, sp, ic = synthetic.small_case(nx=40, ny=16, dx=4000.0, maxiter_picard=60, tol_picard=1e-7)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    f = fields_from_oracle(om, g)
    om.update_velocities()
    s = VelocitySolver(g, sp, precision="mixed")
    t0 = time.perf_counter()
    assert s.selftest_watchdog()
    assert time.perf_counter() - t0 < 60.0
    st = s.solve(p, f)
    assert st["status"] == 0, st
    assert uv_err(f, om) < 1e-6
    s.close()
