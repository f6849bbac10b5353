"""The opt-in pipelined coarse CG (WAVI_COARSE_PIPELINED_CHEBYSHEV, k_pcg_persistent): its requirements are
checked when a context is made; its solves are checked against the reference's FP64 solve and against the
single-reduction Chebyshev solver it pipelines.  The FP64 oracle states its iteration (coarse variant 5,
tests/test_oracle_coarse.py).  Measured on GB300: it reaches the reference's fixed point, but with 1.35x
(40 x 16) to 1.96x (37 x 13) the coarse iterations of the single-reduction solver, and 1.46x on the
640 x 80 benchmark (5810 against 3989) at 10.45 against 10.77 us per iteration, so it is not the default."""
import numpy as np
import pytest

from helpers import fields_from_oracle, uv_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


CASES = {
    "full": dict(nx=40, ny=16, dx=4000.0, mask="full"),
    "ragged": dict(nx=37, ny=13, dx=3000.0, mask="full"),
    "channel": dict(nx=96, ny=32, dx=2000.0, mask="full"),
}
# Picard tolerance per case: on the 96 x 32 channel the reference algorithm itself does not reach 1e-6
# within 100 Picard iterations (the oracle's residual oscillates between 3.6e-6 and 9e-6); there the GPU
# solves run the same 100 iterations and are compared with the oracle's at that point
TOL = {"full": 1e-7, "ragged": 1e-7, "channel": 1e-6}


def _setup(oracle, name, **kw):
    from wavi_gb300 import synthetic
    g, bed, p, sp, ic = synthetic.small_case(**{**CASES[name], **kw})
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    return g, p, sp, om


def test_pipelined_needs_mixed_precision_and_16x16_tiles(oracle):
    """Rejected, without a launch, in FP64 and with 32 x 32 tiles (levels 4)."""
    from wavi_gb300.abi import WaviError
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, "full")
    with pytest.raises(WaviError, match="WAVI_ERR_ARGUMENT"):
        VelocitySolver(g, sp, precision="fp64", coarse_solver="pipelined_chebyshev")
    from wavi_gb300.config import SolverParams
    with pytest.raises(WaviError, match="WAVI_ERR_ARGUMENT"):
        VelocitySolver(g, SolverParams(levels=4), precision="mixed", coarse_solver="pipelined_chebyshev")


@pytest.mark.parametrize("name", list(CASES))
def test_pipelined_converged_solve_matches_reference(oracle, name):
    """The pipelined coarse solve changes the V-cycle, not the fixed point: the converged mixed solve (the
    reference's plain Picard iteration and coarse tolerance, like the oracle's) agrees with the reference's
    FP64 solve to 1e-6.  Its restarts from the true residual and the FP32 drift of its
    recurrences cost coarse iterations: at most 2.5x those of the single-reduction Chebyshev solve with the
    same 3 Chebyshev steps (GB300: 1.35x and 1.96x on the first two cases)."""
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, name, maxiter_picard=100, tol_picard=TOL[name])
    f0 = fields_from_oracle(om, g)
    om.update_velocities()
    converged = om.stats()["picard_iterations"] < 100
    stats = {}
    for solver in ("srcg_chebyshev", "pipelined_chebyshev"):
        f = {k: np.array(v, copy=True, order="F") for k, v in f0.items()}
        s = VelocitySolver(g, sp, precision="mixed", coarse_solver=solver, cheb_steps=3, picard_accel="plain",
                           coarse_forcing="fixed")
        st = s.solve(p, f)
        s.close()
        print(name, solver, st["picard_iterations"], st["coarse_cg_iterations"], st["rel_residual"], uv_err(f, om))
        assert (st["status"] == 0) == converged, (solver, st)
        assert st["coarse_solver"] == solver
        assert uv_err(f, om) < 1e-6, (solver, st)
        stats[solver] = st
    a, b = stats["srcg_chebyshev"], stats["pipelined_chebyshev"]
    assert b["coarse_cg_iterations"] <= 2.5 * a["coarse_cg_iterations"], (a, b)
