"""Parity at the benchmark's own configuration: the 640 x 80 (1 km, nσ = 4) channel solved to
||b - A u|| / ||b|| < 1e-6 (update_velocities.jl:59-65) from the benchmark's state, against the FP64
oracle's converged solve of the same state (tests/golden/c2_oracle_solution.npz, made by
tests/golden/make_c2_solution.py; the oracle takes minutes, so its result is a committed fixture).

  FP64, the reference algorithm (cg! coarse solve)          same Picard count, within 1e-9
  FP64, single-reduction Chebyshev coarse solve              within 1e-6 (another V-cycle, same fixed point)
  mixed precision (the benchmark's solve)                    within 1e-6

Relative error = ||(u, v) - (u, v)_oracle||_2 / ||(u, v)_oracle||_2 over the whole u and v grids."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "c2_oracle_solution.npz")


@pytest.fixture(scope="module")
def c2():
    sys.path.insert(0, os.path.dirname(HERE))
    import bench
    import __graft_entry__ as ge
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_c2_solution import fingerprints
    pkg = ge.load_package()
    m = bench.build_state(pkg)
    snap = {k: np.array(v, copy=True) for k, v in m.fields.items()}
    from wavi_gb300.model import release_solver
    release_solver(m)
    ref = np.load(FIXTURE)
    # the state rebuilt here is the one the oracle solved (numpy's seeded streams are stable; elementwise
    # math may differ in the last bit between machines)
    assert np.allclose(fingerprints(snap), ref["fingerprints"], rtol=1e-12, atol=0.0)
    return m, snap, ref


def _solve(m, snap, precision, coarse_solver="auto"):
    from wavi_gb300.gpu import ALL_FIELDS, VelocitySolver
    f = {k: np.array(snap[k], copy=True, order="F") for k in ALL_FIELDS}
    s = VelocitySolver(m.grid, m.solver_params, precision=precision, coarse_solver=coarse_solver)
    st = s.solve(m.params, f)
    s.close()
    return f, st


def _err(f, ref):
    num = np.sqrt(np.sum((f["u"] - ref["u"]) ** 2) + np.sum((f["v"] - ref["v"]) ** 2))
    return num / np.sqrt(np.sum(ref["u"] ** 2) + np.sum(ref["v"] ** 2))


def test_c2_fp64_reference_algorithm_matches_oracle(c2):
    m, snap, ref = c2
    f, st = _solve(m, snap, "fp64")
    err = _err(f, ref)
    print("fp64 cg!", err, st)
    assert st["status"] == 0, st
    assert st["coarse_solver"] == "cg"
    assert st["picard_iterations"] == int(ref["picard_iterations"]), st
    assert err < 1e-9, (err, st)


def test_c2_fp64_single_reduction_chebyshev_matches_oracle(c2):
    m, snap, ref = c2
    f, st = _solve(m, snap, "fp64", "srcg_chebyshev")
    err = _err(f, ref)
    print("fp64 srcg_chebyshev", err, st)
    assert st["status"] == 0, st
    assert err < 1e-6, (err, st)


def test_c2_mixed_matches_oracle(c2):
    m, snap, ref = c2
    f, st = _solve(m, snap, "mixed")
    err = _err(f, ref)
    print("mixed", err, st)
    assert st["status"] == 0, st
    assert err < 1e-6, (err, st)
