"""Anderson acceleration of the Picard loop (wavi_options.picard_accel = WAVI_PICARD_ANDERSON) and the
adaptive coarse tolerance (wavi_options.coarse_forcing = WAVI_FORCING_ADAPTIVE), the mixed defaults,
through the C ABI, against the oracle's restatement of the same iteration and against the oracle's fixed
point.

  FP64, the reference's cg! coarse solve, accelerated, with   the oracle's loop with the same options:
  the fixed and the adaptive coarse tolerance                 Picard count within 1, velocities within 1e-7
  mixed precision, accelerated                                the oracle's fixed point (solved to 1e-11)
                                                              within 1e-6, in fewer Picard iterations
                                                              than the plain mixed solve
  640 x 80 benchmark state, mixed, accelerated                tests/golden/c2_oracle_fixed_point.npz
                                                              within 1e-6

Both sides stop on the reference's residual test (update_velocities.jl:59-65); a converged accelerated
solve therefore meets the same criterion as the reference's, but along another path, so it is compared
with the fixed point, not with the point where the plain iteration stops.  Errors are relative 2-norms
over the whole u and v grids.
"""
import os
import sys

import numpy as np
import pytest

from helpers import fields_from_oracle, uv_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    "full": dict(nx=40, ny=16, dx=4000.0, mask="full"),
    "disc": dict(nx=24, ny=24, dx=4000.0, mask="disc"),
    "fixed": dict(nx=20, ny=20, dx=5000.0, mask="disc", fixed=True),
}


def _setup(oracle, name, **kw):
    from wavi_gb300 import synthetic
    c = dict(CASES[name])
    c.update(kw)
    g, bed, p, sp, ic = synthetic.small_case(**c)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    return g, p, sp, om


def _oracle_solve(oracle, om, depth, forcing=False):
    oracle.set_anderson(depth)
    oracle.set_coarse_forcing(forcing)
    try:
        om.update_velocities()
    finally:
        oracle.set_anderson(0)
        oracle.set_coarse_forcing(False)
    return om.stats()


@pytest.mark.parametrize("forcing", ["fixed", "adaptive"])
@pytest.mark.parametrize("name", list(CASES))
def test_fp64_anderson_follows_oracle(oracle, name, forcing):
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, name, maxiter_picard=80, tol_picard=1e-7)
    f = fields_from_oracle(om, g)
    s = VelocitySolver(g, sp, precision="fp64", picard_accel="anderson", coarse_forcing=forcing)
    st = s.solve(p, f)
    s.close()
    ost = _oracle_solve(oracle, om, 3, forcing == "adaptive")
    err = uv_err(f, om)
    print(name, forcing, "fp64 anderson vs oracle", err, st["picard_iterations"], ost["picard_iterations"],
          st["anderson_steps"], st["coarse_cg_iterations"], ost["coarse_cg_iterations"])
    assert st["status"] == 0, st
    assert st["anderson_steps"] > 0 and st["coarse_forcing"] == forcing
    assert abs(st["picard_iterations"] - ost["picard_iterations"]) <= 1, (st, ost)
    assert err < 1e-7, (err, st, ost)


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_anderson_reaches_fixed_point(oracle, name):
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, name, maxiter_picard=200, tol_picard=1e-11)
    f0 = fields_from_oracle(om, g)
    ost = _oracle_solve(oracle, om, 3)  # the fixed point, to 1e-11
    assert ost["rel_residual"] < 1e-11, ost
    sp.tol_picard, sp.maxiter_picard = 1e-6, 100
    res = {}
    for accel, forcing in (("plain", "fixed"), ("anderson", "fixed"), ("auto", "auto")):
        f = {k: np.array(a, copy=True) for k, a in f0.items()}
        s = VelocitySolver(g, sp, precision="mixed", picard_accel=accel, coarse_forcing=forcing)
        st = s.solve(p, f)
        s.close()
        res[accel] = (uv_err(f, om), st)
        print(name, accel, forcing, res[accel][0], st["picard_iterations"], st["anderson_steps"],
              st["coarse_cg_iterations"])
        assert st["status"] == 0, st
    for accel in ("anderson", "auto"):
        err, st = res[accel]
        assert err < 1e-6, res
        assert st["anderson_steps"] > 0
        assert st["picard_iterations"] < res["plain"][1]["picard_iterations"], res
    # the mixed defaults: Anderson and the adaptive coarse tolerance, fewer coarse iterations again
    assert res["auto"][1]["picard_accel"] == "anderson" and res["auto"][1]["coarse_forcing"] == "adaptive"
    assert res["auto"][1]["coarse_cg_iterations"] < res["anderson"][1]["coarse_cg_iterations"], res


def test_anderson_options_are_checked():
    from wavi_gb300 import abi, synthetic
    from wavi_gb300.gpu import VelocitySolver
    g, bed, p, sp, ic = synthetic.small_case(nx=24, ny=12)
    for kw in (dict(picard_accel="anderson", anderson_depth=6), dict(picard_accel="anderson", anderson_depth=-1)):
        with pytest.raises(abi.WaviError):
            VelocitySolver(g, sp, precision="mixed", **kw)
    s = VelocitySolver(g, sp, precision="mixed", picard_accel="anderson", anderson_depth=5)
    s.close()
    lib = abi.load_library()
    import ctypes as C
    for field, bad in (("picard_accel", 3), ("coarse_forcing", 3), ("coarse_forcing", -1)):
        opt = abi.Options(0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0)
        setattr(opt, field, bad)
        ctx = C.c_void_p()
        desc, spc = g.descriptor(), sp.to_c()
        assert lib.wavi_ctx_create(C.byref(desc.desc), C.byref(spc), C.byref(opt), C.byref(ctx)) != 0, field


def test_c2_mixed_anderson_matches_oracle_fixed_point():
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import bench
    import __graft_entry__ as ge
    from make_c2_solution import fingerprints
    from wavi_gb300.gpu import ALL_FIELDS, VelocitySolver
    from wavi_gb300.model import release_solver
    pkg = ge.load_package()
    m = bench.build_state(pkg)
    snap = {k: np.array(v, copy=True) for k, v in m.fields.items()}
    release_solver(m)
    ref = np.load(os.path.join(HERE, "golden", "c2_oracle_fixed_point.npz"))
    assert np.allclose(fingerprints(snap), ref["fingerprints"], rtol=1e-12, atol=0.0)
    f = {k: np.array(snap[k], copy=True, order="F") for k in ALL_FIELDS}
    s = VelocitySolver(m.grid, m.solver_params, precision="mixed")  # the defaults: Anderson, adaptive tolerance
    st = s.solve(m.params, f)
    s.close()
    num = np.sqrt(np.sum((f["u"] - ref["u"]) ** 2) + np.sum((f["v"] - ref["v"]) ** 2))
    err = num / np.sqrt(np.sum(ref["u"] ** 2) + np.sum(ref["v"] ** 2))
    print("c2 mixed anderson vs the oracle's fixed point", err, st)
    assert st["status"] == 0, st
    assert st["anderson_steps"] > 0
    assert err < 1e-6, (err, st)
