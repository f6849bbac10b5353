"""Time stepping through the product path: the host mirror of update_state!/run_simulation! with the GPU
velocity solve (float64), against the reference's MISMIP+ golden file and against the CPU oracle.

  * MISMIP+ 100 years (1000 steps of dt = 0.1, maxiter_picard = 1), the reference's version-update test
    (test/version_update_test_verification/test_version_updates.jl:6-97).  The early steps run coarse CGs
    of up to 1000 iterations whose result depends at the 1e-5 level on the summation order of their dot
    products (the oracle matches the golden file to sqrt(eps) only when it follows Julia's OpenBLAS order;
    the GPU sums in a tree), and the coupled run keeps that difference: GPU vs golden and GPU vs oracle
    are held to the level a different summation order gives (measured 1.2e-4 in u).
  * The 8 km channel (80 x 10, seeded bed and thickness): one Picard-converged solve, then 200 steps of
    dt = 0.5 yr with maxiter_picard = 1, against the oracle.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))

GOLDEN_TOL = {"h": 2e-5, "u": 2.5e-4, "v": 5e-5, "viscosity": 5e-4, "grounded_fraction": 5e-5, "bed_speed": 2.5e-4}
GOLDEN_KEYS = {"h": "h", "u": "u", "v": "v", "viscosity": "eta_av", "grounded_fraction": "grounded_fraction",
               "bed_speed": "bed_speed"}


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_mismip_golden_through_gpu(oracle, pkg):
    from wavi_gb300 import config
    from wavi_gb300.model import GPUParallelSpec, Model, Simulation, release_solver, run_simulation
    from wavi_gb300.synthetic import mismip_plus_bed
    g = config.Grid(nx=80, ny=10, nσ=4, x0=0.0, y0=-40000.0, dx=8000.0, dy=8000.0, u_iszero=["north"],
                    v_iszero=["west", "east"])
    p = config.Params(default_thickness=100.0, accumulation_rate=0.3, default_temperature=265.700709)
    sp = config.SolverParams(maxiter_picard=1)
    m = Model(g, lambda x, y: float(mismip_plus_bed(x, y)), p, sp, parallel_spec=GPUParallelSpec(precision="fp64"))
    sim = Simulation(m, config.TimesteppingParams(dt=0.1, end_time=100.0))
    run_simulation(sim)
    release_solver(m)
    gold = np.load(os.path.join(HERE, "golden", "mismip_100yr_v1_8_3.npz"))
    for name, key in GOLDEN_KEYS.items():
        assert _rel(m.fields[key], gold[name]) < GOLDEN_TOL[name], name
    om = oracle.build_model(g, lambda x, y: float(mismip_plus_bed(x, y)), p, sp)
    om.run(1000, 0.1)
    for name, key in GOLDEN_KEYS.items():
        assert _rel(m.fields[key], om.field(key)) < GOLDEN_TOL[name], key


def test_channel_c1_converged_then_200_steps(oracle, pkg):
    from wavi_gb300 import config, synthetic
    from wavi_gb300.model import (GPUParallelSpec, Model, Simulation, release_solver, run_simulation,
                                  update_state)
    g, bed, p, sp, ic = synthetic.channel_c1(tol_picard=1e-5, maxiter_picard=30)
    m = Model(g, bed, p, sp, ic, parallel_spec=GPUParallelSpec(precision="fp64"))
    om = oracle.build_model(g, bed, p, sp, ic)
    update_state(m)  # one Picard-converged (or 30-iteration) solve
    om.update_state()
    assert m.last_stats["picard_iterations"] == om.stats()["picard_iterations"]
    assert _rel(m.fields["u"], om.field("u")) < 1e-6
    release_solver(m)
    m.solver_params = config.SolverParams(maxiter_picard=1)
    sim = Simulation(m, config.TimesteppingParams(dt=0.5, n_iter_total=200))
    run_simulation(sim)
    release_solver(m)
    oracle.lib().oracle_set_params(om.h, __import__("ctypes").byref(p.to_c()),
                                   __import__("ctypes").byref(config.SolverParams(maxiter_picard=1).to_c()), 0.0)
    om.run(200, 0.5)
    for key in ("h", "u", "v", "eta_av", "bed_speed"):
        assert _rel(m.fields[key], om.field(key)) < 1e-5, key
