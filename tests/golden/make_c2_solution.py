"""Make tests/golden/c2_oracle_solution.npz: the FP64 oracle's Picard-converged velocity solve of the
640 x 80 (1 km, nσ = 4) channel, the benchmark's workload, on the exact state the benchmark solves.

The state is bench.build_state()'s: the seeded 8 km channel refined to 1 km, at the model's initial
state (u = 0, default viscosity, the reference's initial all-true wavelet coarse space) after the
update_state! steps that precede the solve.  The oracle solves it with the benchmark's solver
parameters (tol_picard = 1e-6 on ||b - A u|| / ||b||, update_velocities.jl:59-65; maxiter_picard = 100;
the reference's defaults otherwise, SolverParams.jl:2-13) and the reference's own algorithm
(update_velocities.jl:11-29 with the V-cycle of Wavelets/update_preconditioners.jl:54-83).

Saved: u (641 x 80) and v (640 x 81) in float64; the Picard count, final relative residual and coarse-CG
iterations; fingerprints of the inputs (norms of h, bed-dependent fields and glen_b) so that a test can
confirm it rebuilt the same state; and the oracle's single-thread time of the whole solve and of its first
SAMPLE_PICARD Picard iterations, whose ratio scales the benchmark's bounded CPU sample (those iterations,
timed on the benchmark machine's host cores) to a whole solve.  The oracle takes a few minutes on one core.

Usage:  python tests/golden/make_c2_solution.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "c2_oracle_solution.npz")

FINGERPRINT_FIELDS = ("h", "s", "grounded_fraction", "weertman_c", "gu_h", "gv_h", "glen_b")
SAMPLE_PICARD = 2


def fingerprints(fields):
    return np.array([float(np.linalg.norm(np.asarray(fields[k], np.float64).ravel())) for k in FINGERPRINT_FIELDS])


def main():
    sys.path.insert(0, ROOT)
    import bench
    import __graft_entry__ as ge
    pkg = ge.load_package()
    oracle = ge.load_oracle()
    from wavi_gb300 import synthetic
    m = bench.build_state(pkg)
    snap = {k: np.array(v, copy=True) for k, v in m.fields.items()}
    g, bed, p, sp, ic = synthetic.channel_c2(tol_picard=bench.TOL_PICARD, maxiter_picard=bench.MAXITER_PICARD)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    # the oracle's own steps before the solve give the benchmark's state; check it, then solve
    for k in FINGERPRINT_FIELDS + ("u", "v", "eta", "beta", "quad_f2", "dsdh", "gu_s", "gv_s"):
        if not np.array_equal(np.asarray(om.field(k)), np.asarray(snap[k])):
            raise SystemExit(f"the oracle's pre-solve state differs from the benchmark's in {k}")
    t0 = time.perf_counter()
    om.update_velocities()
    sec = time.perf_counter() - t0
    st = om.stats()
    u, v = np.array(om.field("u"), order="F"), np.array(om.field("v"), order="F")
    # the first SAMPLE_PICARD Picard iterations of the same solve, timed alone
    g2, bed2, p2, sp2, ic2 = synthetic.channel_c2(tol_picard=bench.TOL_PICARD, maxiter_picard=SAMPLE_PICARD)
    om2 = oracle.build_model(g2, bed2, p2, sp2, ic2)
    om2.pre_solve()
    t0 = time.perf_counter()
    om2.update_velocities()
    sample_sec = time.perf_counter() - t0
    np.savez_compressed(OUT, u=u, v=v, picard_iterations=st["picard_iterations"],
                        rel_residual=st["rel_residual"], coarse_cg_iterations=st["coarse_cg_iterations"],
                        tol_picard=bench.TOL_PICARD, maxiter_picard=bench.MAXITER_PICARD,
                        fingerprint_fields=np.array(FINGERPRINT_FIELDS), fingerprints=fingerprints(snap),
                        oracle_seconds=sec, sample_picard=SAMPLE_PICARD, sample_seconds=sample_sec,
                        cg_history=np.array(st["cg_history"]))
    print(f"{OUT}: picard {st['picard_iterations']}, rel residual {st['rel_residual']:.3e}, "
          f"coarse cg {st['coarse_cg_iterations']}, {sec:.1f} s; first {SAMPLE_PICARD} Picard iterations "
          f"{sample_sec:.1f} s")


if __name__ == "__main__":
    main()
