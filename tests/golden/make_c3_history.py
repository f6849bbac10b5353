"""Make tests/golden/c3_oracle_history.npz: the FP64 oracle's first Picard iterations on the large single
domain, 2560 x 320 at 250 m with nσ = 8 (log-normal C with a 20 km correlation length, A from a 243-268 K
vertical temperature profile; wavi_gb300.synthetic.channel_c3), from the model's initial state.

It records, per Picard iteration, the relative residual ||b - A u|| / ||b|| before the correction
(update_velocities.jl:59-65), the relative update ||du|| / ||u|| of the correction, and the coarse-CG
iteration count of the V-cycle (Wavelets/update_preconditioners.jl:54-83, cg! capped at maxiter_coarse =
1000, SolverParams.jl:2-13).  The GPU's FP64 solve of the same state is compared with it: whether the
reference algorithm itself stalls at this size (every coarse solve at maxiter_coarse) is a property of
the algorithm, and the oracle settles it.  A whole solve is far beyond a test's budget on the CPU
(about a minute and a half per Picard iteration on one core), so only the first iterations are kept.

Usage:  python tests/golden/make_c3_history.py [picard_iterations]   (default 5)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "c3_oracle_history.npz")
FINGERPRINT_FIELDS = ("h", "s", "grounded_fraction", "weertman_c", "gu_h", "gv_h", "glen_b")


def c3_state(pkg):
    """The host model of the 2560 x 320 case after the update_state! steps before the solve."""
    from wavi_gb300 import synthetic
    from wavi_gb300.model import GPUParallelSpec, Model, pre_solve
    g, bed, p, sp, ic = synthetic.channel_c3(tol_picard=1e-6, maxiter_picard=30)
    m = Model(g, bed, p, sp, ic, parallel_spec=GPUParallelSpec(precision="fp64"))
    pre_solve(m)
    return m, (g, bed, p, sp, ic)


def fingerprints(fields):
    return np.array([float(np.linalg.norm(np.asarray(fields[k], np.float64).ravel())) for k in FINGERPRINT_FIELDS])


def main():
    k = int(sys.argv[1]) if len(sys.argv) > 1 else 5
    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge
    pkg = ge.load_package()
    oracle = ge.load_oracle()
    m, (g, bed, p, sp, ic) = c3_state(pkg)
    snap = {f: np.array(v, copy=True) for f, v in m.fields.items()}
    from dataclasses import replace
    om = oracle.build_model(g, bed, p, replace(sp, maxiter_picard=k), ic)
    om.pre_solve()
    # the oracle's own steps before the solve agree with the host model's to rounding (glen_b's exp of the
    # temperature profile may differ in the last bit); the solve starts from the host model's exact state,
    # the one the GPU solves
    sys.path.insert(0, os.path.dirname(HERE))
    from helpers import SOLVE_FIELDS
    for f in SOLVE_FIELDS:
        a, b = np.asarray(om.field(f)), np.asarray(snap[f])
        d = float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))
        if d > 1e-13:
            raise SystemExit(f"the oracle's pre-solve state differs from the host model's in {f} by {d:.1e}")
        om.field(f)[...] = b
    t0 = time.perf_counter()
    om.update_velocities()
    sec = time.perf_counter() - t0
    st = om.stats()
    np.savez_compressed(OUT, rel_history=np.array(st["rel_history"]), update_history=np.array(st["update_history"]),
                        cg_history=np.array(st["cg_history"]), picard_iterations=k,
                        maxiter_coarse=sp.maxiter_coarse, fingerprints=fingerprints(snap),
                        fingerprint_fields=np.array(FINGERPRINT_FIELDS), oracle_seconds=sec)
    print(f"{OUT}: {k} Picard iterations in {sec:.0f} s")
    print("rel residual", st["rel_history"])
    print("rel update  ", st["update_history"])
    print("coarse cg   ", st["cg_history"])


if __name__ == "__main__":
    main()
