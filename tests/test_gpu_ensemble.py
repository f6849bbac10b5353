"""Ensembles through the C ABI (wavi_ensemble_*): ragged members solved concurrently give each member's
own solve, checked against the FP64 oracle member by member."""
import numpy as np
import pytest

from helpers import fields_from_oracle, to_dev, from_dev, uv_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MEMBERS = [
    dict(nx=40, ny=16, dx=4000.0, mask="full", seed=0),
    dict(nx=24, ny=24, dx=4000.0, mask="disc", seed=1),
    dict(nx=37, ny=13, dx=3000.0, mask="full", seed=2),
    dict(nx=20, ny=20, dx=5000.0, mask="disc", fixed=True, seed=3),
    dict(nx=64, ny=20, dx=4000.0, mask="full", seed=4),
    dict(nx=30, ny=30, dx=4000.0, mask="disc", seed=5),
]


def _members(oracle, **kw):
    from wavi_gb300 import synthetic
    out = []
    for m in MEMBERS:
        g, bed, p, sp, ic = synthetic.small_case(**m, **kw)
        om = oracle.build_model(g, bed, p, sp, ic)
        om.pre_solve()
        out.append((g, p, sp, om, fields_from_oracle(om, g)))
    return out


@pytest.mark.parametrize("concurrency", [1, 4, 16])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-6)])
def test_ensemble_members_match_oracle(oracle, precision, tol, concurrency):
    from wavi_gb300.ensemble import EnsembleSolver
    mem = _members(oracle, maxiter_picard=80, tol_picard=1e-7)
    ens = EnsembleSolver([m[0] for m in mem], [m[2] for m in mem], precision=precision, concurrency=concurrency)
    tensors = [to_dev(m[4], torch) for m in mem]
    stats = ens.solve_device([m[1] for m in mem], tensors)
    for k, (g, p, sp, om, f) in enumerate(mem):
        from_dev(tensors[k], f)
        om.update_velocities()
        assert stats[k]["status"] == 0, (k, stats[k])
        assert uv_err(f, om) < tol, (k, uv_err(f, om), stats[k])
    ens.close()


def test_ensemble_matches_single_solves(oracle):
    """A member's result does not depend on the other members or on how many run at once."""
    from wavi_gb300.ensemble import EnsembleSolver
    from wavi_gb300.gpu import VelocitySolver
    mem = _members(oracle, maxiter_picard=3)
    ens = EnsembleSolver([m[0] for m in mem], [m[2] for m in mem], precision="fp64", concurrency=3,
                         coarse_kernel="iterations")
    tensors = [to_dev(m[4], torch) for m in mem]
    ens.solve_device([m[1] for m in mem], tensors)
    for k, (g, p, sp, om, f) in enumerate(mem):
        s = VelocitySolver(g, sp, precision="fp64", coarse_kernel="iterations")
        t = to_dev(f, torch)
        s.solve_device(p, t)
        for name in ("u", "v", "eta", "wu_correction_coarse"):
            a, b = tensors[k][name].cpu().numpy(), t[name].cpu().numpy()
            assert np.array_equal(a, b), (k, name, np.abs(a - b).max())
        s.close()
    ens.close()


def test_ensemble_reports_the_failing_member(oracle):
    from wavi_gb300.abi import WaviError
    from wavi_gb300.ensemble import EnsembleSolver
    mem = _members(oracle, maxiter_picard=2)
    ens = EnsembleSolver([m[0] for m in mem], [m[2] for m in mem], precision="mixed", concurrency=2)
    params = [m[1] for m in mem]
    import dataclasses
    params[3] = dataclasses.replace(params[3], glen_n=0.0)
    with pytest.raises(WaviError, match="member 3"):
        ens.solve_device(params, [to_dev(m[4], torch) for m in mem])
    # the ensemble stays usable
    stats = ens.solve_device([m[1] for m in mem], [to_dev(m[4], torch) for m in mem])
    assert len(stats) == len(mem)
    ens.close()


def test_autotune_picks_a_candidate(oracle):
    from wavi_gb300.ensemble import autotune
    mem = _members(oracle, maxiter_picard=5)
    cands = (dict(concurrency=2, coarse_kernel="auto"), dict(concurrency=6, coarse_kernel="iterations"))
    best, timings = autotune([m[0] for m in mem], [m[2] for m in mem], [m[1] for m in mem],
                             lambda: [to_dev(m[4], torch) for m in mem], candidates=cands, picard=2, finalists=1,
                             sync=torch.cuda.synchronize)
    # two capped solves, then the whole solve of the faster one, which is the choice
    assert best in cands and len(timings) == 3 and all(t > 0 for t, _, _ in timings)
    assert [st for _, _, st in timings] == ["capped", "capped", "whole"]
    assert timings[2][1] == best == min(timings[:2], key=lambda t: t[0])[1]


@pytest.fixture(scope="module")
def ragged_members(oracle):
    """Three of the smallest members of the benchmark's 256-member ragged ensemble (77 x 24, 147 x 17 and
    84 x 28 at 2 km), with the oracle's converged solves (tol 1e-6, about 17 s of oracle time)."""
    from wavi_gb300 import synthetic
    ens = synthetic.ensemble_members()
    out = []
    for k in (186, 45, 160):
        g, bed, p, sp, ic = ens[k]
        om = oracle.build_model(g, bed, p, sp, ic)
        om.pre_solve()
        f = fields_from_oracle(om, g)
        om.update_velocities()
        out.append((g, p, sp, om, f))
    return out


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-7), ("mixed", 2e-6)])
def test_benchmark_ensemble_members_match_oracle(ragged_members, precision, tol):
    """Members of the measured ensemble itself, solved together at the benchmark's tolerance, against the
    oracle's own converged solves of the same members."""
    from wavi_gb300.ensemble import EnsembleSolver
    mem = ragged_members
    ens = EnsembleSolver([m[0] for m in mem], [m[2] for m in mem], precision=precision, concurrency=3)
    tensors = [to_dev(m[4], torch) for m in mem]
    stats = ens.solve_device([m[1] for m in mem], tensors)
    for k, (g, p, sp, om, f) in enumerate(mem):
        got = {name: np.array(a, copy=True, order="F") for name, a in f.items()}  # f stays the initial state
        from_dev(tensors[k], got)
        assert stats[k]["status"] == 0 and stats[k]["rel_residual"] < sp.tol_picard, (k, stats[k])
        assert uv_err(got, om) < tol, (k, uv_err(got, om), stats[k], om.stats()["picard_iterations"])
    ens.close()
