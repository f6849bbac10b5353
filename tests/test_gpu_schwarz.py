"""Restricted additive Schwarz (wavi_gb300.schwarz, the reference's SharedMemorySpec) through the GPU: the
subdomains solved by their own velocity-solver contexts or as ensemble members, and the global residual
test by a one-iteration solve, against the same loop driven by the oracle (the host logic is covered by
tests/test_schwarz.py).  A subdomain's adaptive coarse space can be empty after update_wavelets!; the
ensemble staging keeps such a member's compact correction addressable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


class _OracleSubdomain:
    def __init__(self, om):
        self.om = om
        self.fields = {"u": om.field("u"), "v": om.field("v")}


def _models(oracle):
    """A host model on the GPU spec and its oracle twin, after the steps before the solve."""
    from dataclasses import replace
    from wavi_gb300 import synthetic
    from wavi_gb300.model import GPUParallelSpec, Model, pre_solve
    g, bed, p, sp, ic = synthetic.small_case(nx=32, ny=16, dx=4000.0)
    sp = replace(sp, maxiter_picard=4, tol_picard=1e-7)
    m = Model(g, bed, p, sp, ic, parallel_spec=GPUParallelSpec(precision="fp64"))
    pre_solve(m)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    return m, om


def _oracle_loop(oracle, om, m_host, spec):
    """The same Schwarz loop with the oracle relinearising and solving (tests/test_schwarz.py)."""
    from wavi_gb300.schwarz import update_velocities_schwarz
    iu, iv = om.mask("u_inner").astype(bool), om.mask("v_inner").astype(bool)

    def residual(model):
        om.field("u")[...] = model.fields["u"]
        om.field("v")[...] = model.fields["v"]
        om.inner_update()
        bu, bv = om.rhs()
        au, av = om.apply_operator(model.fields["u"] * iu, model.fields["v"] * iv)
        r = np.concatenate([(bu - au)[iu], (bv - av)[iv]])
        return float(np.linalg.norm(r) / np.linalg.norm(np.concatenate([bu[iu], bv[iv]])))
    return update_velocities_schwarz(m_host, spec, global_residual=residual, solve=lambda s: s.om.update_state(),
                                     make=lambda *a: _OracleSubdomain(oracle.build_model(*a)))


@pytest.mark.parametrize("batched", [False, True])
def test_schwarz_loop_on_the_gpu_follows_the_oracle(oracle, batched):
    """Four Picard iterations of the Schwarz loop, 2 x 2 subdomains: the GPU (subdomains by their own
    contexts, or as ensemble members; FP64) and the oracle give the same residual history to 1e-6 and the
    same velocities to 1e-6."""
    from wavi_gb300.model import Model
    from wavi_gb300.schwarz import (EnsembleSubdomainSolver, SchwarzSpec, build_subdomains, gpu_global_residual,
                                    release_residual_solver, update_velocities_schwarz)
    spec = SchwarzSpec(ngridsx=2, ngridsy=2, overlap=2, niterations=1)
    m, om = _models(oracle)
    host = Model(m.grid, m.fields["b"], m.params, m.solver_params)
    for k in ("h", "grounded_fraction", "u", "v", "eta"):
        host.fields[k][...] = m.fields[k]
    gpu_hist, ora_hist = [], []

    def gpu_residual(model):
        gpu_hist.append(gpu_global_residual(model))
        return gpu_hist[-1]

    kw = {}
    if batched:
        kw["solve_all"] = EnsembleSubdomainSolver(build_subdomains(m, spec), precision="fp64")
    update_velocities_schwarz(m, spec, global_residual=gpu_residual, **kw)
    release_residual_solver(m)
    _oracle_loop(oracle, om, host, spec)
    ora_hist = [host.last_stats["rel_residual"]]
    assert len(gpu_hist) == 4
    assert abs(gpu_hist[-1] - ora_hist[-1]) <= 1e-6 + 1e-3 * ora_hist[-1]
    du = m.fields["u"] - host.fields["u"]
    dv = m.fields["v"] - host.fields["v"]
    ref = np.sqrt(np.sum(host.fields["u"] ** 2) + np.sum(host.fields["v"] ** 2))
    err = np.sqrt(np.sum(du ** 2) + np.sum(dv ** 2)) / ref
    assert err < 1e-6
