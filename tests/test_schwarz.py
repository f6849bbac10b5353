"""The restricted-additive-Schwarz decomposition (wavi_gb300.schwarz) against the reference's
SharedMemorySpec (src/SharedMemorySpec.jl): subdomain ranges, cut-boundary Dirichlet points, the partition
of unity, and restriction followed by damped prolongation.  Host logic only (no GPU)."""
import numpy as np
import pytest

from helpers import SOLVE_FIELDS, fields_from_oracle


def _model(nx=32, ny=8):
    from wavi_gb300 import synthetic
    from wavi_gb300.model import Model
    g, bed, p, sp, ic = synthetic.small_case(nx=nx, ny=ny, dx=4000.0)
    m = Model(g, bed, p, sp, ic)
    rng = np.random.default_rng(2)
    m.fields["u"][...] = rng.standard_normal(m.fields["u"].shape)
    m.fields["v"][...] = rng.standard_normal(m.fields["v"].shape)
    return m


def test_subdomain_ranges():
    from wavi_gb300.schwarz import SchwarzSpec, subdomain_range
    spec = SchwarzSpec(ngridsx=4, ngridsy=2, overlap=2)
    assert subdomain_range(32, 8, 1, 1, spec) == (0, 10, 0, 6)   # block 1..8 (x), 1..4 (y), + overlap, clipped
    assert subdomain_range(32, 8, 2, 2, spec) == (6, 18, 2, 8)
    assert subdomain_range(32, 8, 4, 1, spec) == (22, 32, 0, 6)
    with pytest.raises(ValueError):
        subdomain_range(30, 8, 1, 1, spec)
    with pytest.raises(IndexError):
        subdomain_range(32, 8, 5, 1, spec)
    for bad in (dict(overlap=0), dict(ngridsx=0), dict(niterations=-1)):
        with pytest.raises(ValueError):
            SchwarzSpec(**bad)


@pytest.mark.parametrize("ngx,ngy,overlap", [(4, 2, 2), (2, 2, 1), (8, 1, 2), (2, 4, 1), (1, 1, 3)])
def test_partitions_of_unity_add_to_one(ngx, ngy, overlap):
    """Summed over the subdomains (embedded in the global grids), the u- and v-grid weights are 1 at every
    point: the ramps of neighbours (over 2 overlap u points, 2 overlap - 1 v points) add up across each
    overlap."""
    from wavi_gb300.schwarz import SchwarzSpec, partition_of_unity, subdomain_range
    nx, ny = 32, 8
    spec = SchwarzSpec(ngridsx=ngx, ngridsy=ngy, overlap=overlap)
    su, sv = np.zeros((nx + 1, ny)), np.zeros((nx, ny + 1))
    for ig in range(1, ngx + 1):
        for jg in range(1, ngy + 1):
            i0, i1, j0, j1 = subdomain_range(nx, ny, ig, jg, spec)
            e = (ig == 1, ig == ngx, jg == 1, jg == ngy)
            su[i0:i1 + 1, j0:j1] += partition_of_unity(i1 - i0 + 1, j1 - j0, *e, 2 * overlap, 2 * overlap - 1)
            sv[i0:i1, j0:j1 + 1] += partition_of_unity(i1 - i0, j1 - j0 + 1, *e, 2 * overlap - 1, 2 * overlap)
    assert np.allclose(su, 1.0, rtol=0, atol=1e-14) and np.allclose(sv, 1.0, rtol=0, atol=1e-14)


def test_partition_of_unity_shape_and_ramps():
    from wavi_gb300.schwarz import partition_of_unity
    p = partition_of_unity(9, 5, False, True, True, True, 4, 1)
    assert p.shape == (9, 5)
    assert np.allclose(p[:, 0], [0.0, 0.25, 0.5, 0.75, 1.0, 1.0, 1.0, 1.0, 1.0])
    assert np.allclose(p[4, :], 1.0)
    with pytest.raises(ValueError):
        partition_of_unity(4, 5, False, False, True, True, 2, 1)


def test_subdomain_problem_crops_and_fixes_the_cut_boundaries():
    from wavi_gb300.model import Model
    from wavi_gb300.schwarz import SchwarzSpec, subdomain_problem, subdomain_range
    m = _model()
    spec = SchwarzSpec(ngridsx=4, ngridsy=2, overlap=2)
    grid, bed, params, ic = subdomain_problem(m, 2, 1, spec)
    i0, i1, j0, j1 = subdomain_range(32, 8, 2, 1, spec)
    assert (grid.nx, grid.ny) == (i1 - i0, j1 - j0)
    assert grid.x0 == m.grid.x0 + i0 * m.grid.dx and grid.y0 == m.grid.y0
    assert np.array_equal(bed, m.fields["b"][i0:i1, j0:j1])
    assert np.array_equal(ic.initial_u_veloc, m.fields["u"][i0:i1 + 1, j0:j1])
    assert np.array_equal(ic.initial_v_veloc, m.fields["v"][i0:i1, j0:j1 + 1])
    assert np.array_equal(ic.initial_viscosity, m.fields["eta"][i0:i1, j0:j1, :])
    # subdomain (2, 1) of 4 x 2: cut boundaries west, east and north; the south edge is the domain's own
    assert grid.u_isfixed[0, :].all() and grid.u_isfixed[-1, :].all() and grid.u_isfixed[:, -1].all()
    assert grid.v_isfixed[0, :].all() and grid.v_isfixed[-1, :].all() and grid.v_isfixed[:, -1].all()
    assert not grid.v_isfixed[1:-1, 0].any()
    assert np.array_equal(params.weertman_c, m.weertman_c_param[i0:i1, j0:j1])
    sub = Model(grid, bed, params, m.solver_params, ic)  # a valid model of its own
    assert sub.fields["u"].shape == (grid.nx + 1, grid.ny)


def test_prolongation_rejects_an_overlap_wider_than_the_ramps_fit():
    """An interior subdomain of 4 + 2 x 3 cells has 11 u points, fewer than its two ramps of 6: the
    reference's partition of unity asserts against it, and so does this one."""
    from wavi_gb300.model import Model
    from wavi_gb300.schwarz import SchwarzSpec, prolong_velocities, subdomain_problem
    m = _model()
    spec = SchwarzSpec(ngridsx=8, ngridsy=1, overlap=3)
    grid, bed, params, ic = subdomain_problem(m, 2, 1, spec)
    with pytest.raises(ValueError):
        prolong_velocities(m, Model(grid, bed, params, m.solver_params, ic), 2, 1, spec)


@pytest.mark.parametrize("damping", [0.0, 0.3])
def test_restrict_then_prolong_reproduces_the_global_velocities(damping):
    """With every subdomain holding the global velocities (no solve in between), a Schwarz update —
    damping, then the weighted prolongation of every subdomain — gives back the global velocities."""
    from wavi_gb300.model import Model
    from wavi_gb300.schwarz import SchwarzSpec, prolong_velocities, restrict_velocities, subdomain_problem
    m = _model()
    u0, v0 = m.fields["u"].copy(), m.fields["v"].copy()
    spec = SchwarzSpec(ngridsx=4, ngridsy=2, overlap=2, niterations=1, damping=damping)
    subs = {}
    for ig in range(1, 5):
        for jg in range(1, 3):
            grid, bed, params, ic = subdomain_problem(m, ig, jg, spec)
            subs[ig, jg] = Model(grid, bed, params, m.solver_params, ic)
            restrict_velocities(subs[ig, jg], m, ig, jg, spec)
    m.fields["u"] *= damping
    m.fields["v"] *= damping
    for (ig, jg), sub in subs.items():
        prolong_velocities(m, sub, ig, jg, spec)
    assert np.allclose(m.fields["u"], u0, rtol=0, atol=1e-13) and np.allclose(m.fields["v"], v0, rtol=0, atol=1e-13)


class _OracleSubdomain:
    """A subdomain model held by the oracle, with the velocity views the restriction and prolongation use."""

    def __init__(self, om):
        self.om = om
        self.fields = {"u": om.field("u"), "v": om.field("v")}


def _converged_global(oracle):
    from dataclasses import replace
    from wavi_gb300 import synthetic
    from wavi_gb300.model import Model
    g, bed, p, sp, ic = synthetic.small_case(nx=32, ny=16, dx=4000.0)
    sp = replace(sp, tol_picard=1e-10, maxiter_picard=200)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.update_state()
    m = Model(g, bed, p, sp, ic)
    for k in ("u", "v", "eta", "h", "grounded_fraction"):
        m.fields[k][...] = om.field(k)
    return m


def _uv_dist(m, u, v):
    return np.sqrt(np.sum((m.fields["u"] - u) ** 2) + np.sum((m.fields["v"] - v) ** 2)) / \
        np.sqrt(np.sum(u ** 2) + np.sum(v ** 2))


@pytest.fixture(scope="module")
def converged(oracle):
    m = _converged_global(oracle)
    return m, m.fields["u"].copy(), m.fields["v"].copy()


@pytest.mark.parametrize("ngx,ngy,overlap", [(2, 2, 2), (4, 2, 2)])
def test_ras_sweep_contracts_a_perturbation(oracle, converged, ngx, ngy, overlap):
    """One Schwarz sweep with the oracle solving the subdomains (halo velocities held at the global values)
    brings a 20 % perturbation of the converged global velocities at least 4x closer to them."""
    from wavi_gb300.schwarz import SchwarzSpec, build_subdomains, ras_sweeps
    m, u, v = converged
    rng = np.random.default_rng(1)
    m.fields["u"][...] = u * (1 + 0.2 * rng.standard_normal(u.shape))
    m.fields["v"][...] = v * (1 + 0.2 * rng.standard_normal(v.shape))
    d0 = _uv_dist(m, u, v)
    spec = SchwarzSpec(ngridsx=ngx, ngridsy=ngy, overlap=overlap, niterations=1, damping=0.0)
    subs = build_subdomains(m, spec, make=lambda *a: _OracleSubdomain(oracle.build_model(*a)))
    ras_sweeps(m, spec, subs, solve=lambda s: s.om.update_state())
    assert _uv_dist(m, u, v) < d0 / 4


def test_ras_sweep_of_the_solution_moves_it_by_the_edge_viscosity_only(oracle, converged):
    """The converged global solution is a fixed point of a sweep up to the subdomains' edge-cell viscosity
    (their strain rates miss the corners beyond the cut): well under 1 %, for damping 0 and 0.5."""
    from wavi_gb300.schwarz import SchwarzSpec, build_subdomains, ras_sweeps
    m, u, v = converged
    for damping in (0.0, 0.5):
        m.fields["u"][...] = u
        m.fields["v"][...] = v
        spec = SchwarzSpec(ngridsx=2, ngridsy=2, overlap=2, niterations=1, damping=damping)
        subs = build_subdomains(m, spec, make=lambda *a: _OracleSubdomain(oracle.build_model(*a)))
        ras_sweeps(m, spec, subs, solve=lambda s: s.om.update_state())
        assert _uv_dist(m, u, v) < 3e-3 * (1 - damping) + 1e-12


class _OracleEnsemble:
    """A stand-in with EnsembleSolver.solve_device's contract (lists of params and of member field dicts of
    flat column-major tensors, solved in place) whose members the oracle solves, on CPU tensors."""

    def __init__(self, oracle, subs):
        self.oracle, self.subs = oracle, list(subs)

    def solve_device(self, params, tensors):
        import torch
        stats = []
        for sub, p, t in zip(self.subs, params, tensors):
            g = sub.grid
            om = self.oracle.build_model(g, sub.fields["b"], p, sub.solver_params)
            for name in SOLVE_FIELDS + ("gu_residual", "gv_residual"):
                om.field(name)[...] = t[name].numpy().reshape(om.field(name).shape, order="F")
            for w in ("wu", "wv"):
                mask = t[f"{w}_mask"].numpy().reshape(om.mask(f"{w}_mask").shape, order="F")
                om.mask(f"{w}_mask")[...] = mask
                full = np.zeros(mask.shape, order="F")
                full.ravel(order="F")[mask.ravel(order="F") != 0] = t[f"{w}_correction_coarse"].numpy()
                om.field(f"{w}_correction_full")[...] = full
            om.update_velocities()
            for name, a in fields_from_oracle(om, g).items():
                t[name] = torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F")))
            stats.append({"status": 0})
        return stats


def test_ensemble_batched_sweep_matches_per_subdomain_sweep(oracle, converged):
    """The sweep with the subdomains' velocity solves batched as ensemble members (host Models; their
    pre- and post-solve steps on the host) gives the global velocities of the per-subdomain sweep (the
    oracle's whole update_state per subdomain), with the oracle solving in both, for two sweeps."""
    from wavi_gb300.model import Model
    from wavi_gb300.schwarz import EnsembleSubdomainSolver, SchwarzSpec, build_subdomains, ras_sweeps
    m, u, v = converged
    rng = np.random.default_rng(3)
    pu = u * (1 + 0.1 * rng.standard_normal(u.shape))
    pv = v * (1 + 0.1 * rng.standard_normal(v.shape))
    spec = SchwarzSpec(ngridsx=2, ngridsy=2, overlap=2, niterations=2, damping=0.2)
    out = []
    for batched in (False, True):
        m.fields["u"][...] = pu
        m.fields["v"][...] = pv
        if batched:
            subs = build_subdomains(m, spec, make=lambda *a: Model(*a))
            solver = EnsembleSubdomainSolver(subs, ensemble=_OracleEnsemble(oracle, subs.values()), device="cpu")
            ras_sweeps(m, spec, subs, solve_all=solver)
        else:
            subs = build_subdomains(m, spec, make=lambda *a: _OracleSubdomain(oracle.build_model(*a)))
            ras_sweeps(m, spec, subs, solve=lambda s: s.om.update_state())
        out.append((m.fields["u"].copy(), m.fields["v"].copy()))
    (ua, va), (ub, vb) = out
    m.fields["u"][...], m.fields["v"][...] = pu, pv
    assert _uv_dist(m, ua, va) > 1e-2  # the sweeps moved the velocities
    m.fields["u"][...], m.fields["v"][...] = ub, vb
    assert _uv_dist(m, ua, va) < 1e-10


def _oracle_global_residual(oracle, m):
    """inner_update! and ‖b − A u‖/‖b‖ over the interior points, by the oracle, on the host model's velocities
    (the reference's precondition! residual test, update_velocities.jl:50-62)."""
    om = m._oracle
    iu, iv = om.mask("u_inner").astype(bool), om.mask("v_inner").astype(bool)

    def residual(model):
        om.field("u")[...] = model.fields["u"]
        om.field("v")[...] = model.fields["v"]
        om.inner_update()
        bu, bv = om.rhs()
        au, av = om.apply_operator(model.fields["u"] * iu, model.fields["v"] * iv)
        r = np.concatenate([(bu - au)[iu], (bv - av)[iv]])
        return float(np.linalg.norm(r) / np.linalg.norm(np.concatenate([bu[iu], bv[iv]])))
    return residual


def _global_model(oracle, **sp_kw):
    from dataclasses import replace
    from wavi_gb300 import synthetic
    from wavi_gb300.model import Model
    g, bed, p, sp, ic = synthetic.small_case(nx=32, ny=16, dx=4000.0)
    sp = replace(sp, **sp_kw)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    m = Model(g, bed, p, sp, ic)
    for k in ("h", "grounded_fraction", "u", "v", "eta"):
        m.fields[k][...] = om.field(k)
    m._oracle = om
    return m


def test_schwarz_picard_loop_reduces_the_global_residual(oracle):
    """update_velocities! with SharedMemorySpec, the oracle relinearising and solving the subdomains: from
    the cold start (relative residual 1) the global residual falls below 2 % within three Picard iterations
    and keeps falling, and the loop stops at maxiter_picard without converging (the sweeps level off, as
    the reference's do, above tol_picard)."""
    from wavi_gb300.schwarz import SchwarzSpec, update_velocities_schwarz
    m = _global_model(oracle, maxiter_picard=6)
    hist = []
    base = _oracle_global_residual(oracle, m)

    def residual(model):
        hist.append(base(model))
        return hist[-1]

    spec = SchwarzSpec(ngridsx=2, ngridsy=2, overlap=2, niterations=1)
    converged, rel, its = update_velocities_schwarz(
        m, spec, global_residual=residual, solve=lambda s: s.om.update_state(),
        make=lambda *a: _OracleSubdomain(oracle.build_model(*a)))
    assert not converged and its == 6 and rel == hist[-1]
    assert hist[0] > 0.5 and min(hist[1:4]) < 0.05 and hist[-1] < hist[3]


def test_schwarz_picard_loop_stops_when_the_residual_passes(oracle):
    """A model that already passes the residual test stops after the test, with no sweep."""
    from wavi_gb300.schwarz import SchwarzSpec, update_velocities_schwarz
    m = _global_model(oracle)
    calls = []
    converged, rel, its = update_velocities_schwarz(
        m, SchwarzSpec(ngridsx=2, ngridsy=2, overlap=2, niterations=1), global_residual=lambda model: 1e-9,
        solve=lambda s: calls.append(s), make=lambda *a: _OracleSubdomain(oracle.build_model(*a)))
    assert converged and its == 1 and rel == 1e-9 and not calls


def test_gpu_global_residual_undoes_the_correction(pkg, monkeypatch):
    """The GPU residual test runs a one-iteration solve and keeps what it relinearised, but restores the
    velocities and the coarse cache that its V-cycle correction changed (a stand-in solver here)."""
    from wavi_gb300 import gpu, schwarz, synthetic
    from wavi_gb300.model import Model
    made = []

    class FakeSolver:
        def __init__(self, grid, solver_params, **kw):
            made.append(solver_params.maxiter_picard)

        def solve(self, params, fields):
            fields["eta"][...] = 7.0              # relinearised
            fields["u"][...] += 1.0               # the correction
            fields["v"][...] += 1.0
            fields["wu_correction_coarse"] = np.ones(3)
            return {"rel_residual": 0.25}

        def close(self):
            pass

    monkeypatch.setattr(gpu, "VelocitySolver", FakeSolver)
    g, bed, p, sp, ic = synthetic.small_case(nx=12, ny=6)
    m = Model(g, bed, p, sp, ic)
    u0, v0, c0 = m.fields["u"].copy(), m.fields["v"].copy(), np.array(m.fields["wu_correction_coarse"])
    assert schwarz.gpu_global_residual(m) == 0.25
    assert made == [1]
    assert np.array_equal(m.fields["u"], u0) and np.array_equal(m.fields["v"], v0)
    assert np.array_equal(m.fields["wu_correction_coarse"], c0) and (m.fields["eta"] == 7.0).all()
    schwarz.gpu_global_residual(m)
    assert made == [1]  # one context per model
    schwarz.release_residual_solver(m)


def test_schwarz_spec_is_a_parallel_spec(pkg, monkeypatch):
    """A model whose parallel spec is a SchwarzSpec (the reference's SharedMemorySpec) takes the Schwarz
    path in update_velocities; its subdomain models get the spec's subdomain_spec, a GPU spec by default."""
    from wavi_gb300 import schwarz, synthetic
    from wavi_gb300.model import GPUParallelSpec, Model, update_velocities
    g, bed, p, sp, ic = synthetic.small_case(nx=32, ny=16, dx=4000.0)
    spec = schwarz.SchwarzSpec(ngridsx=2, ngridsy=2, overlap=2, niterations=1)
    assert isinstance(spec.subdomain_spec, GPUParallelSpec)
    m = Model(g, bed, p, sp, ic, parallel_spec=spec)
    calls = []
    monkeypatch.setattr(schwarz, "update_velocities_schwarz", lambda model, s: calls.append((model, s)))
    update_velocities(m)
    assert calls == [(m, spec)]
    subs = schwarz.build_subdomains(m, spec)
    assert all(s.parallel_spec is spec.subdomain_spec for s in subs.values())
    with pytest.raises(TypeError):
        update_velocities(Model(g, bed, p, sp, ic, parallel_spec=object()))


def test_member_staging_keeps_an_empty_coarse_space_addressable(pkg):
    """A subdomain whose wavelet mask is empty has zero-length compact corrections; they are staged with one
    unused entry (a zero-length tensor has no device address, which the library rejects) and come back with
    count(mask) entries."""
    torch = pytest.importorskip("torch")
    from wavi_gb300 import schwarz
    from wavi_gb300.gpu import ALL_FIELDS
    fields = {k: np.zeros((3, 2)) for k in ALL_FIELDS}
    fields["wu_mask"] = np.zeros((3, 2), np.uint8)
    fields["wv_mask"] = np.array([[1, 0], [0, 1], [0, 0]], np.uint8)
    fields["wu_correction_coarse"] = np.zeros(0)
    fields["wv_correction_coarse"] = np.array([2.0, 3.0])
    t = schwarz._member_tensors(fields, "cpu")
    assert t["wu_correction_coarse"].numel() == 1 and t["wv_correction_coarse"].numel() == 2
    t["wv_correction_coarse"] += 1.0
    schwarz._member_fields_back(fields, t)
    assert fields["wu_correction_coarse"].shape == (0,)
    assert np.array_equal(fields["wv_correction_coarse"], [3.0, 4.0])
