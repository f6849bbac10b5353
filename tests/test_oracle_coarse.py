"""The oracle's restatements of the GPU library's opt-in coarse solvers (single-reduction CG, Jacobi on
diag(R A P), Chebyshev steps) and of the pipelined CG a GPU kernel is to follow, checked on the CPU against
first principles: the probed diagonal against the explicitly assembled coarse matrix, and the
single-reduction and pipelined solves against the reference's cg! on the same problem."""
import numpy as np
import pytest


@pytest.fixture
def reference_cg(oracle):
    yield
    oracle.set_coarse_variant("cg")


def _relinearised(oracle, nx, ny, seed=3, mask="full", drop=0.3):
    from wavi_gb300 import synthetic
    g, bed, p, sp, ic = synthetic.small_case(nx=nx, ny=ny, mask=mask)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    rng = np.random.default_rng(seed)
    om.field("u")[...] = 50 * rng.standard_normal(om.field("u").shape)
    om.field("v")[...] = 20 * rng.standard_normal(om.field("v").shape)
    # a coarse space with holes, as the wavelet threshold leaves it after a solve
    for name in ("wu_mask", "wv_mask"):
        m = om.mask(name)
        m[...] = (rng.uniform(size=m.shape) > drop).astype(np.uint8)
    om.inner_update()
    return g, om


def _coarse_matrix(om, g):
    """R A P assembled column by column (UWavelets.jl restriction/prolongation, update_preconditioners.jl:176-193)."""
    iu = om.mask("u_inner").astype(bool)
    iv = om.mask("v_inner").astype(bool)
    wu = om.mask("wu_mask").astype(bool).ravel(order="F")
    wv = om.mask("wv_mask").astype(bool).ravel(order="F")
    nu = (g.nx + 1) * g.ny
    idx = np.concatenate([np.flatnonzero(wu), nu + np.flatnonzero(wv)])

    def apply(cfull):
        cu = cfull[:nu].reshape((g.nx + 1, g.ny), order="F")
        cv = cfull[nu:].reshape((g.nx, g.ny + 1), order="F")
        fu, fv = om.haar(0, 0, cu) * iu, om.haar(1, 0, cv) * iv
        au, av = om.apply_operator(fu, fv)
        return np.concatenate([om.haar(0, 1, au * iu).ravel(order="F"), om.haar(1, 1, av * iv).ravel(order="F")])

    n = idx.size
    M = np.zeros((n, n))
    for k in range(n):
        e = np.zeros(nu + g.nx * (g.ny + 1))
        e[idx[k]] = 1.0
        M[:, k] = apply(e)[idx]
    return M, idx


@pytest.mark.parametrize("shape", [(12, 8), (19, 7)])
def test_probed_coarse_diagonal_is_exact(oracle, shape):
    g, om = _relinearised(oracle, *shape)
    M, idx = _coarse_matrix(om, g)
    du, dv = om.coarse_diag()
    d = np.concatenate([du.ravel(order="F"), dv.ravel(order="F")])
    assert np.allclose(M, M.T, rtol=0, atol=1e-9 * np.abs(M).max())  # R A P is symmetric
    ref = np.diag(M)
    assert np.all(ref < 0)  # and negative definite
    assert np.max(np.abs(d[idx] - ref)) <= 1e-12 * np.max(np.abs(ref))
    off = np.ones(d.size, bool)
    off[idx] = False
    assert np.all(d[off] == 0.0)


@pytest.mark.parametrize("variant", ["srcg", "srcg_jacobi", "srcg_chebyshev", "pipelined_chebyshev"])
def test_single_reduction_coarse_solves_reach_the_reference_fixed_point(oracle, reference_cg, variant):
    from wavi_gb300 import synthetic
    sols = {}
    for v in ("cg", variant):
        oracle.set_coarse_variant(v)
        g, bed, p, sp, ic = synthetic.small_case(nx=40, ny=16, maxiter_picard=60, tol_picard=1e-7)
        om = oracle.build_model(g, bed, p, sp, ic)
        om.pre_solve()
        om.update_velocities()
        st = om.stats()
        assert st["rel_residual"] < 1e-7, (v, st)
        sols[v] = (np.array(om.field("u")), np.array(om.field("v")), st)
    (u0, v0, s0), (u1, v1, s1) = sols["cg"], sols[variant]
    err = np.sqrt(np.sum((u1 - u0) ** 2) + np.sum((v1 - v0) ** 2)) / np.sqrt(np.sum(u0 ** 2) + np.sum(v0 ** 2))
    assert err < 1e-6
    if variant == "srcg_jacobi":  # the preconditioner must pay for itself
        assert s1["coarse_cg_iterations"] < 0.75 * s0["coarse_cg_iterations"]
    if variant in ("srcg_chebyshev", "pipelined_chebyshev"):  # two more operator applications per iteration
        assert s1["coarse_cg_iterations"] < s0["coarse_cg_iterations"] / 3


@pytest.mark.parametrize("mask", ["full", "disc"])
def test_pipelined_cg_follows_the_single_reduction_iterates(oracle, reference_cg, mask):
    """Pipelined CG (variant 5) and single-reduction CG (variant 4) with the same Chebyshev preconditioner
    produce the same Krylov iterates in exact arithmetic between variant 5's restarts: in FP64 their
    Picard counts agree, the restarts (after each hundredfold fall of |r|) cost at most 20 % more coarse
    iterations (measured 14 % and 12 %), and their converged velocities agree to the Picard tolerance."""
    from wavi_gb300 import synthetic
    sols = {}
    for v in ("srcg_chebyshev", "pipelined_chebyshev"):
        oracle.set_coarse_variant(v)
        g, bed, p, sp, ic = synthetic.small_case(nx=40, ny=16, mask=mask, maxiter_picard=60, tol_picard=1e-7)
        om = oracle.build_model(g, bed, p, sp, ic)
        om.pre_solve()
        om.update_velocities()
        sols[v] = (np.array(om.field("u")), np.array(om.field("v")), om.stats())
    (u0, v0, s0), (u1, v1, s1) = sols["srcg_chebyshev"], sols["pipelined_chebyshev"]
    assert s1["picard_iterations"] == s0["picard_iterations"]
    assert s0["coarse_cg_iterations"] <= s1["coarse_cg_iterations"] <= 1.2 * s0["coarse_cg_iterations"]
    err = np.sqrt(np.sum((u1 - u0) ** 2) + np.sum((v1 - v0) ** 2)) / np.sqrt(np.sum(u0 ** 2) + np.sum(v0 ** 2))
    assert err < 1e-9


def test_oracle_keeps_the_last_coarse_problem(oracle, reference_cg):
    """coarse_b and coarse_x0 hold the last V-cycle's coarse right-hand side and starting point: sized as
    the coarse space, the first V-cycle starting cold, the second from the first one's correction."""
    from wavi_gb300 import synthetic
    g, bed, p, sp, ic = synthetic.small_case(nx=24, ny=12, maxiter_picard=1)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    om.update_velocities()
    n = int(om.mask("wu_mask").sum() + om.mask("wv_mask").sum())
    b, x0 = np.array(om.field("coarse_b")), np.array(om.field("coarse_x0"))
    assert b.shape == x0.shape == (n,) and np.linalg.norm(b) > 0 and not x0.any()
    wu = np.asarray(om.field("wu_correction_full")).ravel(order="F")[om.mask("wu_mask").ravel(order="F") != 0]
    wv = np.asarray(om.field("wv_correction_full")).ravel(order="F")[om.mask("wv_mask").ravel(order="F") != 0]
    om.update_velocities()
    assert np.array_equal(np.array(om.field("coarse_x0")), np.concatenate([wu, wv]))
