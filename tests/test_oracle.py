"""The CPU oracle pinned against the reference's own tests and golden files (no GPU).

  pos_fraction KATs            test/test_utils.jl:4-31
  Kronecker product vs kron    test/test_kronecker.jl:3-35
  σ-quadrature identities      test/test_fields.jl:71-76
  MISMIP+ 100-year golden      test/version_update_test_verification/test_version_updates.jl:6-97
  iceberg analytic state       test/verification_tests/iceberg_test.jl, test/verification_tests.jl:3-10
  MISMIP+ Ice0 grounding line  test/verification_tests/MISMIP_PLUS_Ice0.jl, test/verification_tests.jl:14-36
                               (opt-in: WAVI_SLOW_TESTS=1)
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_pos_fraction_kats(oracle):
    z = np.array([[-1.0, -1, -1], [-1, 1, -1], [-1, -1, -1]])
    h, u, v = oracle.pos_fraction(z)
    assert np.array_equal(h, [[0, 0, 0], [0, 0.5, 0], [0, 0, 0]])
    assert np.array_equal(u, [[0, 0, 0], [0, 0.25, 0], [0, 0.25, 0], [0, 0, 0]])
    assert np.array_equal(v, [[0, 0, 0, 0], [0, 0.25, 0.25, 0], [0, 0, 0, 0]])
    mask = np.array([[0, 0, 0], [0, 1, 0], [0, 0, 0]])
    for zz in (z, np.ones((3, 3))):
        h, u, v = oracle.pos_fraction(zz, mask)
        assert np.array_equal(h, [[0, 0, 0], [0, 1.0, 0], [0, 0, 0]])
        assert np.array_equal(u, [[0, 0, 0], [0, 0.5, 0], [0, 0.5, 0], [0, 0, 0]])
        assert np.array_equal(v, [[0, 0, 0, 0], [0, 0.5, 0.5, 0], [0, 0, 0, 0]])


def test_kronecker_matches_explicit_kron(oracle):
    rng = np.random.default_rng(0)
    nbig, nsmall = 300, 30
    A = rng.standard_normal((nbig, nsmall)) * (rng.random((nbig, nsmall)) < 0.05)
    B = rng.standard_normal((nsmall, nbig)) * (rng.random((nsmall, nbig)) < 0.05)
    x = rng.standard_normal(nbig * nsmall)
    for P, Q in ((A, B), (B, A)):
        y0 = np.kron(P, Q) @ x
        y1 = oracle.kron_apply(P, Q, x)
        assert np.allclose(y0, y1, rtol=1e-12, atol=1e-12)


def test_sigma_quadrature(pkg):
    for sig in (np.linspace(0, 1, 10), np.linspace(0, 1, 10) ** 2):
        g = pkg.Grid(nx=10, ny=10, nσ=10, σ=sig)
        assert np.isclose(g.quadrature_weights.sum(), 1.0)
        assert np.isclose(g.quadrature_weights @ g.σ, 0.5)


def _mismip_golden_model(oracle, pkg):
    from wavi_gb300.synthetic import mismip_plus_bed
    g = pkg.Grid(nx=80, ny=10, nσ=4, x0=0.0, y0=-40000.0, dx=8000.0, dy=8000.0, u_iszero=["north"],
                 v_iszero=["west", "east"])
    p = pkg.Params(default_thickness=100.0, accumulation_rate=0.3, default_temperature=265.700709)
    sp = pkg.SolverParams(maxiter_picard=1)
    return oracle.build_model(g, lambda x, y: float(mismip_plus_bed(x, y)), p, sp)


# The reference's own test (test_version_updates.jl:90-97) asks for Julia's isapprox: norm(a - b) <=
# sqrt(eps) * max(norm(a), norm(b)).  The oracle meets it on every field once its coarse-CG dot products
# and norms follow the summation order of the OpenBLAS kernels Julia calls (wavi_oracle.cpp, g_sum_order):
# a coarse CG of hundreds of iterations carries that order into a 1e-5 difference that 1000 coupled solves
# keep.  Other Julia versions' golden files differ from v1.8.3 by 16 % in u and are not used.
RTOL_JULIA = float(np.sqrt(np.finfo(np.float64).eps))
GOLDEN_KEYS = {"h": "h", "u": "u", "v": "v", "viscosity": "eta_av", "grounded_fraction": "grounded_fraction",
               "bed_speed": "bed_speed"}


def isapprox(a, b, rtol=RTOL_JULIA):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def test_mismip_golden_1000_steps(oracle, pkg):
    m = _mismip_golden_model(oracle, pkg)
    m.run(1000, 0.1)
    gold = np.load(os.path.join(HERE, "golden", "mismip_100yr_v1_8_3.npz"))
    for name, key in GOLDEN_KEYS.items():
        r = np.linalg.norm(m.field(key) - gold[name]) / np.linalg.norm(gold[name])
        assert isapprox(m.field(key), gold[name]), (name, r)


def test_operator_symmetric_negative_definite(oracle, pkg):
    from wavi_gb300 import synthetic
    g, bed, p, sp, ic = synthetic.small_case(nx=20, ny=12, mask="disc")
    m = oracle.build_model(g, bed, p, sp, ic)
    m.pre_solve()
    rng = np.random.default_rng(1)
    m.field("u")[...] = 30 * rng.standard_normal(m.field("u").shape)
    m.inner_update()
    inner_u, inner_v = m.mask("u_inner").astype(bool), m.mask("v_inner").astype(bool)
    xs = []
    for _ in range(2):
        xu = rng.standard_normal((g.nx + 1, g.ny)) * inner_u
        xv = rng.standard_normal((g.nx, g.ny + 1)) * inner_v
        xs.append((xu, xv))
    (xu, xv), (yu, yv) = xs
    axu, axv = m.apply_operator(xu, xv)
    ayu, ayv = m.apply_operator(yu, yv)
    lhs = np.sum(axu * yu) + np.sum(axv * yv)
    rhs = np.sum(xu * ayu) + np.sum(xv * ayv)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))
    assert np.sum(axu * xu) + np.sum(axv * xv) < 0  # the reference's operator is negative definite


def test_haar_forward_inverts_reverse(oracle, pkg):
    from wavi_gb300 import synthetic
    g, bed, p, sp, ic = synthetic.small_case(nx=37, ny=13)
    m = oracle.build_model(g, bed, p, sp, ic)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((g.nx + 1, g.ny))
    y = m.haar(0, 2, m.haar(0, 0, x))  # dwt(idwt(x))
    assert np.allclose(y, x, atol=1e-13)
    # idwtᵀ is the transpose of idwt
    z = rng.standard_normal((g.nx + 1, g.ny))
    assert np.isclose(np.sum(m.haar(0, 0, x) * z), np.sum(x * m.haar(0, 1, z)), rtol=1e-12)


def test_converged_solve_reaches_tolerance(oracle, pkg):
    from wavi_gb300 import synthetic
    g, bed, p, sp, ic = synthetic.small_case(nx=24, ny=12, maxiter_picard=60, tol_picard=1e-6)
    m = oracle.build_model(g, bed, p, sp, ic)
    m.pre_solve()
    m.update_velocities()
    st = m.stats()
    assert st["rel_residual"] < 1e-6
    assert 1 < st["picard_iterations"] < 60


def test_iceberg_reaches_the_analytic_steady_state(oracle, pkg):
    """The reference's iceberg verification (test/verification_tests.jl:3-10, iceberg_test.jl): 1000 yr of
    dt = 0.1 time steps with one Picard iteration each reach the closed-form steady state to the
    reference's tolerances (h 1e-4, u and v 3e-4, relative)."""
    from wavi_gb300 import synthetic
    g, bed, p, sp, ic = synthetic.iceberg_case()
    om = oracle.build_model(g, bed, p, sp, ic)
    om.run(10000, 0.1)
    h0, u0, v0 = synthetic.iceberg_analytic(g)
    hm = np.asarray(g.h_mask, bool)
    um, vm = om.mask("u_mask").astype(bool), om.mask("v_mask").astype(bool)
    assert synthetic.relative_error(om.field("h"), h0, hm) < 1.0e-4
    assert synthetic.relative_error(om.field("u"), u0, um) < 3.0e-4
    assert synthetic.relative_error(om.field("v"), v0, vm) < 3.0e-4


@pytest.mark.skipif(not os.environ.get("WAVI_SLOW_TESTS"),
                    reason="20 000 oracle time steps (~4.5 min); WAVI_SLOW_TESTS=1")
def test_mismip_plus_ice0_grounding_line(oracle, pkg):
    """The reference's MISMIP+ Ice0 verification (test/verification_tests.jl:14-36,
    verification_tests/MISMIP_PLUS_Ice0.jl): 10 000 yr of dt = 0.5 from a 100 m slab on the 8 km channel.
    The grounding line crosses every row, is symmetric about the centre line to 1e-4, and lies in the
    reference's loose bands (the tight bands are marked broken there at this resolution)."""
    m = _mismip_golden_model(oracle, pkg)
    m.run(20000, 0.5)
    g = pkg.Grid(nx=80, ny=10, nσ=4, x0=0.0, y0=-40000.0, dx=8000.0, dy=8000.0)
    from wavi_gb300.model import grounding_line_x
    glx = grounding_line_x(np.asarray(m.field("haf")), g.xxh)
    ny = 10
    assert glx.size == ny
    t = glx[[0, ny // 2 - 1, ny // 2, ny - 1]]
    assert (t[3] - t[0]) / (t[3] + t[0]) < 1e-4 and (t[1] - t[2]) / (t[1] + t[2]) < 1e-4
    assert 480000 < t[0] < 550000 and 480000 < t[3] < 550000
    assert 430000 < t[1] < 490000 and 430000 < t[2] < 490000


def test_c2_fixture_is_a_converged_solve_of_the_benchmark_state(oracle, pkg):
    """tests/golden/c2_oracle_solution.npz (the oracle's converged 640 x 80 solve, which the GPU parity tests
    at the benchmark's configuration compare against): made from the benchmark's own state (input
    fingerprints), and its velocities meet the reference's stopping rule ||b - A(u) u|| / ||b|| < tol_picard
    (update_velocities.jl:59-65) when the oracle relinearises at them (inner_update!, :32-45, repeated
    until the viscosity has settled)."""
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import bench
    from make_c2_solution import fingerprints
    from wavi_gb300 import synthetic
    ref = np.load(os.path.join(HERE, "golden", "c2_oracle_solution.npz"))
    m = bench.build_state(pkg)
    assert np.allclose(fingerprints(m.fields), ref["fingerprints"], rtol=1e-12, atol=0.0)
    g, bed, p, sp, ic = synthetic.channel_c2(tol_picard=bench.TOL_PICARD, maxiter_picard=bench.MAXITER_PICARD)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    for k in ("u", "v"):
        om.field(k)[...] = ref[k]
    # viscosity, drag and F2 iterate from their previous values (update_velocities.jl:227-283): repeated
    # relinearisations at the fixed velocities bring them to their fixed point for those velocities
    for _ in range(40):
        om.inner_update()
    bu, bv = om.rhs()
    iu, iv = om.mask("u_inner").astype(bool), om.mask("v_inner").astype(bool)
    au, av = om.apply_operator(ref["u"] * iu, ref["v"] * iv)
    r = np.concatenate([(bu - au)[iu], (bv - av)[iv]])
    rel = np.linalg.norm(r) / np.linalg.norm(np.concatenate([bu[iu], bv[iv]]))
    assert rel < float(ref["tol_picard"]), rel
    assert int(ref["picard_iterations"]) == 40


def test_golden_file_sensitivity_to_the_coarse_cg_summation_order(oracle, pkg):
    """Why the GPU's FP64 time stepping is held to the golden file at 2.5e-4 (u) rather than at Julia's
    sqrt(eps): 1000 coupled solves, each with a coarse CG of hundreds of iterations, carry the summation
    order of its dot products into the result.  The oracle alone, with a plain left-to-right sum instead of
    the OpenBLAS kernel's order that the reference's machine used, moves from the golden file by the same
    order (measured: u 1.2e-4, ηav 3.0e-4; 3.6e-9 and 1.5e-8 in the default order)."""
    gold = np.load(os.path.join(HERE, "golden", "mismip_100yr_v1_8_3.npz"))
    oracle.lib().oracle_set_sum_order(0)
    try:
        m = _mismip_golden_model(oracle, pkg)
        m.run(1000, 0.1)
    finally:
        oracle.lib().oracle_set_sum_order(3)
    err_u = np.linalg.norm(m.field("u") - gold["u"]) / np.linalg.norm(gold["u"])
    assert 1e-5 < err_u < 1e-3, err_u
    assert not isapprox(m.field("u"), gold["u"])


def test_anderson_restatement_converges_faster_and_closer(oracle, pkg):
    """The oracle's restatement of the opt-in Anderson acceleration (3 columns, from the first Picard
    iteration below a relative residual of 0.3) on the 8 km channel (80 x 10, nσ = 4): the reference's
    stopping rule (update_velocities.jl:59-65) is met in fewer Picard iterations (measured 24 against 39)
    and nearer the fixed point (solved to 1e-11) than by the reference's plain iteration (1.1e-7 against
    1.8e-6: a linearly converging iteration stops about rel / (1 - rate) from its fixed point)."""
    from wavi_gb300 import synthetic

    def solve(depth, tol):
        g, bed, p, sp, ic = synthetic.channel_c1(tol_picard=tol, maxiter_picard=200)
        m = oracle.build_model(g, bed, p, sp, ic)
        m.pre_solve()
        oracle.set_coarse_variant("srcg_chebyshev")
        oracle.set_chebyshev(5)
        oracle.set_anderson(depth)
        try:
            m.update_velocities()
        finally:
            oracle.set_anderson(0)
            oracle.set_coarse_variant("cg")
            oracle.set_chebyshev()
        return m.stats(), np.concatenate([np.ravel(m.field("u")), np.ravel(m.field("v"))])

    st_fp, x_fp = solve(3, 1e-11)
    assert st_fp["rel_residual"] < 1e-11
    st_plain, x_plain = solve(0, 1e-6)
    st_aa, x_aa = solve(3, 1e-6)
    err = lambda x: np.linalg.norm(x - x_fp) / np.linalg.norm(x_fp)
    assert st_plain["rel_residual"] < 1e-6 and st_aa["rel_residual"] < 1e-6
    assert st_aa["picard_iterations"] <= 0.75 * st_plain["picard_iterations"], (st_aa, st_plain)
    assert err(x_aa) < 0.2 * err(x_plain), (err(x_aa), err(x_plain))


def test_c2_fixed_point_fixture(oracle, pkg):
    """tests/golden/c2_oracle_fixed_point.npz (make_c2_fixed_point.py): the oracle's solve of the benchmark
    state to a relative residual below 1e-11; the reference algorithm's own solve at the benchmark's 1e-6
    (c2_oracle_solution.npz) lies within a few 1e-6 of it."""
    fp = np.load(os.path.join(HERE, "golden", "c2_oracle_fixed_point.npz"))
    plain = np.load(os.path.join(HERE, "golden", "c2_oracle_solution.npz"))
    assert float(fp["rel_residual"]) < 1e-11
    assert np.array_equal(fp["fingerprints"], plain["fingerprints"])
    den = np.sqrt(np.sum(fp["u"] ** 2) + np.sum(fp["v"] ** 2))
    d = np.sqrt(np.sum((plain["u"] - fp["u"]) ** 2) + np.sum((plain["v"] - fp["v"]) ** 2)) / den
    assert np.isclose(d, float(fp["reference_stop_distance"]), rtol=1e-6)
    assert d < 1e-5


def test_adaptive_coarse_tolerance_restatement(oracle, pkg):
    """The oracle's restatement of the opt-in adaptive coarse tolerance (max(tol_coarse, min(0.1, 0.1 rel)))
    on the 8 km channel, with and without the Anderson acceleration: the same Picard count (within 1), the
    same distance from the fixed point (within a factor 2 and below 1e-6 with the acceleration), and at
    least a quarter fewer coarse iterations (measured 2 791 -> 1 857 plain, 1 897 -> 1 224 accelerated)."""
    from wavi_gb300 import synthetic

    def solve(depth, forcing, tol=1e-6):
        g, bed, p, sp, ic = synthetic.channel_c1(tol_picard=tol, maxiter_picard=200)
        m = oracle.build_model(g, bed, p, sp, ic)
        m.pre_solve()
        oracle.set_coarse_variant("srcg_chebyshev")
        oracle.set_chebyshev(5)
        oracle.set_anderson(depth)
        oracle.set_coarse_forcing(forcing)
        try:
            m.update_velocities()
        finally:
            oracle.set_anderson(0)
            oracle.set_coarse_forcing(False)
            oracle.set_coarse_variant("cg")
            oracle.set_chebyshev()
        return m.stats(), np.concatenate([np.ravel(m.field("u")), np.ravel(m.field("v"))])

    _, x_fp = solve(3, False, 1e-11)
    err = lambda x: np.linalg.norm(x - x_fp) / np.linalg.norm(x_fp)
    for depth in (0, 3):
        st0, x0 = solve(depth, False)
        st1, x1 = solve(depth, True)
        assert st1["rel_residual"] < 1e-6
        assert abs(st1["picard_iterations"] - st0["picard_iterations"]) <= 1, (st0, st1)
        assert st1["coarse_cg_iterations"] <= 0.75 * st0["coarse_cg_iterations"], (st0, st1)
        assert err(x1) < 2 * err(x0) + 1e-8, (err(x0), err(x1))
    assert err(x1) < 1e-6


@pytest.mark.parametrize("case", ["disc", "fixed"])
def test_accelerated_loop_on_masked_domains(oracle, pkg, case):
    """The oracle's restatement of the mixed defaults' iteration (Anderson acceleration, 3 columns, with the
    adaptive coarse tolerance) on a masked disc with calving fronts on every side, and on the same disc with
    Dirichlet lines (u, v fixed on a centre line): the reference's stopping rule is met in fewer Picard and
    coarse iterations than by the reference's plain loop, and within 1e-6 of the fixed point (solved to
    1e-11)."""
    from wavi_gb300 import synthetic
    kw = dict(nx=24, ny=24, dx=4000.0, mask="disc") if case == "disc" else dict(nx=20, ny=20, dx=5000.0, mask="disc",
                                                                                 fixed=True)

    def solve(depth, forcing, tol):
        g, bed, p, sp, ic = synthetic.small_case(**kw, tol_picard=tol, maxiter_picard=200)
        m = oracle.build_model(g, bed, p, sp, ic)
        m.pre_solve()
        oracle.set_coarse_variant("srcg_chebyshev")
        oracle.set_chebyshev(5)
        oracle.set_anderson(depth)
        oracle.set_coarse_forcing(forcing)
        try:
            m.update_velocities()
        finally:
            oracle.set_anderson(0)
            oracle.set_coarse_forcing(False)
            oracle.set_coarse_variant("cg")
            oracle.set_chebyshev()
        return m.stats(), np.concatenate([np.ravel(m.field("u")), np.ravel(m.field("v"))])

    _, x_fp = solve(3, False, 1e-11)
    st0, _ = solve(0, False, 1e-6)
    st1, x1 = solve(3, True, 1e-6)
    assert st1["rel_residual"] < 1e-6
    assert st1["picard_iterations"] < st0["picard_iterations"], (st0, st1)
    assert st1["coarse_cg_iterations"] < 0.6 * st0["coarse_cg_iterations"], (st0, st1)
    assert np.linalg.norm(x1 - x_fp) < 1e-6 * np.linalg.norm(x_fp)
