"""The host-side mirror (numpy update_state! neighbours) against the oracle; no GPU."""
import numpy as np
import pytest


def test_pos_fraction_numpy_matches_oracle(oracle, pkg):
    from wavi_gb300.model import pos_fraction
    rng = np.random.default_rng(3)
    for shape in ((3, 3), (17, 9), (40, 21)):
        z = rng.standard_normal(shape)
        mask = rng.random(shape) > 0.2
        for mk in (None, mask):
            a = pos_fraction(z, mk)
            b = oracle.pos_fraction(z, mk)
            for x, y in zip(a, b):
                assert np.allclose(x, y, rtol=0, atol=1e-15)


@pytest.mark.parametrize("mask", ["full", "disc"])
def test_pre_solve_matches_oracle(oracle, pkg, mask):
    from wavi_gb300 import synthetic
    from wavi_gb300.model import Model, pre_solve
    g, bed, p, sp, ic = synthetic.small_case(nx=26, ny=14, mask=mask)
    m = Model(g, bed, p, sp, ic)
    om = oracle.build_model(g, bed, p, sp, ic)
    pre_solve(m)
    om.pre_solve()
    for k in ("s", "haf", "grounded_fraction", "weertman_c", "dsdh", "accumulation", "basal_melt", "gu_h", "gu_s",
              "gv_h", "gv_s", "gu_grounded_fraction", "gv_grounded_fraction", "glen_b", "quad_f2", "eta_av"):
        assert np.allclose(m.fields[k], om.field(k), rtol=1e-14, atol=1e-12), k


def test_update_wavelets_matches_oracle(oracle, pkg):
    from wavi_gb300 import synthetic
    from wavi_gb300.model import Model, update_wavelets
    g, bed, p, sp, ic = synthetic.small_case(nx=37, ny=21)
    m = Model(g, bed, p, sp, ic)
    om = oracle.build_model(g, bed, p, sp, ic)
    rng = np.random.default_rng(4)
    u = 40 * rng.standard_normal((g.nx + 1, g.ny))
    v = 15 * rng.standard_normal((g.nx, g.ny + 1))
    m.fields["u"][...] = u
    m.fields["v"][...] = v
    om.field("u")[...] = u
    om.field("v")[...] = v
    update_wavelets(m)
    om.update_wavelets()
    assert np.array_equal(m.fields["wu_mask"].astype(bool), om.mask("wu_mask").astype(bool))
    assert np.array_equal(m.fields["wv_mask"].astype(bool), om.mask("wv_mask").astype(bool))


def test_grid_boundary_strings(pkg):
    g = pkg.Grid(nx=5, ny=4, u_iszero=["north"], v_iszero=["west", "east"])
    assert g.u_iszero[0, :].all() and not g.u_iszero[1:, :].any()
    assert g.v_iszero[:, 0].all() and g.v_iszero[:, -1].all() and not g.v_iszero[:, 1:-1].any()
    with pytest.raises(ValueError):
        pkg.Grid(nx=5, ny=4, h_mask=np.ones((4, 4), bool))
    with pytest.raises(AssertionError):
        pkg.SolverParams(n_iter_viscosity=3)


@pytest.mark.parametrize("mask", ["full", "disc"])
def test_post_solve_and_thickness_step_match_oracle(oracle, pkg, mask):
    """The host mirror's steps after the velocity solve — h-grid, bed and surface velocities, dh/dt, the
    wavelet coarse space (update_state.jl:17-19) — and update_thickness! (run_simulation.jl:24-42) give the
    oracle's values on the same velocities and relinearised fields."""
    from wavi_gb300 import synthetic
    from wavi_gb300.model import Model, Simulation, post_solve_steps, pre_solve, update_thickness
    from wavi_gb300.config import TimesteppingParams
    g, bed, p, sp, ic = synthetic.small_case(nx=26, ny=14, mask=mask)
    m = Model(g, bed, p, sp, ic)
    om = oracle.build_model(g, bed, p, sp, ic)
    rng = np.random.default_rng(5)
    u = 50 * rng.standard_normal((g.nx + 1, g.ny))
    v = 20 * rng.standard_normal((g.nx, g.ny + 1))
    om.field("u")[...] = u
    om.field("v")[...] = v
    om.pre_solve()
    om.inner_update()
    pre_solve(m)
    m.fields["u"][...] = u
    m.fields["v"][...] = v
    for k in ("beta", "quad_f1", "quad_f2"):
        m.fields[k][...] = om.field(k)
    post_solve_steps(m)
    om.post_solve()
    for k in ("uh", "vh", "ub", "vb", "us", "vs", "dhdt"):
        assert np.allclose(m.fields[k], om.field(k), rtol=1e-13, atol=1e-12), k
    assert np.array_equal(m.fields["wu_mask"].astype(bool), om.mask("wu_mask").astype(bool))
    assert np.array_equal(m.fields["wv_mask"].astype(bool), om.mask("wv_mask").astype(bool))
    dt = 0.5
    update_thickness(Simulation(m, TimesteppingParams(dt=dt, end_time=dt)))
    om.update_thickness(dt)
    assert np.allclose(m.fields["h"], om.field("h"), rtol=1e-14, atol=1e-12)


def test_volume_above_floatation_closed_form(pkg):
    """The reference's known answer (test/test_utils.jl:33-42): 500 m of ice on a bed 200 m below sea level
    over 20 x 25 cells of 1 km²."""
    from wavi_gb300.model import Model, volume_above_floatation
    g = pkg.Grid(nx=20, ny=25, dx=1000.0, dy=1000.0)
    m = Model(g, -200.0 * np.ones((20, 25)), initial_conditions=pkg.InitialConditions(
        initial_thickness=500.0 * np.ones((20, 25))))
    vaf = volume_above_floatation(m.fields["h"], m.fields["b"], m.params, m.grid)
    assert np.isclose(vaf, (500.0 - (1028.0 / 918.0) * 200.0) * 25 * 20 * 1000.0 ** 2, rtol=1e-14)


def test_grounding_line_x_interpolates_the_sign_change(pkg):
    """get_glx (src/utilities.jl:417-426) on a height above floatation that falls linearly along x and
    crosses zero at a known x in each row, plus a row crossing twice (both crossings, in x order)."""
    from wavi_gb300.model import grounding_line_x
    nx, ny, dx = 10, 3, 1000.0
    xxh = np.repeat(((np.arange(nx) + 0.5) * dx)[:, None], ny, axis=1)
    x0 = np.array([3200.0, 5600.0, 7100.0])
    haf = (x0[None, :] - xxh) * 0.01
    haf[8, 2] = 5.0  # row 3 grounds again at cell 9 and floats at cell 10
    glx = grounding_line_x(haf, xxh)
    assert np.allclose(glx[:2], x0[:2]) and np.isclose(glx[2], x0[2]) and glx.size == 4
    assert 8500.0 < glx[3] < 9500.0
