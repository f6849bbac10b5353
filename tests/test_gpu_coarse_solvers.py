"""The opt-in coarse solvers of the persistent coarse kernel (single-reduction CG, Jacobi-preconditioned
single-reduction CG) against the oracle's restatements of the same iterations, and the mixed-precision default
(single-reduction Jacobi) against the reference's FP64 solve.  Through the C ABI."""
import numpy as np
import pytest

from helpers import fields_from_oracle, rel, to_dev, uv_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CASES = {
    "full": dict(nx=40, ny=16, dx=4000.0, mask="full"),
    "disc": dict(nx=24, ny=24, dx=4000.0, mask="disc"),
    "fixed": dict(nx=20, ny=20, dx=5000.0, mask="disc", fixed=True),
    "ragged": dict(nx=37, ny=13, dx=3000.0, mask="full"),
}


@pytest.fixture
def reference_cg(oracle):
    yield
    oracle.set_coarse_variant("cg")


def _setup(oracle, name, **kw):
    from wavi_gb300 import synthetic
    c = dict(CASES[name])
    c.update(kw)
    g, bed, p, sp, ic = synthetic.small_case(**c)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    return g, p, sp, om


def _uv(u, v):
    return np.concatenate([np.asarray(u).ravel(order="F"), np.asarray(v).ravel(order="F")])


@pytest.mark.parametrize("name", list(CASES))
def test_coarse_diagonal_matches_oracle(oracle, name):
    """diag(R A P) from the quadratic form (k_coarse_diag) against the oracle's probing, on a coarse space
    with holes."""
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, name)
    rng = np.random.default_rng(11)
    om.field("u")[...] = 50 * rng.standard_normal(om.field("u").shape)
    om.field("v")[...] = 20 * rng.standard_normal(om.field("v").shape)
    for m in ("wu_mask", "wv_mask"):
        om.mask(m)[...] = (rng.uniform(size=om.mask(m).shape) > 0.3).astype(np.uint8)
    f = fields_from_oracle(om, g)
    om.inner_update()
    du, dv = om.coarse_diag()
    ref = _uv(du, dv)
    for prec, tol in (("fp64", 1e-12), ("mixed", 2e-5)):
        s = VelocitySolver(g, sp, precision=prec)
        s.relinearise_device(p, to_dev(f, torch))
        d = torch.zeros(ref.size, dtype=torch.float64 if prec == "fp64" else torch.float32, device="cuda")
        s.coarse_diagonal_device(d, prec)
        got = d.double().cpu().numpy()
        assert rel(got, ref) < tol, prec
        assert np.all(got[ref == 0] == 0), prec
        s.close()


KERNEL_SOLVERS = [("persistent", "srcg"), ("persistent", "srcg_jacobi"), ("persistent", "srcg_chebyshev"),
                  ("persistent_global", "srcg"), ("persistent_global", "srcg_jacobi"),
                  ("persistent_global", "srcg_chebyshev")]


@pytest.mark.parametrize("kernel,solver", KERNEL_SOLVERS)
@pytest.mark.parametrize("name", list(CASES))
def test_single_reduction_fixed_cg_count_matches_oracle(oracle, reference_cg, name, solver, kernel):
    """One Picard iteration whose coarse solve runs exactly 10 single-reduction iterations (tol_coarse = 0),
    in FP64 on both sides: the same recurrences, so the velocities agree to rounding.  (Masking makes some
    Haar basis functions coincide on the interior, so R A P of a masked grid can be singular; with the
    Jacobi preconditioner and tol_coarse = 0, 25 iterations amplify rounding along that null space until
    the oracle alone moves by up to 8e-5 when only its summation order changes.  After 10 iterations it
    moves by < 1e-13, and real solves stop at tol_coarse.)"""
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, name, maxiter_picard=1, maxiter_coarse=10, tol_coarse=0.0)
    f = fields_from_oracle(om, g)
    s = VelocitySolver(g, sp, precision="fp64", coarse_kernel=kernel, coarse_solver=solver)
    st = s.solve(p, f)
    oracle.set_coarse_variant(solver)
    if solver == "srcg_chebyshev":  # the library's default step count for this kernel (5 or 3)
        assert st["cheb_steps"] == (5 if kernel == "persistent" else 3), st
        oracle.set_chebyshev(st["cheb_steps"])
    try:
        om.update_velocities()
    finally:
        oracle.set_chebyshev()
    ost = om.stats()
    assert st["picard_iterations"] == 1
    assert st["coarse_cg_iterations"] == ost["coarse_cg_iterations"] == 10
    assert uv_err(f, om) < 1e-10
    wu = np.asarray(om.field("wu_correction_full")).ravel(order="F")[f["wu_mask"].ravel(order="F") != 0]
    assert rel(f["wu_correction_coarse"], wu) < 1e-8
    s.close()


@pytest.mark.parametrize("kernel,solver", KERNEL_SOLVERS)
@pytest.mark.parametrize("name", list(CASES))
def test_single_reduction_converged_solve_matches_reference(oracle, name, solver, kernel):
    """The single-reduction coarse solves change the V-cycle, not the fixed point: converged FP64 and mixed
    solves agree with the reference's (cg!) FP64 solve to 1e-6.  On the disc grids R A P is singular and the
    FP32 coarse solves drift along its null space; the mixed solve converges because a coarse solve that
    ends above its tolerance does not become the next warm start (without that rule these cases stall at
    ~1e-6 with every coarse solve at maxiter_coarse)."""
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, name, maxiter_picard=80, tol_picard=1e-7)
    f0 = fields_from_oracle(om, g)
    om.update_velocities()
    ost = om.stats()
    for prec in ("fp64", "mixed"):
        f = {k: np.array(v, copy=True, order="F") for k, v in f0.items()}
        s = VelocitySolver(g, sp, precision=prec, coarse_kernel=kernel, coarse_solver=solver)
        st = s.solve(p, f)
        assert st["status"] == 0, (prec, st)
        assert uv_err(f, om) < 1e-6, (prec, st, ost)
        if name == "full" and solver == "srcg_chebyshev":  # (masked coarse spaces blunt the gain)
            # fewer coarse iterations per V-cycle than cg! (the Picard counts may differ in mixed precision)
            per = st["coarse_cg_iterations"] / st["picard_iterations"]
            assert per < 0.7 * ost["coarse_cg_iterations"] / ost["picard_iterations"], (prec, st, ost)
        s.close()


@pytest.mark.parametrize("steps", [3, 5])
def test_chebyshev_on_the_global_memory_kernel_matches_the_register_kernel(oracle, steps):
    """The Chebyshev coarse solve with its vectors in global memory (k_srcg_cheb_global, the kernel of grids
    too large for the register-resident one) and in registers (k_srcg_persistent): one Picard iteration
    with a fixed count of 10 coarse iterations in FP64 at the same step count, the same iterates to
    rounding."""
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, "full", maxiter_picard=1, maxiter_coarse=10, tol_coarse=0.0)
    f0 = fields_from_oracle(om, g)
    out = {}
    for kernel in ("persistent", "persistent_global"):
        f = {k: np.array(v, copy=True, order="F") for k, v in f0.items()}
        s = VelocitySolver(g, sp, precision="fp64", coarse_kernel=kernel, coarse_solver="srcg_chebyshev",
                           cheb_steps=steps)
        st = s.solve(p, f)
        s.close()
        assert st["coarse_cg_iterations"] == 10 and st["coarse_solver"] == "srcg_chebyshev", st
        assert st["cheb_steps"] == steps and st["coarse_kernel"] == kernel, st
        out[kernel] = np.concatenate([f["u"].ravel(), f["v"].ravel()])
    a, b = out["persistent"], out["persistent_global"]
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(a)


def test_mixed_default_is_chebyshev(oracle):
    """The mixed default coarse solver is the Chebyshev single-reduction CG, on full and on masked domains;
    FP64 keeps the reference's cg!."""
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, "disc", maxiter_picard=2)
    s = VelocitySolver(g, sp, precision="fp64")
    assert s.solve(p, fields_from_oracle(om, g))["coarse_solver"] == "cg"
    s.close()
    for name, want in (("full", "srcg_chebyshev"), ("disc", "srcg_chebyshev"), ("fixed", "srcg_chebyshev")):
        g, p, sp, om = _setup(oracle, name, maxiter_picard=2)
        f = fields_from_oracle(om, g)
        s = VelocitySolver(g, sp, precision="mixed")
        st = s.solve(p, f)
        assert st["coarse_solver"] == want, (name, st)
        # 5 Chebyshev steps in the register-resident kernel, 3 with the vectors in global memory
        assert st["coarse_kernel"] == "persistent" and st["cheb_steps"] == 5, (name, st)
        s.close()
    s = VelocitySolver(g, sp, precision="mixed", coarse_kernel="persistent_global")
    st = s.solve(p, fields_from_oracle(om, g))
    assert st["coarse_kernel"] == "persistent_global" and st["cheb_steps"] == 3, st
    s.close()


def test_single_reduction_solvers_need_the_persistent_kernel(oracle):
    from wavi_gb300.abi import WaviError
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, "full")
    for solver in ("srcg", "srcg_jacobi", "srcg_chebyshev"):
        with pytest.raises(WaviError, match="WAVI_ERR_ARGUMENT"):
            VelocitySolver(g, sp, precision="mixed", coarse_kernel="iterations", coarse_solver=solver)
    # auto falls back to the reference recurrence with per-iteration kernels
    s = VelocitySolver(g, sp, precision="mixed", coarse_kernel="iterations")
    f = fields_from_oracle(om, g)
    assert s.solve(p, f)["status"] in (0, -4)
    s.close()


def test_chebyshev_step_count_option(oracle):
    """wavi_options.cheb_steps: an even count (the preconditioner would not stay positive definite) is
    rejected; 3 and 5 steps both converge to the reference's FP64 solution."""
    from wavi_gb300.abi import WaviError
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, "full", maxiter_picard=80, tol_picard=1e-7)
    with pytest.raises(WaviError, match="WAVI_ERR_ARGUMENT"):
        VelocitySolver(g, sp, precision="mixed", coarse_solver="srcg_chebyshev", cheb_steps=4)
    f0 = fields_from_oracle(om, g)
    om.update_velocities()
    for steps in (3, 5):
        f = {k: np.array(v, copy=True, order="F") for k, v in f0.items()}
        s = VelocitySolver(g, sp, precision="mixed", coarse_solver="srcg_chebyshev", cheb_steps=steps)
        st = s.solve(p, f)
        s.close()
        assert st["status"] == 0 and uv_err(f, om) < 1e-6, (steps, st)


@pytest.mark.parametrize("solver", ["srcg_jacobi", "srcg_chebyshev"])
@pytest.mark.parametrize("name", ["full", "ragged"])
def test_fp64_coarse_sums_converge_to_the_reference(oracle, name, solver):
    """WAVI_SUMS_FP64: the mixed coarse CG with every dot-product term, sum and CG scalar in FP64 (the FP32
    vectors unchanged) reaches the reference's fixed point to 1e-6, as the float-float default does."""
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, name, maxiter_picard=80, tol_picard=1e-7)
    f0 = fields_from_oracle(om, g)
    om.update_velocities()
    for sums in ("float_float", "fp64"):
        f = {k: np.array(v, copy=True, order="F") for k, v in f0.items()}
        s = VelocitySolver(g, sp, precision="mixed", coarse_solver=solver, coarse_sums=sums)
        st = s.solve(p, f)
        s.close()
        print(name, solver, sums, st["picard_iterations"], st["coarse_cg_iterations"], uv_err(f, om))
        assert st["status"] == 0, (sums, st)
        assert uv_err(f, om) < 1e-6, (sums, st)


def test_fp64_coarse_sums_need_the_single_reduction_register_kernel(oracle):
    from wavi_gb300.abi import WaviError
    from wavi_gb300.config import SolverParams
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, "full")
    for kw in (dict(coarse_solver="cg"), dict(coarse_solver="pipelined_chebyshev"),
               dict(coarse_solver="srcg_jacobi", coarse_kernel="persistent_global"),
               dict(coarse_solver="srcg_jacobi", coarse_kernel="iterations")):
        with pytest.raises(WaviError, match="WAVI_ERR_ARGUMENT"):
            VelocitySolver(g, sp, precision="mixed", coarse_sums="fp64", **kw)
    with pytest.raises(WaviError, match="WAVI_ERR_ARGUMENT"):  # 32 x 32 tiles
        VelocitySolver(g, SolverParams(levels=4), precision="mixed", coarse_sums="fp64", coarse_solver="srcg_jacobi")
    s = VelocitySolver(g, sp, precision="fp64", coarse_sums="fp64")  # FP64 contexts sum in FP64 anyway
    s.close()


@pytest.mark.parametrize("kernel", ["persistent", "persistent_global"])
@pytest.mark.parametrize("name", ["full", "disc"])
def test_fp64_coarse_solve_in_the_mixed_vcycle(oracle, name, kernel):
    """WAVI_SUMS_FP64_SOLVE: the mixed V-cycle with its coarse CG in FP64 (the FP64 contexts' kernels on the
    FP64 coefficients, the restricted residual widened and the solution narrowed): the converged solve
    reaches the reference's fixed point to 1e-6 and uses the FP64 coarse kernel's stopping rule."""
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, name, maxiter_picard=80, tol_picard=1e-7)
    f0 = fields_from_oracle(om, g)
    om.update_velocities()
    f = {k: np.array(v, copy=True, order="F") for k, v in f0.items()}
    s = VelocitySolver(g, sp, precision="mixed", coarse_kernel=kernel, coarse_sums="fp64_solve")
    st = s.solve(p, f)
    s.close()
    print(name, kernel, st["picard_iterations"], st["coarse_cg_iterations"], st["coarse_solver"], uv_err(f, om))
    assert st["status"] == 0, st
    assert st["coarse_solver"] == "srcg_chebyshev"
    assert uv_err(f, om) < 1e-6, st


def test_fp64_coarse_solve_needs_a_persistent_kernel(oracle):
    from wavi_gb300.abi import WaviError
    from wavi_gb300.gpu import VelocitySolver
    g, p, sp, om = _setup(oracle, "full")
    for kw in (dict(coarse_kernel="iterations"), dict(coarse_solver="pipelined_chebyshev")):
        with pytest.raises(WaviError, match="WAVI_ERR_ARGUMENT"):
            VelocitySolver(g, sp, precision="mixed", coarse_sums="fp64_solve", **kw)
