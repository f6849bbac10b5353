"""Adjoint and tangent linear of the converged solve (wavi_adjoint_device, wavi_tangent_device) on the
GPU: the dot-product test <J v, w> = <v, Jᵀ w>, and the gradient of the speed misfit
J = ½ Σ (|u| − u_obs)² against central finite differences of tightly converged forward solves."""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


class Case:
    def __init__(self, **kw):
        from wavi_gb300 import synthetic
        from wavi_gb300.gpu import VelocitySolver
        self.g, self.bed, self.p, self.sp, self.ic = synthetic.small_case(**kw, tol_picard=1e-11, maxiter_picard=600)
        self.solver = VelocitySolver(self.g, self.sp, precision="fp64")

    def solve(self, dlogc=None, dloga=None):
        """Model state for C·exp(dlogc), A·exp(dloga) (per cell), solved to the fixed point."""
        from wavi_gb300.model import GPUParallelSpec, Model, pre_solve, release_solver
        g = self.g
        p = self.p
        c = np.full((g.nx, g.ny), float(p.weertman_c)) if np.isscalar(p.weertman_c) else np.array(p.weertman_c)
        a = np.full((g.nx, g.ny), float(p.glen_a_ref)) if np.isscalar(p.glen_a_ref) else np.array(p.glen_a_ref)
        if dlogc is not None:
            c = c * np.exp(dlogc)
        if dloga is not None:
            a = a * np.exp(dloga)
        p2 = dataclasses.replace(p, weertman_c=np.asfortranarray(c), glen_a_ref=np.asfortranarray(a))
        m = Model(g, self.bed, p2, self.sp, self.ic, parallel_spec=GPUParallelSpec(precision="fp64"))
        pre_solve(m)
        f = {k: np.array(v, copy=True, order="F") for k, v in m.fields.items()}
        release_solver(m)
        st = self.solver.solve(m.params, f)
        assert st["status"] == 0, st
        self.m = m
        return m.params, f


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))).cuda()


@pytest.mark.parametrize("kw", [dict(nx=40, ny=16, dx=4000.0, mask="full"), dict(nx=37, ny=13, dx=3000.0, mask="full")])
def test_dot_product_test(kw):
    case = Case(**kw)
    g = case.g
    params, f = case.solve()
    rng = np.random.default_rng(12)
    vc, va = rng.standard_normal((g.nx, g.ny)), rng.standard_normal((g.nx, g.ny))
    wu = np.where(case.m.u_inner, rng.standard_normal((g.nx + 1, g.ny)), 0.0)
    wv = np.where(case.m.v_inner, rng.standard_normal((g.nx, g.ny + 1)), 0.0)
    du = torch.zeros((g.nx + 1) * g.ny, dtype=torch.float64, device="cuda")
    dv = torch.zeros(g.nx * (g.ny + 1), dtype=torch.float64, device="cuda")
    st_t = case.solver.tangent_device(params, _dev(vc), _dev(va), du, dv, tol=1e-12)
    gc = torch.zeros(g.nx * g.ny, dtype=torch.float64, device="cuda")
    ga = torch.zeros_like(gc)
    st_a = case.solver.adjoint_device(params, _dev(wu), _dev(wv), gc, ga, tol=1e-12)
    lhs = float(torch.dot(du, _dev(wu)) + torch.dot(dv, _dev(wv)))
    rhs = float(torch.dot(gc, _dev(vc)) + torch.dot(ga, _dev(va)))
    print("dot test", lhs, rhs, st_t, st_a)
    assert st_t["status"] == 0 and st_a["status"] == 0
    assert abs(lhs - rhs) <= 1e-8 * max(abs(lhs), abs(rhs))


def test_gradient_matches_central_differences():
    from wavi_gb300.misfit import misfit, misfit_gradient, speed
    case = Case(nx=40, ny=16, dx=4000.0, mask="full")
    g = case.g
    params, f0 = case.solve()
    m = case.m
    s0, _, _ = speed(f0["u"], f0["v"], m.u_mask, m.v_mask, m.h_mask)
    rng = np.random.default_rng(4)
    s_obs = s0 * (1.0 + 0.02 * rng.standard_normal(s0.shape))
    gu, gv = misfit_gradient(f0["u"], f0["v"], m.u_mask, m.v_mask, m.h_mask, s_obs)
    gc = torch.zeros(g.nx * g.ny, dtype=torch.float64, device="cuda")
    ga = torch.zeros_like(gc)
    st = case.solver.adjoint_device(params, _dev(gu), _dev(gv), gc, ga, tol=1e-12)
    assert st["status"] == 0, st
    grad_c = gc.cpu().numpy().reshape((g.nx, g.ny), order="F")
    grad_a = ga.cpu().numpy().reshape((g.nx, g.ny), order="F")
    h = 1e-3
    for k in range(3):
        drng = np.random.default_rng(100 + k)
        vc, va = drng.standard_normal((g.nx, g.ny)), drng.standard_normal((g.nx, g.ny))
        ad = float(np.sum(grad_c * vc) + np.sum(grad_a * va))
        _, fp = case.solve(h * vc, h * va)
        jp = misfit(fp["u"], fp["v"], m.u_mask, m.v_mask, m.h_mask, s_obs)
        _, fm = case.solve(-h * vc, -h * va)
        jm = misfit(fm["u"], fm["v"], m.u_mask, m.v_mask, m.h_mask, s_obs)
        fd = (jp - jm) / (2 * h)
        print("direction", k, "adjoint", ad, "central difference", fd)
        assert abs(ad - fd) <= 1e-4 * abs(fd), (k, ad, fd)


def test_adjoint_preconditions():
    from wavi_gb300 import synthetic
    from wavi_gb300.abi import WaviError
    from wavi_gb300.gpu import VelocitySolver
    g, bed, p, sp, ic = synthetic.small_case(nx=24, ny=12)
    s = VelocitySolver(g, sp, precision="mixed")
    z = torch.zeros(max((g.nx + 1) * g.ny, g.nx * (g.ny + 1)), dtype=torch.float64, device="cuda")
    with pytest.raises(WaviError, match="float64"):
        s.adjoint_device(p, z, z, z, z)
    s.close()
    s = VelocitySolver(g, sp, precision="fp64")
    with pytest.raises(WaviError, match="no converged solve"):
        s.adjoint_device(p, z, z, z, z)
    s.close()


def test_autograd_function_backward_is_the_adjoint():
    """torch.autograd through VelocityFunction: the gradient of <w, (u, v)> agrees with the tangent linear,
    <∇, dθ> = <w, J dθ>."""
    from wavi_gb300.autograd import Problem, VelocityFunction
    case = Case(nx=40, ny=16, dx=4000.0, mask="full")
    g = case.g
    c0, a0 = float(case.p.weertman_c), float(case.p.glen_a_ref)
    prob = Problem(case.solver, lambda C, A: case.solve(np.log(C / c0), np.log(A / a0)), tol=1e-12)
    logC = torch.full((g.nx * g.ny,), np.log(c0), dtype=torch.float64, device="cuda", requires_grad=True)
    logA = torch.full((g.nx * g.ny,), np.log(a0), dtype=torch.float64, device="cuda", requires_grad=True)
    u, v = VelocityFunction.apply(logC, logA, prob)
    rng = np.random.default_rng(21)
    wu = _dev(np.where(case.m.u_inner, rng.standard_normal((g.nx + 1, g.ny)), 0.0))
    wv = _dev(np.where(case.m.v_inner, rng.standard_normal((g.nx, g.ny + 1)), 0.0))
    (torch.dot(wu, u) + torch.dot(wv, v)).backward()
    vc, va = rng.standard_normal((g.nx, g.ny)), rng.standard_normal((g.nx, g.ny))
    du = torch.zeros((g.nx + 1) * g.ny, dtype=torch.float64, device="cuda")
    dv = torch.zeros(g.nx * (g.ny + 1), dtype=torch.float64, device="cuda")
    case.solver.tangent_device(case.m.params, _dev(vc), _dev(va), du, dv, tol=1e-12)
    lhs = float(torch.dot(wu, du) + torch.dot(wv, dv))
    rhs = float(torch.dot(logC.grad, _dev(vc)) + torch.dot(logA.grad, _dev(va)))
    assert abs(lhs - rhs) <= 1e-8 * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("kw,coarse", [(dict(nx=40, ny=16, dx=4000.0, mask="full"), "auto"),
                                       (dict(nx=37, ny=13, dx=3000.0, mask="full"), "auto"),
                                       (dict(nx=40, ny=16, dx=4000.0, mask="full"), "srcg_chebyshev")])
def test_fp32_preconditioner_gives_the_fp64_gradient(kw, coarse):
    """The adjoint's FGMRES preconditioned by an FP32 V-cycle (wavi_options.adjoint_precond) and by the
    solve's own FP64 V-cycle: both stop at the same FP64 residual (1e-12), so the gradients agree to that
    level; the FP32 preconditioner may take a few more iterations.  Also with the Chebyshev coarse solve,
    whose power vector the FP32 V-cycle restarts from zero."""
    from wavi_gb300.gpu import VelocitySolver
    case = Case(**kw)
    g = case.g
    params, _ = case.solve()
    m = case.m
    rng = np.random.default_rng(31)
    wu = np.where(m.u_inner, rng.standard_normal((g.nx + 1, g.ny)), 0.0)
    wv = np.where(m.v_inner, rng.standard_normal((g.nx, g.ny + 1)), 0.0)
    out = {}
    for prec in ("fp64", "fp32"):
        s = VelocitySolver(g, case.sp, precision="fp64", adjoint_precond=prec, coarse_solver=coarse)
        st = s.solve(params, {k: np.array(v, copy=True, order="F") for k, v in m.fields.items()})
        assert st["status"] == 0, st
        gc = torch.zeros(g.nx * g.ny, dtype=torch.float64, device="cuda")
        ga = torch.zeros_like(gc)
        ast = s.adjoint_device(params, _dev(wu), _dev(wv), gc, ga, tol=1e-12)
        s.close()
        assert ast["status"] == 0, (prec, ast)
        out[prec] = (torch.cat([gc, ga]).cpu().numpy(), ast)
        print(prec, ast)
    a, b = out["fp64"][0], out["fp32"][0]
    assert np.linalg.norm(a - b) <= 1e-9 * np.linalg.norm(a), np.linalg.norm(a - b) / np.linalg.norm(a)
