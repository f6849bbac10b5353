"""wavi_residual_noalloc: the allocation-free residual entry point, for callers that cannot call
cudaMalloc (a framework owning the device heap through its own pool, code under stream capture or in a
callback, a service with a fixed device-memory budget).  It takes every input and output from the
caller and keeps its reduction scratch in a static device array.

Checked on two calls in a row against the existing entry point (wavi_apply_operator_device on a
relinearised float64 context) and against the FP64 oracle's operator (op_fun!, utilities.jl:61-145) on
the same x and b, which shares none of the library's stencil code: r = b - A x and ||r||^2 to the
operator tests' 1e-12.  This file sorts last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import fields_from_oracle, rel, to_dev

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _operator_arrays(om, g):
    """The operator's device coefficient arrays, folded exactly as the reference folds its crops
    (update_rheological_operators!), taken from the oracle's relinearised model."""
    um, vm = om.mask("u_mask").astype(bool), om.mask("v_mask").astype(bool)
    cat = lambda a, b: np.concatenate([np.asarray(a).ravel(order="F"), np.asarray(b).ravel(order="F")])
    arrs = {
        "heta_h": -np.asarray(om.field("dneg_heta_h")).ravel(order="F"),
        "heta_c": -np.asarray(om.field("dneg_heta_c")).ravel(order="F"),
        "dimp": np.asarray(om.field("dimplicit")).ravel(order="F"),
        "beta_m": -cat(om.field("gu_dnegbeff"), om.field("gv_dnegbeff")),
        "h_m": cat(np.where(um, om.field("gu_h"), 0.0), np.where(vm, om.field("gv_h"), 0.0)),
    }
    dev = {k: torch.from_numpy(np.ascontiguousarray(v + 0.0)).cuda() for k, v in arrs.items()}
    inner = cat(om.mask("u_inner"), om.mask("v_inner")).astype(np.uint8)
    dev["inner"] = torch.from_numpy(inner).cuda()
    return dev, inner.astype(bool)


@pytest.mark.parametrize("name", ["full", "disc"])
def test_residual_noalloc_matches_operator_entry_point_and_oracle(oracle, name):
    from wavi_gb300 import abi, synthetic
    from wavi_gb300.gpu import VelocitySolver
    case = dict(nx=40, ny=16, dx=4000.0, mask="full") if name == "full" else dict(nx=24, ny=24, dx=4000.0, mask="disc")
    g, bed, p, sp, ic = synthetic.small_case(**case)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    rng = np.random.default_rng(11)
    om.field("u")[...] = 50 * rng.standard_normal(om.field("u").shape)
    om.field("v")[...] = 20 * rng.standard_normal(om.field("v").shape)
    f = fields_from_oracle(om, g)
    solver = VelocitySolver(g, sp, precision="fp64")
    solver.relinearise_device(p, to_dev(f, torch))  # the existing entry point's coefficients
    om.inner_update()
    dev, inner = _operator_arrays(om, g)
    lib = abi.load_library()
    desc = abi.OperatorDesc(g.nx, g.ny, g.dx, g.dy, *(C.c_void_p(dev[k].data_ptr()) for k in
                                                      ("heta_h", "heta_c", "dimp", "beta_m", "h_m", "inner")))
    n = inner.size
    nu = (g.nx + 1) * g.ny
    for call in range(2):  # the static scratch is shared: the second call must not see the first's state
        xh = rng.standard_normal(n) * inner
        bh = rng.standard_normal(n) * 1e3 * inner
        x = torch.from_numpy(xh).cuda()
        b = torch.from_numpy(bh).cuda()
        y = torch.zeros_like(x)
        solver.apply_operator_device(x, y, "fp64")
        r_ref = (b - y).cpu().numpy() * inner
        rr_ref = float(np.sum(r_ref ** 2))
        # the oracle's own operator on the same x: independent of the library's stencil helpers
        ou, ov = om.apply_operator(xh[:nu].reshape((g.nx + 1, g.ny), order="F"),
                                   xh[nu:].reshape((g.nx, g.ny + 1), order="F"))
        r_orc = (bh - np.concatenate([np.asarray(ou).ravel(order="F"), np.asarray(ov).ravel(order="F")])) * inner
        rr_orc = float(np.sum(r_orc ** 2))
        r = torch.full_like(x, float("nan"))
        rr = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        st = lib.wavi_residual_noalloc(C.byref(desc), C.c_void_p(x.data_ptr()), C.c_void_p(b.data_ptr()),
                                       C.c_void_p(r.data_ptr()), C.c_void_p(rr.data_ptr()), None)
        assert st == 0, lib.wavi_last_error(None)
        torch.cuda.synchronize()
        assert rel(r.cpu().numpy(), r_ref) < 1e-12, call
        assert abs(float(rr.item()) - rr_ref) <= 1e-12 * rr_ref, call
        assert rel(r.cpu().numpy(), r_orc) < 1e-12, call
        assert abs(float(rr.item()) - rr_orc) <= 1e-12 * rr_orc, call
    solver.close()


def test_residual_noalloc_rejects_grids_beyond_its_scratch():
    from wavi_gb300 import abi
    lib = abi.load_library()
    big = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(big.data_ptr())
    nx, ny = 32 * 129 - 1, 8 * 128  # 129 x 129 = 16641 tiles > 16384
    desc = abi.OperatorDesc(nx, ny, 1000.0, 1000.0, p, p, p, p, p, p)
    st = lib.wavi_residual_noalloc(C.byref(desc), p, p, p, p, None)
    assert st == -1
    assert b"too large" in lib.wavi_last_error(None)
