"""Parity at the largest configuration's full size (2560 x 320 at 250 m, nσ = 8: 1.6 M velocity unknowns),
where a whole oracle solve is out of a test's reach but single steps are not.

  relinearisation (inner_update!, update_velocities.jl:32-45) and one application of the momentum
  operator (op_fun!, utilities.jl:61-145) at a nonzero velocity field: GPU FP64 against the oracle on the
  same inputs, to the small-grid tests' 1e-12 (1e-11 for the viscosity and quadratures)
  the operator's symmetry <Ax, y> = <x, Ay> and sign (declared isposdef, update_velocities.jl:396; the
  reference's operator is negative definite)
  the Haar transforms (update_wavelets.jl:38-89): dwt(idwt x) = x, and idwtᵀ the transpose of idwt
  the FP32 operator of a mixed context within FP32 rounding of the FP64 one
"""
import os
import sys

import numpy as np
import pytest

from helpers import SOLVE_FIELDS, rel

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))


def _cat(u, v):
    return np.concatenate([np.asarray(u).ravel(order="F"), np.asarray(v).ravel(order="F")])


@pytest.fixture(scope="module")
def c3(oracle):
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import __graft_entry__ as ge
    from make_c3_history import c3_state
    from wavi_gb300.model import release_solver
    pkg = ge.load_package()
    m, (g, bed, p, sp, ic) = c3_state(pkg)
    release_solver(m)
    rng = np.random.default_rng(21)
    f = {k: np.array(m.fields[k], copy=True, order="F") for k in m.fields}
    f["u"][...] = 40.0 * rng.standard_normal(f["u"].shape) * m.u_mask
    f["v"][...] = 15.0 * rng.standard_normal(f["v"].shape) * m.v_mask
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    for k in SOLVE_FIELDS:  # the host model's exact state (its glen_b may differ from the oracle's in the last bit)
        om.field(k)[...] = f[k]
    return m, g, p, sp, f, om, rng


def _dev(f):
    out = {}
    for k, a in f.items():
        arr = np.asarray(a)
        dt = np.uint8 if k in ("wu_mask", "wv_mask") else np.float64
        out[k] = torch.from_numpy(np.ascontiguousarray(arr.astype(dt).ravel(order="F"))).cuda()
    return out


def test_relinearise_and_operator_match_oracle_at_full_size(c3):
    from wavi_gb300.gpu import ALL_FIELDS, VelocitySolver
    m, g, p, sp, f, om, rng = c3
    s = VelocitySolver(g, sp, precision="fp64")
    t = _dev({k: f[k] for k in ALL_FIELDS})
    s.relinearise_device(p, t)
    om.inner_update()
    for k in ("shelf_strain_rate", "av_speed", "bed_speed", "beta", "tau_bed"):
        got = t[k].cpu().numpy().reshape(np.asarray(om.field(k)).shape, order="F")
        assert rel(got, om.field(k)) < 1e-12, k
    for k in ("eta", "eta_av", "quad_f1", "quad_f2", "beta_eff", "gu_beta_eff", "gv_beta_eff"):
        got = t[k].cpu().numpy().reshape(np.asarray(om.field(k)).shape, order="F")
        assert rel(got, om.field(k)) < 1e-11, k
    iu, iv = m.u_inner.astype(bool), m.v_inner.astype(bool)
    xu = rng.standard_normal((g.nx + 1, g.ny)) * iu
    xv = rng.standard_normal((g.nx, g.ny + 1)) * iv
    ref = _cat(*om.apply_operator(xu, xv))
    x = torch.from_numpy(_cat(xu, xv)).cuda()
    y = torch.zeros_like(x)
    s.apply_operator_device(x, y, "fp64")
    assert rel(y.cpu().numpy(), ref) < 1e-12
    s.close()


def test_float_relinearise_matches_oracle_at_full_size(c3):
    """The mixed context's float relinearisation (integer conversions of the FP64 fields, FP64 velocity
    differences, the float chain) on the 2560 x 320, nσ = 8 state against the oracle's FP64 one, within
    float rounding of each field."""
    from wavi_gb300.gpu import ALL_FIELDS, VelocitySolver
    m, g, p, sp, f, om, rng = c3
    s = VelocitySolver(g, sp, precision="mixed")
    t = _dev({k: f[k] for k in ALL_FIELDS})
    s.relinearise_device(p, t)
    for k in SOLVE_FIELDS:  # the oracle back at the fixture's state (an earlier test relinearised it)
        om.field(k)[...] = f[k]
    om.inner_update()
    for k in ("shelf_strain_rate", "av_speed", "bed_speed", "beta", "tau_bed", "eta", "eta_av", "quad_f1",
              "quad_f2", "beta_eff", "gu_beta_eff", "gv_beta_eff"):
        got = t[k].cpu().numpy().reshape(np.asarray(om.field(k)).shape, order="F")
        assert rel(got, om.field(k)) < 2e-6, (k, rel(got, om.field(k)))
    s.close()


def test_operator_symmetry_sign_and_fp32_at_full_size(c3):
    from wavi_gb300.gpu import ALL_FIELDS, VelocitySolver
    m, g, p, sp, f, om, rng = c3
    s = VelocitySolver(g, sp, precision="fp64")
    s.relinearise_device(p, _dev({k: f[k] for k in ALL_FIELDS}))
    sm = VelocitySolver(g, sp, precision="mixed", viscosity="fp64")  # the same coefficients, rounded to FP32
    sm.relinearise_device(p, _dev({k: f[k] for k in ALL_FIELDS}))
    inner = torch.from_numpy(_cat(m.u_inner, m.v_inner).astype(np.float64)).cuda()
    x = torch.randn(inner.numel(), dtype=torch.float64, device="cuda") * inner
    z = torch.randn(inner.numel(), dtype=torch.float64, device="cuda") * inner
    ax, az = torch.zeros_like(x), torch.zeros_like(x)
    torch.cuda.synchronize()  # the library runs on its context's own stream: x and z must be written first
    s.apply_operator_device(x, ax, "fp64")
    s.apply_operator_device(z, az, "fp64")
    lhs, rhs = float(torch.dot(ax, z)), float(torch.dot(x, az))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))
    assert float(torch.dot(ax, x)) < 0
    ax32 = torch.zeros_like(x, dtype=torch.float32)
    x32 = x.float()
    torch.cuda.synchronize()
    sm.apply_operator_device(x32, ax32, "mixed")
    assert float(torch.linalg.norm(ax32.double() - ax) / torch.linalg.norm(ax)) < 1e-5
    s.close()
    sm.close()


def test_haar_transforms_at_full_size(c3):
    from wavi_gb300.gpu import VelocitySolver
    m, g, p, sp, f, om, rng = c3
    s = VelocitySolver(g, sp, precision="fp64")
    n = (g.nx + 1) * g.ny + g.nx * (g.ny + 1)
    ones = torch.ones(n, dtype=torch.uint8, device="cuda")
    x = torch.randn(n, dtype=torch.float64, device="cuda")
    z = torch.randn(n, dtype=torch.float64, device="cuda")
    px, back, rz = torch.zeros_like(x), torch.zeros_like(x), torch.zeros_like(x)
    torch.cuda.synchronize()  # the library runs on its context's own stream
    s.haar_device(0, x, px, ones)      # idwt x
    s.haar_device(2, px, back, ones)   # dwt(idwt x)
    assert float(torch.linalg.norm(back - x) / torch.linalg.norm(x)) < 1e-13
    s.haar_device(1, z, rz, ones)      # idwtᵀ z
    lhs, rhs = float(torch.dot(px, z)), float(torch.dot(x, rz))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))
    # and against the oracle's transform of the u grid
    xu = x[:(g.nx + 1) * g.ny].cpu().numpy().reshape((g.nx + 1, g.ny), order="F")
    ref = np.asarray(om.haar(0, 0, xu)).ravel(order="F")
    assert rel(px[:(g.nx + 1) * g.ny].cpu().numpy(), ref) < 1e-13
    s.close()
