"""update_wavelets! (Wavelets/update_wavelets.jl:6-32) on the device, one step on identical inputs.

The device time stepping (wavi_run_device) rebuilds the adaptive coarse space after every solve: the
forward Haar transform of the model-masked velocities, then |w| >= wavelet_threshold.  The mask is byte
output, so on the same velocities it must equal the oracle's exactly.  wavi_update_wavelets_device runs
those two kernels of the time step on velocities the test gives it (the oracle's converged solution, and
random fields scaled so that many coefficients lie near the threshold)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CASES = {
    "full": dict(nx=40, ny=16, dx=4000.0, mask="full"),
    "disc": dict(nx=24, ny=24, dx=4000.0, mask="disc"),
    "ragged": dict(nx=37, ny=13, dx=3000.0, mask="full"),
}


def _cat(u, v):
    return np.concatenate([np.asarray(u).ravel(order="F"), np.asarray(v).ravel(order="F")])


@pytest.mark.parametrize("name", list(CASES))
def test_device_wavelet_mask_is_bit_exact(oracle, name):
    from wavi_gb300 import synthetic
    from wavi_gb300.gpu import VelocitySolver
    g, bed, p, sp, ic = synthetic.small_case(**CASES[name], maxiter_picard=80, tol_picard=1e-7)
    om = oracle.build_model(g, bed, p, sp, ic)
    om.pre_solve()
    om.update_velocities()
    s = VelocitySolver(g, sp, precision="fp64")
    rng = np.random.default_rng(12)
    fields = [(np.array(om.field("u"), order="F"), np.array(om.field("v"), order="F"))]
    for scale in (10.0, 30.0):
        fields.append((scale * rng.standard_normal(om.field("u").shape),
                       scale * rng.standard_normal(om.field("v").shape)))
    near = 0
    for u, v in fields:
        om.field("u")[...] = u
        om.field("v")[...] = v
        om.update_wavelets()
        ref = _cat(om.mask("wu_mask"), om.mask("wv_mask")).astype(np.uint8)
        uv = torch.from_numpy(_cat(u, v)).cuda()
        out = torch.full((ref.size,), 7, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()  # the library runs on its context's own stream: the fill must be done first
        s.update_wavelets_device(uv, out)
        got = out.cpu().numpy()
        assert got.max() <= 1
        assert np.array_equal(got, ref), int(np.sum(got != ref))
        # coefficients within 5 % of the threshold: the comparison is not decided far from it
        um, vm = om.mask("u_mask").astype(float), om.mask("v_mask").astype(float)
        wav = _cat(om.haar(0, 2, um * u), om.haar(1, 2, vm * v))
        near += int(np.sum(np.abs(np.abs(wav) - sp.wavelet_threshold) < 0.05 * sp.wavelet_threshold))
    s.close()
    assert near > 10, near
