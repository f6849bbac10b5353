"""File formats around the solve (wavi_gb300.io): the reference's write_vel dump for MITgcm
(src/Simulations/run_simulation.jl:107-124) and the JLD2 dataset reader."""
import os

import numpy as np
import pytest


def test_write_vel_layout_and_round_trip(tmp_path, pkg):
    from wavi_gb300.io import read_vel, write_vel
    rng = np.random.default_rng(5)
    nx, ny = 7, 4
    u = np.asfortranarray(rng.standard_normal((nx + 1, ny)))
    v = np.asfortranarray(rng.standard_normal((nx, ny + 1)))
    fu, fv = write_vel(str(tmp_path / "run"), u, v)
    assert os.path.basename(fu) == "run_U.bin" and os.path.basename(fv) == "run_V.bin"
    raw = open(fu, "rb").read()
    assert len(raw) == 8 * nx * ny  # u[1:end-1, :]: the last column of u points is not written
    assert raw[:8] == np.array([u[0, 0]], dtype=">f8").tobytes()  # big-endian (hton)
    assert raw[8:16] == np.array([u[1, 0]], dtype=">f8").tobytes()  # column-major
    ur, vr = read_vel(str(tmp_path / "run"), nx, ny)
    assert np.array_equal(ur, u[:-1, :]) and np.array_equal(vr, v[:, :-1])
    with pytest.raises(ValueError):
        write_vel(str(tmp_path / "bad"), v, u)


def test_read_jld2_matches_the_committed_golden_fixtures(pkg):
    """The reader against the reference's own JLD2 golden files (when a reference checkout is named by
    WAVI_REFERENCE_DIR): the datasets equal the committed .npz fixtures made from them."""
    ref = os.environ.get("WAVI_REFERENCE_DIR")
    src = os.path.join(ref or "", "test", "version_update_test_verification")
    if not ref or not os.path.isdir(src):
        pytest.skip("no reference checkout (WAVI_REFERENCE_DIR)")
    from wavi_gb300.io import read_jld2
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    for ver in ("1_5_1", "1_8_3"):
        got = read_jld2(os.path.join(src, f"v{ver}_MISMIP_100yr_output_8kmres_maxiter1_timesteppt1.jld2"))
        want = np.load(os.path.join(here, f"mismip_100yr_v{ver}.npz"))
        for k in want.files:
            assert np.array_equal(got[k], want[k]), (ver, k)
