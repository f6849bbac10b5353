"""File formats around the solve (wavi_gb300.io): the reference's write_vel dump for MITgcm
(src/Simulations/run_simulation.jl:107-124), the JLD2 reader and writer, and the output files of
run_simulation! (src/OutputParams/output_writing.jl)."""
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


def test_lookup3_known_answers(pkg):
    """Jenkins' lookup3 hashlittle self-test values (lookup3.c, driver5), the checksum of HDF5 metadata."""
    from wavi_gb300.io import lookup3
    assert lookup3(b"") == 0xDEADBEEF
    assert lookup3(b"Four score and seven years ago") == 0x17770551
    assert lookup3(b"Four score and seven years ago", 1) == 0xCD628161


@pytest.mark.parametrize("ver", ["v1_5_1", "v1_6_1", "v1_6_2", "v1_8_3"])
def test_write_jld2_rebuilds_the_reference_golden_files_byte_for_byte(tmp_path, pkg, ver):
    """write_jld2 on the arrays of the reference's golden JLD2 files (the committed fixtures), in their
    link order and with their header's Julia version, gives files whose SHA-256 equals the reference
    files' (recorded by make_golden.py); reading them back gives the arrays."""
    import hashlib
    import json
    from wavi_gb300.io import read_jld2, write_jld2
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    rec = json.load(open(os.path.join(here, "jld2_files.json")))[ver]
    z = np.load(os.path.join(here, f"mismip_100yr_{ver}.npz"))
    fn = str(tmp_path / "out.jld2")
    n = write_jld2(fn, {k: z[k] for k in rec["links"]}, rec["julia_version"])
    data = open(fn, "rb").read()
    assert n == len(data) == rec["bytes"]
    assert hashlib.sha256(data).hexdigest() == rec["sha256"]
    back = read_jld2(fn)
    assert list(back) == sorted(rec["links"])
    for k in rec["links"]:
        assert back[k].shape == z[k].shape and np.array_equal(back[k], z[k]), k


def test_write_jld2_contiguous_and_checksummed(tmp_path, pkg):
    """Arrays above the compact limit go contiguous after their object header (a 640 x 80 field, a 3-D
    sigma field), small ones stay compact; the reader checks every checksum and rejects a flipped byte."""
    from wavi_gb300.io import COMPACT_LIMIT, ChecksumError, read_jld2, write_jld2
    rng = np.random.default_rng(9)
    arrays = {"u": rng.standard_normal((641, 80)), "eta": rng.standard_normal((64, 20, 4)),
              "small": rng.standard_normal((3, 5)), "x": np.arange(7.0)}
    assert arrays["u"].nbytes > COMPACT_LIMIT and arrays["small"].nbytes <= COMPACT_LIMIT
    fn = str(tmp_path / "big.jld2")
    write_jld2(fn, arrays)
    back = read_jld2(fn)
    for k, a in arrays.items():
        assert back[k].shape == a.shape and np.array_equal(back[k], a), k
    data = bytearray(open(fn, "rb").read())
    data[600] ^= 1  # inside the first object header
    open(fn, "wb").write(bytes(data))
    with pytest.raises(ChecksumError):
        read_jld2(fn)
    with pytest.raises(ValueError):
        write_jld2(fn, {"i": np.arange(3)})
    with pytest.raises(ValueError):
        write_jld2(fn, {"e": np.zeros((0, 3))})


def test_output_params_mirror_the_reference_constructor(tmp_path, pkg):
    """OutputParams (src/OutputParams/OutputParams.jl:34-70) and set_n_iter_out! (Simulation.jl:62-66)."""
    from wavi_gb300.config import OutputParams
    op = OutputParams(output_path=str(tmp_path / "new"), output_freq=2.0)
    assert os.path.isdir(tmp_path / "new") and op.output_path.endswith("/")
    assert op.set_n_iter_out(0.5, 40).n_iter_out == 4
    assert OutputParams(output_path=str(tmp_path)).set_n_iter_out(0.5, 40).n_iter_out == 41  # Inf: never
    assert OutputParams(output_path=str(tmp_path), zip_format="zip").zip_format == "none"
    for bad in (dict(output_freq=0.0), dict(output_freq=-1.0), dict(output_format="nc")):
        with pytest.raises(ValueError):
            OutputParams(output_path=str(tmp_path), **bad)


def _sim(tmp_path, fmt="jld2", **kw):
    from wavi_gb300 import synthetic
    from wavi_gb300.config import OutputParams, TimesteppingParams
    from wavi_gb300.model import Model, Simulation
    g, bed, p, sp, ic = synthetic.small_case(nx=12, ny=6)
    m = Model(g, bed, p, sp, ic)
    op = OutputParams(outputs={"h": m.fields["h"], "u": m.fields["u"]}, output_path=str(tmp_path),
                      prefix="run", output_format=fmt, **kw)
    return Simulation(m, TimesteppingParams(dt=0.25, n_iter_total=6), op)


@pytest.mark.parametrize("fmt", ["jld2", "mat"])
def test_write_output_names_and_contents(tmp_path, pkg, fmt):
    """write_output (output_writing.jl:7-27): the outputs, t rounded to 3 decimals, and the h-grid x, y in
    <path><prefix><n_iter as 10 digits>.<format>."""
    from wavi_gb300.io import read_jld2, write_output
    sim = _sim(tmp_path, fmt)
    sim.n_iter, sim.time = 3, 0.7500004
    fn = write_output(sim)
    assert fn == str(tmp_path) + "/run0000000003." + fmt
    if fmt == "jld2":
        got = read_jld2(fn)
    else:
        from scipy.io import loadmat
        got = loadmat(fn, squeeze_me=False)
    f, g = sim.model.fields, sim.model.grid
    assert float(np.squeeze(got["t"])) == 0.75
    for k, want in (("h", f["h"]), ("u", f["u"]), ("x", g.xxh), ("y", g.yyh)):
        assert np.array_equal(np.asarray(got[k]), want), k


def test_run_simulation_writes_outputs_on_the_reference_schedule(tmp_path, pkg, monkeypatch):
    """run_simulation! (run_simulation.jl:61-100): the initial output with output_start, one every
    n_iter_out steps, the MITgcm velocity dump after the last step; outputs read the fields' current values.
    The time step is a stand-in that changes h, so the schedule is checked without a velocity solve."""
    from wavi_gb300 import model as M
    from wavi_gb300.io import read_jld2, read_vel

    def fake_timestep(sim):
        sim.model.fields["h"][...] += 1.0
        sim.n_iter += 1
        sim.time += sim.timestepping_params.dt

    monkeypatch.setattr(M, "timestep", fake_timestep)
    monkeypatch.chdir(tmp_path)
    sim = _sim(tmp_path, output_freq=0.5, output_start=True, dump_vel=True)
    h0 = sim.model.fields["h"].copy()
    M.run_simulation(sim)
    names = sorted(n for n in os.listdir(tmp_path) if n.endswith(".jld2"))
    assert names == [f"run{i:010d}.jld2" for i in (0, 2, 4, 6)]
    for i in (0, 2, 4, 6):
        got = read_jld2(str(tmp_path / f"run{i:010d}.jld2"))
        assert np.array_equal(got["h"], h0 + i) and float(got["t"]) == round(0.25 * i, 3)
    nx, ny = sim.model.grid.nx, sim.model.grid.ny
    u, _ = read_vel("run", nx, ny)
    assert np.array_equal(u, sim.model.fields["u"][:-1, :])


def test_device_copy_back_keeps_field_references(pkg):
    """Fields coming back from a device-resident run are written into the model's arrays in place, so an
    output that holds a reference to a field sees the new values."""
    from wavi_gb300.model import _assign_field
    f = {"h": np.zeros((3, 2), order="F"), "wu_mask": np.zeros((4, 2), bool)}
    ref_h, ref_m = f["h"], f["wu_mask"]
    _assign_field(f, "h", np.ones((3, 2)))
    _assign_field(f, "wu_mask", np.ones((4, 2), np.uint8))
    _assign_field(f, "dhdt", np.full((3, 2), 2.0))
    assert f["h"] is ref_h and (ref_h == 1).all() and f["wu_mask"] is ref_m and ref_m.all()
    assert (f["dhdt"] == 2).all()


@pytest.mark.parametrize("fmt", ["jld2", "mat"])
@pytest.mark.filterwarnings("ignore:found an output variable")
def test_zip_output_merges_the_output_files_into_netcdf(tmp_path, pkg, monkeypatch, fmt):
    """zip_output (src/OutputParams/zipping_output.jl): after the run the output files become one NetCDF
    file with dimensions x, y, TIME, the coordinate variables and their attributes, and each nx x ny output
    over (x, y, TIME) — stored (TIME, y, x) — with the values of every output step."""
    from scipy.io import netcdf_file
    from wavi_gb300 import model as M

    def fake_timestep(sim):
        sim.model.fields["h"][...] += 1.0
        sim.n_iter += 1
        sim.time += sim.timestepping_params.dt

    monkeypatch.setattr(M, "timestep", fake_timestep)
    sim = _sim(tmp_path, fmt, output_freq=0.5, output_start=True, zip_format="nc")
    h0 = sim.model.fields["h"].copy()
    M.run_simulation(sim)
    g = sim.model.grid
    with netcdf_file(str(tmp_path / "run.nc"), "r", mmap=False) as ds:
        assert (ds.dimensions["x"], ds.dimensions["y"], ds.dimensions["TIME"]) == (g.nx, g.ny, 4)
        assert np.array_equal(ds.variables["x"][:], g.xxh[:, 0]) and np.array_equal(ds.variables["y"][:], g.yyh[0, :])
        assert np.allclose(ds.variables["TIME"][:], [0.0, 0.5, 1.0, 1.5])
        assert ds.variables["TIME"].units == b"years" and ds.variables["x"].units == b"m"
        assert ds.variables["h"].dimensions == ("TIME", "y", "x")
        h = ds.variables["h"][:].copy()
        assert "u" not in ds.variables  # (nx + 1) x ny: not on the h grid, skipped as in the reference
    for i in range(4):
        assert np.array_equal(h[i].T, h0 + 2 * i)
