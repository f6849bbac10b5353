"""Generate the committed golden fixtures for the MISMIP+ 100-year version-update test.

The reference pins its whole time-stepping loop (and therefore 1000 coupled velocity solves) with
four JLD2 files, ``test/version_update_test_verification/v1_*_MISMIP_100yr_output_8kmres_maxiter1_timesteppt1.jld2``
(compared in ``test/version_update_test_verification/test_version_updates.jl:90-97``).  JLD2 files are HDF5
files; every dataset there is a little-endian float64 array stored compact or contiguous.  This script reads them with
the package's minimal HDF5 reader (``wavi_gb300.io.read_jld2``) and writes ``mismip_100yr_<julia version>.npz`` next to
itself, and ``jld2_files.json``: each file's header Julia version, link order and SHA-256, so that a test can rebuild the
files byte for byte with ``wavi_gb300.io.write_jld2``.  It reads the reference checkout and is run by hand
on a machine that has it; the tests elsewhere only need the ``.npz`` files.

Usage:  python tests/golden/make_golden.py <path-to-reference-checkout>
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from wavi_gb300.io import HDF5Reader, read_jld2  # noqa: E402

NAMES = ("h", "u", "v", "viscosity", "grounded_fraction", "bed_speed")
SHAPES = {"h": (80, 10), "u": (81, 10), "v": (80, 11), "viscosity": (80, 10),
          "grounded_fraction": (80, 10), "bed_speed": (80, 10)}


def read_golden(path):
    out = read_jld2(path, NAMES)
    for name in NAMES:
        if out[name].shape != SHAPES[name]:
            raise ValueError(f"{name}: shape {out[name].shape} != {SHAPES[name]}")
    return out


def file_record(path):
    """What a byte-exact rebuild of the file needs besides the arrays: the Julia version in its JLD2
    header, its root group's link order, and its SHA-256."""
    with open(path, "rb") as f:
        d = f.read()
    rd = HDF5Reader(d)
    julia = d[d.index(b"(Julia ") + 7:d.index(b" 64-bit")].decode()
    return {"julia_version": julia, "links": list(rd.links()), "sha256": hashlib.sha256(d).hexdigest(),
            "bytes": len(d)}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the WAVI.jl source tree>")
    ref = sys.argv[1]
    src = os.path.join(ref, "test", "version_update_test_verification")
    here = os.path.dirname(os.path.abspath(__file__))
    records = {}
    for ver in ("1_5_1", "1_6_1", "1_6_2", "1_8_3"):
        fn = os.path.join(src, f"v{ver}_MISMIP_100yr_output_8kmres_maxiter1_timesteppt1.jld2")
        g = read_golden(fn)
        out = os.path.join(here, f"mismip_100yr_v{ver}.npz")
        if not os.path.exists(out) or any(not np.array_equal(np.load(out)[k], g[k]) for k in NAMES):
            np.savez_compressed(out, **g)
        records[f"v{ver}"] = file_record(fn)
        print(ver, {k: (v.shape, float(np.abs(v).max())) for k, v in g.items()})
    with open(os.path.join(here, "jld2_files.json"), "w") as f:
        json.dump(records, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
