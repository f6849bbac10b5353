"""Generate the committed golden fixtures for the MISMIP+ 100-year version-update test.

The reference pins its whole time-stepping loop (and therefore 1000 coupled velocity solves) with
four JLD2 files, ``test/version_update_test_verification/v1_*_MISMIP_100yr_output_8kmres_maxiter1_timesteppt1.jld2``
(compared in ``test/version_update_test_verification/test_version_updates.jl:90-97``).  JLD2 files are HDF5
files; every dataset there is a little-endian float64 array stored compact or contiguous.  This script carries a minimal
HDF5 reader (superblock v2/v3, version-2 object headers, link messages, compact and contiguous data layouts) and writes
``mismip_100yr_<julia version>.npz`` next to itself.  It reads the reference checkout and is run by hand
in a container that has it; the GPU machine only sees the ``.npz`` files.

Usage:  python tests/golden/make_golden.py [path-to-reference-checkout]
"""
import os
import struct
import sys

import numpy as np

NAMES = ("h", "u", "v", "viscosity", "grounded_fraction", "bed_speed")
SHAPES = {"h": (80, 10), "u": (81, 10), "v": (80, 11), "viscosity": (80, 10),
          "grounded_fraction": (80, 10), "bed_speed": (80, 10)}


class HDF5Reader:
    """Just enough HDF5 to walk a JLD2 root group and pull out contiguous float64 datasets."""

    def __init__(self, data: bytes):
        self.d = data
        sb = data.find(b"\x89HDF\r\n\x1a\n")
        if sb < 0:
            raise ValueError("no HDF5 superblock")
        ver = data[sb + 8]
        if ver not in (2, 3):
            raise ValueError(f"unsupported superblock version {ver}")
        self.so, self.sl = data[sb + 9], data[sb + 10]
        p = sb + 12
        self.base, = struct.unpack_from("<Q", data, p)
        root_rel, = struct.unpack_from("<Q", data, p + 24)
        self.root = self.base + root_rel

    def _messages(self, addr):
        d = self.d
        if d[addr:addr + 4] != b"OHDR":
            raise ValueError(f"expected OHDR at {addr}")
        flags = d[addr + 5]
        p = addr + 6
        if flags & 0x20:
            p += 16
        if flags & 0x10:
            p += 4
        nsz = 1 << (flags & 3)
        chunk = int.from_bytes(d[p:p + nsz], "little")
        p += nsz
        end = p + chunk
        while p + 4 <= end:
            mtype = d[p]
            msize, = struct.unpack_from("<H", d, p + 1)
            mflags = d[p + 3]
            p += 4
            if flags & 0x04:
                p += 2
            yield mtype, d[p:p + msize], mflags
            p += msize

    def links(self):
        out = {}
        for mtype, body, _ in self._messages(self.root):
            if mtype != 6:  # link message
                continue
            flags = body[1]
            q = 2
            ltype = 0
            if flags & 0x08:
                ltype = body[q]
                q += 1
            if flags & 0x04:
                q += 8
            if flags & 0x10:
                q += 1
            nlen_sz = 1 << (flags & 3)
            nlen = int.from_bytes(body[q:q + nlen_sz], "little")
            q += nlen_sz
            name = body[q:q + nlen].decode()
            q += nlen
            if ltype == 0:
                addr, = struct.unpack_from("<Q", body, q)
                out[name] = self.base + addr
        return out

    def dataset(self, addr):
        dims = None
        raw = None
        for mtype, body, _ in self._messages(addr):
            if mtype == 1:  # dataspace
                ver, rank = body[0], body[1]
                q = 4 if ver == 2 else 8
                dims = struct.unpack_from("<" + "Q" * rank, body, q)
            elif mtype == 8:  # data layout (version 3/4): class 0 compact, 1 contiguous
                cls = body[1]
                if cls == 0:
                    size, = struct.unpack_from("<H", body, 2)
                    raw = body[4:4 + size]
                elif cls == 1:
                    data_addr, size = struct.unpack_from("<QQ", body, 2)
                    raw = self.d[self.base + data_addr:self.base + data_addr + size]
                else:
                    raise ValueError("chunked layout not supported")
        if raw is None or dims is None:
            raise ValueError("dataset without a readable layout")
        n = int(np.prod(dims))
        if len(raw) != 8 * n:
            raise ValueError("dataset is not float64")
        # HDF5 lists dimensions slowest first; JLD2 writes Julia's column-major arrays with the
        # dimensions reversed, so the raw bytes are already in Julia (x fastest) order.
        return np.frombuffer(raw, dtype="<f8").copy(), tuple(reversed(dims))


def read_golden(path):
    rd = HDF5Reader(open(path, "rb").read())
    links = rd.links()
    out = {}
    for name in NAMES:
        arr, shape = rd.dataset(links[name])
        if shape != SHAPES[name]:
            raise ValueError(f"{name}: shape {shape} != {SHAPES[name]}")
        out[name] = arr.reshape(shape, order="F")
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    src = os.path.join(ref, "test", "version_update_test_verification")
    here = os.path.dirname(os.path.abspath(__file__))
    for ver in ("1_5_1", "1_6_1", "1_6_2", "1_8_3"):
        fn = os.path.join(src, f"v{ver}_MISMIP_100yr_output_8kmres_maxiter1_timesteppt1.jld2")
        g = read_golden(fn)
        np.savez_compressed(os.path.join(here, f"mismip_100yr_v{ver}.npz"), **g)
        print(ver, {k: (v.shape, float(np.abs(v).max())) for k, v in g.items()})


if __name__ == "__main__":
    main()
