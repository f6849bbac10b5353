"""File formats around the velocity solve: the MITgcm velocity dump and JLD2 datasets.

write_vel / read_vel
    The reference's ``write_vel`` (src/Simulations/run_simulation.jl:107-124), which hands the final
    velocities to MITgcm's STREAMICE in the coupled model: ``<prefix>_U.bin`` holds gu.u without its last
    column of points (u[1:end-1, :], nx x ny) and ``<prefix>_V.bin`` gv.v without its last row (v[:, 1:end-1],
    nx x ny), each as big-endian float64 in Julia's column-major order, nothing else in the file.

read_jld2
    The float64 datasets of a JLD2 file's root group (JLD2 files are HDF5 files: superblock v2/v3,
    version-2 object headers, link messages, compact or contiguous data layouts), as Julia-shaped arrays.
    Enough for the reference's golden and output files, which store each field as a plain float64 array;
    chunked or compressed datasets, and JLD2's serialised Julia structs, are not read.
"""
import struct

import numpy as np


def write_vel(prefix, u, v):
    """Write ``<prefix>_U.bin`` and ``<prefix>_V.bin`` as the reference's write_vel does; u is the
    (nx + 1) x ny u-grid field, v the nx x (ny + 1) v-grid field.  Returns the two file names."""
    u = np.asarray(u, dtype=np.float64)
    v = np.asarray(v, dtype=np.float64)
    if u.ndim != 2 or v.ndim != 2 or u.shape[0] != v.shape[0] + 1 or v.shape[1] != u.shape[1] + 1:
        raise ValueError(f"expected u (nx+1, ny) and v (nx, ny+1), got {u.shape} and {v.shape}")
    names = (f"{prefix}_U.bin", f"{prefix}_V.bin")
    for fn, a in zip(names, (u[:-1, :], v[:, :-1])):
        with open(fn, "wb") as f:
            f.write(np.ascontiguousarray(a.ravel(order="F"), dtype=">f8").tobytes())
    return names


def read_vel(prefix, nx, ny):
    """Read a write_vel pair back: (u[:nx, :ny], v[:nx, :ny]) as native float64 nx x ny arrays."""
    out = []
    for fn in (f"{prefix}_U.bin", f"{prefix}_V.bin"):
        a = np.fromfile(fn, dtype=">f8")
        if a.size != nx * ny:
            raise ValueError(f"{fn}: {a.size} values, expected {nx * ny}")
        out.append(a.astype(np.float64).reshape((nx, ny), order="F"))
    return tuple(out)


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



def read_jld2(path, names=None):
    """The float64 datasets of the JLD2 file's root group (or those in ``names``) as a dict of arrays in
    Julia's shape and column-major order.  Datasets that are not plain float64 arrays are skipped unless
    named, in which case they raise."""
    with open(path, "rb") as f:
        rd = HDF5Reader(f.read())
    links = rd.links()
    out = {}
    for name in (names if names is not None else sorted(links)):
        if name not in links:
            raise KeyError(name)
        try:
            arr, shape = rd.dataset(links[name])
        except ValueError:
            if names is not None:
                raise
            continue
        out[name] = arr.reshape(shape, order="F")
    return out
