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

write_jld2
    The inverse for float64 arrays: the file JLD2's ``@save`` writes for a set of Float64 arrays (the
    reference's output and golden files, ``test/version_update_test_verification/*.jld2``).  The layout is
    the 512-byte JLD2 header, an HDF5 version-2 superblock, one version-2 object header per array (fill
    value, dataspace, IEEE float64 datatype and a compact or contiguous data layout) in link order, and
    the root group's object header (link info, group info, one link per array, and a 16-byte NIL message
    that keeps room for a header continuation) last.  Every object header and the superblock end in the
    HDF5 lookup3 checksum.  Rebuilding the reference's four golden JLD2 files from their arrays gives them
    byte for byte.

write_output, zip_output
    run_simulation!'s periodic output files (src/OutputParams/output_writing.jl:7-27) in JLD2 (or MAT), and
    their merge into one NetCDF file (src/OutputParams/zipping_output.jl), written in the classic NetCDF
    format (64-bit offsets) by scipy where the reference's NCDatasets writes NetCDF-4: the same dimensions,
    variables, attributes and values, readable by any NetCDF library.
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


class ChecksumError(ValueError):
    """An HDF5 superblock or object header whose stored lookup3 checksum does not match its bytes."""


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
        if struct.unpack_from("<I", data, sb + 44)[0] != lookup3(data[sb:sb + 44]):
            raise ChecksumError("superblock checksum mismatch")
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
        if struct.unpack_from("<I", d, end)[0] != lookup3(d[addr:end]):
            raise ChecksumError(f"object header checksum mismatch at {addr}")
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



def lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' lookup3 ``hashlittle`` (2006, public domain), the checksum of HDF5's version-2
    metadata: 12-byte little-endian blocks mixed into three 32-bit words, the last (partial, zero-padded)
    block followed by the final avalanche; an empty tail after full blocks skips the final step."""
    M = 0xFFFFFFFF

    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & M

    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & M
    p = 0
    while n - p > 12:
        x, y, z = struct.unpack_from("<III", data, p)
        a = (a + x) & M
        b = (b + y) & M
        c = (c + z) & M
        a = (a - c) & M; a ^= rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 4); b = (b + a) & M
        p += 12
    if n - p == 0:
        return c
    x, y, z = struct.unpack("<III", data[p:] + bytes(12 - (n - p)))
    a = (a + x) & M
    b = (b + y) & M
    c = (c + z) & M
    c ^= b; c = (c - rot(b, 14)) & M
    a ^= c; a = (a - rot(c, 11)) & M
    b ^= a; b = (b - rot(a, 25)) & M
    c ^= b; c = (c - rot(b, 16)) & M
    a ^= c; a = (a - rot(c, 4)) & M
    b ^= a; b = (b - rot(a, 14)) & M
    c ^= b; c = (c - rot(b, 24)) & M
    return c


_JLD2_BASE = 512          # the HDF5 base address: the superblock follows the 512-byte JLD2 header
_UNDEF = b"\xff" * 8      # HDF5's undefined address
# IEEE little-endian float64: class 1 version 3, byte order LE, padding 0, mantissa normalised (implied
# leading 1), sign at bit 63; size 8; bit offset 0, precision 64, exponent at bit 52 of 11 bits, mantissa at
# bit 0 of 52 bits, exponent bias 1023
_F64_TYPE = bytes([0x31, 0x20, 0x3F, 0x00]) + struct.pack("<IHHBBBBI", 8, 0, 64, 52, 11, 0, 52, 1023)
_FILL_VALUE = bytes([3, 0x09])    # fill value message v3: allocation early, fill never written, undefined
COMPACT_LIMIT = 8192              # arrays up to this many bytes are stored inside their object header


def _object_header(messages):
    """A version-2 object header ("OHDR", no times or attribute phases) holding ``messages`` (type, flags,
    body), with the chunk-size field of the fewest bytes that fit, and its lookup3 checksum."""
    chunk = b"".join(bytes([t]) + struct.pack("<H", len(body)) + bytes([fl]) + body for t, fl, body in messages)
    for code, width in ((0, 1), (1, 2), (2, 4), (3, 8)):
        if len(chunk) < (1 << (8 * width)):
            break
    head = b"OHDR" + bytes([2, code]) + len(chunk).to_bytes(width, "little")
    out = head + chunk
    return out + struct.pack("<I", lookup3(out))


def write_jld2(path, arrays, julia_version="1.8.3"):
    """Write the float64 arrays (and float64 scalars) of ``arrays`` (a name -> value mapping, in the order
    the links are to be listed) as JLD2's ``@save`` does: each array's dimensions reversed into HDF5
    order, its column-major bytes stored compact (up to COMPACT_LIMIT bytes) or contiguous right after its
    object header.
    ``julia_version`` only fills the header's informational "(Julia x.y.z 64-bit LE)" field."""
    header = b"HDF5-based Julia Data Format, version 0.1.1\x00 (Julia " + julia_version.encode() + b" 64-bit LE)\x00"
    if len(header) > _JLD2_BASE:
        raise ValueError("julia_version too long")
    body = bytearray()            # everything after the superblock, addressed from the base
    pos = 48                      # the version-2 superblock is 48 bytes
    links = []
    for name, a in arrays.items():
        a = np.asarray(a)
        if a.dtype != np.float64 or a.size == 0:
            raise ValueError(f"{name}: only non-empty float64 arrays and float64 scalars are written")
        raw = np.ascontiguousarray(a.ravel(order="F")).astype("<f8").tobytes()
        dims = tuple(reversed(a.shape))
        # dataspace v2: a simple space of the reversed dimensions, or the scalar space of a 0-d value
        space = bytes([2, len(dims), 0, 1 if dims else 0]) + struct.pack("<" + "Q" * len(dims), *dims)
        msgs = [(5, 0, _FILL_VALUE), (1, 0, space), (3, 1, _F64_TYPE)]
        if len(raw) <= COMPACT_LIMIT:
            obj = _object_header(msgs + [(8, 0, bytes([4, 0]) + struct.pack("<H", len(raw)) + raw)])
        else:
            probe = _object_header(msgs + [(8, 0, bytes([4, 1]) + bytes(16))])
            obj = _object_header(msgs + [(8, 0, bytes([4, 1]) + struct.pack("<QQ", pos + len(probe), len(raw)))])
            obj += raw
        links.append((name, pos))
        body += obj
        pos += len(obj)
    root_msgs = [(2, 0, bytes([0, 0]) + _UNDEF + _UNDEF), (10, 0, bytes([0, 0]))]
    for name, addr in links:
        nb = name.encode()
        if len(nb) > 255:
            raise ValueError(f"{name}: link names up to 255 bytes")
        root_msgs.append((6, 0, bytes([1, 0x10, 1, len(nb)]) + nb + struct.pack("<Q", addr)))
    root_msgs.append((0, 0, bytes(16)))
    root = _object_header(root_msgs)
    root_addr = pos
    body += root
    eof = _JLD2_BASE + 48 + len(body)
    sb = b"\x89HDF\r\n\x1a\n" + bytes([2, 8, 8, 0]) + struct.pack("<Q", _JLD2_BASE) + _UNDEF + \
        struct.pack("<QQ", eof, root_addr)
    sb += struct.pack("<I", lookup3(sb))
    with open(path, "wb") as f:
        f.write(header + bytes(_JLD2_BASE - len(header)) + sb + bytes(body))
    return eof


def read_jld2(path, names=None):
    """The float64 datasets of the JLD2 file's root group (or those in ``names``) as a dict of arrays in
    Julia's shape and column-major order.  Datasets that are not plain float64 arrays are skipped unless
    named, in which case they raise; a checksum mismatch always raises (ChecksumError)."""
    with open(path, "rb") as f:
        rd = HDF5Reader(f.read())
    links = rd.links()
    out = {}
    for name in (names if names is not None else sorted(links)):
        if name not in links:
            raise KeyError(name)
        try:
            arr, shape = rd.dataset(links[name])
        except ChecksumError:
            raise
        except ValueError:
            if names is not None:
                raise
            continue
        out[name] = arr.reshape(shape, order="F")
    return out


def write_output(sim):
    """write_output (src/OutputParams/output_writing.jl:7-27): the Simulation's outputs, plus the time
    rounded to 3 decimals ("t") and the h-grid coordinates ("x", "y") unless an output of that name
    exists, to ``<output_path><prefix><n_iter, 10 digits>.jld2`` (or ``.mat``).  The "mat" format is
    written by scipy.io.savemat (MAT version 5).  Returns the file name."""
    op, model = sim.output_params, sim.model
    out = {str(k): np.array(v, dtype=np.float64) for k, v in op.outputs.items()}
    out.setdefault("t", np.float64(round(sim.time, 3)))
    out.setdefault("x", np.asarray(model.grid.xxh, np.float64))
    out.setdefault("y", np.asarray(model.grid.yyh, np.float64))
    fname = f"{op.output_path}{op.prefix}{sim.n_iter:010d}"  # (Bool or integer outputs are written as float64)
    if op.output_format == "jld2":
        fname += ".jld2"
        write_jld2(fname, out)
    else:
        from scipy.io import savemat
        fname += ".mat"
        savemat(fname, out)
    print(f"outputting at timestep number {sim.n_iter}")
    return fname


def _read_output(fname):
    """An output file as a dict (get_output_as_dict, zipping_output.jl:58-66)."""
    if fname.endswith(".mat"):
        from scipy.io import loadmat
        return {k: v for k, v in loadmat(fname).items() if not k.startswith("__")}
    return read_jld2(fname)


def make_ncfile(output_format, folder, nc_name, prefix):
    """make_ncfile and make_ncfile_from_filenames (zipping_output.jl:82-158): the files of ``folder`` named
    <prefix>*.<output_format>, in name order (so in time step order), merged into ``nc_name``.  Dimensions
    x and y (the first column of the h-grid x and the first row of its y) and TIME (each file's t), their
    coordinate variables with the reference's attributes, and every output of size nx x ny as a variable
    over (x, y, TIME) in Julia's order, which the file stores slowest first as (TIME, y, x).  Outputs of
    another size are skipped with a warning, as in the reference.  Returns the file name, or None when
    there are no files."""
    import os
    import warnings
    from scipy.io import netcdf_file
    names = sorted(f for f in os.listdir(folder) if f.endswith(output_format) and f.startswith(prefix))
    if not names:
        print("attempted to zip the outputs to nc format, but did not find any files...")
        return None
    files = [os.path.join(folder, f) for f in names]
    first = _read_output(files[0])
    x = np.asarray(first["x"], np.float64)[:, 0]
    y = np.asarray(first["y"], np.float64)[0, :]
    t = np.array([float(np.squeeze(_read_output(f)["t"])) for f in files])
    if os.path.isfile(nc_name):
        os.remove(nc_name)
    with netcdf_file(nc_name, "w", version=2) as ds:
        ds.createDimension("x", x.size)
        ds.createDimension("y", y.size)
        ds.createDimension("TIME", t.size)
        for name, dim, vals, longname, units in (("x", "x", x, "x co-ordinates of ice grid points (h grid)", "m"),
                                                 ("y", "y", y, "y co-ordinates of ice grid points (h grid)", "m"),
                                                 ("TIME", "TIME", t, "Time", "years")):
            v = ds.createVariable(name, "d", (dim,))
            v[:] = vals
            v.longname = longname
            v.units = units
        for key in first:
            if key in ("x", "y", "t"):
                continue
            a = np.asarray(first[key])
            if a.shape != (x.size, y.size):
                warnings.warn(f"found an output variable ({key}) whose spatial dimensions ({a.shape}) do not match "
                              "the co-ordinates. Skipping this variable from the nc output...")
                continue
            dtype = "b" if a.dtype == np.bool_ else a.dtype.char
            v = ds.createVariable(key, dtype, ("TIME", "y", "x"))
            for i, f in enumerate(files):
                d = np.asarray(_read_output(f)[key])
                v[i, :, :] = (d.astype(np.int8) if d.dtype == np.bool_ else d).T
    return nc_name


def zip_output(sim):
    """zip_output (zipping_output.jl:162-169): with zip_format "nc", the run's output files merged into
    <output_path><prefix>.nc."""
    op = sim.output_params
    if op is None or op.zip_format != "nc":
        return None
    return make_ncfile(op.output_format, op.output_path, f"{op.output_path}{op.prefix}.nc", op.prefix)
