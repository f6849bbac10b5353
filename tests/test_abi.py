"""The C-ABI library builds, loads, exports every symbol include/*.h declares, and its structs match the
ctypes mirror.  No compute call is made (this runs without a GPU)."""
import ctypes as C
import os
import subprocess

import pytest


@pytest.fixture(scope="module")
def lib(pkg):
    from wavi_gb300 import abi, build
    build.build_library()
    return abi.load_library()


def test_exports_every_header_symbol(lib, pkg):
    from wavi_gb300 import abi
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    declared = abi.header_symbols()
    assert declared, "no declarations found"
    missing = [s for s in declared if s not in exported]
    assert not missing, missing


def test_struct_layout_matches_header(lib, pkg):
    from wavi_gb300 import abi
    sizes = (C.c_int32 * 8)()
    n = lib.wavi_abi_struct_sizes(sizes, 8)
    names = ("wavi_grid_desc", "wavi_params", "wavi_solver_params", "wavi_options", "wavi_fields", "wavi_stats")
    mirror = (abi.GridDesc, abi.Params, abi.SolverParams, abi.Options, abi.Fields, abi.Stats)
    assert n == len(names)
    for i, (nm, st) in enumerate(zip(names, mirror)):
        assert sizes[i] == C.sizeof(st), nm


def test_no_device_is_an_error_not_a_crash(lib, pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from wavi_gb300 import abi, synthetic
    g, bed, p, sp, ic = synthetic.small_case()
    desc = g.descriptor()
    ctx = C.c_void_p()
    st = lib.wavi_ctx_create(C.byref(desc.desc), C.byref(sp.to_c()), C.byref(abi.Options(0, 0, 0, 0)), C.byref(ctx))
    assert st in (-7, -2)
    assert lib.wavi_last_error(None)
    assert lib.wavi_ctx_destroy(None) == 0


def test_coarse_solver_names_match_the_header_enum(pkg):
    """abi.COARSE_SOLVERS (the names the Python host and the tests use) against wavi_coarse_solver."""
    import re
    from wavi_gb300 import abi
    here = os.path.dirname(os.path.abspath(__file__))
    text = open(os.path.join(os.path.dirname(here), "include", "wavi_gpu.h")).read()
    body = text[text.index("typedef enum wavi_coarse_solver"):text.index("} wavi_coarse_solver;")]
    enum = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"WAVI_COARSE_(\w+)\s*=\s*(\d+)", body)}
    assert enum == {k: v for k, v in abi.COARSE_SOLVERS.items()}, (enum, abi.COARSE_SOLVERS)


def test_ctx_create_rejects_bad_arguments_before_touching_a_device(lib, pkg):
    """wavi_ctx_create checks its arguments before any CUDA call: each bad argument is WAVI_ERR_ARGUMENT (-1)
    with a message from wavi_last_error(NULL), with or without a GPU."""
    import dataclasses
    from wavi_gb300 import abi, synthetic
    g, bed, p, sp, ic = synthetic.small_case()
    desc = g.descriptor()
    ctx = C.c_void_p()

    def create(d=desc.desc, s=sp, opt=abi.Options(0, 0, 0, 0), out=True):
        return lib.wavi_ctx_create(C.byref(d), C.byref(s.to_c()), C.byref(opt), C.byref(ctx) if out else None)

    assert create(out=False) == -1
    small = abi.GridDesc.from_buffer_copy(desc.desc)
    small.nx = 1
    assert create(d=small) == -1 and b"nx" in lib.wavi_last_error(None)
    assert create(s=dataclasses.replace(sp, levels=5)) == -1 and b"levels" in lib.wavi_last_error(None)
    assert create(opt=abi.Options(0, 7, 0, 0)) == -1 and b"precision" in lib.wavi_last_error(None)
    nomask = abi.GridDesc.from_buffer_copy(desc.desc)
    nomask.h_mask = None
    assert create(d=nomask) == -1
    assert not ctx.value  # no context was made


def test_residual_noalloc_rejects_bad_arguments_before_touching_a_device(lib, pkg):
    """wavi_residual_noalloc checks its arguments before any CUDA call (the pointers are not dereferenced
    before then): null arguments, a grid below 2 x 2, and a grid beyond the static scratch's 16384 tiles
    of 32 x 8 points are WAVI_ERR_ARGUMENT (-1) with a message."""
    from wavi_gb300 import abi
    buf = (C.c_double * 4)()
    p = C.cast(buf, C.c_void_p)
    ok = abi.OperatorDesc(16, 8, 1000.0, 1000.0, p, p, p, p, p, p)
    assert lib.wavi_residual_noalloc(None, p, p, p, p, None) == -1
    assert lib.wavi_residual_noalloc(C.byref(ok), None, p, p, p, None) == -1
    assert b"null" in lib.wavi_last_error(None)
    nocoef = abi.OperatorDesc(16, 8, 1000.0, 1000.0, p, None, p, p, p, p)
    assert lib.wavi_residual_noalloc(C.byref(nocoef), p, p, p, p, None) == -1
    tiny = abi.OperatorDesc(1, 8, 1000.0, 1000.0, p, p, p, p, p, p)
    assert lib.wavi_residual_noalloc(C.byref(tiny), p, p, p, p, None) == -1
    big = abi.OperatorDesc(32 * 129 - 1, 8 * 128, 1000.0, 1000.0, p, p, p, p, p, p)  # 129 x 129 tiles
    assert lib.wavi_residual_noalloc(C.byref(big), p, p, p, p, None) == -1
    assert b"too large" in lib.wavi_last_error(None)


def test_ensemble_create_rejects_bad_arguments_before_touching_a_device(lib, pkg):
    """wavi_ensemble_create: no members, null arrays, host-driven launches (members run as graphs) and a
    member grid that its context rejects are WAVI_ERR_ARGUMENT (-1) before any CUDA call; the message
    names the member."""
    from wavi_gb300 import abi, synthetic
    g, bed, p, sp, ic = synthetic.small_case()
    d = g.descriptor()
    grids = (abi.GridDesc * 2)(d.desc, d.desc)
    sps = (abi.SolverParams * 2)(sp.to_c(), sp.to_c())
    ens = C.c_void_p()
    graphs = abi.Options(0, 0, 1, 0)
    assert lib.wavi_ensemble_create(0, grids, sps, C.byref(graphs), 4, C.byref(ens)) == -1
    assert lib.wavi_ensemble_create(2, None, sps, C.byref(graphs), 4, C.byref(ens)) == -1
    assert lib.wavi_ensemble_create(2, grids, sps, C.byref(abi.Options(0, 0, 0, 0)), 4, C.byref(ens)) == -1
    assert b"graphs" in lib.wavi_last_error(None)
    grids[0].nx = 1
    assert lib.wavi_ensemble_create(2, grids, sps, C.byref(graphs), 4, C.byref(ens)) == -1
    assert b"member 0" in lib.wavi_last_error(None)
    assert not ens.value


def test_every_entry_point_rejects_a_null_context(lib, pkg):
    """Each entry point that takes a context (or an ensemble) returns WAVI_ERR_ARGUMENT (-1) for a null one,
    before touching anything; destroying a null context or ensemble is a no-op."""
    calls = {
        "wavi_solve_velocities": (None, None, None, None),
        "wavi_solve_velocities_device": (None, None, None, None),
        "wavi_relinearise_device": (None, None, None),
        "wavi_apply_operator_device": (None, 0, None, None),
        "wavi_time_operator_device": (None, 0, None, None, 1, None),
        "wavi_time_relinearise_device": (None, 1, None, None),
        "wavi_op_diagonal_device": (None, 0, None),
        "wavi_selftest_watchdog": (None, None),
        "wavi_selftest_conversions": (None, 1, None),
        "wavi_coarse_diagonal_device": (None, 0, None),
        "wavi_adjoint_device": (None, None, None, None, None, None, 1e-10, 10, None),
        "wavi_tangent_device": (None, None, None, None, None, None, 1e-10, 10, None),
        "wavi_run_device": (None, None, 1.0, 1, None, None, None, None),
        "wavi_haar_device": (None, 0, None, None, None),
        "wavi_update_wavelets_device": (None, None, None),
        "wavi_ensemble_solve_device": (None, None, None, None),
    }
    for name, args in calls.items():
        assert getattr(lib, name)(*args) == -1, name
    assert lib.wavi_ctx_destroy(None) == 0 and lib.wavi_ensemble_destroy(None) == 0


def _header_struct_fields(text, name):
    """Field names, in order, of `typedef struct name { ... } name;` in the header (comments dropped)."""
    import re
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "int32_t a, b" / "double x, y" / "const uint8_t* p, *q": the last word of each comma-separated part
        for part in decl.split(","):
            fields.append(re.split(r"[\s*]+", part.strip())[-1])
    return fields


@pytest.mark.parametrize("cname,mirror", [("wavi_options", "Options"), ("wavi_stats", "Stats"),
                                          ("wavi_solver_params", "SolverParams"), ("wavi_params", "Params")])
def test_ctypes_mirror_field_order_matches_header(pkg, cname, mirror):
    """The ctypes structs list the header's fields in the header's order (equal sizes alone would not catch
    two int32 fields swapped, e.g. a new option added in the wrong place)."""
    from wavi_gb300 import abi
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(root, "include", "wavi_gpu.h")) as fh:
        text = fh.read()
    want = _header_struct_fields(text, cname)
    have = [f[0] for f in getattr(abi, mirror)._fields_]
    assert have == want, (cname, have, want)


def _julia_struct_fields(text, name):
    """Field names, in order, of `struct name` / `mutable struct name` ... `end` in the Julia binding."""
    import re
    m = re.search(r"(?:mutable )?struct %s\n(.*?)\nend" % name, text, re.S)
    body = re.sub(r"#.*", "", m.group(1))
    return [f.split("::")[0].strip() for f in re.findall(r"\b\w+::\w+(?:\{[^}]*\})?", body)]


@pytest.mark.parametrize("jname,cname", [("WaviOptions", "wavi_options"), ("WaviStats", "wavi_stats"),
                                         ("WaviSolverParams", "wavi_solver_params"), ("WaviParams", "wavi_params"),
                                         ("WaviGridDesc", "wavi_grid_desc")])
def test_julia_binding_structs_match_header(jname, cname):
    """The Julia binding documented in INTEGRATION.md declares the header's struct fields in the header's
    order (the layout its ccall passes)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(root, "include", "wavi_gpu.h")) as fh:
        header = fh.read()
    with open(os.path.join(root, "INTEGRATION.md")) as fh:
        julia = fh.read()
    assert _julia_struct_fields(julia, jname) == _header_struct_fields(header, cname)
