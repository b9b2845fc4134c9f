"""C-ABI library: loads, exports every symbol the public header declares,
and validates arguments with the reference's error messages before touching
the GPU.  CPU only (no compute calls)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(sc_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("sc_mesh_create", "sc_deposit", "sc_solve", "sc_interpolate_field", "sc_kick"):
        assert n in names


def test_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_python_binding_covers_header(lib):
    import spacecharge_gb300._lib as L

    assert set(declared_symbols()) <= set(L.SIGNATURES), set(declared_symbols()) - set(L.SIGNATURES)


def test_julia_binding_calls_declared_symbols():
    """Every ccall in the Julia package names an entry point of the header,
    and its deposit-mode table matches the header's SC_DEPOSIT_* values."""
    src = open(os.path.join(ROOT, "spacecharge.jl_gb300", "julia", "SpaceChargeGB300", "src",
                            "SpaceChargeGB300.jl")).read()
    called = set(re.findall(r"ccall\(\(:(sc_\w+),", src))
    assert called and called <= set(declared_symbols()), called - set(declared_symbols())
    hdr = open(os.path.join(ROOT, "include", "spacecharge_gb300.h")).read()
    modes = {k.lower(): int(v) for k, v in re.findall(r"#define SC_DEPOSIT_(\w+)\s+(\d+)", hdr)}
    jl = {k: int(v) for k, v in re.findall(r":(\w+) => Cint\((\d+)\)", src)}
    assert jl == modes


def test_python_constants_match_header():
    """Every integer constant the Python binding defines has the header's
    value (status codes, precisions, dtypes, deposit modes, FFT engines,
    FP64 arithmetic modes)."""
    hdr = open(os.path.join(ROOT, "include", "spacecharge_gb300.h")).read()
    defs = {k: int(v) for k, v in re.findall(r"#define (SC_[A-Z0-9_]+)\s+(-?\d+)\b", hdr)}
    src = open(os.path.join(ROOT, "spacecharge.jl_gb300", "python", "spacecharge_gb300", "_lib.py")).read()
    py = {k: int(v) for k, v in re.findall(r"^(SC_[A-Z0-9_]+) = (-?\d+)\s*$", src, re.M)}
    assert py and all(k in defs for k in py), set(py) - set(defs)
    assert {k: defs[k] for k in py} == py
    # the Julia wrapper's FP64 arithmetic modes
    jl = open(os.path.join(ROOT, "spacecharge.jl_gb300", "julia", "SpaceChargeGB300", "src",
                           "SpaceChargeGB300.jl")).read()
    m = re.search(r"mode === :fp64 \? Cint\((\d+)\) : mode === :df32 \? Cint\((\d+)\)", jl)
    assert m and (int(m.group(1)), int(m.group(2))) == (defs["SC_FP64_ARITH_FP64"], defs["SC_FP64_ARITH_DF32"])


def test_version(lib):
    assert lib.sc_version() >= 10000


def _grid(*g):
    return (C.c_int32 * 3)(*g)


def _d3(*v):
    return (C.c_double * 3)(*v)


@pytest.mark.parametrize("g", [(0, 2, 2), (2, 0, 2), (2, 2, 0), (1, 2, 2), (2, 1, 2), (2, 2, 1)])
def test_grid_validation(lib, g):  # test/test_mesh.jl:78-83
    out = C.c_void_p()
    st = lib.sc_mesh_create(_grid(*g), _d3(0, 0, 0), _d3(1, 1, 1), 1.0, 0.0, 2, C.byref(out))
    assert st == 1
    assert lib.sc_last_error() == b"All elements of grid_size must be at least 2."


@pytest.mark.parametrize("lo,hi", [((0, 0, 0), (0, 0, 0)), ((1, 1, 1), (0, 0, 0))])
def test_bounds_validation(lib, lo, hi):  # test_mesh.jl:92-93
    out = C.c_void_p()
    st = lib.sc_mesh_create(_grid(2, 2, 2), _d3(*lo), _d3(*hi), 1.0, 0.0, 2, C.byref(out))
    assert st == 1
    assert lib.sc_last_error() == b"max_bounds must be strictly greater than min_bounds for all dimensions."


def test_auto_bounds_validation(lib):  # test_mesh.jl:86
    st = lib.sc_auto_bounds(_grid(2, 2, 2), None, None, None, 0, 1, None, None, None, None)
    assert st == 1 and lib.sc_last_error() == b"Particle arrays cannot be empty."
    st = lib.sc_auto_bounds(_grid(2, 1, 2), None, None, None, 0, 1, None, None, None, None)
    assert st == 1 and lib.sc_last_error() == b"All elements of grid_size must be at least 2."


def test_python_host_validation(sc):
    """The Python host raises SpaceChargeError (the ErrorException analogue)
    with the reference's messages, before any device work."""
    with pytest.raises(sc.SpaceChargeError, match="at least 2"):
        sc.Mesh3D((1, 2, 2), [0.0], [0.0], [0.0])
    with pytest.raises(sc.SpaceChargeError, match="cannot be empty"):
        sc.Mesh3D((2, 2, 2), [], [], [])
    with pytest.raises(sc.SpaceChargeError, match="same length"):
        sc.Mesh3D((4, 4, 4), [0.0, 1.0], [0.0], [0.0])
    with pytest.raises(sc.SpaceChargeError, match="strictly greater"):
        sc.Mesh3D((2, 2, 2), (1, 1, 1), (0, 0, 0))
    with pytest.raises(sc.SpaceChargeError, match="unknown precision"):
        sc.Mesh3D((2, 2, 2), (0, 0, 0), (1, 1, 1), precision="bf16")


def test_null_mesh(lib):
    assert lib.sc_solve(None, 0, None) == 1
    assert lib.sc_deposit(None, None, None, None, None, 0, 1, 1, 0, None) == 1
    assert lib.sc_mesh_set_bounds(None, _d3(0, 0, 0), _d3(1, 1, 1)) == 1
    assert lib.sc_last_error() == b"mesh is NULL"
    assert lib.sc_mesh_refit(None, None, None, None, 1, 1, None) == 1
