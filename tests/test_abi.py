"""The C ABI: the library builds, loads, exports every symbol of include/sph_gb300.h,
and the ctypes mirrors match the C struct layout (checked by compiling the header
with gcc). No compute calls: these run without a GPU."""

import ctypes
import os
import re
import subprocess

import pytest

from jaxsph_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sph_gb300.h")


def header_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(sph_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return ctypes.CDLL(_build.LIB_PATH)


def test_every_declared_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_lib.EXPORTS)


def test_abi_version_and_error_string(lib):
    lib.sph_abi_version.restype = ctypes.c_int
    assert lib.sph_abi_version() == 7
    lib.sph_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.sph_last_error(), bytes)


def test_status_bits_match_the_header():
    src = open(HEADER).read()
    bits = dict(re.findall(r"^#define SPH_(\w+) (0x[0-9a-f]+)u", src, re.M))
    assert len(bits) >= 11 and "ERR_HOST" in bits
    for name, value in bits.items():
        assert getattr(_lib, name) == int(value, 16), name
    assert len(set(bits.values())) == len(bits)  # every bit distinct


def test_enum_values_match_the_header():
    src = open(HEADER).read()
    enums = dict(re.findall(r"SPH_(\w+) = (\d+)", src))
    assert len(enums) >= 20
    for name, value in enums.items():
        group, _, member = name.partition("_")
        if group in ("KERNEL", "SOLVER"):
            mirror = getattr(_lib, group + "S")[member]
        else:
            mirror = getattr(_lib, name)
        assert mirror == int(value), name


def test_create_rejects_bad_arguments_without_touching_the_gpu(lib):
    lib.sph_create.restype = ctypes.c_int
    cfg = _lib.SphConfig(dim=4)
    case = _lib.SphCase(n=10)
    h = ctypes.c_void_p()
    rc = lib.sph_create(ctypes.byref(cfg), ctypes.byref(case), 1, ctypes.byref(h))
    assert rc & _lib.ERR_INVALID_ARG and not h.value
    lib.sph_last_error.restype = ctypes.c_char_p
    assert b"dimension" in lib.sph_last_error()


def test_struct_layout_matches_c(tmp_path):
    prog = tmp_path / "layout.c"
    fields = {
        "SphConfig": [f[0] for f in _lib.SphConfig._fields_],
        "SphCase": [f[0] for f in _lib.SphCase._fields_],
        "SphStateView": [f[0] for f in _lib.SphStateView._fields_],
        "SphNLCapacity": [f[0] for f in _lib.SphNLCapacity._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sph_gb300.h"',
             "int main(void) {"]
    for s, fs in fields.items():
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f in fs:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0; }")
    prog.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    c = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    for s, fs in fields.items():
        cls = getattr(_lib, s)
        assert int(c[s]) == ctypes.sizeof(cls), s
        for f in fs:
            assert int(c[f"{s}.{f}"]) == getattr(cls, f).offset, f"{s}.{f}"


@pytest.mark.skipif(__import__("torch").cuda.is_available(),
                    reason="argument checks only: run where no kernel can launch")
@pytest.mark.parametrize("dim,n,box,cutoff,capacity,word", [
    (4, 100, 1.0, 0.1, 1000, b"dimension"),
    (2, 0, 1.0, 0.1, 1000, b"particle count"),
    (2, 65537, 1.0, 0.1, 1000, b"particle count"),
    (2, 100, 1.0, 0.1, -1, b"capacity"),
    (3, 100, 1.0, 0.005, 1000, b"cell"),
])
def test_noalloc_rejects_bad_arguments_before_any_gpu_work(lib, dim, n, box, cutoff, capacity,
                                                            word):
    fn = lib.sph_nl_edges_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                   ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                   ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    boxes = (ctypes.c_double * 3)(box, box, box)
    # host placeholders: the checks reject the call before anything is read
    dummy = ctypes.create_string_buffer(64)
    addr = ctypes.addressof(dummy)
    rc = fn(dim, boxes, cutoff, 0, addr, n, addr, capacity, addr, None, None)
    assert rc == _lib.ERR_INVALID_ARG
    lib.sph_last_error.restype = ctypes.c_char_p
    assert word in lib.sph_last_error()


def _valid_case():
    c = _lib.SphCase(n=100, r_cutoff=0.15, dx=0.05, h=0.05, dt=1e-4, dt_solver=1e-4,
                     c_ref=10.0, eos=_lib.EOS_TAIT, p_ref=100.0, rho_ref=1.0, gamma=1.0,
                     u_ref=1.0, eta_limiter=3.0)
    c.box[0] = c.box[1] = c.box[2] = 1.0
    return c


@pytest.mark.parametrize("field,value,word", [
    ("kernel", 5, b"kernel"),
    ("solver", 7, b"solver"),
    ("nl_backend", 3, b"nl_backend"),
    ("verlet_skin", 0.7, b"verlet_skin"),
    ("case.n", 0, b"at least one particle"),
    ("case.r_cutoff", 0.0, b"r_cutoff"),
    ("case.box", -1.0, b"box"),
    ("case.bc_kind", 9, b"bc_kind"),
    ("case.g_kind", 9, b"g_kind"),
])
def test_create_validates_config_and_cases_before_allocating(lib, field, value, word):
    """Every rejected configuration returns SPH_ERR_INVALID_ARG with a message
    and no handle, before the first device allocation."""
    lib.sph_create.restype = ctypes.c_int
    lib.sph_last_error.restype = ctypes.c_char_p
    cfg = _lib.SphConfig(dim=2, kernel=0, solver=0, capacity_multiplier=1.25, verlet_skin=0.1)
    case = _valid_case()
    if field.startswith("case."):
        name = field[5:]
        if name == "box":
            case.box[0] = value
        else:
            setattr(case, name, value)
    else:
        setattr(cfg, field, value)
    h = ctypes.c_void_p()
    rc = lib.sph_create(ctypes.byref(cfg), ctypes.byref(case), 1, ctypes.byref(h))
    assert rc == _lib.ERR_INVALID_ARG and not h.value
    assert word in lib.sph_last_error()


def test_handle_entry_points_reject_a_null_handle(lib):
    lib.sph_last_error.restype = ctypes.c_char_p
    assert lib.sph_step(None, 1, None) == _lib.ERR_INVALID_ARG
    assert lib.sph_forward(None, None) == _lib.ERR_INVALID_ARG
    assert lib.sph_nl_update(None, None) == _lib.ERR_INVALID_ARG
    fmt = ctypes.c_int32(-1)
    assert lib.sph_list_format(None, ctypes.byref(fmt)) == _lib.ERR_INVALID_ARG
    assert fmt.value == -1
    assert lib.sph_snapshot_init(None, 1) == _lib.ERR_INVALID_ARG
    assert lib.sph_snapshot_save(None, 0, None) == _lib.ERR_INVALID_ARG
    assert lib.sph_snapshot_restore(None, 0, None) == _lib.ERR_INVALID_ARG
    assert lib.sph_set_force_variant(None, _lib.FORCE_STAGED) == _lib.ERR_INVALID_ARG
    assert b"null" in lib.sph_last_error() or b"slot" in lib.sph_last_error()
    cfg = _lib.SphConfig(dim=2)
    h = ctypes.c_void_p()
    assert lib.sph_create(ctypes.byref(cfg), None, 0, ctypes.byref(h)) == _lib.ERR_INVALID_ARG
