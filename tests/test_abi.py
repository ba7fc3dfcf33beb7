"""The C ABI library without a GPU: it builds for sm_103a, loads, exports
every function include/ocpx.h declares, and refuses to run compute without a
device instead of falling back to anything."""
import ctypes as C
import os
import re

import pytest

import parity as P
from opencaeporox_gb300 import build, fim

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ocpx.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    text = re.sub(r"#[^\n]*", " ", text)
    names = re.findall(r"\b(ocpx_[A-Za-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    return C.CDLL(build.build())


def test_header_declares_the_abi():
    names = declared_functions()
    assert "ocpx_create" in names and "ocpx_step" in names and len(names) >= 25


def test_library_exports_every_declared_function(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_binds_only_declared_functions():
    assert set(fim.EXPORTS) <= set(declared_functions())


def test_no_device_is_an_error_not_a_fallback(lib):
    from conftest import _cuda_available
    lib.ocpx_abi_version.restype = C.c_int
    assert lib.ocpx_abi_version() >= 1
    if _cuda_available():
        pytest.skip("a device is present")
    fx = P.load_fixture("bo_10x10x3")
    model, grid = fim.model_and_grid_from_dump(fx)
    with pytest.raises(fim.OcpxError, match="NO_DEVICE"):
        fim.FimContext(model, grid)


def test_python_parameter_names_match_the_header():
    """fim.PARAMS names and numbers every ocpx_param of the header, and no other."""
    text = open(HEADER).read()
    enum = re.search(r"typedef enum ocpx_param \{(.*?)\}", text, flags=re.S).group(1)
    declared = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"OCPX_PARAM_([A-Z0-9_]+)\s*=\s*(\d+)", enum)}
    assert declared == fim.PARAMS


STRUCTS = {"ocpx_well": "Well", "ocpx_table": "Table", "ocpx_model_desc": "ModelDesc", "ocpx_grid_desc": "GridDesc",
           "ocpx_report": "Report", "ocpx_norms": "Norms", "ocpx_change_max": "ChangeMax",
           "ocpx_solve_report": "SolveReport", "ocpx_nr_control": "NRControl"}


def test_python_structs_match_the_header(tmp_path):
    """Every struct the Python mirror passes through the ABI has the size and
    alignment the C compiler gives the header's struct, and each field sits
    at the C offset of the field of the same name."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    for cname, pname in STRUCTS.items():
        lines.append(f'printf("{cname} size %zu align %zu\\n", sizeof({cname}), _Alignof({cname}));')
        for fname, _ in getattr(fim, pname)._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    got = {}
    for line in out:
        parts = line.split()
        if parts[1] == "size":
            got[(parts[0], "size")] = int(parts[2])
            got[(parts[0], "align")] = int(parts[4])
        else:
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, pname in STRUCTS.items():
        st = getattr(fim, pname)
        assert C.sizeof(st) == got[(cname, "size")], cname
        assert C.alignment(st) == got[(cname, "align")], cname
        for fname, _ in st._fields_:
            assert getattr(st, fname).offset == got[(cname, fname)], (cname, fname)


def test_create_options_are_checked_before_the_device():
    """ocpx_create_ex checks its options with the descriptions, before it
    looks for a device: a wrong struct_size and the recompute option on a
    black-oil model are refused (OCPX_INVALID_ARG); a compositional model
    with the option passes the checks (OCPX_NO_DEVICE here)."""
    from conftest import _cuda_available
    if _cuda_available():
        pytest.skip("a device is present")
    bo = P.load_fixture("bo_10x10x3")
    model, grid = fim.model_and_grid_from_dump(bo)
    with pytest.raises(fim.OcpxError, match="INVALID_ARG.*compositional"):
        fim.FimContext(model, grid, recompute=True)
    comp = P.load_fixture("comp6_8x8x3")
    m2, g2 = fim.model_and_grid_from_dump(comp)
    with pytest.raises(fim.OcpxError, match="NO_DEVICE"):
        fim.FimContext(m2, g2, recompute=True)
    lib = fim.load_library()
    md, keep1 = m2.desc()
    gd, keep2 = g2.desc()
    opt = fim.Options(C.sizeof(fim.Options) - 4, 1)
    h = C.c_void_p()
    st = lib.ocpx_create_ex(C.byref(md), C.byref(gd), -1, C.byref(opt), C.byref(h))
    assert fim.STATUS_NAMES[st] == "INVALID_ARG"
    assert b"struct_size" in lib.ocpx_last_error()


def test_solve_entry_points_refuse_a_null_context(lib):
    """The enqueue-only solve and its report check their arguments before
    any device work."""
    lib.ocpx_linsolve_async.argtypes = [C.c_void_p, C.c_double, C.c_int]
    lib.ocpx_linsolve_report.argtypes = [C.c_void_p, C.POINTER(fim.SolveReport)]
    lib.ocpx_last_error.restype = C.c_char_p
    rep = fim.SolveReport()
    assert lib.ocpx_linsolve_async(None, 1e-10, 10) != 0
    assert b"null context" in lib.ocpx_last_error()
    assert lib.ocpx_linsolve_report(None, C.byref(rep)) != 0
    assert b"null argument" in lib.ocpx_last_error()
