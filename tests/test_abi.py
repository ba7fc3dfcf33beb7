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
