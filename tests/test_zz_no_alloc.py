"""ocpx_relres_noalloc (static device scratch, no allocation) against the
context entry point ocpx_calres, on consecutive calls.

The file sorts last so that it also runs after every other GPU test in the
same process; it passes alone as well.  The inputs are copied to device
buffers the test allocates; the call under test allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import fim, synthetic

pytestmark = pytest.mark.gpu

OCPX_OK, OCPX_INVALID_ARG = 0, 5
MAX_CELLS = 2097152  # OCPX_RELRES_NOALLOC_MAX_CELLS


class _Cudart:
    def __init__(self):
        for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        else:
            raise RuntimeError("libcudart not found")
        self.rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.rt.cudaFree.argtypes = [C.c_void_p]
        self.rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.bufs = []

    def to_device(self, a):
        a = np.ascontiguousarray(a, np.float64)
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), max(a.nbytes, 8)) == 0
        assert self.rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0  # host to device
        self.bufs.append(p)
        return p

    def empty(self, n):
        return self.to_device(np.zeros(n))

    def to_host(self, p, n):
        out = np.empty(n)
        assert self.rt.cudaMemcpy(out.ctypes.data, p, out.nbytes, 2) == 0  # device to host
        return out

    def free(self):
        for p in self.bufs:
            self.rt.cudaFree(p)
        self.bufs = []


def _bind(lib):
    f = lib.ocpx_relres_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.POINTER(fim.Norms)]
    f.restype = C.c_int
    return f


def _calres_case(ctx, dt):
    """Residual and norms from the context entry point."""
    n = ctx.cal_res(dt)
    return dict(res=ctx.get("RES"), rockVp=ctx.get("ROCKVP"), Nt=ctx.get("NT"), relV=ctx.get("RES_REL_V"),
                relN=ctx.get("RES_REL_N"), norms=(n.maxRelRes_V, n.maxId_V, n.maxRelRes_N, n.maxId_N))


def _fixture_case(name):
    fx = P.load_fixture(name)
    model, grid = fim.model_and_grid_from_dump(fx)
    it = P.iterations(fx)[0]
    js = P.jac_state(fx, it)
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(js)
        return _calres_case(ctx, float(js["dt"][0])), model.nc


def _synthetic_case(nx, ny, nz, ncomp=6, seed=2):
    """A grid large enough for many reduction blocks (PTN start, pores filled)."""
    model = synthetic.comp_model(ncomp, seed)
    grid = synthetic.comp_grid(nx, ny, nz)
    st = synthetic.comp_initial_state(grid, ncomp, seed)
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(st)
        ctx.update_property()
        scale = ctx.get("ROCKVP") / ctx.get("VF")
        Ni = (st["Ni"].reshape(grid.nb, -1) * scale[:, None]).ravel()
        st.update(Ni=Ni, lNi=Ni * 0.999, Nt=Ni.reshape(grid.nb, -1).sum(axis=1))
        ctx.load_state(st)
        ctx.update_property()
        return _calres_case(ctx, 0.1), model.nc


def _noalloc(f, rt, case, nc):
    nb = case["rockVp"].size
    d_res, d_vp, d_nt = rt.to_device(case["res"]), rt.to_device(case["rockVp"]), rt.to_device(case["Nt"])
    d_v, d_n = rt.empty(nb), rt.empty(nb)
    out = fim.Norms()
    st = f(d_res, d_vp, d_nt, nb, nc + 1, d_v, d_n, None, C.byref(out))
    assert st == OCPX_OK
    return dict(relV=rt.to_host(d_v, nb), relN=rt.to_host(d_n, nb),
                norms=(out.maxRelRes_V, out.maxId_V, out.maxRelRes_N, out.maxId_N))


def _same(got, ref):
    assert got["norms"] == ref["norms"]
    assert np.array_equal(got["relV"], ref["relV"])
    assert np.array_equal(got["relN"], ref["relN"])


def test_noalloc_matches_calres_on_consecutive_calls(gpu_lib):
    f = _bind(gpu_lib)
    rt = _Cudart()
    try:
        cases = [_fixture_case("comp6_8x8x3"), _fixture_case("bo_10x10x3"), _synthetic_case(40, 40, 10)]
        # consecutive calls on different inputs and sizes (one block, one block, eight blocks),
        # then the first input again: every call must leave the scratch ready for the next
        for case, nc in cases + cases[:1]:
            _same(_noalloc(f, rt, case, nc), case)
        # two calls in a row on the same input give the same answer
        big, nc = cases[2]
        a, b = _noalloc(f, rt, big, nc), _noalloc(f, rt, big, nc)
        _same(a, big)
        _same(b, big)
    finally:
        rt.free()


def test_noalloc_rejects_sizes_beyond_scratch(gpu_lib):
    f = _bind(gpu_lib)
    rt = _Cudart()
    try:
        d = rt.empty(4)
        out = fim.Norms()
        assert f(d, d, d, MAX_CELLS + 1, 4, d, d, None, C.byref(out)) == OCPX_INVALID_ARG
        assert f(d, d, d, 0, 4, d, d, None, C.byref(out)) == OCPX_INVALID_ARG
    finally:
        rt.free()
