"""The C ABI without a GPU: the library builds and loads, exports every
symbol the headers declare, validates arguments before touching CUDA, and
its host-side set-up (element matrices, load) matches the reference's."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden, relerr
import topopt_gb300 as tp

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared(path):
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;", src, flags=re.M)
    return [n for n in names if not n.startswith("__")]


@pytest.fixture(scope="module")
def lib():
    return tp.load()


def test_library_loads(lib):
    assert os.path.exists(tp.LIB_PATH)


def test_exports_every_declared_symbol():
    libs = {"topopt_gb300.h": [tp.LIB_PATH]}
    ref = [os.path.join(tp.PKG, "libtopopt_ref%s.so" % f) for f in ("32", "64")]
    libs["topopt_ref_api.h"] = ref
    for h in HEADERS:
        names = declared(h)
        assert names, h
        for so in libs.get(os.path.basename(h), [tp.LIB_PATH]):
            L = ctypes.CDLL(so)
            missing = [n for n in names if not hasattr(L, n)]
            assert not missing, "%s lacks %s" % (os.path.basename(so), missing)


def test_default_params_are_the_references(lib):
    p = tp.TpParams()
    lib.tp_default_params(ctypes.byref(p))
    assert (p.nelx, p.nely, p.nelz, p.nl) == (48, 24, 24, 4)
    assert p.volfrac == float(np.float32(0.2)) and p.rmin == 1.5
    assert p.cgtol == float(np.float32(1e-5)) and p.cgmax == 1000
    assert (p.nswp, p.omega, p.precision, p.nrhs) == (4, 0.6, 0, 1)


@pytest.mark.parametrize("field,value", [("nl", 1), ("nelx", 7), ("nrhs", 0), ("precision", 5), ("rmin", 0.0)])
def test_create_rejects_bad_arguments(lib, field, value):
    p = tp.TpParams()
    lib.tp_default_params(ctypes.byref(p))
    setattr(p, field, value)
    ctx = ctypes.c_void_p()
    assert lib.tp_create(ctypes.byref(p), ctypes.byref(ctx)) == 1  # TP_ERR_ARG, before any CUDA call
    assert not ctx.value


@pytest.mark.parametrize("setter", ["tp_set_fine_variant", "tp_set_fine_arith", "tp_set_coarse_solve_variant",
                                    "tp_set_coarse_arith", "tp_set_coarse_order"])
def test_selectors_reject_bad_arguments(lib, setter):
    """The kernel and arithmetic selectors check their arguments before any
    CUDA call: no context, or a choice other than 0 and 1, is TP_ERR_ARG."""
    f = getattr(lib, setter)
    f.argtypes = [ctypes.c_void_p, ctypes.c_int]
    assert f(None, 0) == 1
    assert f(None, 1) == 1
    assert f(None, 2) == 1


def test_status_strings(lib):
    assert lib.tp_status_string(0) == b"ok"
    assert lib.tp_status_string(4) == b"coarse matrix not positive definite"


@pytest.mark.parametrize("l", [0, 1, 2, 3])
def test_element_matrices_match_reference(lib, l):
    ke = golden("ke.npz")
    out = np.zeros(576 * 8 ** l)
    assert lib.tp_element_matrix_tables(l, 0.3, out.ctypes.data_as(ctypes.c_void_p)) == 0
    if l < 2:
        assert relerr(out, ke["ke_%d" % l]) < 1e-14
    assert relerr(out[ke["ke_%d_idx" % l]], ke["ke_%d_val" % l]) < 1e-13
    assert out.sum() == pytest.approx(float(ke["ke_%d_sum" % l]), rel=1e-12, abs=1e-12)


def test_reference_load(lib):
    g = golden("kernels_16x8x8_l3.npz")
    F = np.zeros(3 * 17 * 9 * 9)
    assert lib.tp_reference_load(16, 8, 8, F.ctypes.data_as(ctypes.c_void_p)) == 0
    assert relerr(F, g["load"]) == 0.0
