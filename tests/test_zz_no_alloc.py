"""tp_filter_T_noalloc: the density-filter adjoint for callers that cannot
allocate device memory, such as applications that keep all of the GPU's
memory in an arena of their own and forbid libraries to call cudaMalloc, or
loops with a fixed time budget. Its result must match the context-based
tp_filter_T on two calls in a row, although the fixed scratch array still holds
the previous call's data, and the reference's own adjoint on the golden
fixture. Collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from conftest import golden, relerr
import topopt_gb300 as tp

pytestmark = pytest.mark.gpu


def test_no_alloc_filter_adjoint_matches_context_path(cuda):
    torch = cuda
    L = tp.load()
    L.tp_filter_T_noalloc.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    L.tp_filter_T_noalloc_max_elements.restype = ctypes.c_long
    rng = np.random.default_rng(42)
    for shape, rmin in (((32, 16, 16), 1.5), ((24, 8, 16), 2.5)):
        ctx = tp.TopOpt(*shape, 2, rmin=rmin)
        for call in range(2):  # two calls in a row share the scratch array
            v = torch.from_numpy(rng.uniform(-1.0, 1.0, ctx.nelem())).cuda()
            expect = ctx.filter_T(v).cpu().numpy()
            got = v.clone()
            st = L.tp_filter_T_noalloc(shape[0], shape[1], shape[2], rmin, ctypes.c_void_p(got.data_ptr()), None)
            assert st == 0
            torch.cuda.synchronize()
            assert relerr(got.cpu().numpy(), expect) < 1e-14, (shape, call)
        ctx.close()
    # against the reference's own filter adjoint (golden fixture, 16x8x8)
    g = golden("kernels_16x8x8_l3.npz")
    for tag, rmin in (("15", 1.5), ("25", 2.5)):
        for call in range(2):
            v = torch.from_numpy(g["x"].copy()).cuda()
            assert L.tp_filter_T_noalloc(16, 8, 8, rmin, ctypes.c_void_p(v.data_ptr()), None) == 0
            torch.cuda.synchronize()
            assert relerr(v.cpu().numpy(), g["filterT_" + tag]) < 1e-14, (tag, call)
    # a radius wider than the grid reaches every element, as the box rule gives
    v0 = rng.uniform(-1.0, 1.0, 4 * 2 * 6)
    ctx = tp.TopOpt(4, 2, 6, 2, rmin=40.0)
    want = ctx.filter_T(torch.from_numpy(v0).cuda()).cpu().numpy()
    ctx.close()
    v = torch.from_numpy(v0.copy()).cuda()
    assert L.tp_filter_T_noalloc(4, 2, 6, 40.0, ctypes.c_void_p(v.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert relerr(v.cpu().numpy(), want) < 1e-14
    # sizes beyond the fixed scratch, and unusable radii, are rejected
    # without touching the data
    big = L.tp_filter_T_noalloc_max_elements() + 1
    v = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert L.tp_filter_T_noalloc(big, 1, 1, 1.5, ctypes.c_void_p(v.data_ptr()), None) == 1
    for bad in (0.0, -1.0, float("inf"), float("nan")):
        assert L.tp_filter_T_noalloc(4, 2, 2, bad, ctypes.c_void_p(v.data_ptr()), None) == 1
