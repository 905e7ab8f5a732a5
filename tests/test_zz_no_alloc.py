"""tp_filter_T_noalloc: the density-filter adjoint for callers that cannot
allocate device memory (code being captured into a CUDA graph, or an
application whose device memory belongs to another allocator). Its result must
match the context-based tp_filter_T on consecutive calls, although the fixed
scratch array still holds the previous call's data. Collected last so that a
run stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from conftest import relerr
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
    # sizes beyond the fixed scratch are rejected without touching the data
    big = L.tp_filter_T_noalloc_max_elements() + 1
    v = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert L.tp_filter_T_noalloc(big, 1, 1, 1.5, ctypes.c_void_p(v.data_ptr()), None) == 1
