"""Failure detection made on the host, with no GPU fault: a coarse matrix
that is not positive definite, a NaN in the load or the design, and an
allocation that fails during set-up. The reference checks none of these
(stencil_assembly.c:435,476 ignore CHOLMOD's status; stencil_solvers.c:334
runs its CG loop to the cap whatever the residual); here each returns its
status code, and the context keeps working once the input is good again."""
import numpy as np
import pytest

from conftest import relerr
import topopt_gb300 as tp

pytestmark = pytest.mark.gpu

SHAPE, NL = (32, 16, 16), 3  # coarsest level 8x4x4 elements, 675 DOFs


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def _smooth(shape):
    nx, ny, nz = shape
    i, k, j = np.meshgrid(np.arange(nx), np.arange(nz), np.arange(ny), indexing="ij")
    return (0.3 + 0.1 * np.sin(2 * np.pi * i / nx) * np.cos(2 * np.pi * j / ny)).ravel()


def _coarse_csr(ctx, torch):
    """The coarsest operator (fixed rows and columns replaced by the identity)
    as a dense-then-CSR host matrix, column by column through tp_apply."""
    lc = ctx.nl - 1
    n = ctx.ndof(lc)
    K = np.zeros((n, n))
    e = torch.zeros(n, dtype=torch.float64, device="cuda")
    for j in range(n):
        e.zero_()
        e[j] = 1.0
        K[:, j] = ctx.apply(lc, e).cpu().numpy()
    rows, cols = np.nonzero(K)
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, rows + 1, 1)
    return np.cumsum(rowptr).astype(np.int32), cols.astype(np.int32), K[rows, cols].copy(), K


def test_non_spd_coarse_csr_reports_not_spd_and_recovers(cuda):
    torch = cuda
    ctx = tp.TopOpt(*SHAPE, NL)
    ctx.upload("xphys", _smooth(SHAPE))
    ctx.assemble()
    rowptr, col, val, K = _coarse_csr(ctx, torch)
    lc = ctx.nl - 1
    b = _dev(torch, np.random.default_rng(3).uniform(-1, 1, ctx.ndof(lc)))
    assert ctx.coarse_factor_csr(rowptr, col, val) == 0
    good = ctx.coarse_solve_factored(b).cpu().numpy()
    assert relerr(K @ good, b.cpu().numpy()) < 1e-10
    # a negative diagonal entry half-way down the matrix: the factor meets a
    # non-positive pivot there (the single-launch factor still runs to its end)
    r = ctx.ndof(lc) // 2
    bad = val.copy()
    q = np.nonzero(col[rowptr[r]:rowptr[r + 1]] == r)[0][0] + rowptr[r]
    bad[q] = -abs(bad[q]) - 1.0
    assert ctx.coarse_factor_csr(rowptr, col, bad) == 4
    assert "pivot" in ctx.L.tp_error_message(ctx.ctx).decode()
    # the next good factorisation gives the same solution, bit for bit
    assert ctx.coarse_factor_csr(rowptr, col, val) == 0
    assert np.array_equal(ctx.coarse_solve_factored(b).cpu().numpy(), good)
    ctx.close()


def test_indefinite_design_is_reported_until_replaced(cuda):
    """Negative densities give negative moduli E(x) = Emin + x^3 (E0 - Emin),
    so the coarsest operator is not positive definite: every call that
    assembles reports TP_ERR_NOT_SPD (none solves with the failed factor), and
    uploading a good design restores the earlier results exactly."""
    torch = cuda
    ctx = tp.TopOpt(*SHAPE, NL)
    x = _smooth(SHAPE)
    lc = ctx.nl - 1
    b = _dev(torch, np.random.default_rng(4).uniform(-1, 1, ctx.ndof(lc)))
    ctx.upload("xphys", x)
    good = ctx.coarse_solve(b).cpu().numpy()
    ctx.upload("xphys", -np.ones_like(x))
    for call in (ctx.assemble, lambda: ctx.coarse_solve(b), lambda: ctx.vcycle(_dev(torch, np.ones(ctx.ndof(0))))):
        with pytest.raises(tp.TopOptError) as e:
            call()
        assert e.value.status == 4
    ctx.upload("xphys", x)
    assert np.array_equal(ctx.coarse_solve(b).cpu().numpy(), good)
    ctx.close()


@pytest.mark.parametrize("device_loop", [0, 1])
def test_nan_in_load_reports_nonfinite(cuda, device_loop):
    """A NaN in the host load vector, uploaded as it is: the solve (host-driven
    or graph-launched) and the design iteration return TP_ERR_NONFINITE after
    one CG iteration instead of running to the cap; with the load restored the
    run gives the same compliance as a fresh context."""
    ctx = tp.TopOpt(*SHAPE, NL)
    ctx.set_device_loop(device_loop)
    F = ctx.download("F")
    bad = F.copy()
    bad[np.argmax(np.abs(F))] = np.nan
    ctx.upload("F", bad)
    for graph in (0, 1):
        ctx.set_graph_solve(2 if graph == 0 else 1)
        with pytest.raises(tp.TopOptError) as e:
            ctx.solve()
        assert e.value.status == 6
    ctx.set_graph_solve(0)
    with pytest.raises(tp.TopOptError) as e:
        ctx.design_iteration()
    assert e.value.status == 6
    ctx.upload("F", F)
    ctx.init_design()
    c1 = ctx.design_iteration().c
    ref = tp.TopOpt(*SHAPE, NL)
    ref.set_device_loop(device_loop)
    assert ref.design_iteration().c == c1
    ref.close()
    ctx.close()


def test_nan_in_design_is_reported(cuda):
    ctx = tp.TopOpt(*SHAPE, NL)
    x = np.full(ctx.nelem(), 0.2)
    x[ctx.nelem() // 3] = np.nan
    ctx.upload("xphys", x)
    with pytest.raises(tp.TopOptError) as e:
        ctx.design_iteration()
    assert e.value.status in (4, 6)  # a NaN pivot, or a NaN residual
    ctx.close()


def test_failed_allocation_reports_alloc_and_leaks_nothing(cuda):
    torch = cuda
    base = tp.fault_alloc(0)
    ctx = tp.TopOpt(*SHAPE, NL)
    total = tp.fault_alloc(0) - base  # allocations one context makes
    ctx.close()
    assert total > 10 and tp.fault_alloc(0) == base
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    ks = sorted(set(list(range(1, total + 1, max(1, total // 16))) + [total]))
    for k in ks:
        tp.fault_alloc(k)
        with pytest.raises(tp.TopOptError) as e:
            tp.TopOpt(*SHAPE, NL)
        assert e.value.status == 3, k
        assert tp.fault_alloc(0) == base, k  # the failed context freed what it held
    tp.fault_alloc(total + 1)  # one past the last allocation: set-up succeeds
    ok = tp.TopOpt(*SHAPE, NL)
    tp.fault_alloc(0)
    ok.close()
    assert tp.fault_alloc(0) == base
    torch.cuda.synchronize()
    assert abs(torch.cuda.mem_get_info()[0] - free0) < (8 << 20)
