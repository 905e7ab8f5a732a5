"""The coarsest-level direct solve on grids whose coarsest level spans many
solve blocks (608 rows on 152 SMs: 4 per SM), one of them with a half
bandwidth wider than a block (the forward sweep then reads the solution of
the two previous blocks).

The single cooperative launch (both triangular sweeps, grid barriers between
the block steps) is checked against the two-launch block solve, against the
oracle's band Cholesky and by applying the coarsest operator to the solution;
repeated solves must agree bit for bit. Its bounded barrier waits are checked
by host-side fault injection: a barrier that waits for one arrival too many
gives up, the call reports TP_ERR_TIMEOUT and the context stays usable."""
import numpy as np
import pytest

from conftest import relerr
import topopt_gb300 as tp

pytestmark = pytest.mark.gpu

# (shape, levels): coarsest 16x8x8 elements (n = 4131, half bandwidth 275,
# 7 blocks of 608) and 16x16x16 elements (n = 14739, half bandwidth 923, 25)
CASES = [((64, 32, 32), 3), ((64, 64, 64), 3)]


def _smooth(shape, seed=0):
    nx, ny, nz = shape
    i, k, j = np.meshgrid(np.arange(nx), np.arange(nz), np.arange(ny), indexing="ij")
    ph = np.random.default_rng(seed).uniform(0, 2 * np.pi, 3)
    x = 0.3 + 0.1 * np.sin(2 * np.pi * i / nx + ph[0]) * np.cos(2 * np.pi * j / ny + ph[1]) \
        + 0.1 * np.sin(2 * np.pi * k / nz + ph[2])
    return x.ravel()


@pytest.fixture(scope="module", params=CASES, ids=["64x32x32_l3", "64x64x64_l3"])
def case(request, cuda):
    shape, nl = request.param
    ctx = tp.TopOpt(*shape, nl)
    x = _smooth(shape)
    ctx.upload("xphys", x)
    ctx.assemble()
    yield ctx, x, cuda
    ctx.close()


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def test_single_launch_against_block_launches(case):
    ctx, x, torch = case
    lc = ctx.nl - 1
    rhs = np.random.default_rng(5).uniform(-1, 1, ctx.ndof(lc))
    b = _dev(torch, rhs)
    ctx.set_coarse_solve_variant(1)
    s1 = ctx.coarse_solve(b).cpu().numpy()
    ctx.set_coarse_solve_variant(0)
    s0 = ctx.coarse_solve(b).cpu().numpy()
    assert np.array_equal(s0, ctx.coarse_solve(b).cpu().numpy())  # fixed summation order
    assert relerr(s0, s1) < 1e-10
    back = ctx.apply(lc, _dev(torch, s0)).cpu().numpy()
    assert relerr(back, rhs) < 1e-8


def test_single_launch_against_oracle(case):
    from oracle import Oracle
    ctx, x, torch = case
    if ctx.shape != (64, 32, 32):
        pytest.skip("the oracle's band Cholesky is timed for the smaller grid only")
    lc = ctx.nl - 1
    rhs = np.random.default_rng(6).uniform(-1, 1, ctx.ndof(lc))
    ctx.set_coarse_solve_variant(0)
    sol = ctx.coarse_solve(_dev(torch, rhs)).cpu().numpy()
    ref, st = Oracle(*ctx.shape, ctx.nl).coarse_direct(lc, x, rhs)
    assert st == 0
    assert relerr(sol, ref) < 1e-9


def test_double_single_factor(case):
    """The factor and the block inverses in double-single arithmetic (the
    mixed form's default; about 48 bits against FP64's 53): the solution
    stays within 1e-8 of the FP64 factor's and solves the system to 1e-8."""
    ctx, x, torch = case
    lc = ctx.nl - 1
    rhs = np.random.default_rng(7).uniform(-1, 1, ctx.ndof(lc))
    b = _dev(torch, rhs)
    ctx.set_coarse_solve_variant(0)
    s64 = ctx.coarse_solve(b).cpu().numpy()
    try:
        ctx.set_coarse_arith(1)
        ctx.assemble()
        sds = ctx.coarse_solve(b).cpu().numpy()
    finally:
        ctx.set_coarse_arith(0)
        ctx.assemble()
    assert 0 < relerr(sds, s64) < 1e-8
    back = ctx.apply(lc, _dev(torch, sds)).cpu().numpy()
    assert relerr(back, rhs) < 1e-8


def test_barrier_wait_gives_up(case):
    ctx, x, torch = case
    if ctx.shape != (64, 32, 32):
        pytest.skip("one grid suffices")
    lc = ctx.nl - 1
    rhs = np.random.default_rng(7).uniform(-1, 1, ctx.ndof(lc))
    b = _dev(torch, rhs)
    ctx.set_coarse_solve_variant(0)
    good = ctx.coarse_solve(b).cpu().numpy()
    ctx.fault_coarse_barrier(20000, 1)  # every barrier waits for an arrival that never comes
    with pytest.raises(tp.TopOptError) as e:
        ctx.coarse_solve(b)
    assert e.value.status == 7 and "barrier" in str(e.value)
    ctx.fault_coarse_barrier(0, 0)
    assert np.array_equal(ctx.coarse_solve(b).cpu().numpy(), good)  # the context is usable


def test_factor_wait_gives_up(case):
    """The single-launch factorisation's waits are bounded: with a budget of one
    poll the first wait for the chain CTA's diagonal tile runs out, every CTA
    leaves, and the assembly reports TP_ERR_TIMEOUT; with the default budget the
    next assembly gives the same factor as before, bit for bit."""
    ctx, x, torch = case
    if ctx.shape != (64, 32, 32):
        pytest.skip("one grid suffices")
    lc = ctx.nl - 1
    b = _dev(torch, np.random.default_rng(8).uniform(-1, 1, ctx.ndof(lc)))
    ctx.set_coarse_solve_variant(0)
    good = ctx.coarse_solve(b).cpu().numpy()
    ctx.fault_coarse_barrier(1, 0)
    with pytest.raises(tp.TopOptError) as e:
        ctx.assemble()
    assert e.value.status == 7 and "wait" in str(e.value)
    ctx.fault_coarse_barrier(0, 0)
    ctx.assemble()
    assert np.array_equal(ctx.coarse_solve(b).cpu().numpy(), good)


@pytest.mark.parametrize("shape", [(64, 32, 32), (60, 32, 32)], ids=["halves_8_8", "halves_7_8"])
def test_dissected_order_against_natural(cuda, shape):
    """The dissected coarse factor (the middle x node plane as the separator;
    17 and 16 node planes, so halves of 8 and 8 and of 7 and 8 planes) against
    the natural band: the solutions agree to rounding but not bit for bit (so
    the dissected path ran), repeated solves agree bit for bit, and the
    solution solves the system; the form with the halves swept one after the
    other gives the same solution to rounding."""
    torch = cuda
    ctx = tp.TopOpt(*shape, 3)
    try:
        ctx.upload("xphys", _smooth(shape))
        lc = ctx.nl - 1
        rhs = np.random.default_rng(9).uniform(-1, 1, ctx.ndof(lc))
        b = _dev(torch, rhs)
        ctx.set_coarse_order(0)
        ctx.assemble()
        s0 = ctx.coarse_solve(b).cpu().numpy()
        ctx.set_coarse_order(1)
        ctx.assemble()
        s1 = ctx.coarse_solve(b).cpu().numpy()
        assert np.array_equal(s1, ctx.coarse_solve(b).cpu().numpy())
        assert 0 < relerr(s1, s0) < 1e-10
        back = ctx.apply(lc, _dev(torch, s1)).cpu().numpy()
        assert relerr(back, rhs) < 1e-8
        # the same factor, the halves' sweeps one after the other (the form
        # taken where a phase of both halves does not fit the shared memory)
        ctx.set_coarse_order(2)
        ctx.assemble()
        s2 = ctx.coarse_solve(b).cpu().numpy()
        assert relerr(s2, s1) < 1e-12
    finally:
        ctx.close()
