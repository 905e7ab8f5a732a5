"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference's C), plus known-answer
properties of the operators. CPU only."""
import os

import numpy as np
import pytest

from conftest import CGTOL, VOLFRAC, golden, relerr
from oracle import Oracle, Reference, nnodes


@pytest.fixture(scope="module")
def ke():
    return golden("ke.npz")


@pytest.mark.parametrize("l", [0, 1, 2, 3])
def test_ke_tables(ke, l):
    k = Oracle.ke(l)
    if l < 2:
        assert np.array_equal(k, ke["ke_%d" % l])  # bit-exact restatement
    assert np.array_equal(k[ke["ke_%d_idx" % l]], ke["ke_%d_val" % l])
    assert k.sum() == pytest.approx(float(ke["ke_%d_sum" % l]), rel=1e-14, abs=1e-14)
    assert np.abs(k).sum() == pytest.approx(float(ke["ke_%d_abssum" % l]), rel=1e-14)


KERNEL_CASES = [("kernels_16x8x8_l3.npz", (16, 8, 8), 3), ("kernels_32x16x16_l4.npz", (32, 16, 16), 4)]


@pytest.fixture(scope="module", params=KERNEL_CASES, ids=["16x8x8_l3", "32x16x16_l4"])
def case(request):
    name, shape, nl = request.param
    return golden(name), Oracle(*shape, nl)


def test_fixed_dofs_and_load(case):
    g, o = case
    for l in range(o.nl):
        assert np.array_equal(o.fixed_dofs(l), g["fixed_%d" % l])
    assert relerr(o.load(), g["load"]) == 0.0


def test_operators(case):
    g, o = case
    x = g["x"]
    for l in range(o.nl):
        assert relerr(o.apply(l, x, g["u_%d" % l]), g["apply_%d" % l]) < 1e-13
        if l >= 2:
            assert relerr(o.apply(l, x, g["u_%d" % l], masked=True), g["apply_csr_%d" % l]) < 1e-13
        assert relerr(o.inv_diag(l, x), g["invdiag_%d" % l]) < 1e-13


def test_transfers_and_smoother(case):
    g, o = case
    for l in range(o.nl - 1):
        assert relerr(o.restrict(l, g["u_%d" % l]), g["restrict_%d" % l]) == 0.0
        assert relerr(o.prolong(l, g["uc_%d" % l]), g["prolong_%d" % l]) == 0.0
        if "smooth_%d" % l in g:
            assert relerr(o.smooth(l, g["x"], 4, 0.6, g["b_%d" % l], g["u_%d" % l]), g["smooth_%d" % l]) < 1e-13


def test_compliance_filter_oc(case):
    g, o = case
    c, dc = o.compliance(g["x"], g["u_c"])
    assert c == pytest.approx(float(g["c"]), rel=1e-13)
    assert relerr(dc, g["dc"]) < 1e-13
    for tag, rmin in (("15", 1.5), ("25", 2.5)):
        assert relerr(o.filter(rmin, g["x"]), g["filter_" + tag]) == 0.0
        assert relerr(o.filter_T(rmin, g["x"]), g["filterT_" + tag]) == 0.0
    xn = o.oc_update(g["oc_x"], g["oc_dv"], g["oc_dc"], float(g["oc_g"]))
    assert relerr(xn, g["oc_xnew"]) < 1e-12


def test_state_solve(case):
    g, o = case
    u, it, rr, st = o.solve(g["solve_x"], g["load"], None, 4, CGTOL)
    assert st == 0
    assert it == int(g["solve_iters"])
    assert relerr(u, g["solve_u"]) < 1e-9


@pytest.mark.parametrize("name,shape,nl", [("history_48x24x24_l3.npz", (48, 24, 24), 3),
                                           ("history_32x16x16_l4.npz", (32, 16, 16), 4)])
def test_design_history(name, shape, nl):
    g = golden(name)
    loops, h, xp, _ = Oracle.run(*shape, VOLFRAC, 1.5, nl, CGTOL, 20, want_fields=True)
    assert loops == int(g["loops"])
    np.testing.assert_array_equal(h["cgiters"], g["cgiters"])
    assert np.max(np.abs(h["c"] - g["c"]) / g["c"]) < 1e-10
    assert np.max(np.abs(h["vol"] - g["vol"])) < 1e-10
    assert np.max(np.abs(xp - g["xphys"])) < 1e-7


# ---- known answers of the operators (independent of the fixtures) ----

@pytest.fixture(scope="module")
def small():
    return Oracle(8, 4, 4, 3)


def test_operator_symmetry_on_free_dofs(small):
    o = small
    rng = np.random.default_rng(5)
    x = rng.uniform(0.01, 1, o.nelem())
    free = np.ones(o.ndof(0), bool)
    free[o.fixed_dofs(0)] = False
    a = rng.uniform(-1, 1, o.ndof(0)) * free
    b = rng.uniform(-1, 1, o.ndof(0)) * free
    lhs = a @ o.apply(0, x, b)
    rhs = b @ o.apply(0, x, a)
    assert lhs == pytest.approx(rhs, rel=1e-13)


def test_rigid_translation_in_kernel(small):
    o = small
    x = np.full(o.nelem(), 0.7)
    for d in range(3):
        u = np.zeros(o.ndof(0))
        u[d::3] = 1.0
        y = o.apply(0, x, u)
        free = np.ones(o.ndof(0), bool)
        free[o.fixed_dofs(0)] = False
        assert np.max(np.abs(y[free])) < 1e-13


def test_restriction_is_prolongation_transpose(small):
    o = small
    rng = np.random.default_rng(6)
    for l in range(o.nl - 1):
        a = rng.uniform(-1, 1, o.ndof(l))
        b = rng.uniform(-1, 1, o.ndof(l + 1))
        assert o.restrict(l, a) @ b == pytest.approx(a @ o.prolong(l, b), rel=1e-13)


def test_filter_rows_sum_to_one_and_adjoint(small):
    o = small
    rng = np.random.default_rng(7)
    for rmin in (1.5, 2.5):
        assert np.allclose(o.filter(rmin, np.ones(o.nelem())), 1.0, rtol=0, atol=1e-14)
        a = rng.uniform(0, 1, o.nelem())
        b = rng.uniform(0, 1, o.nelem())
        assert o.filter(rmin, a) @ b == pytest.approx(a @ o.filter_T(rmin, b), rel=1e-13)


def test_sensitivity_finite_difference(small):
    """dc/dxPhys by central differences of c(x) = u^T K(x) u at fixed u."""
    o = small
    rng = np.random.default_rng(8)
    x = rng.uniform(0.1, 1, o.nelem())
    u = rng.uniform(-1, 1, o.ndof(0))
    _, dc = o.compliance(x, u)
    h = 1e-6
    for e in rng.choice(o.nelem(), 8, replace=False):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        fd = (o.compliance(xp, u)[0] - o.compliance(xm, u)[0]) / (2 * h)
        # c = sum E u^T KE u, dc reported as -dE/dx u^T KE u
        assert -dc[e] == pytest.approx(fd, rel=1e-6)


# ---- the oracle against the compiled reference, where it was built here ----

REF64 = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "libref64.so")


@pytest.mark.skipif(not os.path.exists(REF64), reason="reference not built in this checkout")
def test_oracle_matches_reference_build():
    shape, nl = (16, 8, 8), 3
    o, r = Oracle(*shape, nl), Reference(*shape, nl)
    rng = np.random.default_rng(11)
    x = rng.uniform(0.01, 1, o.nelem())
    for l in range(nl):
        u = rng.uniform(-1, 1, o.ndof(l))
        assert relerr(o.apply(l, x, u), r.apply(l, x, u)) < 1e-13
    # a mildly graded design; rough random fields stall the reference's CG
    i = np.arange(o.nelem())
    xs = 0.2 + 0.05 * np.sin(i * 0.37)
    F = r.load()
    uo, io, _, _ = o.solve(xs, F)
    ur, ir, _ = r.solve(xs, F)
    assert io == ir and relerr(uo, ur) < 1e-9
    assert nnodes(*shape, 0) * 3 == o.ndof(0)
