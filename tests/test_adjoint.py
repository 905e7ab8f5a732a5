"""Adjoint sensitivities through the C ABI, wrapped in a torch.autograd.Function
(test harness only): compliance c(x) = F^T U with K(xPhys) U = F and
xPhys = H x / Hs, and the volume V(x) = sum(xPhys) / n, on 64x32x32 elements
(-l 4) with i.i.d. U[0.01, 1] design variables (seed 0), density filters with
rmin 1.5 and 2.5.

Checks: the gradients against the reference's own sensitivities (golden
fixture from its C: dc/dxPhys, dc/dx = H^T(dc/Hs), dv = H^T(1/Hs)), and
against central finite differences with h = 1e-6 on 64 seeded elements.
Compliance is self-adjoint, so its adjoint solve is the state solve; the
general form (tp_element_sensitivity with an adjoint field from
tp_solve_rhs) is checked on a non-self-adjoint objective c2 = L^T U."""
import numpy as np
import pytest

from conftest import golden
import topopt_gb300 as tp

pytestmark = pytest.mark.gpu

SHAPE, NL = (64, 32, 32), 4


class Compliance:
    """torch.autograd.Function over the C ABI (built lazily to keep torch optional)."""

    @staticmethod
    def make(torch):
        class _C(torch.autograd.Function):
            @staticmethod
            def forward(fctx, x, g, warm):
                xd = x.detach().to("cuda", torch.float64).contiguous()
                xphys = g.filter(xd)
                g.set_field("xphys", xphys)
                if warm is None:
                    g.upload("U", np.zeros(g.ndof(0)))
                else:
                    g.set_field("U", warm)
                it, rr, st = g.solve()
                assert st == 0, "CG did not converge"
                c = g.compliance()  # U^T K U, element by element
                # 2 F^T U - U^T K U equals c at the exact solution and errs only
                # to second order in the solve error, as central differences with
                # h = 1e-6 need
                fu = float(np.dot(g.download("F"), g.download("U")))
                dc = torch.from_numpy(g.download("dc")).cuda()
                fctx.save_for_backward(g.filter_T(dc))
                return torch.tensor(2.0 * fu - c, dtype=torch.float64, device=x.device)

            @staticmethod
            def backward(fctx, grad):
                (dcdx,) = fctx.saved_tensors
                return grad * dcdx.to(grad.device), None, None

        return _C


@pytest.fixture(scope="module")
def design(cuda):
    n = SHAPE[0] * SHAPE[1] * SHAPE[2]
    x = np.random.default_rng(0).uniform(0.01, 1.0, n)
    ref = golden("adjoint_64x32x32_l4.npz")
    assert x.sum() == pytest.approx(float(ref["x_sum"]), rel=1e-15)  # same generator stream
    return x, ref


@pytest.mark.parametrize("rmin,tag", [(1.5, "15"), (2.5, "25")])
def test_gradients_match_reference(design, cuda, rmin, tag):
    torch = cuda
    x, ref = design
    g = tp.TopOpt(*SHAPE, NL, rmin=rmin)
    xd = torch.from_numpy(x).cuda()
    xphys = g.filter(xd)
    g.set_field("xphys", xphys)
    it, rr, st = g.solve()
    assert st == 0 and it == int(ref["iters_" + tag])
    c = g.compliance()
    assert c == pytest.approx(float(ref["c_" + tag]), rel=1e-10)
    dc = g.download("dc")
    idx = ref["idx"]
    assert np.max(np.abs(dc[idx] - ref["dc_" + tag])) / np.max(np.abs(ref["dc_" + tag])) < 1e-9
    dcdx = g.filter_T(torch.from_numpy(dc).cuda()).cpu().numpy()
    assert np.max(np.abs(dcdx[idx] - ref["dcdx_" + tag])) / np.max(np.abs(ref["dcdx_" + tag])) < 1e-9
    assert np.linalg.norm(dcdx) == pytest.approx(float(ref["dcdx_norm_" + tag]), rel=1e-9)
    dv = g.filter_T(torch.ones(g.nelem(), dtype=torch.float64, device="cuda")).cpu().numpy()
    assert np.max(np.abs(dv[idx] - ref["dv_" + tag])) < 1e-13
    g.close()


@pytest.mark.parametrize("h", [1e-5, 1e-6], ids=["h1e-5", "h1e-6"])
@pytest.mark.parametrize("rmin", [1.5, 2.5])
def test_autograd_against_central_differences(design, cuda, rmin, h):
    torch = cuda
    x0, _ = design
    g = tp.TopOpt(*SHAPE, NL, rmin=rmin)
    g.set_cg(1e-12)  # FD needs the state to ~machine precision
    fn = Compliance.make(torch)
    x = torch.from_numpy(x0.copy()).requires_grad_(True)
    c = fn.apply(x, g, None)
    c.backward()
    grad = x.grad.numpy().copy()
    u0 = torch.from_numpy(g.download("U")).cuda()
    # volume: linear in x, its autograd gradient is H^T(1/Hs)/n
    xv = torch.from_numpy(x0.copy()).cuda().requires_grad_(True)
    vol = g_volume(g, torch, xv)
    vol.backward()
    rng = np.random.default_rng(1)
    # central differences: truncation O(h^2) ~ 1e-10 relative at h = 1e-5 (1e-12
    # at the configured h = 1e-6), while the solve's round-off (CG to 1e-12)
    # enters the quotient as noise / h, ten times larger at h = 1e-6
    noise = 1e-5 * (1e-5 / h)
    for e in rng.choice(g.nelem(), 64, replace=False):
        xp, xm = x0.copy(), x0.copy()
        xp[e] += h
        xm[e] -= h
        cp = fn.apply(torch.from_numpy(xp), g, u0).item()
        cm = fn.apply(torch.from_numpy(xm), g, u0).item()
        fd = (cp - cm) / (2 * h)
        assert abs(fd - grad[e]) <= noise * np.max(np.abs(grad)) + 1e-4 * abs(grad[e]), (e, fd, grad[e])
        fdv = (g_volume(g, torch, torch.from_numpy(xp).cuda()).item() -
               g_volume(g, torch, torch.from_numpy(xm).cuda()).item()) / (2 * h)
        # V is linear in x; its difference quotient is limited only by the round-off
        # of a 65,536-term sum changed by ~1e-11 (a few 1e-6 relative at h = 1e-5)
        assert fdv == pytest.approx(xv.grad[e].item(), rel=1e-4 * (1e-5 / h), abs=1e-12)
    g.close()


def g_volume(g, torch, x):
    class _V(torch.autograd.Function):
        @staticmethod
        def forward(fctx, xx):
            xphys = g.filter(xx.detach().contiguous())
            return xphys.sum() / g.nelem()

        @staticmethod
        def backward(fctx, grad):
            ones = torch.ones(g.nelem(), dtype=torch.float64, device="cuda")
            return grad * g.filter_T(ones) / g.nelem()

    return _V.apply(x)


def test_non_self_adjoint_objective(design, cuda):
    """c2 = L^T U with L != F needs a second solve K lam = L; its gradient
    wrt xPhys is -3 (E0-Emin) xPhys^2 lam_e^T KE u_e (tp_element_sensitivity)."""
    torch = cuda
    x0, _ = design
    g = tp.TopOpt(*SHAPE, NL, rmin=1.5)
    g.set_cg(1e-12)
    rng = np.random.default_rng(3)
    Lvec = np.zeros(g.ndof(0))
    free = np.ones(g.ndof(0), bool)
    free[g.fixed_dofs(0)] = False
    Lvec[free] = rng.uniform(-1, 1, free.sum()) * (rng.uniform(0, 1, free.sum()) < 0.01)
    xphys0 = g.filter(torch.from_numpy(x0).cuda())

    def c2(xphys):
        g.set_field("xphys", xphys)
        g.upload("U", np.zeros(g.ndof(0)))
        it, rr, st = g.solve()
        assert st == 0
        return float(Lvec @ g.download("U"))

    c2(xphys0)
    u = torch.from_numpy(g.download("U")).cuda()
    lam, it, rr, st = g.solve_rhs(torch.from_numpy(Lvec).cuda())
    assert st == 0
    sens = g.element_sensitivity(u, lam).cpu().numpy()
    h = 1e-6
    for e in np.random.default_rng(4).choice(g.nelem(), 16, replace=False):
        xp, xm = xphys0.clone(), xphys0.clone()
        xp[e] += h
        xm[e] -= h
        fd = (c2(xp) - c2(xm)) / (2 * h)
        # d(L^T U)/dxPhys_e = -lam^T (dK/dxPhys_e) U = sens_e (sens carries the minus sign)
        assert abs(fd - sens[e]) <= 1e-5 * np.max(np.abs(sens)) + 1e-4 * abs(sens[e]), (e, fd, sens[e])
    g.close()
