"""The element-centric, sum-factorised level-0 kernel against the node-centric
stencil and the oracle, through the C ABI, on grids that exercise its launch
plan: y extents that are and are not multiples of the 32-thread warp (the
columns shared by two warps go through shared memory), z extents that split
unevenly into row groups, single-element-thick slabs, and a y extent past
the kernel's envelope (falls back to the stencil)."""
import numpy as np
import pytest

from conftest import relerr
import topopt_gb300 as tp

pytestmark = pytest.mark.gpu

SHAPES = [(16, 66, 6), (8, 32, 10), (12, 64, 4), (6, 8, 30), (10, 96, 2), (4, 256, 4), (4, 258, 4),
          (2, 2, 2)]


def _rand(g, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.01, 1.0, g.nelem()), rng.uniform(-1.0, 1.0, g.ndof(0))


@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
def test_apply_fp64_matches_stencil(cuda, shape):
    torch = cuda
    g = tp.TopOpt(*shape, 2)
    x, u = _rand(g, 0)
    g.upload("xphys", x)
    ud = torch.from_numpy(u).cuda()
    y_ec = g.apply(0, ud).cpu().numpy()
    g.set_fine_variant(1)
    y_nc = g.apply(0, ud).cpu().numpy()
    assert relerr(y_ec, y_nc) < 1e-13
    b = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, g.ndof(0))).cuda()
    s_nc = g.smooth(0, 3, 0.6, b, ud).cpu().numpy()
    g.set_fine_variant(0)
    s_ec = g.smooth(0, 3, 0.6, b, ud).cpu().numpy()
    assert relerr(s_ec, s_nc) < 1e-12
    g.close()


@pytest.mark.parametrize("shape", SHAPES[:4], ids=["x".join(map(str, s)) for s in SHAPES[:4]])
def test_apply_against_oracle(cuda, shape):
    from oracle import Oracle
    torch = cuda
    g = tp.TopOpt(*shape, 2)
    x, u = _rand(g, 2)
    g.upload("xphys", x)
    y = g.apply(0, torch.from_numpy(u).cuda()).cpu().numpy()
    assert relerr(y, Oracle(*shape, 2).apply(0, x, u)) < 1e-12
    g.close()


@pytest.mark.parametrize("shape", SHAPES[:4], ids=["x".join(map(str, s)) for s in SHAPES[:4]])
def test_apply_double_single(cuda, shape):
    """Double vectors worked on as pairs of floats (the mixed form's default
    for its CG matvec and residual): FP64 in, FP64 out, about 48 bits in
    between -- five to six orders of magnitude closer to the FP64 oracle than
    the FP32 operator. A smooth field, whose K u cancels most of |K| |u|,
    loses what that cancellation costs and stays well inside 1e-10. The
    FP64 switch gives back the FP64 result."""
    from oracle import Oracle
    torch = cuda
    g = tp.TopOpt(*shape, 2, precision=tp.TP_MIXED)
    o = Oracle(*shape, 2)
    x, u = _rand(g, 7)
    g.upload("xphys", x)
    nx, ny, nz = (s + 1 for s in shape)
    i, k, j = np.meshgrid(np.arange(nx), np.arange(nz), np.arange(ny), indexing="ij")  # [x][z][y] node order
    smooth = np.stack([np.sin(0.3 * i + 0.2 * j) * np.cos(0.1 * k) + 2.0, np.cos(0.2 * i) + 0.5 * j / ny,
                       np.sin(0.25 * k + 0.1 * i)], axis=-1).reshape(-1)
    assert smooth.size == g.ndof(0)
    for v, tol in ((u, 1e-12), (smooth, 1e-10)):
        ref = o.apply(0, x, v)
        y_ds = g.apply(0, torch.from_numpy(v).cuda()).cpu().numpy()
        assert relerr(y_ds, ref) < tol
    g.set_fine_arith(0)
    y64 = g.apply(0, torch.from_numpy(u).cuda()).cpu().numpy()
    assert relerr(y64, o.apply(0, x, u)) < 1e-12
    g.close()


def test_fp64_form_opting_into_double_single(cuda):
    """The FP64 form with tp_set_fine_arith(1): its V-cycle's level-0 Jacobi
    sweeps and residual run in double-single too. A V-cycle agrees with the
    FP64 one to 1e-10 and the cantilever solve takes the same CG iterations."""
    torch = cuda
    shape = (16, 64, 12)
    g = tp.TopOpt(*shape, 2)
    x, _ = _rand(g, 8)
    g.upload("xphys", x)
    g.assemble()
    r = torch.from_numpy(np.random.default_rng(9).uniform(-1, 1, g.ndof(0))).cuda()
    z64 = g.vcycle(r).cpu().numpy()
    g.set_fine_arith(1)
    zds = g.vcycle(r).cpu().numpy()
    assert 0 < relerr(zds, z64) < 1e-10
    runs = []
    for arith in (0, 1):
        g.set_fine_arith(arith)
        g.init_design()
        g.upload("U", np.zeros(g.ndof(0)))
        it, rr, st = g.solve()
        assert st == 0 and rr < 1e-5
        runs.append((it, g.download("U")))
    assert runs[0][0] == runs[1][0]
    assert relerr(runs[1][1], runs[0][1]) < 1e-8
    g.close()


@pytest.mark.parametrize("shape", SHAPES[:3], ids=["x".join(map(str, s)) for s in SHAPES[:3]])
def test_apply_fp32(cuda, shape):
    torch = cuda
    g = tp.TopOpt(*shape, 2, precision=tp.TP_MIXED)
    x, u = _rand(g, 3)
    g.upload("xphys", x)
    g.assemble()
    ud = torch.from_numpy(u).cuda()
    y64 = g.apply(0, ud).cpu().numpy()
    y32 = g.apply(0, ud.float()).double().cpu().numpy()
    assert relerr(y32, y64) < 1e-5
    g.set_fine_variant(1)
    y32n = g.apply(0, ud.float()).double().cpu().numpy()
    assert relerr(y32, y32n) < 1e-5
    g.close()


@pytest.mark.parametrize("prec", [tp.TP_FP64, tp.TP_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("shape", [(16, 64, 12), (8, 32, 10), (16, 66, 6)], ids=["16x64x12", "8x32x10", "16x66x6"])
def test_vcycle_matches_stencil(cuda, shape, prec):
    """One V-cycle: the fused Jacobi sweeps and the residual of level 0."""
    torch = cuda
    g = tp.TopOpt(*shape, 2, precision=prec)
    x, _ = _rand(g, 5)
    g.upload("xphys", x)
    g.assemble()
    r = torch.from_numpy(np.random.default_rng(6).uniform(-1, 1, g.ndof(0))).cuda()
    z_ec = g.vcycle(r).cpu().numpy()
    g.set_fine_variant(1)
    z_nc = g.vcycle(r).cpu().numpy()
    assert relerr(z_ec, z_nc) < (1e-12 if prec == tp.TP_FP64 else 1e-4)
    g.close()


def test_autotune_keeps_results(cuda):
    torch = cuda
    g = tp.TopOpt(16, 64, 12, 2, precision=tp.TP_MIXED)
    x, u = _rand(g, 4)
    g.upload("xphys", x)
    g.assemble()
    ud = torch.from_numpy(u).cuda()
    y0 = g.apply(0, ud).cpu().numpy()
    ms = g.autotune()
    assert np.all(ms > 0) and np.all(ms < 1e3)
    g.upload("xphys", x)
    g.assemble()
    y1 = g.apply(0, ud).cpu().numpy()
    # every node is owned by one thread whatever the launch shape, with the
    # same order of accumulation: the result is bit for bit the same
    assert np.array_equal(y0, y1)
    # the cantilever state solve with the tuned shapes and with the stencil
    g.init_design()
    g.upload("U", np.zeros(g.ndof(0)))
    it, rr, st = g.solve()
    assert st == 0 and rr < 1e-5
    u_ec = g.download("U")
    g.set_fine_variant(1)
    g.upload("U", np.zeros(g.ndof(0)))
    it1, rr1, st1 = g.solve()
    assert st1 == 0 and it1 == it
    assert relerr(u_ec, g.download("U")) < 1e-6
    g.close()


PK_SHAPES = SHAPES[:6] + [(8, 128, 16), (6, 40, 22)]


@pytest.mark.parametrize("shape", PK_SHAPES, ids=["x".join(map(str, s)) for s in PK_SHAPES])
def test_packed_fp32_kernel(cuda, shape):
    """The packed FP32 kernel (two z groups per thread in f32x2 arithmetic,
    tp_set_fine_variant(2)) against the one-group kernel and the node-centric
    stencil: the FP32 product, and a V-cycle of the mixed form, whose level-0
    sweeps and residual it runs. Grids with odd group counts leave the second
    lane of the last thread row empty."""
    torch = cuda
    g = tp.TopOpt(*shape, 2, precision=tp.TP_MIXED)
    x, u = _rand(g, 11)
    g.upload("xphys", x)
    g.assemble()
    uf = torch.from_numpy(u).cuda().float()
    r = torch.from_numpy(np.random.default_rng(12).uniform(-1, 1, g.ndof(0))).cuda()
    out = {}
    for variant in (0, 2, 1):
        g.set_fine_variant(variant)
        out[variant] = (g.apply(0, uf).double().cpu().numpy(), g.vcycle(r).cpu().numpy())
    y64 = g.apply(0, torch.from_numpy(u).cuda()).cpu().numpy()
    for variant in (0, 1):
        assert relerr(out[2][0], out[variant][0]) < 1e-5
        assert relerr(out[2][1], out[variant][1]) < 1e-4
    assert relerr(out[2][0], y64) < 1e-5
    g.close()


@pytest.mark.parametrize("shape", [(8, 128, 16), (6, 40, 22), (16, 66, 6)], ids=["8x128x16", "6x40x22", "16x66x6"])
def test_every_fp32_launch_plan(cuda, shape):
    """Every FP32 launch plan the grid allows (one or two z groups per thread,
    b and invD from global memory, staged per CTA or copied ahead per thread,
    both register caps, the moduli staged or in registers, several x
    chunkings), set through tp_set_fine_plan,
    gives the node-centric stencil's product and V-cycle to FP32 accuracy."""
    torch = cuda
    g = tp.TopOpt(*shape, 2, precision=tp.TP_MIXED)
    x, u = _rand(g, 21)
    g.upload("xphys", x)
    g.assemble()
    uf = torch.from_numpy(u).cuda().float()
    r = torch.from_numpy(np.random.default_rng(22).uniform(-1, 1, g.ndof(0))).cuda()
    g.set_fine_variant(1)
    y_ref, z_ref = g.apply(0, uf).double().cpu().numpy(), g.vcycle(r).cpu().numpy()
    g.set_fine_variant(0)
    tried = 0
    for pk in (0, 1):
        for groups in ((1, 2, 4) if pk == 0 else (2, 4)):
            for ncx in (1, 3):
                for own in (0, 1, 2):
                    for occ, es in ((0, 1), (1, 1), (0, 0), (1, 0)):
                        plan = [groups, ncx, own, occ, pk, es]
                        if g.set_fine_plan(0, 2, plan) != 0:
                            continue
                        assert g.set_fine_plan(0, 3, plan) == 0
                        assert g.set_fine_plan(0, 0, [groups, ncx, 0, occ, pk, es]) == 0
                        assert g.fine_plan(0, 2)[:6] == plan
                        tried += 1
                        y = g.apply(0, uf).double().cpu().numpy()
                        z = g.vcycle(r).cpu().numpy()
                        assert relerr(y, y_ref) < 1e-5, plan
                        assert relerr(z, z_ref) < 1e-4, plan
    assert tried >= 8
    assert g.set_fine_plan(0, 1, [2, 1, 0, 0, 1, 1]) == 1  # no packed product with a dot product
    assert g.set_fine_plan(1, 2, [1, 1, 2, 0, 0, 1]) == 1  # per-thread copies are FP32 only
    assert g.set_fine_plan(0, 2, [2, 1, 0, 0, 1, 0]) == 1  # the packed kernel stages its moduli
    g.close()
