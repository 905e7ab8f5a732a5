"""Generates the golden fixtures in tests/golden/ from the reference's own C.

Run in the development container, where the reference tree is mounted:
    bash oracle/build_ref.sh && python tests/golden/make_golden.py [--big]

It loads oracle/_ref/libref64.so (the reference's sources, FP64 typedefs,
CHOLMOD/CBLAS stand-ins) through oracle/ref_driver.c and records inputs and
outputs in the canonical unpadded layout (see oracle/topopt_oracle.h). The
fixtures are the pin for the oracle restatement and for the CUDA path.
--big adds the 128x64x64 (-l 4) 20-iteration history (about 20 minutes);
--config4 writes only the 256x128x128 (-l 4) history (hours), with samples of
the final design instead of the whole field.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
from oracle import Reference  # noqa: E402

F32 = lambda v: float(np.float32(v))  # main() holds volfrac, rmin, cgtol as float


def kernels(shape, nl, seed=0, solve_after=5):
    R = Reference(*shape, nl)
    rng = np.random.default_rng(seed)
    out = {"shape": np.array(shape), "nl": nl}
    x = rng.uniform(0.01, 1.0, R.nelem())
    out["x"] = x
    for l in range(nl):
        out["fixed_%d" % l] = R.fixed_dofs(l)
        u = rng.uniform(-1, 1, R.ndof(l))
        out["u_%d" % l] = u
        out["apply_%d" % l] = R.apply(l, x, u)
        if l >= 2:
            out["apply_csr_%d" % l] = R.apply_csr(l, x, u)
        out["invdiag_%d" % l] = R.inv_diag(l, x)
        if l + 1 < nl:
            out["restrict_%d" % l] = R.restrict(l, u)
            uc = rng.uniform(-1, 1, R.ndof(l + 1))
            out["uc_%d" % l] = uc
            out["prolong_%d" % l] = R.prolong(l, uc)
            if l < 2:
                b = rng.uniform(-1, 1, R.ndof(l))
                out["b_%d" % l] = b
                out["smooth_%d" % l] = R.smooth(l, x, 4, 0.6, b, u)
    out["load"] = R.load()
    u0 = rng.uniform(-1, 1, R.ndof(0))
    out["u_c"] = u0
    c, dc = R.compliance(x, u0)
    out["c"] = c
    out["dc"] = dc
    for tag, rmin in (("15", 1.5), ("25", 2.5)):
        out["filter_" + tag] = R.filter(rmin, x)
        out["filterT_" + tag] = R.filter_T(rmin, x)
    dv = R.filter_T(1.5, np.ones(R.nelem()))
    dcn = -rng.uniform(0.05, 1.0, R.nelem())
    xo = rng.uniform(0.0, 1.0, R.nelem())
    out["oc_x"], out["oc_dv"], out["oc_dc"], out["oc_g"] = xo, dv, dcn, 0.013
    out["oc_xnew"] = R.oc_update(xo, dv, dcn, 0.013)
    # one state solve on a real design: the reference's own xPhys after
    # `solve_after` design iterations on this grid (0: the uniform start),
    # warm-started from zero. On very small grids the reference's
    # preconditioner needs hundreds of iterations on evolved designs, so those
    # use the start design.
    if solve_after > 0:
        _, _, xs, _ = Reference(*shape, nl).run(0.2, 1.5, 1e-5, solve_after, want_fields=True)
    else:
        xs = np.full(R.nelem(), F32(0.2))
    us, it, rr = R.solve(xs, out["load"], None, 4, F32(1e-5))
    out["solve_x"], out["solve_u"], out["solve_iters"], out["solve_relres"] = xs, us, it, rr
    return out


def history(shape, nl, iters, flavour=64):
    R = Reference(*shape, nl, flavour=flavour)
    t = time.time()
    loops, h, xp, u = R.run(0.2, 1.5, 1e-5, iters, want_fields=True)
    h = {k: np.asarray(v) for k, v in h.items()}
    h["seconds"] = time.time() - t
    h["loops"] = loops
    h["xphys"] = xp
    h["shape"] = np.array(shape)
    h["nl"] = nl
    return h


def history_compact(shape, nl, iters):
    """The 20-iteration history of a grid too large to store its fields:
    compliance, volume, change, relres and CG counts in full, and of the final
    xPhys its sum, its 2-norm and 256 seeded samples (default_rng(11))."""
    h = history(shape, nl, iters)
    xp = h.pop("xphys")
    idx = np.sort(np.random.default_rng(11).choice(xp.size, 256, replace=False))
    h.update({"xphys_idx": idx, "xphys_val": xp[idx], "xphys_sum": xp.sum(),
              "xphys_norm": np.linalg.norm(xp)})
    return h


def adjoint(shape=(64, 32, 32), nl=4):
    """Sensitivities of the reference on i.i.d. U[0.01, 1] design variables
    (numpy default_rng(0)) through the density filter, rmin 1.5 and 2.5: the
    compliance, dc/dxPhys and dc/dx = H^T(dc/Hs), and dv = H^T(1/Hs). Only
    seeded samples and norms of the element arrays are stored."""
    R = Reference(*shape, nl)
    n = R.nelem()
    x = np.random.default_rng(0).uniform(0.01, 1.0, n)
    idx = np.sort(np.random.default_rng(7).choice(n, 256, replace=False))
    out = {"shape": np.array(shape), "nl": nl, "x_sum": x.sum(), "x_head": x[:16], "idx": idx}
    F = R.load()
    for tag, rmin in (("15", 1.5), ("25", 2.5)):
        xp = R.filter(rmin, x)
        u, it, rr = R.solve(xp, F, None, 4, F32(1e-5))
        c, dc = R.compliance(xp, u)
        dcdx = R.filter_T(rmin, dc)
        dv = R.filter_T(rmin, np.ones(n))
        out.update({"c_" + tag: c, "iters_" + tag: it, "dc_" + tag: dc[idx], "dcdx_" + tag: dcdx[idx],
                    "dv_" + tag: dv[idx], "dcdx_norm_" + tag: np.linalg.norm(dcdx),
                    "dc_norm_" + tag: np.linalg.norm(dc), "dv_sum_" + tag: dv.sum()})
    return out


def ke_fixture():
    R = Reference(8, 4, 4, 4)
    out = {}
    rng = np.random.default_rng(1)
    for l in range(4):
        k = R.ke(l)
        if l < 2:
            out["ke_%d" % l] = k
        idx = np.sort(rng.choice(k.size, 64, replace=False))
        out["ke_%d_idx" % l] = idx
        out["ke_%d_val" % l] = k[idx]
        out["ke_%d_sum" % l] = k.sum()
        out["ke_%d_abssum" % l] = np.abs(k).sum()
        out["ke_%d_sqsum" % l] = (k * k).sum()
    return out


def main():
    if "--config4" in sys.argv:
        # the headline grid, 256x128x128 -l 4, 20 iterations (hours on 8 cores)
        np.savez_compressed(os.path.join(HERE, "history_256x128x128_l4.npz"),
                            **history_compact((256, 128, 128), 4, 20))
        return
    big = "--big" in sys.argv
    np.savez_compressed(os.path.join(HERE, "ke.npz"), **ke_fixture())
    np.savez_compressed(os.path.join(HERE, "kernels_16x8x8_l3.npz"), **kernels((16, 8, 8), 3, solve_after=0))
    np.savez_compressed(os.path.join(HERE, "kernels_32x16x16_l4.npz"), **kernels((32, 16, 16), 4, seed=3))
    np.savez_compressed(os.path.join(HERE, "history_48x24x24_l3.npz"), **history((48, 24, 24), 3, 20))
    np.savez_compressed(os.path.join(HERE, "history_48x24x24_l3_float.npz"),
                        **history((48, 24, 24), 3, 20, flavour=32))
    np.savez_compressed(os.path.join(HERE, "history_32x16x16_l4.npz"), **history((32, 16, 16), 4, 20))
    if big:
        np.savez_compressed(os.path.join(HERE, "history_128x64x64_l4.npz"), **history((128, 64, 64), 4, 20))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
