"""The reference-signature entry points (include/topopt_ref_api.h).

They take the reference's structs and HOST arrays in its padded layout. The
CPU tests check the host-side set-up (element tables, fixed DOFs, padding,
CSR pattern) against the golden fixtures and, where it was built here, the
reference's own C; the GPU tests drive the operators, the solve and
top3dmgcg through these entry points against the golden fixtures."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, golden, relerr
import topopt_gb300 as tp

UF = ctypes.c_ulong  # uint_fast32_t on LP64 glibc (x86_64 and aarch64)
D = ctypes.c_double


class FixedDofs(ctypes.Structure):
    _fields_ = [("n", UF), ("idx", ctypes.POINTER(UF))]


class GridContext(ctypes.Structure):
    _fields_ = [("E0", D), ("Emin", D), ("nu", D), ("esx", D), ("esy", D), ("esz", D),
                ("nelx", UF), ("nely", UF), ("nelz", UF), ("wrapx", UF), ("wrapy", UF), ("wrapz", UF),
                ("penal", D), ("precomputedKE", ctypes.POINTER(ctypes.POINTER(D))),
                ("fixedDofs", ctypes.POINTER(FixedDofs))]


class GpuNode(ctypes.Structure):
    pass


GpuNode._fields_ = [("id", ctypes.c_int), ("prev", ctypes.POINTER(GpuNode)), ("next", ctypes.POINTER(GpuNode)),
                    ("gc", ctypes.POINTER(GridContext)), ("offset_x", ctypes.c_int), ("x_global", ctypes.c_int)]


class GpuGrid(ctypes.Structure):
    _fields_ = [("num_targets", ctypes.c_int), ("target", ctypes.POINTER(GpuNode))]


class CSR(ctypes.Structure):
    _fields_ = [("nnz", ctypes.c_uint64), ("nrows", ctypes.c_int32), ("rowOffsets", ctypes.POINTER(ctypes.c_int)),
                ("colIndex", ctypes.POINTER(ctypes.c_int)), ("vals", ctypes.POINTER(D))]


def lib64():
    tp.load()
    L = ctypes.CDLL(os.path.join(tp.PKG, "libtopopt_ref64.so"))
    P = ctypes.c_void_p
    L.setupGC.argtypes = [ctypes.POINTER(GridContext), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.freeGC.argtypes = [ctypes.POINTER(GridContext), ctypes.c_int]
    L.gridContextToGPUGrid.argtypes = [ctypes.POINTER(GridContext), ctypes.POINTER(GpuGrid), ctypes.c_int, ctypes.c_int]
    L.computePadding.argtypes = [ctypes.POINTER(GridContext), ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 4 + [ctypes.POINTER(UF)]
    L.allocateSubspaceMatrix.argtypes = [GridContext, ctypes.c_int, ctypes.POINTER(CSR)]
    L.assembleSubspaceMatrix.argtypes = [GridContext, ctypes.c_int, P, CSR, P]
    L.applyStateOperator_stencil.argtypes = [ctypes.POINTER(GpuNode), P, P, P]
    L.applyStateOperatorSubspace_halo.argtypes = [ctypes.POINTER(GpuNode), ctypes.c_int, P, P, P]
    L.projectToCoarserGrid_halo.argtypes = [ctypes.POINTER(GpuNode), ctypes.c_int, P, P]
    L.projectToFinerGrid_halo.argtypes = [ctypes.POINTER(GpuNode), ctypes.c_int, P, P]
    L.assembleInvertedMatrixDiagonalSubspace_halo.argtypes = [ctypes.POINTER(GpuNode), P, ctypes.c_int, P]
    L.getComplianceAndSensetivity_halo.argtypes = [ctypes.POINTER(GpuNode), P, P, P, P]
    L.applyDensityFilter.argtypes = [GridContext, D, P, P]
    L.applyDensityFilterGradient.argtypes = [GridContext, D, P]
    return L


def padded_dims(nelx, nely, nelz, l):
    ex, ey, ez = nelx >> l, nely >> l, nelz >> l
    py = (128 - (ey + 1) % 128) % 128
    return ex, ey, ez, ex + 3, ey + py + 3, ez + 3


def vec_to_padded(v, dims):
    ex, ey, ez, wx, wy, wz = dims
    p = np.zeros((wx, wz, wy, 3))
    p[1:ex + 2, 1:ez + 2, 1:ey + 2, :] = v.reshape(ex + 1, ez + 1, ey + 1, 3)
    return p.reshape(-1)


def vec_from_padded(p, dims):
    ex, ey, ez, wx, wy, wz = dims
    return p.reshape(wx, wz, wy, 3)[1:ex + 2, 1:ez + 2, 1:ey + 2, :].reshape(-1).copy()


def el_to_padded(x, dims):
    ex, ey, ez, wx, wy, wz = dims
    p = np.zeros((wx - 1, wz - 1, wy - 1))
    p[1:ex + 1, 1:ez + 1, 1:ey + 1] = x.reshape(ex, ez, ey)
    return p.reshape(-1)


def el_from_padded(p, dims):
    ex, ey, ez, wx, wy, wz = dims
    return p.reshape(wx - 1, wz - 1, wy - 1)[1:ex + 1, 1:ez + 1, 1:ey + 1].reshape(-1).copy()


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.fixture(scope="module")
def grid():
    L = lib64()
    gc = GridContext()
    nl = 3
    L.setupGC(ctypes.byref(gc), nl, 16, 8, 8)
    return L, gc, nl


def test_setup_matches_reference_data(grid):
    L, gc, nl = grid
    g = golden("kernels_16x8x8_l3.npz")
    ke = golden("ke.npz")
    k0 = np.ctypeslib.as_array(gc.precomputedKE[0], shape=(576,))
    assert relerr(k0, ke["ke_0"]) < 1e-14
    dims0 = padded_dims(16, 8, 8, 0)
    assert (gc.wrapx, gc.wrapy, gc.wrapz) == dims0[3:]
    for l in range(nl):
        fd = gc.fixedDofs[l]
        idx = np.ctypeslib.as_array(fd.idx, shape=(fd.n,)).astype(np.int64)
        ex, ey, ez, wx, wy, wz = padded_dims(16, 8, 8, l)
        node, c = idx // 3, idx % 3
        i, k, j = node // (wy * wz) - 1, (node % (wy * wz)) // wy - 1, node % wy - 1
        canon = 3 * ((i * (ez + 1) + k) * (ey + 1) + j) + c
        assert np.array_equal(canon, g["fixed_%d" % l])
    ncell, wx, wy, wz, nd = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), UF()
    L.computePadding(ctypes.byref(gc), 1, ctypes.byref(ncell), ctypes.byref(wx), ctypes.byref(wy), ctypes.byref(wz),
                     ctypes.byref(nd))
    _, _, _, ewx, ewy, ewz = padded_dims(16, 8, 8, 1)
    assert (ewx, ewy, ewz) == (11, 130, 7)  # y padded so that nely_1 + 1 + pad = 128
    assert (ncell.value, wx.value, wy.value, wz.value) == (2, ewx, ewy, ewz) and nd.value == 3 * ewx * ewy * ewz


REF64 = os.path.join(ROOT, "oracle", "_ref", "libref64.so")


@pytest.mark.skipif(not os.path.exists(REF64), reason="reference not built in this checkout")
def test_csr_pattern_matches_reference(grid):
    L, gc, nl = grid
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Reference
    R = Reference(16, 8, 8, nl)
    x = np.full(16 * 8 * 8, 0.3)
    nnz = R.L.ref_csr(R.h, 2, x.ctypes.data_as(ctypes.POINTER(D)), None, None, None)
    rp = np.zeros(3 * 5 * 3 * 3 + 1, np.int32)
    ci = np.zeros(nnz, np.int32)
    va = np.zeros(nnz)
    R.L.ref_csr(R.h, 2, x.ctypes.data_as(ctypes.POINTER(D)), rp.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                ci.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), va.ctypes.data_as(ctypes.POINTER(D)))
    M = CSR()
    L.allocateSubspaceMatrix(gc, 2, ctypes.byref(M))
    assert M.nnz == nnz and M.nrows == len(rp) - 1
    assert np.array_equal(np.ctypeslib.as_array(M.rowOffsets, shape=(len(rp),)), rp)
    assert np.array_equal(np.ctypeslib.as_array(M.colIndex, shape=(nnz,)), ci)


@pytest.mark.skipif(not os.path.exists(REF64), reason="reference not built in this checkout")
@pytest.mark.parametrize("flavour", [32, 64])
@pytest.mark.parametrize("shape", [(16, 8, 8), (12, 6, 10)])
def test_vtk_files_match_reference_bytes(tmp_path, flavour, shape):
    """The two .vtu writers (stencil_optimization.c:399-598) of the drop-in
    library and of the reference's own build, given the same padded density
    array, write the same bytes (host code only: no GPU call)."""
    tp.load()
    ours = ctypes.CDLL(os.path.join(tp.PKG, "libtopopt_ref%d.so" % flavour))
    ref = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref%d.so" % flavour))
    dt = np.float64 if flavour == 64 else np.float32
    dims = padded_dims(*shape, 0)
    rho = np.random.default_rng(9).uniform(0.0, 1.0, (dims[3] - 1) * (dims[4] - 1) * (dims[5] - 1)).astype(dt)
    for fn in ("writeDensityVtkFile", "writeDensityVtkFileWithHalo"):
        files = []
        for tag, lib in (("ours", ours), ("ref", ref)):
            f = getattr(lib, fn)
            f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_char_p]
            path = tmp_path / ("%s_%s.vtu" % (fn, tag))
            f(shape[0], shape[1], shape[2], ptr(rho), os.fsencode(str(path)))
            files.append(path.read_bytes())
        assert len(files[0]) > 1000 and files[0] == files[1], fn


# ---------------------------------------------------------------- GPU ----
@pytest.mark.gpu
def test_operators_through_reference_signatures(grid, cuda):
    L, gc, nl = grid
    g = golden("kernels_16x8x8_l3.npz")
    gg = GpuGrid()
    gg.num_targets = 1
    L.gridContextToGPUGrid(ctypes.byref(gc), ctypes.byref(gg), nl, 0)
    node = gg.target
    d0 = padded_dims(16, 8, 8, 0)
    xp = el_to_padded(g["x"], d0)
    for l in range(nl):
        dl = padded_dims(16, 8, 8, l)
        u = vec_to_padded(g["u_%d" % l], dl)
        out = np.zeros_like(u)
        if l == 0:
            L.applyStateOperator_stencil(node, ptr(xp), ptr(u), ptr(out))
            assert relerr(vec_from_padded(out, dl), g["apply_0"]) < 1e-10
        elif l == 1:
            L.applyStateOperatorSubspace_halo(node, l, ptr(xp), ptr(u), ptr(out))
            assert relerr(vec_from_padded(out, dl), g["apply_1"]) < 1e-10
        diag = np.zeros_like(u)
        L.assembleInvertedMatrixDiagonalSubspace_halo(node, ptr(xp), l, ptr(diag))
        assert relerr(vec_from_padded(diag, dl), g["invdiag_%d" % l]) < 1e-10
        if l + 1 < nl:
            dc = padded_dims(16, 8, 8, l + 1)
            rc = np.zeros(3 * dc[3] * dc[4] * dc[5])
            L.projectToCoarserGrid_halo(node, l, ptr(u), ptr(rc))
            assert relerr(vec_from_padded(rc, dc), g["restrict_%d" % l]) < 1e-14
            uc = vec_to_padded(g["uc_%d" % l], dc)
            pf = np.zeros_like(u)
            L.projectToFinerGrid_halo(node, l, ptr(uc), ptr(pf))
            assert relerr(vec_from_padded(pf, dl), g["prolong_%d" % l]) < 1e-14
    U = vec_to_padded(g["u_c"], d0)
    c = np.zeros(1)
    dcp = np.zeros_like(xp)
    L.getComplianceAndSensetivity_halo(node, ptr(xp), ptr(U), ptr(c), ptr(dcp))
    assert abs(c[0] - float(g["c"])) / abs(float(g["c"])) < 1e-10
    assert relerr(el_from_padded(dcp, d0), g["dc"]) < 1e-10
    out = np.zeros_like(xp)
    L.applyDensityFilter(gc, 1.5, ptr(xp), ptr(out))
    assert relerr(el_from_padded(out, d0), g["filter_15"]) < 1e-14
    v = xp.copy()
    L.applyDensityFilterGradient(gc, 2.5, ptr(v))
    assert relerr(el_from_padded(v, d0), g["filterT_25"]) < 1e-14


@pytest.mark.gpu
def test_top3dmgcg_summary_line(cuda):
    """top3d's own call on the 48x24x24 grid (-x 12 -y 6 -z 6 -l 3), through
    the float-typed library a caller compiled against the reference's headers
    would link; the printed compliance agrees with the reference's run."""
    g = golden("history_48x24x24_l3.npz")
    code = ("import ctypes; L = ctypes.CDLL(%r); "
            "L.top3dmgcg.argtypes = [ctypes.c_ulong]*3 + [ctypes.c_float]*2 + [ctypes.c_ulong, ctypes.c_float, "
            "ctypes.c_ulong, ctypes.c_int, ctypes.c_int, ctypes.c_int]; "
            "L.top3dmgcg(48, 24, 24, 0.2, 1.5, 3, 1e-5, 200, 0, 0, 20)") % os.path.join(tp.PKG, "libtopopt_ref32.so")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    fields = r.stdout.split()
    loop, c, vol = int(fields[0]), float(fields[1]), float(fields[2])
    assert loop == int(g["loops"])
    assert c == pytest.approx(float(g["c"][-1]), abs=2e-6)
    assert int(fields[5]) == int(np.sum(g["cgiters"]))
