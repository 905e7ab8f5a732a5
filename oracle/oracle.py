"""ctypes bindings for the CPU oracle (test infrastructure only).

`Oracle` wraps oracle/liboracle.so, the plain-C FP64 restatement of the
reference's hot path. `Reference` wraps oracle/_ref/libref{64,32}.so, the
reference's own C compiled by oracle/build_ref.sh (present only where the
reference tree was mounted at build time).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module. Arrays are float64 numpy arrays in the canonical unpadded layout
described in topopt_oracle.h.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_L = ctypes.POINTER(ctypes.c_long)


def _p(a):
    return None if a is None else a.ctypes.data_as(_D)


def build():
    """Compile liboracle.so (and the reference build where it is mounted)."""
    import subprocess
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def dims(nelx, nely, nelz, l):
    return nelx >> l, nely >> l, nelz >> l


def nnodes(nelx, nely, nelz, l):
    ex, ey, ez = dims(nelx, nely, nelz, l)
    return (ex + 1) * (ey + 1) * (ez + 1)


class _OrHistory(ctypes.Structure):
    _fields_ = [("loops", ctypes.c_int),
                ("c", ctypes.c_double * 1024), ("vol", ctypes.c_double * 1024),
                ("change", ctypes.c_double * 1024), ("relres", ctypes.c_double * 1024),
                ("cgiters", ctypes.c_int * 1024), ("seconds", ctypes.c_double * 1024)]


class Oracle:
    """The oracle restatement on one grid (nelx, nely, nelz, nl)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            path = os.path.join(HERE, "liboracle.so")
            if not os.path.exists(path):
                build()
            L = ctypes.CDLL(path)
            V = ctypes.c_void_p
            L.or_create.restype = V
            L.or_create.argtypes = [ctypes.c_int] * 4
            L.or_destroy.argtypes = [V]
            L.or_ke.argtypes = [ctypes.c_double, ctypes.c_int, _D]
            L.or_fixed_dofs.restype = ctypes.c_int
            L.or_fixed_dofs.argtypes = [V, ctypes.c_int, _L]
            L.or_load.argtypes = [V, _D]
            for f in ("or_apply", "or_apply_masked"):
                getattr(L, f).argtypes = [V, ctypes.c_int, _D, _D, _D]
            L.or_inv_diag.argtypes = [V, ctypes.c_int, _D, _D]
            L.or_restrict.argtypes = [V, ctypes.c_int, _D, _D]
            L.or_prolong.argtypes = [V, ctypes.c_int, _D, _D]
            L.or_smooth.argtypes = [V, ctypes.c_int, _D, ctypes.c_int, ctypes.c_double, _D, _D, _D, _D]
            L.or_coarse_direct.restype = ctypes.c_int
            L.or_coarse_direct.argtypes = [V, ctypes.c_int, _D, _D, _D]
            L.or_solve.restype = ctypes.c_int
            L.or_solve.argtypes = [V, _D, _D, _D, ctypes.c_int, ctypes.c_double, _I, _D]
            L.or_compliance.restype = ctypes.c_double
            L.or_compliance.argtypes = [V, _D, _D, _D]
            L.or_filter.argtypes = [V, ctypes.c_double, _D, _D]
            L.or_filter_T.argtypes = [V, ctypes.c_double, _D]
            L.or_oc_update.argtypes = [V, _D, _D, _D, ctypes.c_double, _D]
            L.or_volume.restype = ctypes.c_double
            L.or_volume.argtypes = [V, _D]
            L.or_change.restype = ctypes.c_float
            L.or_change.argtypes = [V, _D, _D]
            L.or_run.restype = ctypes.c_int
            L.or_run.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                      ctypes.c_double, ctypes.c_int,
                                                      ctypes.POINTER(_OrHistory), _D, _D]
            cls._lib = L
        return cls._lib

    def __init__(self, nelx, nely, nelz, nl):
        self.L = self.lib()
        self.shape = (nelx, nely, nelz)
        self.nl = nl
        self.h = self.L.or_create(nelx, nely, nelz, nl)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.or_destroy(self.h)
            self.h = None

    def ndof(self, l=0):
        return 3 * nnodes(*self.shape, l)

    def nelem(self):
        nx, ny, nz = self.shape
        return nx * ny * nz

    @staticmethod
    def ke(l, nu=0.3):
        n = 1 << l
        out = np.zeros(576 * n ** 3)
        Oracle.lib().or_ke(nu, l, _p(out))
        return out

    def fixed_dofs(self, l=0):
        n = self.L.or_fixed_dofs(self.h, l, None)
        out = np.zeros(n, np.int64)
        self.L.or_fixed_dofs(self.h, l, out.ctypes.data_as(_L))
        return out

    def load(self):
        F = np.zeros(self.ndof())
        self.L.or_load(self.h, _p(F))
        return F

    def apply(self, l, x, u, masked=False):
        out = np.zeros(self.ndof(l))
        f = self.L.or_apply_masked if masked else self.L.or_apply
        f(self.h, l, _p(np.ascontiguousarray(x, np.float64)), _p(np.ascontiguousarray(u, np.float64)), _p(out))
        return out

    def inv_diag(self, l, x):
        out = np.zeros(self.ndof(l))
        self.L.or_inv_diag(self.h, l, _p(np.ascontiguousarray(x, np.float64)), _p(out))
        return out

    def restrict(self, l, fine):
        out = np.zeros(self.ndof(l + 1))
        self.L.or_restrict(self.h, l, _p(np.ascontiguousarray(fine, np.float64)), _p(out))
        return out

    def prolong(self, l, coarse):
        out = np.zeros(self.ndof(l))
        self.L.or_prolong(self.h, l, _p(np.ascontiguousarray(coarse, np.float64)), _p(out))
        return out

    def smooth(self, l, x, nswp, omega, b, u):
        invD = self.inv_diag(l, x)
        u = np.array(u, np.float64)
        tmp = np.zeros(self.ndof(l))
        self.L.or_smooth(self.h, l, _p(np.ascontiguousarray(x, np.float64)), nswp, omega, _p(invD),
                         _p(np.ascontiguousarray(b, np.float64)), _p(u), _p(tmp))
        return u

    def coarse_direct(self, l, x, rhs):
        sol = np.zeros(self.ndof(l))
        st = self.L.or_coarse_direct(self.h, l, _p(np.ascontiguousarray(x, np.float64)),
                                     _p(np.ascontiguousarray(rhs, np.float64)), _p(sol))
        return sol, st

    def solve(self, x, b, u0=None, nswp=4, tol=float(np.float32(1e-5))):
        u = np.zeros(self.ndof()) if u0 is None else np.array(u0, np.float64)
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0)
        st = self.L.or_solve(self.h, _p(np.ascontiguousarray(x, np.float64)),
                             _p(np.ascontiguousarray(b, np.float64)), _p(u), nswp, tol,
                             ctypes.byref(it), ctypes.byref(rr))
        return u, it.value, rr.value, st

    def compliance(self, x, u):
        dc = np.zeros(self.nelem())
        c = self.L.or_compliance(self.h, _p(np.ascontiguousarray(x, np.float64)),
                                 _p(np.ascontiguousarray(u, np.float64)), _p(dc))
        return c, dc

    def filter(self, rmin, x):
        out = np.zeros(self.nelem())
        self.L.or_filter(self.h, rmin, _p(np.ascontiguousarray(x, np.float64)), _p(out))
        return out

    def filter_T(self, rmin, v):
        v = np.array(v, np.float64)
        self.L.or_filter_T(self.h, rmin, _p(v))
        return v

    def oc_update(self, x, dv, dc, g):
        xnew = np.zeros(self.nelem())
        self.L.or_oc_update(self.h, _p(np.ascontiguousarray(x, np.float64)),
                            _p(np.ascontiguousarray(dv, np.float64)),
                            _p(np.ascontiguousarray(dc, np.float64)), g, _p(xnew))
        return xnew

    @staticmethod
    def run(nelx, nely, nelz, volfrac, rmin, nl, cgtol, iters, want_fields=False):
        L = Oracle.lib()
        h = _OrHistory()
        ne = nelx * nely * nelz
        xp = np.zeros(ne) if want_fields else None
        u = np.zeros(3 * nnodes(nelx, nely, nelz, 0)) if want_fields else None
        loops = L.or_run(nelx, nely, nelz, volfrac, rmin, nl, cgtol, iters, ctypes.byref(h), _p(xp), _p(u))
        hist = {
            "c": np.array(h.c[:loops]), "vol": np.array(h.vol[:loops]),
            "change": np.array(h.change[:loops]), "relres": np.array(h.relres[:loops]),
            "cgiters": np.array(h.cgiters[:loops]), "seconds": np.array(h.seconds[:loops]),
        }
        return loops, hist, xp, u


class Reference:
    """The reference's own C (oracle/_ref), called through oracle/ref_driver.c."""

    def __init__(self, nelx, nely, nelz, nl, flavour=64):
        path = os.path.join(HERE, "_ref", "libref%d.so" % flavour)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        V = ctypes.c_void_p
        L.ref_create.restype = V
        L.ref_create.argtypes = [ctypes.c_int] * 4
        L.ref_destroy.argtypes = [V]
        L.ref_ke.argtypes = [V, ctypes.c_int, _D]
        L.ref_fixed_dofs.restype = ctypes.c_int
        L.ref_fixed_dofs.argtypes = [V, ctypes.c_int, _L]
        for f in ("ref_matvec", "ref_matvec_csr"):
            getattr(L, f).argtypes = [V, ctypes.c_int, _D, _D, _D]
        L.ref_csr.restype = ctypes.c_long
        L.ref_csr.argtypes = [V, ctypes.c_int, _D, _I, _I, _D]
        L.ref_inv_diag.argtypes = [V, ctypes.c_int, _D, _D]
        L.ref_restrict.argtypes = [V, ctypes.c_int, _D, _D]
        L.ref_prolong.argtypes = [V, ctypes.c_int, _D, _D]
        L.ref_smooth.argtypes = [V, ctypes.c_int, _D, ctypes.c_int, ctypes.c_double, _D, _D]
        L.ref_compliance.argtypes = [V, _D, _D, _D, _D]
        L.ref_filter.argtypes = [V, ctypes.c_double, _D, _D]
        L.ref_filter_T.argtypes = [V, ctypes.c_double, _D]
        L.ref_oc_update.argtypes = [V, _D, _D, _D, ctypes.c_double, _D]
        L.ref_solve.argtypes = [V, _D, _D, _D, ctypes.c_int, ctypes.c_double, _I, _D]
        L.ref_load.argtypes = [V, _D]
        L.ref_run.restype = ctypes.c_int
        L.ref_run.argtypes = [ctypes.c_int] * 3 + [ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                                  ctypes.c_float, ctypes.c_int, _D, _D, _D, _I, _D, _D, _D]
        self.L = L
        self.shape = (nelx, nely, nelz)
        self.nl = nl
        self.h = L.ref_create(nelx, nely, nelz, nl)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_destroy(self.h)
            self.h = None

    def ndof(self, l=0):
        return 3 * nnodes(*self.shape, l)

    def nelem(self):
        nx, ny, nz = self.shape
        return nx * ny * nz

    def ke(self, l):
        out = np.zeros(576 * (1 << l) ** 3)
        self.L.ref_ke(self.h, l, _p(out))
        return out

    def fixed_dofs(self, l=0):
        n = self.L.ref_fixed_dofs(self.h, l, None)
        out = np.zeros(n, np.int64)
        self.L.ref_fixed_dofs(self.h, l, out.ctypes.data_as(_L))
        return out

    def load(self):
        F = np.zeros(self.ndof())
        self.L.ref_load(self.h, _p(F))
        return F

    def apply(self, l, x, u):
        out = np.zeros(self.ndof(l))
        self.L.ref_matvec(self.h, l, _p(np.ascontiguousarray(x, np.float64)),
                          _p(np.ascontiguousarray(u, np.float64)), _p(out))
        return out

    def apply_csr(self, l, x, u):
        out = np.zeros(self.ndof(l))
        self.L.ref_matvec_csr(self.h, l, _p(np.ascontiguousarray(x, np.float64)),
                              _p(np.ascontiguousarray(u, np.float64)), _p(out))
        return out

    def inv_diag(self, l, x):
        out = np.zeros(self.ndof(l))
        self.L.ref_inv_diag(self.h, l, _p(np.ascontiguousarray(x, np.float64)), _p(out))
        return out

    def restrict(self, l, fine):
        out = np.zeros(self.ndof(l + 1))
        self.L.ref_restrict(self.h, l, _p(np.ascontiguousarray(fine, np.float64)), _p(out))
        return out

    def prolong(self, l, coarse):
        out = np.zeros(self.ndof(l))
        self.L.ref_prolong(self.h, l, _p(np.ascontiguousarray(coarse, np.float64)), _p(out))
        return out

    def smooth(self, l, x, nswp, omega, b, u):
        u = np.array(u, np.float64)
        self.L.ref_smooth(self.h, l, _p(np.ascontiguousarray(x, np.float64)), nswp, omega,
                          _p(np.ascontiguousarray(b, np.float64)), _p(u))
        return u

    def compliance(self, x, u):
        c = np.zeros(1)
        dc = np.zeros(self.nelem())
        self.L.ref_compliance(self.h, _p(np.ascontiguousarray(x, np.float64)),
                              _p(np.ascontiguousarray(u, np.float64)), _p(c), _p(dc))
        return c[0], dc

    def filter(self, rmin, x):
        out = np.zeros(self.nelem())
        self.L.ref_filter(self.h, rmin, _p(np.ascontiguousarray(x, np.float64)), _p(out))
        return out

    def filter_T(self, rmin, v):
        v = np.array(v, np.float64)
        self.L.ref_filter_T(self.h, rmin, _p(v))
        return v

    def oc_update(self, x, dv, dc, g):
        xnew = np.zeros(self.nelem())
        self.L.ref_oc_update(self.h, _p(np.ascontiguousarray(x, np.float64)),
                             _p(np.ascontiguousarray(dv, np.float64)),
                             _p(np.ascontiguousarray(dc, np.float64)), g, _p(xnew))
        return xnew

    def solve(self, x, b, u0=None, nswp=4, tol=float(np.float32(1e-5))):
        u = np.zeros(self.ndof()) if u0 is None else np.array(u0, np.float64)
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0)
        self.L.ref_solve(self.h, _p(np.ascontiguousarray(x, np.float64)),
                         _p(np.ascontiguousarray(b, np.float64)), _p(u), nswp, tol,
                         ctypes.byref(it), ctypes.byref(rr))
        return u, it.value, rr.value

    def run(self, volfrac, rmin, cgtol, iters, want_fields=False):
        n = iters
        hc, hv, hch, hr = (np.zeros(n) for _ in range(4))
        hcg = np.zeros(n, np.int32)
        ne = self.nelem()
        xp = np.zeros(ne) if want_fields else None
        u = np.zeros(self.ndof()) if want_fields else None
        nelx, nely, nelz = self.shape
        loops = self.L.ref_run(nelx, nely, nelz, volfrac, rmin, self.nl, cgtol, iters,
                               _p(hc), _p(hv), _p(hch), hcg.ctypes.data_as(_I), _p(hr), _p(xp), _p(u))
        hist = {"c": hc[:loops], "vol": hv[:loops], "change": hch[:loops],
                "relres": hr[:loops], "cgiters": hcg[:loops].astype(np.int64)}
        return loops, hist, xp, u


class ReferenceBench:
    """Timing samples of the reference's own design iteration (oracle/_ref,
    ref_bench_* in oracle/ref_driver.c): the state of its loop on one grid,
    and the seconds of the iteration's fixed part (assembly, diagonals,
    coarse factor, initial residual, one CG iteration), of one more CG
    iteration and of the design update. A design iteration with n CG
    iterations costs fixed + (n - 1) * cg + design."""

    def __init__(self, nelx, nely, nelz, nl, volfrac, rmin, flavour=64):
        path = os.path.join(HERE, "_ref", "libref%d.so" % flavour)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        V = ctypes.c_void_p
        L.ref_bench_create.restype = V
        L.ref_bench_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_float, ctypes.c_float]
        L.ref_bench_destroy.argtypes = [V]
        for f in ("ref_bench_fixed", "ref_bench_cg"):
            getattr(L, f).restype = ctypes.c_double
            getattr(L, f).argtypes = [V]
        L.ref_bench_design.restype = ctypes.c_double
        L.ref_bench_design.argtypes = [V, _D]
        L.ref_bench_kernels.argtypes = [V, _D]
        self.L = L
        self.path = path
        self.h = L.ref_bench_create(nelx, nely, nelz, nl, volfrac, rmin)

    def close(self):
        if getattr(self, "h", None):
            self.L.ref_bench_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def fixed(self):
        return self.L.ref_bench_fixed(self.h)

    def cg(self):
        return self.L.ref_bench_cg(self.h)

    def design(self):
        c = np.zeros(1)
        t = self.L.ref_bench_design(self.h, _p(c))
        return t, float(c[0])

    KERNELS = ("fine_matvec", "level1_matvec", "restrict_0", "prolong_0", "inv_diag_0", "compliance",
               "filter", "filter_T")

    def kernels_ms(self):
        ms = np.zeros(len(self.KERNELS))
        self.L.ref_bench_kernels(self.h, _p(ms))
        return dict(zip(self.KERNELS, (float(v) for v in ms)))
