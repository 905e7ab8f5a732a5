"""ctypes binding of libtopopt_gb300 (the C ABI in include/topopt_gb300.h).

This is the host-side harness used by the tests and bench.py. Device arrays
are torch CUDA tensors (float64 unless a method says otherwise); torch only
provides the memory. Every call goes through the C ABI into the CUDA
kernels; if the shared library is missing the constructor raises, there is
no CPU fallback.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtopopt_gb300.so")

TP_FP64, TP_MIXED = 0, 1
FIELDS = {"x": 0, "xphys": 1, "xnew": 2, "dc": 3, "dv": 4, "F": 5, "U": 6}
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "allocation failed",
          4: "coarse matrix not positive definite", 5: "CG did not converge",
          6: "non-finite value", 7: "device wait timed out", 8: "call out of order"}


class TpParams(ctypes.Structure):
    _fields_ = [("nelx", ctypes.c_int), ("nely", ctypes.c_int), ("nelz", ctypes.c_int),
                ("nl", ctypes.c_int), ("volfrac", ctypes.c_double), ("rmin", ctypes.c_double),
                ("cgtol", ctypes.c_double), ("cgmax", ctypes.c_int), ("nswp", ctypes.c_int),
                ("omega", ctypes.c_double), ("precision", ctypes.c_int), ("nrhs", ctypes.c_int),
                ("device", ctypes.c_int)]


class TpIterInfo(ctypes.Structure):
    _fields_ = [("loop", ctypes.c_int), ("c", ctypes.c_double), ("vol", ctypes.c_double),
                ("change", ctypes.c_double), ("cgiters", ctypes.c_int), ("relres", ctypes.c_double),
                ("ms", ctypes.c_double)]


class TopOptError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


_lib = None


def load():
    """Loads the shared library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        import importlib.util
        spec = importlib.util.spec_from_file_location("tp_build", os.path.join(PKG, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = ctypes.CDLL(LIB_PATH)
    V, P, I, D = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.tp_default_params.argtypes = [ctypes.POINTER(TpParams)]
    L.tp_create.argtypes = [ctypes.POINTER(TpParams), ctypes.POINTER(V)]
    L.tp_destroy.argtypes = [V]
    L.tp_status_string.restype = ctypes.c_char_p
    L.tp_status_string.argtypes = [I]
    L.tp_error_message.restype = ctypes.c_char_p
    L.tp_error_message.argtypes = [V]
    L.tp_sync.argtypes = [V]
    L.tp_ndof.restype = ctypes.c_long
    L.tp_ndof.argtypes = [V, I]
    L.tp_nelem.restype = ctypes.c_long
    L.tp_nelem.argtypes = [V]
    L.tp_device_bytes.restype = ctypes.c_long
    L.tp_device_bytes.argtypes = [V]
    L.tp_field_ptr.restype = ctypes.c_void_p
    L.tp_field_ptr.argtypes = [V, I]
    L.tp_field_written.argtypes = [V, I]
    L.tp_upload.argtypes = [V, I, P, ctypes.c_long]
    L.tp_download.argtypes = [V, I, P, ctypes.c_long]
    L.tp_element_matrices.argtypes = [V, I, P]
    L.tp_fixed_dofs.argtypes = [V, I, P, ctypes.POINTER(ctypes.c_long)]
    L.tp_element_matrix_tables.argtypes = [I, D, P]
    L.tp_reference_load.argtypes = [I, I, I, P]
    for f in ("tp_assemble", "tp_init_design"):
        getattr(L, f).argtypes = [V]
    for f in ("tp_apply", "tp_apply_f32", "tp_restrict", "tp_prolong"):
        getattr(L, f).argtypes = [V, I, P, P]
    L.tp_inv_diag.argtypes = [V, I, P]
    L.tp_smooth.argtypes = [V, I, I, D, P, P]
    L.tp_coarse_solve.argtypes = [V, P, P]
    L.tp_vcycle.argtypes = [V, P, P]
    L.tp_solve.argtypes = [V, ctypes.POINTER(I), ctypes.POINTER(D)]
    L.tp_solve_rhs.argtypes = [V, P, P, ctypes.POINTER(I), ctypes.POINTER(D)]
    L.tp_compliance.argtypes = [V, ctypes.POINTER(D)]
    L.tp_element_sensitivity.argtypes = [V, P, P, P]
    L.tp_filter.argtypes = [V, P, P]
    L.tp_filter_T.argtypes = [V, P]
    L.tp_volume.argtypes = [V, ctypes.POINTER(D)]
    L.tp_oc_update.argtypes = [V, D, ctypes.POINTER(D)]
    L.tp_set_cg.argtypes = [V, D, I, I, D]
    L.tp_set_fine_variant.argtypes = [V, I]
    L.tp_set_fine_arith.argtypes = [V, I]
    L.tp_set_coarse_arith.argtypes = [V, I]
    L.tp_set_coarse_solve_variant.argtypes = [V, I]
    L.tp_set_coarse_order.argtypes = [V, I]
    L.tp_fault_coarse_barrier.argtypes = [V, ctypes.c_long, I]
    L.tp_autotune.argtypes = [V, P]
    L.tp_multiload.argtypes = [I, I, I, I, I, ctypes.c_ulonglong, P]
    L.tp_set_graph_solve.argtypes = [V, I]
    L.tp_set_device_loop.argtypes = [V, I]
    L.tp_get_fine_plan.argtypes = [V, I, I, P]
    L.tp_set_fine_plan.argtypes = [V, I, I, P]
    L.tp_fault_alloc.restype = ctypes.c_long
    L.tp_fault_alloc.argtypes = [ctypes.c_long]
    L.tp_coarse_factor_csr.argtypes = [V, ctypes.c_long, P, P, P]
    L.tp_coarse_solve_factored.argtypes = [V, P, P]
    L.tp_solve_columns.argtypes = [V, P, P]
    L.tp_checkpoint_save.argtypes = [V, ctypes.c_char_p, I]
    L.tp_checkpoint_load.argtypes = [V, ctypes.c_char_p, ctypes.POINTER(I)]
    L.tp_checkpoint_info.argtypes = [ctypes.c_char_p, P]
    L.tp_set_rmin.argtypes = [V, D]
    L.tp_design_iteration.argtypes = [V, ctypes.POINTER(TpIterInfo)]
    L.tp_run.argtypes = [V, I, ctypes.POINTER(TpIterInfo), ctypes.POINTER(I)]
    _lib = L
    return L


def checkpoint_info(path):
    """(nelx, nely, nelz, nl, nrhs, precision, loop) of a checkpoint file, or
    TopOptError if it is missing, truncated or corrupt."""
    info = np.zeros(7, np.int32)
    st = load().tp_checkpoint_info(os.fsencode(path), info.ctypes.data)
    if st != 0:
        raise TopOptError(st, "checkpoint " + str(path))
    return tuple(int(v) for v in info)


def multiload(nelx, nely, nelz, ncase, nload, seed=0):
    """ncase load cases of nload unit nodal forces on the end face x = nelx
    (tp_multiload), as an (ncase, ndof) float64 array."""
    L = load()
    ndof = 3 * (nelx + 1) * (nely + 1) * (nelz + 1)
    F = np.zeros((ncase, ndof))
    st = L.tp_multiload(nelx, nely, nelz, ncase, nload, seed, F.ctypes.data)
    if st != 0:
        raise TopOptError(st, "tp_multiload")
    return F


def fault_alloc(k):
    """Host-side fault injection: the k-th allocation of the library from now
    on fails (0 = off). Returns the number of live library allocations."""
    return load().tp_fault_alloc(k)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class TopOpt:
    """One device context: grid, multigrid hierarchy, design state."""

    def __init__(self, nelx, nely, nelz, nl, precision=TP_FP64, volfrac=None, rmin=1.5,
                 cgtol=None, cgmax=1000, nswp=4, omega=0.6, device=0, nrhs=1):
        self.L = load()
        p = TpParams()
        self.L.tp_default_params(ctypes.byref(p))
        p.nelx, p.nely, p.nelz, p.nl = nelx, nely, nelz, nl
        if volfrac is not None:
            p.volfrac = volfrac
        p.rmin = rmin
        if cgtol is not None:
            p.cgtol = cgtol
        p.cgmax, p.nswp, p.omega = cgmax, nswp, omega
        p.precision = precision
        p.device = device
        p.nrhs = nrhs
        self.nrhs = nrhs
        self.params = p
        self.ctx = ctypes.c_void_p()
        st = self.L.tp_create(ctypes.byref(p), ctypes.byref(self.ctx))
        if st != 0:
            msg = self.L.tp_error_message(self.ctx).decode() if self.ctx else ""
            if self.ctx:
                self.L.tp_destroy(self.ctx)
            self.ctx = None
            raise TopOptError(st, msg)
        self.shape = (nelx, nely, nelz)
        self.nl = nl

    def close(self):
        if getattr(self, "ctx", None):
            self.L.tp_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()

    def _check(self, st, allow=()):
        if st != 0 and st not in allow:
            raise TopOptError(st, self.L.tp_error_message(self.ctx).decode())
        return st

    # sizes
    def ndof(self, level=0):
        return self.L.tp_ndof(self.ctx, level)

    def nelem(self):
        return self.L.tp_nelem(self.ctx)

    def device_bytes(self):
        return self.L.tp_device_bytes(self.ctx)

    # fields
    def upload(self, name, arr):
        a = np.ascontiguousarray(arr, np.float64)
        self._check(self.L.tp_upload(self.ctx, FIELDS[name], a.ctypes.data_as(ctypes.c_void_p), a.size))

    def download(self, name):
        n = self.nelem() if name not in ("F", "U") else self.ndof(0) * self.nrhs
        out = np.zeros(n)
        self._check(self.L.tp_download(self.ctx, FIELDS[name], out.ctypes.data_as(ctypes.c_void_p), n))
        return out

    def field(self, name):
        """Device pointer (int) of a context field."""
        return self.L.tp_field_ptr(self.ctx, FIELDS[name])

    def element_matrices(self, level):
        out = np.zeros(576 * 8 ** level)
        self._check(self.L.tp_element_matrices(self.ctx, level, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def fixed_dofs(self, level):
        n = ctypes.c_long(0)
        self._check(self.L.tp_fixed_dofs(self.ctx, level, None, ctypes.byref(n)))
        out = np.zeros(n.value, np.int64)
        self._check(self.L.tp_fixed_dofs(self.ctx, level, out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n)))
        return out

    def set_cg(self, cgtol, cgmax=1000, nswp=4, omega=0.6):
        self._check(self.L.tp_set_cg(self.ctx, cgtol, cgmax, nswp, omega))

    def set_fine_variant(self, variant):
        """0: element-centric level-0 kernel where it applies; 1: node-centric stencil."""
        self._check(self.L.tp_set_fine_variant(self.ctx, variant))

    def set_fine_arith(self, arith):
        """Level-0 kernel on double vectors: 0 FP64; 1 double-single (default in the mixed form)."""
        self._check(self.L.tp_set_fine_arith(self.ctx, arith))

    def set_coarse_arith(self, arith):
        """Coarsest-level Cholesky: 0 FP64; 1 double-single (default in the mixed form)."""
        self._check(self.L.tp_set_coarse_arith(self.ctx, arith))

    def set_coarse_solve_variant(self, variant):
        """0: coarse triangular sweeps in one cooperative launch; 1: two launches per block step."""
        self._check(self.L.tp_set_coarse_solve_variant(self.ctx, variant))

    def set_coarse_order(self, order):
        """Coarsest-level elimination order: 0 natural band; 1 nested dissection (default);
        2 nested dissection with the halves' sweeps one after the other."""
        self._check(self.L.tp_set_coarse_order(self.ctx, order))

    def fault_coarse_barrier(self, spin, missing):
        """Failure-detection hook: barrier waits give up after spin polls; missing=1 makes them run out."""
        self._check(self.L.tp_fault_coarse_barrier(self.ctx, spin, missing))

    def checkpoint_save(self, path, loop):
        self._check(self.L.tp_checkpoint_save(self.ctx, os.fsencode(path), loop))

    def checkpoint_load(self, path):
        """Restores x, xPhys, U, F; returns the saved design-iteration number."""
        loop = ctypes.c_int(0)
        self._check(self.L.tp_checkpoint_load(self.ctx, os.fsencode(path), ctypes.byref(loop)))
        return loop.value

    def solve_columns(self):
        """(iteration index, relres) of each load case in the last solve."""
        it = np.zeros(self.nrhs, np.int32)
        rr = np.zeros(self.nrhs)
        self._check(self.L.tp_solve_columns(self.ctx, it.ctypes.data, rr.ctypes.data))
        return it, rr

    def set_graph_solve(self, on):
        """1: the CG loop runs as one CUDA graph launch also for a single load."""
        self._check(self.L.tp_set_graph_solve(self.ctx, int(on)))

    def set_device_loop(self, on):
        """1 (default): one host wait per design iteration (graph-launched CG loop
        and OC bisection); 0: host-driven as the reference."""
        self._check(self.L.tp_set_device_loop(self.ctx, int(on)))

    def coarse_factor_csr(self, rowptr, col, val):
        """Band-Cholesky factor of a host CSR of the coarsest level; returns the
        status (0, or 4 for a non-positive pivot) without raising."""
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        return self.L.tp_coarse_factor_csr(self.ctx, len(rowptr) - 1, rowptr.ctypes.data, col.ctypes.data,
                                           val.ctypes.data)

    def coarse_solve_factored(self, rhs):
        import torch
        out = torch.empty_like(rhs)
        self._check(self.L.tp_coarse_solve_factored(self.ctx, _ptr(rhs), _ptr(out)))
        return out

    def fine_plan(self, vec, mode):
        """Level-0 launch plan (groups, x chunks, b/invD staging, register cap,
        packed, E staged, threads in y) for vec 0 = FP32 / 1 = double vectors, mode 0-3."""
        plan = np.zeros(7, np.int32)
        self._check(self.L.tp_get_fine_plan(self.ctx, vec, mode, plan.ctypes.data))
        return [int(v) for v in plan]

    def set_fine_plan(self, vec, mode, plan):
        """Sets a level-0 launch plan (groups, x chunks, staging, register cap, packed,
        E staged); returns the status (1 if the plan does not apply)."""
        p = list(plan[:6]) + [1] * (6 - len(plan[:6]))
        a = np.ascontiguousarray(p, np.int32)
        return self.L.tp_set_fine_plan(self.ctx, vec, mode, a.ctypes.data)

    def autotune(self):
        """Tunes the level-0 launch shapes; returns the best ms per (f32, f64) x mode."""
        ms = np.zeros(8)
        self._check(self.L.tp_autotune(self.ctx, ms.ctypes.data))
        return ms

    def set_rmin(self, rmin):
        self._check(self.L.tp_set_rmin(self.ctx, rmin))

    def set_field(self, name, t):
        """Copies a float64 tensor (any device) into a context field."""
        self.upload(name, t.detach().cpu().numpy())

    # operators on torch CUDA tensors
    def assemble(self):
        self._check(self.L.tp_assemble(self.ctx))

    def apply(self, level, u):
        import torch
        out = torch.empty_like(u)
        f = self.L.tp_apply_f32 if u.dtype == torch.float32 else self.L.tp_apply
        self._check(f(self.ctx, level, _ptr(u), _ptr(out)))
        return out

    def inv_diag(self, level):
        import torch
        out = torch.empty(self.ndof(level), dtype=torch.float64, device="cuda")
        self._check(self.L.tp_inv_diag(self.ctx, level, _ptr(out)))
        return out

    def restrict(self, level, fine):
        import torch
        out = torch.empty(self.ndof(level + 1), dtype=torch.float64, device="cuda")
        self._check(self.L.tp_restrict(self.ctx, level, _ptr(fine), _ptr(out)))
        return out

    def prolong(self, level, coarse):
        import torch
        out = torch.empty(self.ndof(level), dtype=torch.float64, device="cuda")
        self._check(self.L.tp_prolong(self.ctx, level, _ptr(coarse), _ptr(out)))
        return out

    def smooth(self, level, nswp, omega, b, u):
        u = u.clone()
        self._check(self.L.tp_smooth(self.ctx, level, nswp, omega, _ptr(b), _ptr(u)))
        return u

    def coarse_solve(self, rhs):
        import torch
        out = torch.empty_like(rhs)
        self._check(self.L.tp_coarse_solve(self.ctx, _ptr(rhs), _ptr(out)))
        return out

    def vcycle(self, r):
        import torch
        z = torch.empty_like(r)
        self._check(self.L.tp_vcycle(self.ctx, _ptr(r), _ptr(z)))
        return z

    def solve(self):
        it, rr = ctypes.c_int(0), ctypes.c_double(0)
        st = self._check(self.L.tp_solve(self.ctx, ctypes.byref(it), ctypes.byref(rr)), allow=(5,))
        return it.value, rr.value, st

    def solve_rhs(self, rhs, x0=None):
        import torch
        sol = torch.zeros_like(rhs) if x0 is None else x0.clone()
        it, rr = ctypes.c_int(0), ctypes.c_double(0)
        st = self._check(self.L.tp_solve_rhs(self.ctx, _ptr(rhs), _ptr(sol), ctypes.byref(it),
                                             ctypes.byref(rr)), allow=(5,))
        return sol, it.value, rr.value, st

    def compliance(self):
        c = ctypes.c_double(0)
        self._check(self.L.tp_compliance(self.ctx, ctypes.byref(c)))
        return c.value

    def element_sensitivity(self, u, w):
        import torch
        out = torch.empty(self.nelem(), dtype=torch.float64, device="cuda")
        self._check(self.L.tp_element_sensitivity(self.ctx, _ptr(u), _ptr(w), _ptr(out)))
        return out

    def filter(self, x):
        import torch
        out = torch.empty_like(x)
        self._check(self.L.tp_filter(self.ctx, _ptr(x), _ptr(out)))
        return out

    def filter_T(self, v):
        v = v.clone()
        self._check(self.L.tp_filter_T(self.ctx, _ptr(v)))
        return v

    def volume(self):
        v = ctypes.c_double(0)
        self._check(self.L.tp_volume(self.ctx, ctypes.byref(v)))
        return v.value

    def oc_update(self, g):
        ch = ctypes.c_double(0)
        self._check(self.L.tp_oc_update(self.ctx, g, ctypes.byref(ch)))
        return ch.value

    def init_design(self):
        self._check(self.L.tp_init_design(self.ctx))

    def design_iteration(self):
        info = TpIterInfo()
        self._check(self.L.tp_design_iteration(self.ctx, ctypes.byref(info)))
        return info

    def run(self, max_iterations):
        hist = (TpIterInfo * max(1, max_iterations))()
        loops = ctypes.c_int(0)
        self._check(self.L.tp_run(self.ctx, max_iterations, hist, ctypes.byref(loops)))
        return [hist[i] for i in range(loops.value)]


# ---------------------------------------------------------------------------
# The reference-signature drop-in libraries (include/topopt_ref_api.h):
# ctypes mirrors of the reference's structs (definitions.h:31-53,
# gpu_definitions.h:7-37, stencil_assembly.h:8-27) and of its padded host
# layout (gpu_definitions.c:67-92).
UF = ctypes.c_ulong  # uint_fast32_t on LP64 glibc (x86_64 and aarch64)


class FixedDofs(ctypes.Structure):
    _fields_ = [("n", UF), ("idx", ctypes.POINTER(UF))]


class GridContext(ctypes.Structure):
    _fields_ = [("E0", ctypes.c_double), ("Emin", ctypes.c_double), ("nu", ctypes.c_double),
                ("esx", ctypes.c_double), ("esy", ctypes.c_double), ("esz", ctypes.c_double),
                ("nelx", UF), ("nely", UF), ("nelz", UF), ("wrapx", UF), ("wrapy", UF), ("wrapz", UF),
                ("penal", ctypes.c_double), ("precomputedKE", ctypes.POINTER(ctypes.POINTER(ctypes.c_double))),
                ("fixedDofs", ctypes.POINTER(FixedDofs))]


class GpuNode(ctypes.Structure):
    pass


GpuNode._fields_ = [("id", ctypes.c_int), ("prev", ctypes.POINTER(GpuNode)), ("next", ctypes.POINTER(GpuNode)),
                    ("gc", ctypes.POINTER(GridContext)), ("offset_x", ctypes.c_int), ("x_global", ctypes.c_int)]


class GpuGrid(ctypes.Structure):
    _fields_ = [("num_targets", ctypes.c_int), ("target", ctypes.POINTER(GpuNode))]


class CSR(ctypes.Structure):
    _fields_ = [("nnz", ctypes.c_uint64), ("nrows", ctypes.c_int32), ("rowOffsets", ctypes.POINTER(ctypes.c_int)),
                ("colIndex", ctypes.POINTER(ctypes.c_int)), ("vals", ctypes.POINTER(ctypes.c_double))]


def padded_dims(nelx, nely, nelz, level=0):
    """(ex, ey, ez, wrapx, wrapy, wrapz) of a level in the reference's padded
    layout: a one-node halo on every side, y padded to a multiple of 128."""
    ex, ey, ez = nelx >> level, nely >> level, nelz >> level
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


def load_ref_api(flavour=64):
    """libtopopt_ref<flavour>.so with argument types for the entry points of
    the reference's design loop (stencil_optimization.c:13-223)."""
    load()
    L = ctypes.CDLL(os.path.join(PKG, "libtopopt_ref%d.so" % flavour))
    P, D, I = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
    R = D if flavour == 64 else ctypes.c_float
    L.setupGC.argtypes = [ctypes.POINTER(GridContext), I, I, I, I]
    L.freeGC.argtypes = [ctypes.POINTER(GridContext), I]
    L.gridContextToGPUGrid.argtypes = [ctypes.POINTER(GridContext), ctypes.POINTER(GpuGrid), I, I]
    L.freeGPUGrid.argtypes = [ctypes.POINTER(GpuGrid), I]
    L.solveStateMG_halo.argtypes = [ctypes.POINTER(GpuGrid), P, I, I, R, P, ctypes.POINTER(I),
                                    ctypes.POINTER(ctypes.c_float), P, P]
    L.compute_volume.restype = R
    L.compute_volume.argtypes = [GridContext, P]
    L.getComplianceAndSensetivity_halo.argtypes = [ctypes.POINTER(GpuNode), P, P, P, P]
    L.applyDensityFilterGradient.argtypes = [GridContext, R, P]
    L.applyDensityFilter.argtypes = [GridContext, R, P, P]
    L.update_solution.argtypes = [P, P, P, P, I, R]
    L.compute_change.restype = ctypes.c_float
    L.compute_change.argtypes = [P, P, I]
    L.topopt_ref_transfer_bytes.argtypes = [ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long), I]
    return L


class RefLoop:
    """The reference's design loop body (stencil_optimization.c:148-189)
    through the drop-in entry points, on host arrays in the reference's padded
    layout: the caller of the reference's C API, unchanged. FP64 flavour."""

    def __init__(self, nelx, nely, nelz, nl, volfrac, rmin, cgtol):
        self.L = load_ref_api(64)
        self.nl, self.volfrac, self.rmin, self.cgtol = nl, volfrac, rmin, cgtol
        self.gc = GridContext()
        self.L.setupGC(ctypes.byref(self.gc), nl, nelx, nely, nelz)
        self.gpu = GpuGrid()
        self.gpu.num_targets = 1
        self.L.gridContextToGPUGrid(ctypes.byref(self.gc), ctypes.byref(self.gpu), nl, 0)
        self.dims = padded_dims(nelx, nely, nelz, 0)
        ex, ey, ez, wx, wy, wz = self.dims
        self.nelem_padded = (wx - 1) * (wy - 1) * (wz - 1)
        self.nelem = nelx * nely * nelz
        F = np.zeros(3 * (nelx + 1) * (nely + 1) * (nelz + 1))
        load().tp_reference_load(nelx, nely, nelz, F.ctypes.data)
        self.F = vec_to_padded(F, self.dims)
        self.dv = np.ones(self.nelem_padded)
        self.L.applyDensityFilterGradient(self.gc, rmin, self.dv.ctypes.data)
        self.reset()

    def reset(self):
        """x = xPhys = volfrac on the real elements, U = 0 (:97-137). The
        arrays are allocated once and refilled, as the reference's loop
        allocates them once: a device copy into pages that were never
        touched waits on their first faults."""
        x0 = el_to_padded(self.volfrac * np.ones(self.nelem), self.dims)
        if getattr(self, "x", None) is None:
            self.x, self.xPhys = np.empty_like(x0), np.empty_like(x0)
            self.xnew, self.dc = np.empty(self.nelem_padded), np.empty(self.nelem_padded)
            self.U = np.empty_like(self.F)
        np.copyto(self.x, x0)
        np.copyto(self.xPhys, x0)
        self.xnew.fill(0.0)
        self.dc.fill(0.0)
        self.U.fill(0.0)

    def iteration(self):
        L = self.L
        it, res, c = ctypes.c_int(0), ctypes.c_float(0), ctypes.c_double(0)
        L.solveStateMG_halo(ctypes.byref(self.gpu), self.xPhys.ctypes.data, 4, self.nl, self.cgtol, None,
                            ctypes.byref(it), ctypes.byref(res), self.F.ctypes.data, self.U.ctypes.data)
        vol = L.compute_volume(self.gc, self.xPhys.ctypes.data)
        L.getComplianceAndSensetivity_halo(self.gpu.target, self.xPhys.ctypes.data, self.U.ctypes.data,
                                           ctypes.byref(c), self.dc.ctypes.data)
        L.applyDensityFilterGradient(self.gc, self.rmin, self.dc.ctypes.data)
        vol /= float(self.nelem)
        g = vol - self.volfrac
        L.update_solution(self.x.ctypes.data, self.xnew.ctypes.data, self.dv.ctypes.data, self.dc.ctypes.data,
                          self.nelem_padded, g)
        change = L.compute_change(self.x.ctypes.data, self.xnew.ctypes.data, self.nelem_padded)
        L.applyDensityFilter(self.gc, self.rmin, self.x.ctypes.data, self.xPhys.ctypes.data)
        return {"c": c.value, "vol": vol, "change": change, "cgiters": it.value}

    def transfer_bytes(self, reset=False):
        h, d = ctypes.c_long(0), ctypes.c_long(0)
        self.L.topopt_ref_transfer_bytes(ctypes.byref(h), ctypes.byref(d), 1 if reset else 0)
        return h.value, d.value

    def close(self):
        if getattr(self, "gc", None) is not None:
            self.L.freeGPUGrid(ctypes.byref(self.gpu), self.nl)
            self.L.freeGC(ctypes.byref(self.gc), self.nl)
            self.gc = None
