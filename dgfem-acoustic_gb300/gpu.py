"""ctypes binding of the GPU solver C ABI (include/dgfem_gb300.h).

The binding loads the in-tree libdgfem_gb300.so and fails loudly when it is
missing or when no CUDA device is usable; there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libdgfem_gb300.so")
_lib = None

DG_FP64, DG_FP32 = 0, 1
ERRORS = {1: "DG_ERR_ARG", 2: "DG_ERR_CUDA", 3: "DG_ERR_MESH", 4: "DG_ERR_NONFINITE", 5: "DG_ERR_TIMEOUT"}

# Every entry point declared in include/dgfem_gb300.h.
SYMBOLS = ["dg_create", "dg_destroy", "dg_last_error", "dg_get_info", "dg_set_state", "dg_get_state",
           "dg_set_sources", "dg_set_source_values", "dg_set_observers", "dg_snapshot", "dg_run", "dg_run_euler",
           "dg_step_index", "dg_set_step_index", "dg_rhs", "dg_cell_means", "dg_face_info", "dg_stream",
           "dg_bench_steps", "dg_set_wait_limit", "dg_tune", "dg_tune_cache_stats", "dg_tune_cache_clear", "dg_host_alloc", "dg_host_free", "dg_kernel_info", "dg_vtu_writer_create", "dg_vtu_write_async",
           "dg_vtu_writer_flush", "dg_vtu_writer_destroy", "dg_vtu_writer_last_error", "dg_vtu_writer_stats", "dg_residuals_noalloc", "dg_batch_create", "dg_batch_destroy",
           "dg_batch_last_error", "dg_batch_info", "dg_batch_set_state", "dg_batch_get_state",
           "dg_batch_set_sources", "dg_batch_set_observers", "dg_batch_run", "dg_batch_bench", "dg_batch_set_fused",
           "dg_batch_fused",
           "dg_mlp_create", "dg_mlp_destroy", "dg_mlp_last_error", "dg_mlp_param_count", "dg_mlp_set_params",
           "dg_mlp_get_params", "dg_mlp_forward", "dg_mlp_forward_device", "dg_mlp_gradient", "dg_mlp_set_data",
           "dg_mlp_train", "dg_mlp_set_tensor_cores", "dg_mlp_tensor_cores"]


class MeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("order", C.c_int), ("nodes_per_elem", C.c_int),
                ("n_nodes", C.c_int64), ("xyz", C.POINTER(C.c_double)),
                ("n_elems", C.c_int64), ("elem_nodes", C.POINTER(C.c_int64)),
                ("n_groups", C.c_int), ("group_bc", C.POINTER(C.c_int)),
                ("group_offsets", C.POINTER(C.c_int64)), ("group_nodes", C.POINTER(C.c_int64))]


class Phys(C.Structure):
    _fields_ = [("v0", C.c_double * 3), ("rho0", C.c_double), ("c0", C.c_double)]


class Info(C.Structure):
    _fields_ = [("dim", C.c_int), ("order", C.c_int), ("nodes_per_elem", C.c_int), ("n_var", C.c_int),
                ("precision", C.c_int), ("n_elems", C.c_int64), ("n_faces", C.c_int64),
                ("n_boundary_faces", C.c_int64), ("penalty_sign_hist", C.c_int64 * 2),
                ("device_bytes", C.c_int64), ("setup_ms", C.c_double), ("kernel_variant", C.c_int), ("kernel_grid", C.c_int),
                ("n_curved", C.c_int64)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("GPU solver library not built: %s (run __graft_entry__.build())" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        P, D, I64 = C.POINTER, C.c_double, C.c_int64
        L.dg_create.argtypes = [P(MeshDesc), P(Phys), C.c_int, C.c_int, P(C.c_void_p)]
        L.dg_destroy.argtypes = [C.c_void_p]
        L.dg_last_error.argtypes = [C.c_void_p]
        L.dg_last_error.restype = C.c_char_p
        L.dg_get_info.argtypes = [C.c_void_p, P(Info)]
        L.dg_set_state.argtypes = [C.c_void_p, P(D)]
        L.dg_get_state.argtypes = [C.c_void_p, P(D)]
        L.dg_set_sources.argtypes = [C.c_void_p, C.c_int, P(I64), P(I64)]
        L.dg_set_source_values.argtypes = [C.c_void_p, I64, P(D)]
        L.dg_set_observers.argtypes = [C.c_void_p, C.c_int, P(I64), P(I64), P(D)]
        L.dg_snapshot.argtypes = [C.c_void_p]
        L.dg_run.argtypes = [C.c_void_p, I64, D, P(D), P(D)]
        L.dg_run_euler.argtypes = [C.c_void_p, I64, D, P(D), P(D)]
        L.dg_step_index.argtypes = [C.c_void_p]
        L.dg_step_index.restype = I64
        L.dg_set_step_index.argtypes = [C.c_void_p, I64]
        L.dg_rhs.argtypes = [C.c_void_p, P(D), D, P(D)]
        L.dg_cell_means.argtypes = [C.c_void_p, P(D), P(D), P(D)]
        L.dg_face_info.argtypes = [C.c_void_p, P(I64), P(C.c_int), P(C.c_int)]
        L.dg_stream.argtypes = [C.c_void_p]
        L.dg_stream.restype = C.c_void_p
        L.dg_bench_steps.argtypes = [C.c_void_p, I64, D, I64, P(D), P(D)]
        L.dg_tune.argtypes = [C.c_void_p, C.c_int]
        L.dg_set_wait_limit.argtypes = [C.c_void_p, C.c_int]
        L.dg_tune_cache_stats.argtypes = [P(I64), P(I64), P(I64)]
        L.dg_vtu_writer_create.argtypes = [C.c_void_p, I64, P(D), P(I64), C.c_int, C.c_int, P(C.c_void_p)]
        L.dg_vtu_write_async.argtypes = [C.c_void_p, C.c_char_p]
        L.dg_vtu_writer_flush.argtypes = [C.c_void_p]
        L.dg_vtu_writer_destroy.argtypes = [C.c_void_p]
        L.dg_vtu_writer_last_error.argtypes = [C.c_void_p]
        L.dg_vtu_writer_last_error.restype = C.c_char_p
        L.dg_vtu_writer_stats.argtypes = [C.c_void_p, P(I64), P(C.c_int)]
        L.dg_host_alloc.argtypes = [C.c_size_t, P(C.c_void_p)]
        L.dg_host_free.argtypes = [C.c_void_p]
        L.dg_tune_cache_clear.argtypes = []
        L.dg_tune_cache_clear.restype = None
        L.dg_kernel_info.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
        L.dg_residuals_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, I64, I64, D, C.c_void_p,
                                           C.c_void_p]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64)) if a is not None else None


def _csr(lists, dtype=np.int64):
    off = np.zeros(len(lists) + 1, dtype=np.int64)
    for i, l in enumerate(lists):
        off[i + 1] = off[i] + len(l)
    flat = np.concatenate([np.asarray(l, dtype=dtype) for l in lists]) if off[-1] > 0 else np.zeros(1, dtype)
    return off, np.ascontiguousarray(flat)


class SolverError(RuntimeError):
    pass


def pinned_empty(shape, dtype=np.float64):
    """Uninitialised numpy array in page-locked host memory (dg_host_alloc),
    freed when the array is garbage-collected."""
    import weakref
    dtype = np.dtype(dtype)
    n = int(np.prod(shape))
    ptr = C.c_void_p()
    rc = lib().dg_host_alloc(max(1, n) * dtype.itemsize, C.byref(ptr))
    if rc != 0:
        raise SolverError("dg_host_alloc: %s" % ERRORS.get(rc, rc))
    buf = (C.c_char * (max(1, n) * dtype.itemsize)).from_address(ptr.value)
    weakref.finalize(buf, lib().dg_host_free, ptr.value)
    return np.frombuffer(buf, dtype=dtype, count=n).reshape(shape)


def tune_cache_stats():
    """(hits, misses, entries) of the autotuner's process-wide result cache."""
    h, m, n = C.c_int64(), C.c_int64(), C.c_int64()
    lib().dg_tune_cache_stats(C.byref(h), C.byref(m), C.byref(n))
    return h.value, m.value, n.value


def tune_cache_clear():
    """Forgets the cache's in-process entries and counters."""
    lib().dg_tune_cache_clear()


def residuals_noalloc(u_ptr, snap_ptr, precision, n_var, n_per_var, var_stride, c0, res_ptr, stream=None):
    """dg_residuals_noalloc on caller-owned device pointers (ints); raises on error."""
    L = lib()
    rc = L.dg_residuals_noalloc(C.c_void_p(u_ptr), C.c_void_p(snap_ptr), precision, n_var, n_per_var, var_stride,
                                c0, C.c_void_p(res_ptr), C.c_void_p(stream) if stream else None)
    if rc != 0:
        raise SolverError("dg_residuals_noalloc: %s: %s" % (ERRORS.get(rc, rc), L.dg_last_error(None).decode()))


class Solver:
    """One solver context on one GPU (see include/dgfem_gb300.h)."""

    def __init__(self, mesh, v0=(0.0, 0.0, 0.0), rho0=1.0, c0=1.0, precision=DG_FP64, device=0):
        L = lib()
        xyz = np.ascontiguousarray(mesh["xyz"], dtype=np.float64)
        en = np.ascontiguousarray(mesh["elem_nodes"], dtype=np.int64)
        groups = mesh.get("groups", [])
        gbc = np.array([g[0] for g in groups] or [0], dtype=np.int32)
        goff, gn = _csr([g[1] for g in groups])
        d = MeshDesc()
        d.dim, d.order, d.nodes_per_elem = mesh["dim"], mesh["order"], en.shape[1]
        d.n_nodes, d.xyz = xyz.shape[0], _dp(xyz)
        d.n_elems, d.elem_nodes = en.shape[0], _ip(en)
        d.n_groups, d.group_bc = len(groups), gbc.ctypes.data_as(C.POINTER(C.c_int))
        d.group_offsets, d.group_nodes = _ip(goff), _ip(gn)
        ph = Phys()
        ph.v0 = (C.c_double * 3)(*v0)
        ph.rho0, ph.c0 = rho0, c0
        h = C.c_void_p()
        rc = L.dg_create(C.byref(d), C.byref(ph), precision, device, C.byref(h))
        if rc != 0:
            raise SolverError("dg_create: %s: %s" % (ERRORS.get(rc, rc), L.dg_last_error(None).decode()))
        self.h = h
        self.E, self.np_, self.dim = en.shape[0], en.shape[1], mesh["dim"]
        self.n_obs = 0

    def close(self):
        if getattr(self, "h", None):
            lib().dg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc != 0:
            raise SolverError("%s: %s: %s" % (what, ERRORS.get(rc, rc), lib().dg_last_error(self.h).decode()))

    @property
    def ndof(self):
        return self.E * self.np_

    def info(self):
        i = Info()
        self._ck(lib().dg_get_info(self.h, C.byref(i)), "dg_get_info")
        return {k: (tuple(getattr(i, k)) if k == "penalty_sign_hist" else getattr(i, k)) for k, _ in Info._fields_}

    def set_state(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(4, self.ndof)
        self._ck(lib().dg_set_state(self.h, _dp(u)), "dg_set_state")

    def get_state(self, out=None):
        """State [4][E*Np] in the reference layout; into `out` (float64,
        C-contiguous, e.g. from pinned_empty) when given."""
        if out is None:
            out = np.zeros((4, self.ndof))
        elif out.dtype != np.float64 or not out.flags.c_contiguous or out.size != 4 * self.ndof:
            raise ValueError("out must be a C-contiguous float64 array of 4 * E * Np values")
        self._ck(lib().dg_get_state(self.h, _dp(out)), "dg_get_state")
        return out

    def rhs(self, u, dt):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(4, self.ndof)
        k = np.zeros_like(u)
        self._ck(lib().dg_rhs(self.h, _dp(u), dt, _dp(k)), "dg_rhs")
        return k

    def set_sources(self, dof_lists):
        off, flat = _csr(dof_lists)
        self._ck(lib().dg_set_sources(self.h, len(dof_lists), _ip(off), _ip(flat)), "dg_set_sources")

    def set_source_values(self, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._ck(lib().dg_set_source_values(self.h, v.shape[0], _dp(v)), "dg_set_source_values")

    def set_observers(self, dof_lists, weight_lists):
        off, flat = _csr(dof_lists)
        _, w = _csr(weight_lists, np.float64)
        self._ck(lib().dg_set_observers(self.h, len(dof_lists), _ip(off), _ip(flat), _dp(w)), "dg_set_observers")
        self.n_obs = len(dof_lists)

    def snapshot(self):
        self._ck(lib().dg_snapshot(self.h), "dg_snapshot")

    def run(self, n_steps, dt, euler=False):
        res = np.zeros((max(n_steps, 1), 5))
        obs = np.zeros((max(n_steps, 1), max(self.n_obs, 1), 4))
        fn = lib().dg_run_euler if euler else lib().dg_run
        self._ck(fn(self.h, n_steps, dt, _dp(res), _dp(obs)), "dg_run")
        return res[:n_steps], obs[:n_steps, :self.n_obs]

    @property
    def step(self):
        return lib().dg_step_index(self.h)

    @step.setter
    def step(self, s):
        self._ck(lib().dg_set_step_index(self.h, s), "dg_set_step_index")

    def cell_means(self):
        p, rho, v = np.zeros(self.E), np.zeros(self.E), np.zeros((self.E, 3))
        self._ck(lib().dg_cell_means(self.h, _dp(p), _dp(rho), _dp(v)), "dg_cell_means")
        return p, rho, v

    def face_info(self):
        nf = self.dim + 1
        nbr = np.zeros(self.E * nf, np.int64)
        pen = np.zeros(self.E * nf, np.int32)
        bc = np.zeros(self.E * nf, np.int32)
        self._ck(lib().dg_face_info(self.h, _ip(nbr), pen.ctypes.data_as(C.POINTER(C.c_int)),
                                    bc.ctypes.data_as(C.POINTER(C.c_int))), "dg_face_info")
        return dict(nbr=nbr.reshape(-1, nf), penalty=pen.reshape(-1, nf), bc=bc.reshape(-1, nf))

    def kernel_info(self, variant):
        """(elements per tile, threads, shared bytes, blocks per SM, grid) of a
        stage-kernel variant; elements per tile 0 = not available."""
        out = (C.c_int * 5)()
        self._ck(lib().dg_kernel_info(self.h, variant, out), "dg_kernel_info")
        return tuple(out)

    def tune(self, variant=-2):
        """-2 times every stage-kernel variant on this mesh and keeps the
        fastest, -3 takes a cached result where one exists, -1 / k >= 0 force
        the baseline or variant k."""
        self._ck(lib().dg_tune(self.h, variant), "dg_tune")
        return self.info()["kernel_variant"]

    def set_wait_limit(self, rounds):
        """Polling rounds of each bounded device wait before it gives up
        (default 2**20); a run whose wait gives up raises DG_ERR_TIMEOUT."""
        self._ck(lib().dg_set_wait_limit(self.h, rounds), "dg_set_wait_limit")

    def stream(self):
        return lib().dg_stream(self.h)

    def bench_steps(self, n_steps, dt, flush_bytes=0, kernel_time=True):
        sm, km = C.c_double(), C.c_double()
        self._ck(lib().dg_bench_steps(self.h, n_steps, dt, flush_bytes, C.byref(sm),
                                      C.byref(km) if kernel_time else None), "dg_bench_steps")
        return sm.value, (km.value if kernel_time else None)


def _batch_lib():
    L = lib()
    if getattr(L, "_batch", False):
        return L
    P, D, I64 = C.POINTER, C.c_double, C.c_int64
    L.dg_batch_create.argtypes = [C.c_int, P(MeshDesc), P(Phys), P(D), C.c_int, C.c_int, P(C.c_void_p)]
    L.dg_batch_destroy.argtypes = [C.c_void_p]
    L.dg_batch_last_error.argtypes = [C.c_void_p]
    L.dg_batch_last_error.restype = C.c_char_p
    L.dg_batch_info.argtypes = [C.c_void_p, P(C.c_int), P(I64)]
    L.dg_batch_set_state.argtypes = [C.c_void_p, C.c_int, P(D)]
    L.dg_batch_get_state.argtypes = [C.c_void_p, C.c_int, P(D)]
    L.dg_batch_set_sources.argtypes = [C.c_void_p, C.c_int, C.c_int, P(I64), P(I64), I64, P(D)]
    L.dg_batch_set_observers.argtypes = [C.c_void_p, C.c_int, C.c_int, P(I64), P(I64), P(D)]
    L.dg_batch_run.argtypes = [C.c_void_p, I64, P(D)]
    L.dg_batch_bench.argtypes = [C.c_void_p, I64, P(D)]
    L.dg_batch_set_fused.argtypes = [C.c_void_p, C.c_int]
    L.dg_batch_fused.argtypes = [C.c_void_p]
    L._batch = True
    return L


class VtuWriter:
    """Asynchronous VTU snapshots of a Solver's state (dg_vtu_*): points
    [n][3] and cells [E][dim+1] (corner point indices) describe the VTK mesh;
    write(path) returns once the cell means are enqueued on the GPU, a
    background thread writes the file. compression: 1 zlib, 0 none, -1 zlib
    when available. Close (or flush) before reading the files."""

    def __init__(self, solver, points, cells, compression=-1, slots=0):
        L = lib()
        self.solver = solver
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        cl = np.ascontiguousarray(cells, dtype=np.int64)
        h = C.c_void_p()
        rc = L.dg_vtu_writer_create(solver.h, len(pts), _dp(pts), _ip(cl), compression, slots, C.byref(h))
        if rc != 0:
            raise SolverError("dg_vtu_writer_create: %s" % ERRORS.get(rc, rc))
        self.h = h

    def _ck(self, rc, what):
        if rc != 0:
            raise SolverError("%s: %s: %s" % (what, ERRORS.get(rc, rc), lib().dg_vtu_writer_last_error(self.h).decode()))

    def write(self, path):
        self._ck(lib().dg_vtu_write_async(self.h, str(path).encode()), "dg_vtu_write_async")

    def flush(self):
        self._ck(lib().dg_vtu_writer_flush(self.h), "dg_vtu_writer_flush")

    def stats(self):
        """(files written, compressed)"""
        n, comp = C.c_int64(), C.c_int()
        lib().dg_vtu_writer_stats(self.h, C.byref(n), C.byref(comp))
        return n.value, bool(comp.value)

    def close(self):
        if self.h:
            rc = lib().dg_vtu_writer_destroy(self.h)
            self.h = None
            if rc != 0:
                raise SolverError("dg_vtu_writer_destroy: %s" % ERRORS.get(rc, rc))


class Batch:
    """A batched ensemble of independent instances (dg_batch_* in the ABI).

    instances: list of dict(mesh=<mesh dict>, v0=(..), dt=float); rho0 and c0
    are shared by the batch."""

    def __init__(self, instances, rho0=1.0, c0=1.0, precision=DG_FP64, device=0):
        L = _batch_lib()
        n = len(instances)
        descs = (MeshDesc * n)()
        phys = (Phys * n)()
        dts = (C.c_double * n)()
        self._keep = []
        self.sizes = []
        for i, inst in enumerate(instances):
            mesh = inst["mesh"]
            xyz = np.ascontiguousarray(mesh["xyz"], dtype=np.float64)
            en = np.ascontiguousarray(mesh["elem_nodes"], dtype=np.int64)
            groups = mesh.get("groups", [])
            gbc = np.array([g[0] for g in groups] or [0], dtype=np.int32)
            goff, gn = _csr([g[1] for g in groups])
            self._keep += [xyz, en, gbc, goff, gn]
            d = descs[i]
            d.dim, d.order, d.nodes_per_elem = mesh["dim"], mesh["order"], en.shape[1]
            d.n_nodes, d.xyz = xyz.shape[0], _dp(xyz)
            d.n_elems, d.elem_nodes = en.shape[0], _ip(en)
            d.n_groups, d.group_bc = len(groups), gbc.ctypes.data_as(C.POINTER(C.c_int))
            d.group_offsets, d.group_nodes = _ip(goff), _ip(gn)
            phys[i].v0 = (C.c_double * 3)(*inst.get("v0", (0.0, 0.0, 0.0)))
            phys[i].rho0, phys[i].c0 = rho0, c0
            dts[i] = inst["dt"]
            self.sizes.append((en.shape[0], en.shape[1]))
        h = C.c_void_p()
        rc = L.dg_batch_create(n, descs, phys, dts, precision, device, C.byref(h))
        if rc != 0:
            raise SolverError("dg_batch_create: %s: %s" % (ERRORS.get(rc, rc), L.dg_last_error(None).decode()))
        self.h = h
        self._keep = []
        self.n = n
        self.n_obs = [0] * n

    def close(self):
        if getattr(self, "h", None):
            _batch_lib().dg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc != 0:
            raise SolverError("%s: %s: %s" % (what, ERRORS.get(rc, rc),
                                              _batch_lib().dg_batch_last_error(self.h).decode()))

    def info(self):
        ng, td = C.c_int(), C.c_int64()
        self._ck(_batch_lib().dg_batch_info(self.h, C.byref(ng), C.byref(td)), "dg_batch_info")
        return dict(n_groups=ng.value, total_dofs=td.value)

    def set_state(self, i, u):
        E, npe = self.sizes[i]
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(4, E * npe)
        self._ck(_batch_lib().dg_batch_set_state(self.h, i, _dp(u)), "dg_batch_set_state")

    def get_state(self, i):
        E, npe = self.sizes[i]
        u = np.zeros((4, E * npe))
        self._ck(_batch_lib().dg_batch_get_state(self.h, i, _dp(u)), "dg_batch_get_state")
        return u

    def set_sources(self, i, dof_lists, values):
        off, flat = _csr(dof_lists)
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1, max(len(dof_lists), 1))
        self._ck(_batch_lib().dg_batch_set_sources(self.h, i, len(dof_lists), _ip(off), _ip(flat), v.shape[0],
                                                   _dp(v)), "dg_batch_set_sources")

    def set_observers(self, i, dof_lists, weight_lists):
        off, flat = _csr(dof_lists)
        _, w = _csr(weight_lists, np.float64)
        self._ck(_batch_lib().dg_batch_set_observers(self.h, i, len(dof_lists), _ip(off), _ip(flat), _dp(w)),
                 "dg_batch_set_observers")
        self.n_obs[i] = len(dof_lists)

    def run(self, n_steps):
        tot = sum(n_steps * k * 4 for k in self.n_obs)
        buf = np.zeros(max(tot, 1))
        self._ck(_batch_lib().dg_batch_run(self.h, n_steps, _dp(buf)), "dg_batch_run")
        out, pos = [], 0
        for k in self.n_obs:
            out.append(buf[pos:pos + n_steps * k * 4].reshape(n_steps, k, 4))
            pos += n_steps * k * 4
        return out

    def set_fused(self, on):
        """One launch per RK stage for all element orders (FP32 2-D orders
        2-4) when on, else one stage kernel per order."""
        self._ck(_batch_lib().dg_batch_set_fused(self.h, 1 if on else 0), "dg_batch_set_fused")

    @property
    def fused(self):
        return bool(_batch_lib().dg_batch_fused(self.h))

    def bench(self, n_steps):
        ms = C.c_double()
        self._ck(_batch_lib().dg_batch_bench(self.h, n_steps, C.byref(ms)), "dg_batch_bench")
        return ms.value


def _mlp_lib():
    L = lib()
    if getattr(L, "_mlp", False):
        return L
    P, D, I64, F = C.POINTER, C.c_double, C.c_int64, C.c_float
    L.dg_mlp_create.argtypes = [C.c_int, P(C.c_int), C.c_int, P(C.c_void_p)]
    L.dg_mlp_destroy.argtypes = [C.c_void_p]
    L.dg_mlp_last_error.argtypes = [C.c_void_p]
    L.dg_mlp_last_error.restype = C.c_char_p
    L.dg_mlp_param_count.argtypes = [C.c_void_p]
    L.dg_mlp_param_count.restype = I64
    L.dg_mlp_set_params.argtypes = [C.c_void_p, P(F)]
    L.dg_mlp_get_params.argtypes = [C.c_void_p, P(F)]
    L.dg_mlp_forward.argtypes = [C.c_void_p, P(F), I64, P(F)]
    L.dg_mlp_forward_device.argtypes = [C.c_void_p, C.c_void_p, I64, C.c_void_p, C.c_void_p]
    L.dg_mlp_gradient.argtypes = [C.c_void_p, P(F), P(F), I64, P(F), P(D)]
    L.dg_mlp_set_data.argtypes = [C.c_void_p, P(F), P(F), I64]
    L.dg_mlp_train.argtypes = [C.c_void_p, I64, C.c_int, D, D, D, C.c_uint64, P(D)]
    L.dg_mlp_set_tensor_cores.argtypes = [C.c_void_p, C.c_int]
    L.dg_mlp_tensor_cores.argtypes = [C.c_void_p]
    L._mlp = True
    return L


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Network:
    """Fully connected GELU network on the GPU (dg_mlp_* in the ABI).

    widths: [inputs, hidden..., outputs]. Parameters are one flat float32
    vector, per layer W [out][in] (row-major) then b [out]."""

    def __init__(self, widths, device=0):
        L = _mlp_lib()
        w = (C.c_int * len(widths))(*widths)
        h = C.c_void_p()
        rc = L.dg_mlp_create(len(widths) - 1, w, device, C.byref(h))
        if rc != 0:
            raise SolverError("dg_mlp_create: %s: %s" % (ERRORS.get(rc, rc), L.dg_mlp_last_error(None).decode()))
        self.h = h
        self.widths = list(widths)
        self.n_params = L.dg_mlp_param_count(h)

    def close(self):
        if getattr(self, "h", None):
            _mlp_lib().dg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc != 0:
            raise SolverError("%s: %s: %s" % (what, ERRORS.get(rc, rc), _mlp_lib().dg_mlp_last_error(self.h).decode()))

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32).reshape(-1)
        if p.size != self.n_params:
            raise ValueError("expected %d parameters, got %d" % (self.n_params, p.size))
        self._ck(_mlp_lib().dg_mlp_set_params(self.h, _fp(p)), "dg_mlp_set_params")

    def get_params(self):
        p = np.zeros(self.n_params, dtype=np.float32)
        self._ck(_mlp_lib().dg_mlp_get_params(self.h, _fp(p)), "dg_mlp_get_params")
        return p

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.widths[0])
        y = np.zeros((x.shape[0], self.widths[-1]), dtype=np.float32)
        self._ck(_mlp_lib().dg_mlp_forward(self.h, _fp(x), x.shape[0], _fp(y)), "dg_mlp_forward")
        return y

    def forward_device(self, x_ptr, n, y_ptr, stream=None):
        self._ck(_mlp_lib().dg_mlp_forward_device(self.h, x_ptr, n, y_ptr, stream), "dg_mlp_forward_device")

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.widths[0])
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(x.shape[0], self.widths[-1])
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_double()
        self._ck(_mlp_lib().dg_mlp_gradient(self.h, _fp(x), _fp(t), x.shape[0], _fp(g), C.byref(loss)),
                 "dg_mlp_gradient")
        return g, loss.value

    def set_data(self, x, t):
        self._x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.widths[0])
        self._t = np.ascontiguousarray(t, dtype=np.float32).reshape(self._x.shape[0], self.widths[-1])
        self._ck(_mlp_lib().dg_mlp_set_data(self.h, _fp(self._x), _fp(self._t), self._x.shape[0]), "dg_mlp_set_data")

    def set_tensor_cores(self, on):
        """GEMMs on the tensor cores or on the CUDA cores (the default)."""
        self._ck(_mlp_lib().dg_mlp_set_tensor_cores(self.h, 1 if on else 0), "dg_mlp_set_tensor_cores")

    @property
    def tensor_cores(self):
        return bool(_mlp_lib().dg_mlp_tensor_cores(self.h))

    def train(self, n_steps, batch, lr, lr_final, seed=0, weight_decay=0.0):
        losses = np.zeros(max(n_steps, 1))
        self._ck(_mlp_lib().dg_mlp_train(self.h, n_steps, batch, lr, lr_final, weight_decay, seed, _dp(losses)),
                 "dg_mlp_train")
        return losses[:n_steps]
