"""ctypes binding of the refcpu oracle (oracle/refcpu.h).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py (CPU baseline / reference arm). The product never imports it.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "librefcpu.so")
_lib = None

SRC_SINE, SRC_CALLBACK, SRC_TABLE = 0, 1, 2
SRC_FN = C.CFUNCTYPE(C.c_double, C.c_int, C.c_double, C.c_void_p)


class Input(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("order", C.c_int), ("nodes_per_elem", C.c_int),
        ("n_nodes", C.c_int64), ("xyz", C.POINTER(C.c_double)),
        ("n_elems", C.c_int64), ("elem_nodes", C.POINTER(C.c_int64)),
        ("n_groups", C.c_int), ("group_bc", C.POINTER(C.c_int)),
        ("group_offsets", C.POINTER(C.c_int64)), ("group_nodes", C.POINTER(C.c_int64)),
        ("v0", C.c_double * 3), ("rho0", C.c_double), ("c0", C.c_double),
        ("t_start", C.c_double), ("t_end", C.c_double), ("dt", C.c_double), ("t_rate", C.c_double),
        ("method", C.c_int), ("num_threads", C.c_int),
        ("n_src", C.c_int), ("src_kind", C.POINTER(C.c_int)), ("src_params", C.POINTER(C.c_double)),
        ("src_fn", SRC_FN), ("src_user", C.c_void_p),
        ("src_table_offsets", C.POINTER(C.c_int64)), ("src_table", C.POINTER(C.c_double)),
        ("n_obs", C.c_int), ("obs", C.POINTER(C.c_double)),
        ("n_ic", C.c_int), ("ic", C.POINTER(C.c_double)),
        ("max_steps", C.c_int64),
    ]


class Output(C.Structure):
    _fields_ = [
        ("state", C.POINTER(C.c_double)), ("residuals", C.POINTER(C.c_double)),
        ("times", C.POINTER(C.c_double)), ("obs_trace", C.POINTER(C.c_double)),
        ("snapshot_steps", C.POINTER(C.c_int64)),
        ("steps_done", C.c_int64), ("n_snap", C.c_int64),
        ("setup_seconds", C.c_double), ("loop_seconds", C.c_double),
        ("penalty_sign_hist", C.c_int64 * 2), ("n_faces", C.c_int64), ("n_boundary_faces", C.c_int64),
    ]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle library not built: %s (run __graft_entry__.build())" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        L.refcpu_run.argtypes = [C.POINTER(Input), C.POINTER(Output)]
        L.refcpu_stage.argtypes = [C.POINTER(Input), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.refcpu_faces.argtypes = [C.POINTER(Input), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.refcpu_initial_state.argtypes = [C.POINTER(Input), C.POINTER(C.c_double)]
        L.refcpu_count_steps.argtypes = [C.c_double] * 4 + [C.POINTER(C.c_int64)] * 2
        L.refcpu_rule.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
        L.refcpu_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


class Problem:
    """Numpy-side description of one solver run (mesh + physics + schedule).

    mesh: dict with dim, order, xyz [N,3] f64, elem_nodes [E,Np] i64,
          groups: list of (bc_code, node index array) in ascending tag order.
    """

    def __init__(self, mesh, v0=(0, 0, 0), rho0=1.0, c0=1.0, t_start=0.0, t_end=1.0, dt=0.1,
                 t_rate=0.1, method=0, num_threads=1, sources=(), observers=(), ics=(),
                 src_fn=None, max_steps=-1):
        self.mesh = mesh
        self._keep = []
        xyz = np.ascontiguousarray(mesh["xyz"], dtype=np.float64)
        en = np.ascontiguousarray(mesh["elem_nodes"], dtype=np.int64)
        groups = mesh.get("groups", [])
        gbc = np.array([g[0] for g in groups] or [0], dtype=np.int32)
        goff = np.zeros(len(groups) + 1, dtype=np.int64)
        gnodes = []
        for i, g in enumerate(groups):
            arr = np.asarray(g[1], dtype=np.int64)
            gnodes.append(arr)
            goff[i + 1] = goff[i] + len(arr)
        gn = np.concatenate(gnodes) if gnodes else np.zeros(1, dtype=np.int64)
        # sources: list of dicts {kind, params[8], table}
        kinds = np.array([s["kind"] for s in sources] or [0], dtype=np.int32)
        params = np.zeros((max(1, len(sources)), 8))
        toff = np.zeros(len(sources) + 1, dtype=np.int64)
        tabs = []
        for i, s in enumerate(sources):
            params[i, :len(s["params"])] = s["params"]
            tab = np.asarray(s.get("table", np.zeros((0, 2))), dtype=np.float64).reshape(-1, 2)
            tabs.append(tab)
            toff[i + 1] = toff[i] + len(tab)
        table = np.ascontiguousarray(np.concatenate(tabs) if tabs and toff[-1] > 0 else np.zeros((1, 2)))
        obs = np.ascontiguousarray(np.asarray(observers, dtype=np.float64).reshape(-1, 4))
        ic = np.ascontiguousarray(np.asarray(ics, dtype=np.float64).reshape(-1, 5))
        self._keep += [xyz, en, gbc, goff, gn, kinds, params, toff, table, obs, ic]
        self.src_cb = SRC_FN(src_fn) if src_fn is not None else SRC_FN(lambda i, t, u: 0.0)
        inp = Input()
        inp.dim, inp.order, inp.nodes_per_elem = mesh["dim"], mesh["order"], en.shape[1]
        inp.n_nodes, inp.xyz = xyz.shape[0], _p(xyz, C.c_double)
        inp.n_elems, inp.elem_nodes = en.shape[0], _p(en, C.c_int64)
        inp.n_groups, inp.group_bc = len(groups), _p(gbc, C.c_int)
        inp.group_offsets, inp.group_nodes = _p(goff, C.c_int64), _p(gn, C.c_int64)
        inp.v0 = (C.c_double * 3)(*v0)
        inp.rho0, inp.c0 = rho0, c0
        inp.t_start, inp.t_end, inp.dt, inp.t_rate = t_start, t_end, dt, t_rate
        inp.method, inp.num_threads = method, num_threads
        inp.n_src, inp.src_kind, inp.src_params = len(sources), _p(kinds, C.c_int), _p(params, C.c_double)
        inp.src_fn, inp.src_user = self.src_cb, None
        inp.src_table_offsets, inp.src_table = _p(toff, C.c_int64), _p(table, C.c_double)
        inp.n_obs, inp.obs = obs.shape[0], _p(obs, C.c_double)
        inp.n_ic, inp.ic = ic.shape[0], _p(ic, C.c_double)
        inp.max_steps = max_steps
        self.inp = inp
        self.n_dof = en.shape[0] * en.shape[1]

    def count_steps(self):
        ns, nsn = C.c_int64(), C.c_int64()
        i = self.inp
        lib().refcpu_count_steps(i.t_start, i.t_end, i.dt, i.t_rate, C.byref(ns), C.byref(nsn))
        return ns.value, nsn.value

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("refcpu: " + lib().refcpu_last_error().decode())

    def run(self):
        ns, nsn = self.count_steps()
        if self.inp.max_steps >= 0:
            ns = min(ns, self.inp.max_steps)
        nobs = self.inp.n_obs
        state = np.zeros((4, self.n_dof))
        res = np.zeros((max(ns, 1), 5))
        times = np.zeros(max(ns, 1))
        trace = np.zeros((max(ns, 1), max(nobs, 1), 5))
        snaps = np.zeros(max(nsn, 1), dtype=np.int64)
        out = Output()
        out.state, out.residuals, out.times = _p(state, C.c_double), _p(res, C.c_double), _p(times, C.c_double)
        out.obs_trace, out.snapshot_steps = _p(trace, C.c_double), _p(snaps, C.c_int64)
        self._check(lib().refcpu_run(C.byref(self.inp), C.byref(out)))
        n = out.steps_done
        return dict(state=state, residuals=res[:n], times=times[:n], obs=trace[:n, :nobs],
                    snapshots=snaps[:out.n_snap], steps=n, setup_seconds=out.setup_seconds,
                    loop_seconds=out.loop_seconds, penalty_hist=tuple(out.penalty_sign_hist),
                    n_faces=out.n_faces, n_boundary_faces=out.n_boundary_faces)

    def stage(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(4, self.n_dof)
        k = np.zeros_like(u)
        self._check(lib().refcpu_stage(C.byref(self.inp), _p(u, C.c_double), _p(k, C.c_double)))
        return k

    def initial_state(self):
        u = np.zeros((4, self.n_dof))
        self._check(lib().refcpu_initial_state(C.byref(self.inp), _p(u, C.c_double)))
        return u

    def faces(self):
        E = self.inp.n_elems
        nf = self.inp.dim + 1
        fid = np.zeros(E * nf, dtype=np.int64)
        nbr = np.zeros(E * nf, dtype=np.int64)
        orient = np.zeros(E * nf, dtype=np.int32)
        bc = np.zeros(E * nf, dtype=np.int32)
        pen = np.zeros(E * nf, dtype=np.int32)
        self._check(lib().refcpu_faces(C.byref(self.inp), _p(fid, C.c_int64), _p(nbr, C.c_int64),
                                       _p(orient, C.c_int), _p(bc, C.c_int), _p(pen, C.c_int)))
        sh = (E, nf)
        return dict(face_id=fid.reshape(sh), nbr=nbr.reshape(sh), orient=orient.reshape(sh),
                    bc=bc.reshape(sh), penalty=pen.reshape(sh))


def rule(kind, degree):
    """The oracle's quadrature rule: kind 1 Gauss line (degree = points),
    2 triangle, 3 tetrahedron; returns (points [n][dim], weights [n])."""
    L = lib()
    n = C.c_int()
    if L.refcpu_rule(kind, degree, C.byref(n), None, None) != 0:
        raise RuntimeError(L.refcpu_last_error().decode())
    dim = {1: 1, 2: 2, 3: 3}[kind]
    x = np.zeros(n.value * dim)
    w = np.zeros(n.value)
    L.refcpu_rule(kind, degree, C.byref(n), _p(x, C.c_double), _p(w, C.c_double))
    return x.reshape(n.value, dim), w

