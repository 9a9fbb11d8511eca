"""ctypes binding of the host front end (include/dgfem_host.h).

Mesh and configuration loading, the time schedule, the formula evaluator and
the output writers. Needs no GPU.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libdgfem_host.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("host library not built: %s (run __graft_entry__.build())" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        L.dgh_last_error.restype = C.c_char_p
        L.dgh_mesh_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
        L.dgh_mesh_free.argtypes = [C.c_void_p]
        L.dgh_mesh_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int)]
        for fn, t in (("dgh_mesh_xyz", C.c_double), ("dgh_mesh_node_tags", C.c_int64),
                      ("dgh_mesh_elem_nodes", C.c_int64)):
            getattr(L, fn).argtypes = [C.c_void_p]
            getattr(L, fn).restype = C.POINTER(t)
        L.dgh_mesh_group.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_char_p),
                                     C.POINTER(C.c_int64), C.POINTER(C.POINTER(C.c_int64))]
        L.dgh_mesh_write.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int64, C.POINTER(C.c_double), C.c_int64,
                                     C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_char_p),
                                     C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.dgh_count_steps.argtypes = [C.c_double] * 4 + [C.POINTER(C.c_int64)] * 2
        L.dgh_schedule.argtypes = [C.c_double] * 4 + [C.POINTER(C.c_double), C.POINTER(C.c_ubyte)]
        L.dgh_quadrature.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _err():
    return lib().dgh_last_error().decode()


def load_mesh(path):
    """Reads a .msh file. Returns dict(dim, order, xyz, node_tags, elem_nodes,
    groups=[(tag, name, node_indices)])."""
    L = lib()
    h = C.c_void_p()
    if L.dgh_mesh_load(path.encode(), C.byref(h)) != 0:
        raise RuntimeError(_err())
    try:
        dim, order, npe, ng = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        nn, ne = C.c_int64(), C.c_int64()
        L.dgh_mesh_info(h, C.byref(dim), C.byref(order), C.byref(npe), C.byref(nn), C.byref(ne), C.byref(ng))
        xyz = np.ctypeslib.as_array(L.dgh_mesh_xyz(h), shape=(nn.value * 3,)).reshape(-1, 3).copy()
        tags = np.ctypeslib.as_array(L.dgh_mesh_node_tags(h), shape=(nn.value,)).copy()
        en = np.ctypeslib.as_array(L.dgh_mesh_elem_nodes(h), shape=(ne.value * npe.value,)).reshape(-1, npe.value).copy()
        groups = []
        for g in range(ng.value):
            tag, name, n, ptr = C.c_int(), C.c_char_p(), C.c_int64(), C.POINTER(C.c_int64)()
            L.dgh_mesh_group(h, g, C.byref(tag), C.byref(name), C.byref(n), C.byref(ptr))
            nodes = np.ctypeslib.as_array(ptr, shape=(n.value,)).copy() if n.value else np.zeros(0, np.int64)
            groups.append((tag.value, name.value.decode(), nodes))
        return dict(dim=dim.value, order=order.value, xyz=xyz, node_tags=tags, elem_nodes=en, groups=groups)
    finally:
        L.dgh_mesh_free(h)


def write_mesh(path, dim, order, xyz, elem_nodes, groups):
    """groups: list of (tag, name, face_nodes [nf, nodes_per_face])."""
    L = lib()
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    en = np.ascontiguousarray(elem_nodes, dtype=np.int64)
    tags = (C.c_int * max(1, len(groups)))(*[g[0] for g in groups])
    names = (C.c_char_p * max(1, len(groups)))(*[g[1].encode() for g in groups])
    offs = np.zeros(len(groups) + 1, dtype=np.int64)
    faces = []
    for i, g in enumerate(groups):
        fnodes = np.asarray(g[2], dtype=np.int64)
        faces.append(fnodes.reshape(len(fnodes), -1))
        offs[i + 1] = offs[i] + len(fnodes)
    fn = np.ascontiguousarray(np.concatenate(faces) if faces else np.zeros((1, 1), np.int64), dtype=np.int64)
    rc = L.dgh_mesh_write(path.encode(), dim, order, xyz.shape[0], xyz.ctypes.data_as(C.POINTER(C.c_double)),
                          en.shape[0], en.ctypes.data_as(C.POINTER(C.c_int64)), len(groups), tags, names,
                          offs.ctypes.data_as(C.POINTER(C.c_int64)), fn.ctypes.data_as(C.POINTER(C.c_int64)))
    if rc != 0:
        raise RuntimeError(_err())


def schedule(t_start, t_end, dt, t_rate):
    """Per-step times and snapshot flags of the reference time loop."""
    L = lib()
    ns, nsn = C.c_int64(), C.c_int64()
    L.dgh_count_steps(t_start, t_end, dt, t_rate, C.byref(ns), C.byref(nsn))
    times = np.zeros(ns.value)
    snap = np.zeros(ns.value, dtype=np.uint8)
    L.dgh_schedule(t_start, t_end, dt, t_rate, times.ctypes.data_as(C.POINTER(C.c_double)),
                   snap.ctypes.data_as(C.POINTER(C.c_ubyte)))
    return times, snap.astype(bool)


def _setup_more(L):
    if getattr(L, "_more", False):
        return
    L.dgh_config_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    L.dgh_config_free.argtypes = [C.c_void_p]
    for fn in ("dgh_config_mesh_file", "dgh_config_time_method", "dgh_config_element_type", "dgh_config_precision"):
        getattr(L, fn).argtypes = [C.c_void_p]
        getattr(L, fn).restype = C.c_char_p
    L.dgh_config_numbers.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 7
    for fn in ("dgh_config_num_threads", "dgh_config_num_bc", "dgh_config_num_sources", "dgh_config_num_observers",
               "dgh_config_num_ics"):
        getattr(L, fn).argtypes = [C.c_void_p]
    L.dgh_config_bc.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.dgh_config_source.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                    C.POINTER(C.c_char_p), C.POINTER(C.c_int64), C.POINTER(C.POINTER(C.c_double))]
    L.dgh_config_observer.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    L.dgh_config_ic.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    L.dgh_source_value.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.dgh_source_value.restype = C.c_double
    L.dgh_formula_eval.argtypes = [C.c_char_p, C.c_double, C.POINTER(C.c_double)]
    L.dgh_write_pvd.argtypes = [C.c_char_p] + [C.c_double] * 4
    L.dgh_write_wav.argtypes = [C.c_char_p, C.POINTER(C.c_float), C.c_int64, C.c_uint32]
    L.dgh_read_wav.argtypes = [C.c_char_p, C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.c_int64),
                               C.POINTER(C.c_uint32)]
    L.dgh_free.argtypes = [C.c_void_p]
    L.dgh_write_spectra.argtypes = [C.c_char_p, C.POINTER(C.c_float), C.c_int64, C.c_double]
    L.dgh_spectra.argtypes = [C.POINTER(C.c_float), C.c_int64, C.c_double, C.POINTER(C.c_int64),
                              C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L._more = True


def load_config(path, times=None):
    """Parses a .conf/.json configuration (and its mesh) like the reference.
    With times, also returns source_values[len(times)][n_sources] (NaN where a
    source writes nothing)."""
    L = lib()
    _setup_more(L)
    h = C.c_void_p()
    if L.dgh_config_load(path.encode(), C.byref(h)) != 0:
        raise RuntimeError(_err())
    try:
        nums = [C.c_double() for _ in range(4)]
        v0 = (C.c_double * 3)()
        rho0, c0 = C.c_double(), C.c_double()
        L.dgh_config_numbers(h, *[C.byref(x) for x in nums], v0, C.byref(rho0), C.byref(c0))
        out = dict(mesh_file=L.dgh_config_mesh_file(h).decode(), time_method=L.dgh_config_time_method(h).decode(),
                   element_type=L.dgh_config_element_type(h).decode(), precision=L.dgh_config_precision(h).decode(),
                   t_start=nums[0].value, t_end=nums[1].value, dt=nums[2].value, t_rate=nums[3].value,
                   v0=tuple(v0), rho0=rho0.value, c0=c0.value, num_threads=L.dgh_config_num_threads(h))
        bcs = []
        for i in range(L.dgh_config_num_bc(h)):
            t, ty = C.c_int(), C.c_int()
            L.dgh_config_bc(h, i, C.byref(t), C.byref(ty))
            bcs.append((t.value, ty.value))
        out["bcs"] = bcs
        srcs = []
        for i in range(L.dgh_config_num_sources(h)):
            kind, params = C.c_int(), (C.c_double * 8)()
            formula, rows, tab = C.c_char_p(), C.c_int64(), C.POINTER(C.c_double)()
            L.dgh_config_source(h, i, C.byref(kind), params, C.byref(formula), C.byref(rows), C.byref(tab))
            table = np.ctypeslib.as_array(tab, shape=(rows.value * 2,)).reshape(-1, 2).copy() if rows.value else None
            srcs.append(dict(kind=kind.value, params=list(params), formula=formula.value.decode(), table=table))
        out["sources"] = srcs
        obs = []
        for i in range(L.dgh_config_num_observers(h)):
            v = (C.c_double * 4)()
            L.dgh_config_observer(h, i, v)
            obs.append(tuple(v))
        out["observers"] = obs
        ics = []
        for i in range(L.dgh_config_num_ics(h)):
            v = (C.c_double * 5)()
            L.dgh_config_ic(h, i, v)
            ics.append(tuple(v))
        out["ics"] = ics
        if times is not None:
            out["source_values"] = np.array([[L.dgh_source_value(h, i, float(t)) for i in range(len(srcs))]
                                             for t in times]).reshape(len(times), len(srcs))
        return out
    finally:
        L.dgh_config_free(h)


def formula(expr, t):
    """(ok, value) of the formula evaluator."""
    L = lib()
    _setup_more(L)
    v = C.c_double()
    rc = L.dgh_formula_eval(expr.encode(), t, C.byref(v))
    return rc == 0, v.value


def write_wav(path, samples, rate):
    L = lib()
    _setup_more(L)
    s = np.ascontiguousarray(samples, dtype=np.float32)
    if L.dgh_write_wav(path.encode(), s.ctypes.data_as(C.POINTER(C.c_float)), len(s), rate) != 0:
        raise RuntimeError(_err())


def read_wav(path):
    L = lib()
    _setup_more(L)
    p, n, r = C.POINTER(C.c_float)(), C.c_int64(), C.c_uint32()
    if L.dgh_read_wav(path.encode(), C.byref(p), C.byref(n), C.byref(r)) != 0:
        raise RuntimeError(_err())
    out = np.ctypeslib.as_array(p, shape=(max(n.value, 1),))[:n.value].copy()
    L.dgh_free(p)
    return out, r.value


def spectra(p, dt):
    """(fft rows [nb/2,5], psd rows [nb/2+1,3]) of a pressure trace."""
    L = lib()
    _setup_more(L)
    s = np.ascontiguousarray(p, dtype=np.float32)
    nb = 1
    while nb * 2 <= len(s):
        nb *= 2
    f = np.zeros((nb // 2 + 1, 5))
    q = np.zeros((nb // 2 + 2, 3))
    nbo = C.c_int64()
    if L.dgh_spectra(s.ctypes.data_as(C.POINTER(C.c_float)), len(s), dt, C.byref(nbo),
                     f.ctypes.data_as(C.POINTER(C.c_double)), q.ctypes.data_as(C.POINTER(C.c_double))) != 0:
        raise RuntimeError(_err())
    n = nbo.value
    return f[:n // 2], q[:n // 2 + 1]


def write_spectra(prefix, p, dt):
    L = lib()
    _setup_more(L)
    s = np.ascontiguousarray(p, dtype=np.float32)
    if L.dgh_write_spectra(prefix.encode(), s.ctypes.data_as(C.POINTER(C.c_float)), len(s), dt) != 0:
        raise RuntimeError(_err())


def write_pvd(path, t_start, t_end, dt, t_rate):
    L = lib()
    _setup_more(L)
    if L.dgh_write_pvd(path.encode(), t_start, t_end, dt, t_rate) != 0:
        raise RuntimeError(_err())


def quadrature(kind, degree):
    """The curved-element path's quadrature rule: kind 1 Gauss-Legendre line
    on [-1, 1] with `degree` points, 2 triangle and 3 tetrahedron rule of that
    degree; returns (points [n][dim], weights [n])."""
    L = lib()
    n = C.c_int()
    if L.dgh_quadrature(kind, degree, C.byref(n), None, None) != 0:
        raise RuntimeError(L.dgh_last_error().decode())
    x = np.zeros(n.value * kind)
    w = np.zeros(n.value)
    L.dgh_quadrature(kind, degree, C.byref(n), x.ctypes.data_as(C.POINTER(C.c_double)),
                     w.ctypes.data_as(C.POINTER(C.c_double)))
    return x.reshape(n.value, kind), w

