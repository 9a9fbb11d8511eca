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
