"""Seeded synthetic meshes of the benchmark configurations.

* square(n, half_width, order, jitter, seed): [-a,a]^2 structured n x n grid,
  each cell split into two counter-clockwise triangles, interior vertices
  jittered uniformly by up to jitter*h per axis.
* box(counts, lo, hi, order, jitter, seed): structured box of cubes, each cube
  split into six positively oriented tetrahedra around its main diagonal
  (a conforming split), interior vertices jittered by up to jitter*h.

High-order nodes sit at the straight-sided (affine) Lagrange positions and are
shared between elements; element node lists follow Gmsh's node ordering
(vertices, edge nodes per edge from its first to its second vertex, face
nodes, interior nodes). Boundary groups are the sides of the domain:
(tag, name, node indices, boundary face node lists).
"""
import itertools

import numpy as np

TRI_EDGES = [(0, 1), (1, 2), (2, 0)]
TET_EDGES = [(0, 1), (1, 2), (2, 0), (3, 0), (3, 2), (3, 1)]
TET_FACES = [(0, 2, 1), (0, 1, 3), (0, 3, 2), (3, 1, 2)]


def _simplex_lattice_order(dim, p):
    """Barycentric integer coordinates (b_0..b_dim, sum p) of the element's
    nodes in Gmsh order."""
    nv = dim + 1

    def vert(k):
        b = [0] * nv
        b[k] = p
        return tuple(b)

    pts = [vert(k) for k in range(nv)]
    edges = [(0, 1)] if dim == 1 else TRI_EDGES if dim == 2 else TET_EDGES
    for (a, b) in edges:
        for i in range(1, p):
            c = [0] * nv
            c[a], c[b] = p - i, i
            pts.append(tuple(c))

    def tri_interior(corners, q):
        # interior nodes of a triangle of order q with the given corner vertex
        # ids, in Gmsh's recursive order (an inner triangle of order q-3)
        out = []
        if q < 3:
            return out
        inner = q - 3
        if inner == 0:
            c = [0] * nv
            for v in corners:
                c[v] += 1
            return [tuple(c)]
        # inner triangle vertices (shifted by 1 in each barycentric direction)
        sub = _simplex_lattice_order(2, inner)
        for s in sub:
            c = [0] * nv
            for k, v in enumerate(corners):
                c[v] += s[k] + 1
            out.append(tuple(c))
        return out

    if dim == 1:
        pass
    elif dim == 2:
        pts += tri_interior((0, 1, 2), p)
    else:
        for f in TET_FACES:
            pts += tri_interior(f, p)
        if p >= 4:
            inner = p - 4
            sub = _simplex_lattice_order(3, inner) if inner > 0 else [(0, 0, 0, 0)]
            for s in sub:
                pts.append(tuple(x + 1 for x in s))
    assert len(pts) == len(set(pts)), (dim, p)
    return np.array(pts, dtype=np.int64)


def _face_lattice_order(p):
    return _simplex_lattice_order(2, p) if p > 0 else None


def _build(dim, coarse_int, coarse_xyz, elems, order, sides):
    """Common high-order node construction on a structured coarse grid.

    coarse_int: [V, dim] integer grid coordinates of coarse vertices
    coarse_xyz: [V, 3] physical coordinates
    elems: [E, dim+1] coarse vertex ids (positively oriented)
    sides: list of (tag, name, axis, value) boundary planes in integer coords
    """
    p = order
    lat = _simplex_lattice_order(dim, p)  # [np, dim+1]
    # fine-grid integer coordinates of every element node
    ci = coarse_int[elems]  # [E, dim+1, dim]
    fine = np.einsum("nk,ekd->end", lat, ci)  # [E, np, dim]
    ext = fine.reshape(-1, dim).max(axis=0) + 1
    lin = np.zeros(fine.shape[:2], dtype=np.int64)
    mul = 1
    for d in range(dim - 1, -1, -1):
        lin += fine[:, :, d] * mul
        mul *= int(ext[d])
    uniq, inv = np.unique(lin.reshape(-1), return_inverse=True)
    elem_nodes = inv.reshape(lin.shape).astype(np.int64)
    # physical coordinates: affine combination of the element's vertices
    xv = coarse_xyz[elems]  # [E, dim+1, 3]
    xyz_all = np.einsum("nk,ekx->enx", lat / p, xv)  # [E, np, 3]
    xyz = np.zeros((len(uniq), 3))
    xyz[elem_nodes.reshape(-1)] = xyz_all.reshape(-1, 3)
    fine_u = np.zeros((len(uniq), dim), dtype=np.int64)
    fine_u[elem_nodes.reshape(-1)] = fine.reshape(-1, dim)
    # boundary groups
    faces = TRI_EDGES if dim == 2 else TET_FACES
    flat = _simplex_lattice_order(dim - 1, p)  # face node order (barycentric w.r.t. face corners)
    groups = []
    for (tag, name, axis, value) in sides:
        nodes = np.nonzero(fine_u[:, axis] == value * p)[0]
        fnodes = []
        for lf, fc in enumerate(faces):
            vid = elems[:, list(fc)]
            on = np.all(coarse_int[vid][:, :, axis] == value, axis=1)
            if not on.any():
                continue
            # element-local node of each face lattice point
            loc = []
            for b in flat:
                full = [0] * (dim + 1)
                for k, v in enumerate(fc):
                    full[v] = b[k]
                idx = np.nonzero(np.all(lat == np.array(full), axis=1))[0][0]
                loc.append(idx)
            fnodes.append(elem_nodes[on][:, loc])
        fn = np.concatenate(fnodes) if fnodes else np.zeros((0, len(flat)), np.int64)
        groups.append((tag, name, nodes, fn))
    return dict(dim=dim, order=order, xyz=xyz, elem_nodes=elem_nodes, groups=groups)


def square(n=45, half_width=5.0, order=3, jitter=0.2, seed=1, side_names=None):
    """Config-1 style mesh; all four sides in one group unless side_names given."""
    rng = np.random.default_rng(seed)
    h = 2.0 * half_width / n
    I, J = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="xy")
    ci = np.stack([I.reshape(-1), J.reshape(-1)], axis=1).astype(np.int64)
    xyz = np.zeros((len(ci), 3))
    xyz[:, :2] = -half_width + h * ci
    interior = (ci[:, 0] > 0) & (ci[:, 0] < n) & (ci[:, 1] > 0) & (ci[:, 1] < n)
    xyz[interior, :2] += rng.uniform(-jitter * h, jitter * h, size=(interior.sum(), 2))
    vid = lambda i, j: j * (n + 1) + i
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    ii, jj = ii.reshape(-1), jj.reshape(-1)
    a, b, c, d = vid(ii, jj), vid(ii + 1, jj), vid(ii + 1, jj + 1), vid(ii, jj + 1)
    elems = np.stack([np.stack([a, b, c], 1), np.stack([a, c, d], 1)], axis=1).reshape(-1, 3)
    if side_names is None:
        sides = [(1, "Absorbing", 0, 0), (1, "Absorbing", 0, n), (1, "Absorbing", 1, 0), (1, "Absorbing", 1, n)]
    else:
        sides = [(k + 1, side_names[k], ax, val) for k, (ax, val) in enumerate([(0, 0), (0, n), (1, 0), (1, n)])]
    m = _build(2, ci, xyz, elems, order, sides)
    return _merge_same_tag(m)


def box(counts=(32, 32, 32), lo=(-1, -1, -1), hi=(1, 1, 1), order=3, jitter=0.2, seed=2, side_names=None):
    """Config-2/3 style mesh: six tetrahedra per cube. Sides in the order
    x-, x+, y-, y+, z-, z+ with tags 1..6 (names from side_names)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = counts
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    hvec = (hi - lo) / np.array(counts)
    K, J, I = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    ci = np.stack([I.reshape(-1), J.reshape(-1), K.reshape(-1)], 1).astype(np.int64)
    xyz = lo + ci * hvec
    interior = np.all((ci > 0) & (ci < np.array(counts)), axis=1)
    xyz[interior] += rng.uniform(-jitter, jitter, size=(interior.sum(), 3)) * hvec
    vid = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i
    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ii, jj, kk = ii.reshape(-1), jj.reshape(-1), kk.reshape(-1)
    unit = np.eye(3, dtype=np.int64)
    tets = []
    for perm in itertools.permutations(range(3)):
        p0 = np.zeros(3, np.int64)
        p1 = p0 + unit[perm[0]]
        p2 = p1 + unit[perm[1]]
        p3 = np.ones(3, np.int64)
        vs = [vid(ii + q[0], jj + q[1], kk + q[2]) for q in (p0, p1, p2, p3)]
        # orientation of this permutation's tet (same for every cube)
        M = np.stack([p1 - p0, p2 - p0, p3 - p0], 1)
        if np.linalg.det(M) < 0:
            vs[1], vs[2] = vs[2], vs[1]
        tets.append(np.stack(vs, 1))
    elems = np.stack(tets, 1).reshape(-1, 4)
    names = side_names or ["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"]
    sides = [(k + 1, names[k], ax, val) for k, (ax, val) in
             enumerate([(0, 0), (0, nx), (1, 0), (1, ny), (2, 0), (2, nz)])]
    return _merge_same_tag(_build(3, ci, xyz, elems, order, sides))


def _merge_same_tag(m):
    merged = {}
    order = []
    for (tag, name, nodes, fn) in m["groups"]:
        if tag not in merged:
            merged[tag] = [name, [nodes], [fn]]
            order.append(tag)
        else:
            merged[tag][1].append(nodes)
            merged[tag][2].append(fn)
    m["groups"] = [(t, merged[t][0], np.unique(np.concatenate(merged[t][1])), np.concatenate(merged[t][2]))
                   for t in sorted(order)]
    return m


def solver_groups(mesh, bc_by_name):
    """(bc_code, nodes) list for the solver/oracle from a name -> 'Absorbing'/'Reflecting' map,
    keeping only groups with a recognised type (ascending tag order)."""
    out = []
    for (tag, name, nodes, _fn) in mesh["groups"]:
        t = bc_by_name.get(name)
        if t in ("Absorbing", "Reflecting"):
            out.append((1 if t == "Reflecting" else 0, nodes))
    return out


def min_altitude(mesh):
    """Smallest element altitude of a straight-sided simplex mesh: 2 area /
    longest edge (triangles) or 3 volume / largest face (tetrahedra). This is
    the h_min of the project's time-step rule dt = CFL h_min / ((c0 + |v0|)
    (2p + 1)): the shortest distance a wave crosses an element, which bounds
    the stable explicit step on distorted elements."""
    X = np.asarray(mesh["xyz"], dtype=np.float64)
    dim = mesh.get("dim", 3 if X.shape[1] == 3 and np.ptp(X[:, 2]) > 0 else 2)
    en = np.asarray(mesh["elem_nodes"])[:, :dim + 1]
    P = [X[en[:, i]] for i in range(dim + 1)]
    if dim == 2:
        area = 0.5 * np.abs((P[1][:, 0] - P[0][:, 0]) * (P[2][:, 1] - P[0][:, 1])
                            - (P[1][:, 1] - P[0][:, 1]) * (P[2][:, 0] - P[0][:, 0]))
        L = np.max([np.linalg.norm(P[b] - P[a], axis=1) for a, b in ((0, 1), (1, 2), (2, 0))], axis=0)
        return float((2 * area / L).min())
    V = np.abs(np.einsum("ij,ij->i", P[1] - P[0], np.cross(P[2] - P[0], P[3] - P[0]))) / 6
    A = np.max([0.5 * np.linalg.norm(np.cross(P[b] - P[a], P[c] - P[a]), axis=1)
                for a, b, c in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3))], axis=0)
    return float((3 * V / A).min())


def warp(mesh, amp, center=None, radius=None):
    """Copy of a mesh with every node (vertices and high-order nodes) moved by
    a smooth displacement, which makes the elements it bends curved: the
    high-order nodes leave the straight-sided lattice of their element's
    corners. Without a center, a global quadratic bend: x_d += amp *
    x_{d+1}^2 (cyclic over the mesh's dimensions). With a center and radius, a
    bump amp * (1 - r^2/R^2)^3 along the diagonal inside the ball of radius R;
    elements entirely outside it stay straight-sided."""
    m = dict(mesh)
    X = np.array(mesh["xyz"], dtype=np.float64)
    dim = 3 if np.ptp(X[:, 2]) > 0 else 2
    if center is None:
        Y = X.copy()
        for d in range(dim):
            Y[:, d] += amp * X[:, (d + 1) % dim] ** 2
    else:
        c = np.zeros(3)
        c[:len(center)] = center
        r2 = np.sum((X - c) ** 2, axis=1) / radius ** 2
        f = amp * np.clip(1.0 - r2, 0.0, None) ** 3
        Y = X.copy()
        for d in range(dim):
            Y[:, d] += f / np.sqrt(dim)
    m["xyz"] = Y
    return m


def line(n=100, x0=-5.0, x1=5.0, order=1, jitter=0.0, seed=3, side_names=("left", "right")):
    """1-D mesh of n line elements on [x0, x1] along the x axis, nodes in
    Gmsh's line order (the two end points, then the interior nodes from the
    first to the second). The two end points are the boundary groups
    (tags 1, 2)."""
    rng = np.random.default_rng(seed)
    h = (x1 - x0) / n
    xv = x0 + h * np.arange(n + 1)
    if jitter > 0 and n > 1:
        xv[1:-1] += rng.uniform(-jitter * h, jitter * h, size=n - 1)
    nv = n + 1
    xyz = [np.stack([xv, np.zeros(nv), np.zeros(nv)], axis=1)]
    elems = np.zeros((n, order + 1), dtype=np.int64)
    elems[:, 0] = np.arange(n)
    elems[:, 1] = np.arange(1, n + 1)
    nxt = nv
    for k in range(1, order):
        xk = xv[:-1] + (xv[1:] - xv[:-1]) * k / order
        xyz.append(np.stack([xk, np.zeros(n), np.zeros(n)], axis=1))
        elems[:, 1 + k] = nxt + np.arange(n)
        nxt += n
    xyz = np.concatenate(xyz)
    groups = [(1, side_names[0], np.array([0], np.int64), np.array([[0]], np.int64)),
              (2, side_names[1], np.array([n], np.int64), np.array([[n]], np.int64))]
    return dict(dim=1, order=order, xyz=xyz, elem_nodes=elems, groups=groups)
