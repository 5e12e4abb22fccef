"""Synthetic surface meshes for the collocation BEM path.

Meshes use the reference's flat layout (nihu/core/mesh.hpp:175-193,
``create_mesh(nodes, elements)``): ``nodes`` is an ``(n_nodes, 3)`` float64
array and ``elements`` an ``(n_elems, 5)`` int32 array whose first column is
the element type id (32303 = tria_1, 32404 = quad_1, nihu/core/element.hpp:112-118)
followed by the corner node indices; unused corner slots of triangles hold -1.
Element ids (and so DOF numbers) run in row order (nihu/core/mesh.hpp:155).

All faces are oriented counter-clockwise seen from outside, so the element
normal (dx/dxi x dx/deta) points out of the enclosed volume.
"""
from __future__ import annotations

import numpy as np

TRIA_1 = 32303
QUAD_1 = 32404


def _pack(nodes, faces, type_id):
    faces = np.asarray(faces, dtype=np.int32)
    n, nc = faces.shape
    elems = np.full((n, 5), -1, dtype=np.int32)
    elems[:, 0] = type_id
    elems[:, 1:1 + nc] = faces
    return np.ascontiguousarray(nodes, dtype=np.float64), elems


def icosphere(subdivisions: int, radius: float = 1.0):
    """Unit icosahedron subdivided ``subdivisions`` times, every new vertex
    projected to the sphere after each level: 20 * 4**s flat triangles."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in verts]
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]

        new = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new
    nodes = np.array(v) * radius
    return _pack(nodes, faces, TRIA_1)


def cube_sphere(n: int, radius: float = 1.0):
    """Sphere of 6 n^2 flat quads: every face of the cube [-1, 1]^3 split into
    n x n squares (equiangular spacing), vertices projected to the sphere;
    shared edges share nodes, faces oriented outward."""
    t = np.tan(np.linspace(-np.pi / 4, np.pi / 4, n + 1))
    index = {}
    nodes = []

    def node(p):
        key = tuple(np.round(p, 12))
        if key not in index:
            index[key] = len(nodes)
            nodes.append(p / np.linalg.norm(p))
        return index[key]

    faces = []
    # (normal axis, sign): u, v axes chosen so that u x v = sign * e_axis
    for axis in range(3):
        a1, a2 = (axis + 1) % 3, (axis + 2) % 3
        for sign in (1.0, -1.0):
            grid = np.empty((n + 1, n + 1), dtype=np.int64)
            for i in range(n + 1):
                for j in range(n + 1):
                    p = np.zeros(3)
                    p[axis] = sign
                    p[a1] = t[i]
                    p[a2] = t[j] * sign
                    grid[i, j] = node(p)
            for i in range(n):
                for j in range(n):
                    faces.append((grid[i, j], grid[i + 1, j], grid[i + 1, j + 1], grid[i, j + 1]))
    return _pack(np.array(nodes) * radius, faces, QUAD_1)


def cylinder(n_theta: int, n_z: int, n_ring: int, radius: float = 1.0, length: float = 4.0, smooth: int = 200):
    """Closed cylinder of flat quads: an ``n_theta x n_z`` side grid plus two
    O-grid caps.  Each cap is an ``m x m`` square core (m = n_theta/4) blended
    into the rim circle through ``n_ring`` rings of ``n_theta`` quads.

    Element count: n_theta*n_z + 2*(m*m + n_theta*n_ring).
    Side quads are exact rectangles; cap quads are planar (z = const).
    """
    if n_theta % 4:
        raise ValueError("n_theta must be a multiple of 4")
    m = n_theta // 4
    nodes, faces = [], []

    def add(p):
        nodes.append(p)
        return len(nodes) - 1

    # side: rings of nodes at z_k, angles theta_i
    th = 2 * np.pi * np.arange(n_theta) / n_theta
    zs = np.linspace(-length / 2, length / 2, n_z + 1)
    side = np.empty((n_z + 1, n_theta), dtype=np.int64)
    for k, z in enumerate(zs):
        for i in range(n_theta):
            side[k, i] = add((radius * np.cos(th[i]), radius * np.sin(th[i]), z))
    for k in range(n_z):
        for i in range(n_theta):
            i1 = (i + 1) % n_theta
            # outward normal: d/dxi along +theta, d/deta along +z
            faces.append((side[k, i], side[k, i1], side[k + 1, i1], side[k + 1, i]))

    # caps
    h = 0.5 * radius  # half-width of the square core
    for cap, z in ((0, -length / 2), (1, length / 2)):
        # boundary loop of the square core, counter-clockwise from (-h,-h), n_theta points
        loop = []
        for s in range(4 * m):
            side_i, t = divmod(s, m)
            a = -h + 2 * h * t / m
            loop.append([(a, -h), (h, a), (-a, h), (-h, -a)][side_i])
        # rim angles aligned with the core loop start (corner (-h,-h) at 225 deg)
        rim_th = th + 1.25 * np.pi
        rings = [[None] * n_theta for _ in range(n_ring + 1)]
        for r in range(n_ring + 1):
            s = r / n_ring
            for i in range(n_theta):
                if r == 0:
                    continue
                qx = (1 - s) * loop[i][0] + s * radius * np.cos(rim_th[i])
                qy = (1 - s) * loop[i][1] + s * radius * np.sin(rim_th[i])
                rings[r][i] = (qx, qy)
        # core grid nodes
        core = np.empty((m + 1, m + 1), dtype=np.int64)
        for a in range(m + 1):
            for b in range(m + 1):
                core[a, b] = add((-h + 2 * h * a / m, -h + 2 * h * b / m, z))
        # ring nodes; ring 0 reuses the core boundary, ring n_ring reuses the side
        def loop_node(i):
            side_i, t = divmod(i, m)
            return [core[t, 0], core[m, t], core[m - t, m], core[0, m - t]][side_i]

        ring_ids = [[loop_node(i) for i in range(n_theta)]]
        rim_row = 0 if cap == 0 else n_z
        # rim node for loop index i sits at angle rim_th[i]; find the side node
        rim_map = [int(round((rim_th[i] % (2 * np.pi)) / (2 * np.pi) * n_theta)) % n_theta
                   for i in range(n_theta)]
        for r in range(1, n_ring + 1):
            if r == n_ring:
                ring_ids.append([side[rim_row, rim_map[i]] for i in range(n_theta)])
            else:
                ring_ids.append([add((rings[r][i][0], rings[r][i][1], z)) for i in range(n_theta)])
        quads = []
        for a in range(m):
            for b in range(m):
                quads.append((core[a, b], core[a + 1, b], core[a + 1, b + 1], core[a, b + 1]))
        for r in range(n_ring):
            for i in range(n_theta):
                i1 = (i + 1) % n_theta
                quads.append((ring_ids[r][i], ring_ids[r + 1][i], ring_ids[r + 1][i1], ring_ids[r][i1]))
        # the loops above are counter-clockwise seen from +z: outward for the top cap
        if cap == 0:
            quads = [q[::-1] for q in quads]
        faces += quads
    nodes = np.array(nodes, dtype=np.float64)
    faces = np.asarray(faces, dtype=np.int64)
    # Laplacian smoothing of the cap interiors (rim and side nodes fixed):
    # rounds the square core so that no cap quad is kite-shaped; the
    # nearly singular quad scheme's Newton inverse mapping (the reference's,
    # nihu/core/inverse_mapping.hpp) converges for all neighbour pairs only on
    # such near-parallelogram quads.
    n_side = (n_z + 1) * n_theta
    nbrs = [set() for _ in range(len(nodes))]
    for f in faces[n_theta * n_z:]:
        for a in range(4):
            nbrs[f[a]].add(int(f[(a + 1) % 4]))
            nbrs[f[(a + 1) % 4]].add(int(f[a]))
    free = np.array([v for v in range(n_side, len(nodes))], dtype=np.int64)
    if len(free):
        lists = [np.fromiter(nbrs[v], dtype=np.int64) for v in free]
        for _ in range(smooth):
            new = np.array([nodes[l, :2].mean(axis=0) for l in lists])
            nodes[free, :2] = new
    return _pack(nodes, faces, QUAD_1)


def cylinder_40k():
    """The 40000-quad closed cylinder R=1, L=4: 160 x 200 side grid plus
    O-grid caps of 40*40 core quads and 15 rings of 160 quads each."""
    return cylinder(n_theta=160, n_z=200, n_ring=15)


def element_corners(nodes, elems):
    """(n_elems, 4, 3) corner coordinates (4th corner of a triangle = NaN)."""
    idx = elems[:, 1:5]
    out = np.full((len(elems), 4, 3), np.nan)
    valid = idx >= 0
    out[valid] = nodes[idx[valid]]
    return out


def centroids_and_normals(nodes, elems):
    """Element centres x(domain centre) and unit normals at the centre."""
    c = element_corners(nodes, elems)
    is_quad = elems[:, 0] == QUAD_1
    cen = np.where(is_quad[:, None], np.nanmean(c, axis=1), np.nanmean(c[:, :3], axis=1))
    t1 = np.where(is_quad[:, None], (c[:, 1] + c[:, 2] - c[:, 0] - c[:, 3]) / 4, c[:, 1] - c[:, 0])
    t2 = np.where(is_quad[:, None], (c[:, 2] + c[:, 3] - c[:, 0] - c[:, 1]) / 4, c[:, 2] - c[:, 0])
    n = np.cross(t1, t2)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    return cen, n


def read_off(path, tag=None):
    """Read an OFF surface mesh (nihu/interface/read_off_mesh.hpp): header
    ``OFF``, counts line, node coordinates, then faces ``n i0 .. i(n-1)``.
    Faces with 3 nodes become tria_1, with 4 nodes quad_1."""
    with open(path) as f:
        tokens = f.read().split()
    if not tokens or tokens[0] != "OFF":
        raise RuntimeError("not an OFF file: " + str(path))
    nn, ne = int(tokens[1]), int(tokens[2])
    pos = 4
    nodes = np.array(tokens[pos:pos + 3 * nn], dtype=np.float64).reshape(nn, 3)
    pos += 3 * nn
    elems = np.full((ne, 5), -1, dtype=np.int32)
    for e in range(ne):
        k = int(tokens[pos]); pos += 1
        if k not in (3, 4):
            raise RuntimeError("unsupported OFF face with %d nodes" % k)
        elems[e, 0] = TRIA_1 if k == 3 else QUAD_1
        elems[e, 1:1 + k] = [int(t) for t in tokens[pos:pos + k]]
        pos += k
    return nodes, elems


def plane_wave_neumann(nodes, elems, k: float, directions):
    """Neumann data of the field scattered by a rigid body from plane waves
    p_inc = exp(-i k d.x) (e^{-ikr} convention): q = -dp_inc/dn = i k (d.n) p_inc,
    sampled at the element centres; returns (n_elems, n_directions) complex128."""
    cen, nrm = centroids_and_normals(nodes, elems)
    d = np.asarray(directions, dtype=np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    p_inc = np.exp(-1j * k * (cen @ d.T))
    return np.asfortranarray(1j * k * (nrm @ d.T) * p_inc)


def sphere_directions(count: int, seed: int = 0):
    """``count`` unit vectors uniform on the sphere (seeded)."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((count, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)
