"""Mesh generators, the Fluent .msh writer and initial states.

Every generated face is oriented the way the reference's left/right logic
needs (mesh/MshBlock.cpp:281-305): the area vector (-(y0-y1), x0-x1) of
nodes (n0, n1) points INTO cell c0.  With that orientation the reference's
flags and the geometric ones agree, so generated meshes upwind correctly
with or without the reference's quirks.

A mesh is a dict: node_xy [nN,2], face_nodes [nF,2], face_cells [nF,2]
(c1 = -1 on boundary faces), zones [nz,4] = (id, first face 1-based, last,
type), n_cells, and optionally c1_shift [nF,2] (periodic image shift).
Zone types follow the reference: 2 interior, 3 wall, 5 outlet, 7 symmetry,
10 inlet.
"""
import numpy as np

GAMMA = 1.4
INTERIOR, WALL, OUTLET, SYMMETRY, INLET = 2, 3, 5, 7, 10


def _orient_into_c0(node_xy, face_nodes, face_cells, c0_point):
    """Swap node order where the area vector does not point into c0."""
    a = node_xy[face_nodes[:, 0]]
    b = node_xy[face_nodes[:, 1]]
    d = np.stack([b[:, 1] - a[:, 1], a[:, 0] - b[:, 0]], 1)
    mid = 0.5 * (a + b)
    flip = np.einsum("ij,ij->i", d, mid - c0_point) > 0
    fn = face_nodes.copy()
    fn[flip] = fn[flip][:, ::-1]
    return fn


def reorient(mesh, mode="fluent", seed=0):
    """Copy of ``mesh`` with face node orders reversed: ``"fluent"`` reverses
    every face (area vectors point out of c0, as in the shipped Fluent
    meshes, which the reference's flag logic handles backwards), ``"random"``
    reverses a random half of the faces."""
    m = dict(mesh)
    fn = mesh["face_nodes"].copy()
    if mode == "fluent":
        flip = np.ones(len(fn), bool)
    else:
        flip = np.random.default_rng(seed).random(len(fn)) < 0.5
    fn[flip] = fn[flip][:, ::-1]
    m["face_nodes"] = fn
    return m


def with_zone_types(mesh, old, new):
    """Copy of ``mesh`` with zones of type ``old`` retyped to ``new``."""
    m = dict(mesh)
    z = mesh["zones"].copy()
    z[z[:, 3] == old, 3] = new
    m["zones"] = z
    return m


def sod_strip(nx=1000, ny=4, length=1.0, height=0.01, ends=OUTLET):
    """Quad strip [0,L]x[0,H] of nx*ny cells (Sod tube).  Zones: interior,
    bottom and top walls (slip), left and right ends of type ``ends``."""
    xs = np.linspace(0.0, length, nx + 1)
    ys = np.linspace(0.0, height, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    node_xy = np.stack([X.ravel(), Y.ravel()], 1)
    nid = lambda i, j: i * (ny + 1) + j
    cid = lambda i, j: i * ny + j
    faces, cells, kinds = [], [], []
    # interior vertical faces x = x_i, between cells (i-1, j) and (i, j)
    I, J = np.meshgrid(np.arange(1, nx), np.arange(ny), indexing="ij")
    I, J = I.ravel(), J.ravel()
    faces.append(np.stack([nid(I, J + 1), nid(I, J)], 1))
    cells.append(np.stack([cid(I - 1, J), cid(I, J)], 1))
    # interior horizontal faces y = y_j, between (i, j-1) and (i, j)
    I, J = np.meshgrid(np.arange(nx), np.arange(1, ny), indexing="ij")
    I, J = I.ravel(), J.ravel()
    faces.append(np.stack([nid(I, J), nid(I + 1, J)], 1))
    cells.append(np.stack([cid(I, J - 1), cid(I, J)], 1))
    n_int = sum(len(f) for f in faces)
    bnd = []
    i = np.arange(nx)
    bnd.append((np.stack([nid(i + 1, 0), nid(i, 0)], 1), cid(i, 0), WALL))
    bnd.append((np.stack([nid(i, ny), nid(i + 1, ny)], 1), cid(i, ny - 1), WALL))
    j = np.arange(ny)
    bnd.append((np.stack([nid(0, j), nid(0, j + 1)], 1), cid(0, j), ends))
    bnd.append((np.stack([nid(nx, j + 1), nid(nx, j)], 1), cid(nx - 1, j), ends))
    zones = [(1, 1, n_int, INTERIOR)]
    start = n_int + 1
    for k, (fn, c0, ty) in enumerate(bnd):
        faces.append(fn)
        cells.append(np.stack([c0, -np.ones_like(c0)], 1))
        zones.append((2 + k, start, start + len(fn) - 1, ty))
        start += len(fn)
    face_nodes = np.concatenate(faces).astype(np.int32)
    face_cells = np.concatenate(cells).astype(np.int32)
    # cell centroids for the orientation check
    cc = np.zeros((nx * ny, 2))
    II, JJ = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    cc[cid(II, JJ).ravel()] = np.stack(
        [0.5 * (xs[II] + xs[II + 1]).ravel(), 0.5 * (ys[JJ] + ys[JJ + 1]).ravel()], 1)
    face_nodes = _orient_into_c0(node_xy, face_nodes, face_cells, cc[face_cells[:, 0]])
    return dict(node_xy=node_xy, face_nodes=face_nodes, face_cells=face_cells,
                zones=np.array(zones, np.int32), n_cells=nx * ny)


def _edges_from_tris(tri_nodes, tri_xy):
    """Unique edges of a triangulation given per-triangle node ids."""
    e = np.concatenate([tri_nodes[:, [0, 1]], tri_nodes[:, [1, 2]], tri_nodes[:, [2, 0]]])
    owner = np.tile(np.arange(len(tri_nodes)), 3)
    key = np.sort(e, 1)
    return e, owner, key


def _box_triangulation(nx, ny, lx, ly, jitter, seed):
    """Jittered Delaunay triangles on [0,lx]x[0,ly]: points, triangles,
    unique edges with their cells, and the box side of each boundary edge
    (0 left, 1 right, 2 bottom, 3 top)."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    hx, hy = lx / nx, ly / ny
    X, Y = np.meshgrid(np.linspace(0, lx, nx + 1), np.linspace(0, ly, ny + 1), indexing="ij")
    jx = rng.uniform(-jitter, jitter, X.shape) * hx
    jy = rng.uniform(-jitter, jitter, Y.shape) * hy
    jx[0, :] = jx[-1, :] = 0
    jy[:, 0] = jy[:, -1] = 0
    pts = np.stack([(X + jx).ravel(), (Y + jy).ravel()], 1)
    tri = Delaunay(pts).simplices.astype(np.int64)
    a, b, c = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    area = 0.5 * ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
    tri = tri[np.abs(area) > 1e-14 * hx * hy]
    e, owner, key = _edges_from_tris(tri, pts)
    k = key[:, 0] * len(pts) + key[:, 1]
    order = np.argsort(k, kind="stable")
    ks = k[order]
    first = np.ones(len(ks), bool)
    first[1:] = ks[1:] != ks[:-1]
    grp = np.cumsum(first) - 1
    n_e = grp[-1] + 1
    c0 = np.full(n_e, -1)
    c1 = np.full(n_e, -1)
    en = np.zeros((n_e, 2), np.int64)
    idx_first = order[first]
    c0[:] = owner[idx_first]
    en[:] = e[idx_first]
    second = ~first
    c1[grp[second]] = owner[order[second]]
    interior = c1 >= 0
    mid = pts[en].mean(1)
    tol = 1e-9
    side = np.full(n_e, -1)
    side[~interior & (np.abs(mid[:, 0]) < tol * lx)] = 0
    side[~interior & (np.abs(mid[:, 0] - lx) < tol * lx)] = 1
    side[~interior & (np.abs(mid[:, 1]) < tol * ly)] = 2
    side[~interior & (np.abs(mid[:, 1] - ly) < tol * ly)] = 3
    if np.any(~interior & (side < 0)):
        raise RuntimeError("boundary edge off the box")
    return pts, tri, en, c0, c1, interior, side, mid


def _assemble(pts, tri, en, c0, c1, groups):
    """Faces in zone order: groups = [(edge indices, zone type)], interior
    first; area vectors oriented into c0."""
    faces = np.concatenate([en[s] for s, _ in groups]).astype(np.int32)
    fc = np.stack([np.concatenate([c0[s] for s, _ in groups]),
                   np.concatenate([c1[s] for s, _ in groups])], 1).astype(np.int32)
    zones, start = [], 1
    for zi, (s, ty) in enumerate(groups):
        zones.append((zi + 1, start, start + len(s) - 1, ty))
        start += len(s)
    zones = [z for z in zones if z[2] >= z[1]]
    cen = pts[tri].mean(1)
    fn = _orient_into_c0(pts, faces, fc, cen[fc[:, 0]])
    return dict(node_xy=pts, face_nodes=fn, face_cells=fc,
                zones=np.array(zones, np.int32), n_cells=len(tri))


def tri_box(nx=40, ny=20, lx=4.0, ly=2.0, jitter=0.2, seed=1,
            left=INLET, right=OUTLET, bottom=WALL, top=SYMMETRY):
    """Jittered Delaunay triangles on a box, one boundary zone per side."""
    pts, tri, en, c0, c1, interior, side, _ = _box_triangulation(nx, ny, lx, ly, jitter, seed)
    groups = [(np.where(interior)[0], INTERIOR)]
    groups += [(np.where(side == s)[0], ty) for s, ty in enumerate([left, right, bottom, top])]
    return _assemble(pts, tri, en, c0, c1, groups)


def wedge(cells=20000, angle_deg=10.0, seed=1, length=3.0, height=1.5, ramp_x=0.5,
          jitter=0.2, upstream=WALL):
    """Supersonic compression ramp: the box [0,length]x[0,height] whose floor
    turns up by angle_deg at x = ramp_x, triangulated with about `cells`
    jittered Delaunay triangles (the triangulation of the box, mapped so
    the floor follows the ramp).  Zones: inlet (left), outlet (right and
    top), the floor before the ramp (`upstream`), wall (the ramp).

    upstream = WALL (default): a flat plate from the inlet, so the laminar
    boundary layer develops ahead of the ramp (the classic compression-ramp
    interaction).  SYMMETRY: a slip floor; the boundary layer then starts at
    the ramp corner, and in the laminar cases the slip/no-slip junction
    drives the corner cell towards vacuum (a state the implicit update can
    only leave through the temperature floor, after which its case stalls).
    For inviscid cases both give the same (mirror) boundary."""
    ny = max(4, int(round(np.sqrt(cells * height / (2.0 * length)))))
    nx = max(4, int(round(cells / (2.0 * ny))))
    pts, tri, en, c0, c1, interior, side, mid = _box_triangulation(nx, ny, length, height,
                                                                   jitter, seed)
    t = np.tan(np.radians(angle_deg))
    x, y = pts[:, 0], pts[:, 1]
    yw = np.maximum(0.0, x - ramp_x) * t
    pts = np.stack([x, yw + y * (height - yw) / height], 1)
    floor = side == 2
    groups = [(np.where(interior)[0], INTERIOR),
              (np.where(side == 0)[0], INLET),
              (np.where(floor & (mid[:, 0] < ramp_x))[0], upstream),
              (np.where(floor & (mid[:, 0] >= ramp_x))[0], WALL),
              (np.where((side == 1) | (side == 3))[0], OUTLET)]
    return _assemble(pts, tri, en, c0, c1, groups)


def max_deflection(mach, gamma=GAMMA):
    """Largest ramp angle (degrees) with an attached oblique shock at this
    Mach number (the maximum of the theta-beta-Mach relation)."""
    b = np.linspace(np.arcsin(1.0 / mach) + 1e-9, np.pi / 2, 20001)
    t = np.arctan(2.0 / np.tan(b) * (mach ** 2 * np.sin(b) ** 2 - 1.0)
                  / (mach ** 2 * (gamma + np.cos(2 * b)) + 2.0))
    return float(np.degrees(t.max()))


def post_shock_mach(mach, angle_deg, gamma=GAMMA):
    """Mach number behind the attached weak oblique shock of a ramp of
    angle_deg (theta-beta-Mach relation), or None when the shock detaches."""
    th = np.radians(angle_deg)
    b = np.linspace(np.arcsin(1.0 / mach) + 1e-9, np.pi / 2, 200001)
    t = np.arctan(2.0 / np.tan(b) * (mach ** 2 * np.sin(b) ** 2 - 1.0)
                  / (mach ** 2 * (gamma + np.cos(2 * b)) + 2.0))
    if t.max() < th:
        return None
    beta = b[np.argmax(t >= th)]  # the weak solution: smallest shock angle
    mn1 = mach * np.sin(beta)
    mn2 = np.sqrt((1.0 + 0.5 * (gamma - 1.0) * mn1 ** 2)
                  / (gamma * mn1 ** 2 - 0.5 * (gamma - 1.0)))
    return float(mn2 / np.sin(beta - th))


def wedge_family(n_cases, cells=(20000, 400000), mach=(1.5, 3.0), angle=(5.0, 15.0),
                 reynolds=(1e3, 1e4), seed=20261204, min_post_mach=1.2):
    """Seeded parameters of the compression-ramp family: per case (Mach,
    angle, Re, cells, mesh seed).  An angle whose inviscid flow behind the
    ramp shock is slower than min_post_mach is drawn again: the steady
    problem needs a supersonic outflow outside the boundary layer (the
    outlets extrapolate), and near the detachment angle the laminar
    layer's displacement turns the barely supersonic post-shock flow
    subsonic, so the shock system never settles (Mach 1.6 at 13.2 deg,
    inviscid post-shock Mach 1.07, oscillated between 1e-3 and 2e-2 of its
    first residual for 8,000 iterations)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_cases):
        m = rng.uniform(*mach)
        a = rng.uniform(*angle)
        while (post_shock_mach(m, a) or 0.0) < min_post_mach:
            a = rng.uniform(*angle)
        out.append(dict(mach=m, angle=a, reynolds=rng.uniform(*reynolds),
                        cells=int(rng.uniform(*cells)), seed=seed + 1 + k))
    return out


def freestream(mach, n=None, angle_deg=0.0):
    """Free-stream conserved state, rho = 1, p = 1/gamma (speed of sound 1),
    velocity mach along angle_deg; one row, or n rows."""
    a = np.radians(angle_deg)
    q = primitive_to_q(np.array([1.0]), np.array([mach * np.cos(a)]),
                       np.array([mach * np.sin(a)]), np.array([1.0 / GAMMA]))[0]
    return q if n is None else np.tile(q, (n, 1))


def periodic_delaunay(n=1000, length=10.0, jitter=0.25, seed=20261203):
    """Jittered Delaunay triangulation of the periodic square [0,L)^2.

    Nodes: an n x n lattice with spacing h = L/n, each node moved by
    U(-jitter*h, +jitter*h) per axis from ``numpy.random.default_rng(seed)``.
    The Delaunay triangulation of the lattice plus a periodic ghost layer is
    computed with scipy (Qhull); triangles whose centroid lies in [0,L)^2
    form the mesh.  Every edge becomes one interior face; faces that cross
    the periodic boundary carry c1_shift, the translation that maps cell
    c1's coordinates into the frame of the face (and of c0).  Node
    coordinates are stored per face frame (ghost images are separate nodes).
    """
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    h = length / n
    I, J = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    base = np.stack([I.ravel() * h, J.ravel() * h], 1)
    base = base + rng.uniform(-jitter * h, jitter * h, base.shape)
    # ghost layer of width g nodes on every side
    g = 3
    oi, oj = np.meshgrid(np.arange(-g, n + g), np.arange(-g, n + g), indexing="ij")
    bi, bj = oi % n, oj % n
    sx, sy = (oi - bi) // n, (oj - bj) // n
    src = (bi * n + bj).ravel()
    shift = np.stack([sx.ravel(), sy.ravel()], 1)
    pts = base[src] + shift * length
    tri = Delaunay(pts).simplices.astype(np.int64)
    cen = pts[tri].mean(1)
    inside = np.all((cen >= 0) & (cen < length), 1)
    kept = tri[inside]
    nT = len(kept)
    # edges of the kept triangles, each in its triangle's own frame
    e_pts = np.concatenate([kept[:, [0, 1]], kept[:, [1, 2]], kept[:, [2, 0]]])
    owner = np.tile(np.arange(nT), 3)
    # canonical key of an edge: its base node ids and the periodic offset
    # between its endpoints' frames (the same on both sides of the edge)
    ea, eb = e_pts[:, 0], e_pts[:, 1]
    sa, sb = src[ea], src[eb]
    da, db = shift[ea], shift[eb]
    # orient the key so that the smaller base id comes first
    swap = sa > sb
    k0 = np.where(swap, sb, sa)
    k1 = np.where(swap, sa, sb)
    rel = np.where(swap[:, None], da - db, db - da).astype(np.int64)  # offset of k1 rel. k0
    ekey = ((k0 * (n * n) + k1) * 3 + (rel[:, 0] + 1)) * 3 + (rel[:, 1] + 1)
    eo = np.argsort(ekey, kind="stable")
    eks = ekey[eo]
    first = np.ones(len(eks), bool)
    first[1:] = eks[1:] != eks[:-1]
    if not np.all(first[::2]) or np.any(first[1::2]):
        raise RuntimeError("periodic triangulation is not a closed torus")
    i0 = eo[0::2]
    i1 = eo[1::2]
    c0 = owner[i0]
    c1 = owner[i1]
    # c1_shift: translation mapping c1's frame onto the edge as seen by c0
    pa0 = pts[ea[i0]]
    # endpoint of i1 with the same base id as endpoint a of i0
    same = src[ea[i1]] == src[ea[i0]]
    pa1 = np.where(same[:, None], pts[ea[i1]], pts[eb[i1]])
    c1_shift = pa0 - pa1
    c1_shift = np.round(c1_shift / length) * length
    # frame of each triangle is the positions of its own vertices; nodes per
    # face are the c0-frame positions, deduplicated
    fa = pts[ea[i0]]
    fb = pts[eb[i0]]
    allp = np.concatenate([fa, fb])
    q = np.round(allp / (h * 1e-6)).astype(np.int64)
    _, uidx, inv = np.unique(q[:, 0] * (1 << 31) + q[:, 1], return_index=True,
                             return_inverse=True)
    node_xy = allp[uidx]
    nf = len(i0)
    face_nodes = np.stack([inv[:nf], inv[nf:]], 1).astype(np.int32)
    face_cells = np.stack([c0, c1], 1).astype(np.int32)
    cen_k = pts[kept].mean(1)
    face_nodes = _orient_into_c0(node_xy, face_nodes, face_cells, cen_k[c0])
    zones = np.array([(1, 1, nf, INTERIOR)], np.int32)
    return dict(node_xy=node_xy, face_nodes=face_nodes, face_cells=face_cells,
                zones=zones, n_cells=nT, c1_shift=c1_shift, cell_centroid=cen_k)


def write_msh(path, mesh, crlf=False):
    """Fluent ASCII 2D .msh of the subset the reference reader parses
    (lower-case hex ids, single spaces, interior zone first)."""
    nl = "\r\n" if crlf else "\n"
    xy, fn, fc, zones = mesh["node_xy"], mesh["face_nodes"], mesh["face_cells"], mesh["zones"]
    nN, nF, nC = len(xy), len(fn), int(mesh["n_cells"])
    out = ['(0 "mstcfd meshgen")', "(2 2)",
           f"(10 (0 1 {nN:x} 0 2))", f"(10 (1 1 {nN:x} 1 2)", "("]
    out += [f"{x!r} {y!r}" for x, y in xy.tolist()]
    out += ["))", f"(12 (0 1 {nC:x} 0 0))", f"(12 (2 1 {nC:x} 1 1))",
            f"(13 (0 1 {nF:x} 0 0))"]
    for zi, (zid, st, en, ty) in enumerate(zones.tolist()):
        out.append(f'(0 "zone {zi}")')
        out.append(f"(13 ({zid + 2:x} {st:x} {en:x} {ty:x} 2)(")
        for f in range(st - 1, en):
            a, b = fn[f] + 1
            c0, c1 = fc[f] + 1
            out.append(f"{a:x} {b:x} {c0:x} {c1 if c1 > 0 else 0:x}")
        out.append("))")
    with open(path, "w", newline="") as fh:
        fh.write(nl.join(out) + nl)


# ---------------------------------------------------------------------------
# 3D meshes (host reader only)
# ---------------------------------------------------------------------------
_KUHN = [(0, 1, 3, 7), (0, 1, 5, 7), (0, 2, 3, 7), (0, 2, 6, 7), (0, 4, 5, 7), (0, 4, 6, 7)]
_HEX_FACES = [(0, 2, 6, 4), (1, 3, 7, 5), (0, 1, 5, 4), (2, 3, 7, 6), (0, 1, 3, 2), (4, 5, 7, 6)]


def _box_nodes(nx, ny, nz, length, jitter, seed):
    rng = np.random.default_rng(seed)
    h = length / np.array([nx, ny, nz], float)
    g = np.stack(np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1),
                             indexing="ij"), -1).reshape(-1, 3).astype(float)
    inner = np.all((g > 0) & (g < [nx, ny, nz]), 1)
    j = rng.uniform(-jitter, jitter, g.shape) * inner[:, None]
    xyz = (g + j) * h
    idx = lambda i, k, l: (i * (ny + 1) + k) * (nz + 1) + l
    return xyz, idx


def _assemble3d(xyz, cells_faces, n_cells, side_of, kinds):
    """Unique faces of the cells (node tuples per cell face), boundary faces
    grouped by box side; every area vector points into c0."""
    keys = {}
    faces, fc = [], []
    for c, fl in enumerate(cells_faces):
        for f in fl:
            k = tuple(sorted(f))
            if k in keys:
                fc[keys[k]][1] = c
            else:
                keys[k] = len(faces)
                faces.append(list(f))
                fc.append([c, -1])
    fc = np.array(fc)
    cen = np.zeros((n_cells, 3))
    cnt = np.zeros(n_cells)
    for f, (a, b) in zip(faces, fc):
        m = xyz[f].mean(0)
        for cc in (a, b):
            if cc >= 0:
                cen[cc] += m
                cnt[cc] += 1
    cen /= cnt[:, None]
    # orient into c0: the reference's area vector (n1-n0) x (n2-n0)
    for i, f in enumerate(faces):
        p = xyz[f]
        d = np.cross(p[1] - p[0], p[2] - p[0])
        if np.dot(d, p.mean(0) - cen[fc[i, 0]]) > 0:
            faces[i] = f[::-1]
    interior = fc[:, 1] >= 0
    side = np.array([side_of(xyz[f].mean(0)) if not interior[i] else -1
                     for i, f in enumerate(faces)])
    groups = [np.where(interior)[0]] + [np.where(side == s)[0] for s in range(6)]
    types = [INTERIOR] + list(kinds)
    order = np.concatenate(groups)
    zones, start = [], 1
    for zi, (g, ty) in enumerate(zip(groups, types)):
        if len(g):
            zones.append((zi + 1, start, start + len(g) - 1, ty))
            start += len(g)
    return dict(node_xyz=xyz, faces=[faces[i] for i in order], face_cells=fc[order],
                zones=np.array(zones, np.int32), n_cells=n_cells)


def tet_box(n=4, length=1.0, jitter=0.15, seed=1,
            kinds=(INLET, OUTLET, WALL, WALL, SYMMETRY, SYMMETRY)):
    """n^3 jittered hexahedra split into 6 tetrahedra each (the config-3
    mesh type), one boundary zone per box side (x-, x+, y-, y+, z-, z+)."""
    xyz, idx = _box_nodes(n, n, n, length, jitter, seed)
    cells = []
    for i in range(n):
        for k in range(n):
            for l in range(n):
                v = [idx(i + (c & 1), k + ((c >> 1) & 1), l + ((c >> 2) & 1)) for c in range(8)]
                for t in _KUHN:
                    q = [v[j] for j in t]
                    cells.append([[q[0], q[1], q[2]], [q[0], q[1], q[3]], [q[0], q[2], q[3]],
                                  [q[1], q[2], q[3]]])
    tol = 1e-9 * length

    def side_of(c):
        for d in range(3):
            if abs(c[d]) < tol:
                return 2 * d
            if abs(c[d] - length) < tol:
                return 2 * d + 1
        raise RuntimeError("boundary face off the box")
    return _assemble3d(xyz, cells, len(cells), side_of, kinds)


def hex_box(n=4, length=1.0, jitter=0.0, seed=1,
            kinds=(INLET, OUTLET, WALL, WALL, SYMMETRY, SYMMETRY)):
    """n^3 hexahedra (quadrilateral faces), one boundary zone per side."""
    xyz, idx = _box_nodes(n, n, n, length, jitter, seed)
    cells = []
    for i in range(n):
        for k in range(n):
            for l in range(n):
                v = [idx(i + (c & 1), k + ((c >> 1) & 1), l + ((c >> 2) & 1)) for c in range(8)]
                cells.append([[v[j] for j in f] for f in _HEX_FACES])
    tol = 1e-9 * length

    def side_of(c):
        for d in range(3):
            if abs(c[d]) < tol:
                return 2 * d
            if abs(c[d] - length) < tol:
                return 2 * d + 1
        raise RuntimeError("boundary face off the box")
    return _assemble3d(xyz, cells, len(cells), side_of, kinds)


def tet_grid(n, length=2 * np.pi, jitter=0.15, seed=20261205):
    """Periodic [0, L)^3: an n^3 lattice of hexahedra, each split into 6
    tetrahedra along its main diagonal (the Kuhn subdivision, conforming
    across hexahedra), nodes moved by U(-jitter h, +jitter h) per axis.
    6 n^3 cells, 12 n^3 triangular faces, all interior.

    The faces are enumerated analytically, vectorised over hexahedra: with
    tet T_s = {0, e_s1, e_s1 + e_s2, 7} for an axis permutation s, its face
    opposite e_s1 is shared with T_(s2, s1, s3) and its face opposite
    e_s1 + e_s2 with T_(s1, s3, s2) (both in the same hexahedron); its face
    opposite 7, on the hexahedron's lower side x_s3 = 0, is shared with
    T_(s3, s1, s2) of the hexahedron below along s3.  Every hexahedron owns
    its 6 interior faces and the 6 faces on its lower sides.

    Nodes are the (n+1)^3 unwrapped lattice points (the images at index n
    carry the jitter of index 0 plus L); every face lists its nodes in the
    frame of its c0 (the owning hexahedron's tet) and carries c1_shift =
    x(c0 frame) - x(c1 frame), -L along s3 where the lower side wraps.
    Every area vector points into c0."""
    n = int(n)
    if n < 2 or n > 128:
        raise ValueError("tet_grid: 2 <= n <= 128")
    h = length / n
    n1 = n + 1
    rng = np.random.default_rng(seed)
    jit = rng.uniform(-jitter, jitter, (n ** 3, 3))
    ax = np.arange(n1)
    gi, gj, gk = np.meshgrid(ax, ax, ax, indexing="ij")
    wrap = ((gi % n) * n + (gj % n)) * n + (gk % n)
    xyz = (np.stack([gi, gj, gk], -1).reshape(-1, 3) + jit[wrap.ravel()]) * h
    del gi, gj, gk, wrap
    # tet index of each axis permutation (the order of _KUHN)
    sig = []
    for t in _KUHN:
        a1 = int(np.log2(t[1]))
        a2 = int(np.log2(t[2] - t[1]))
        sig.append((a1, a2, 3 - a1 - a2))
    idx = {s_: i for i, s_ in enumerate(sig)}
    e = [1, 2, 4]  # corner bit of each axis
    local = []  # (tet, partner tet, corners (3), lower side axis or -1)
    for i, (s1, s2, s3) in enumerate(sig):
        for corners, partner in (((0, e[s1] + e[s2], 7), (s2, s1, s3)),
                                 ((0, e[s1], 7), (s1, s3, s2))):
            j = idx[partner]
            if i < j:
                local.append((i, j, corners, -1))
        local.append((i, idx[(s3, s1, s2)], (0, e[s1], e[s1] + e[s2]), s3))
    assert len(local) == 12
    cube = np.arange(n ** 3, dtype=np.int64)
    ci, cj, ck = cube // (n * n), (cube // n) % n, cube % n
    base_u = (ci * n1 + cj) * n1 + ck
    coff = lambda c: (c & 1) * n1 * n1 + ((c >> 1) & 1) * n1 + ((c >> 2) & 1)
    nF = 12 * n ** 3
    faces = np.empty((n ** 3, 12, 3), np.int64)
    fc = np.empty((n ** 3, 12, 2), np.int64)
    shift = np.zeros((n ** 3, 12, 3))
    cidx = (ci, cj, ck)
    for f, (t0, t1, corners, side) in enumerate(local):
        for j, c in enumerate(corners):
            faces[:, f, j] = base_u + coff(c)
        fc[:, f, 0] = 6 * cube + t0
        if side < 0:
            fc[:, f, 1] = 6 * cube + t1
        else:
            nb = list(cidx)
            nb[side] = (cidx[side] - 1) % n
            fc[:, f, 1] = 6 * ((nb[0] * n + nb[1]) * n + nb[2]) + t1
            shift[:, f, side] = np.where(cidx[side] == 0, -length, 0.0)
    faces = faces.reshape(nF, 3)
    fc = fc.reshape(nF, 2)
    shift = shift.reshape(nF, 3)
    # cell centroids (mean of the 4 nodes, own frame)
    kuhn = np.array(_KUHN, np.int64)
    offs = np.array([coff(c) for c in range(8)], np.int64)
    cn = base_u[:, None, None] + offs[kuhn][None, :, :]         # [n^3, 6, 4]
    centroid = xyz[cn.reshape(-1, 4)].mean(1)
    del cn
    # orientation: the area vector (n1-n0) x (n2-n0) points into c0
    p0, p1, p2 = xyz[faces[:, 0]], xyz[faces[:, 1]], xyz[faces[:, 2]]
    nrm = np.cross(p1 - p0, p2 - p0)
    ctr = (p0 + p1 + p2) / 3.0
    del p0, p1, p2
    flip = np.einsum("ij,ij->i", nrm, ctr - centroid[fc[:, 0]]) > 0
    del nrm, ctr
    faces[flip, 1], faces[flip, 2] = faces[flip, 2].copy(), faces[flip, 1].copy()
    return {"node_xyz": xyz, "faces": faces.astype(np.int32),
            "face_cells": fc.astype(np.int32),
            "zones": np.array([[3, 1, nF, INTERIOR]], np.int32), "n_cells": 6 * n ** 3,
            "c1_shift": shift, "cell_centroid": centroid}


def taylor_green(xyz, mach=0.1, rho0=1.0, length=2 * np.pi):
    """Compressible Taylor-Green vortex on [0, 2 pi)^3 (L = 1 per radian):
    u = V0 sin x cos y cos z, v = -V0 cos x sin y cos z, w = 0,
    p = p0 + rho0 V0^2 / 16 (cos 2x + cos 2y)(cos 2z + 2), rho = rho0 p/p0
    (isothermal start), V0 = mach (speed of sound 1: p0 = rho0 / gamma)."""
    x, y, z = (xyz[:, k] * (2 * np.pi / length) for k in range(3))
    v0 = mach
    p0 = rho0 / GAMMA
    u = v0 * np.sin(x) * np.cos(y) * np.cos(z)
    v = -v0 * np.cos(x) * np.sin(y) * np.cos(z)
    w = np.zeros_like(u)
    p = p0 + rho0 * v0 ** 2 / 16.0 * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2.0)
    rho = rho0 * p / p0
    E = p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return np.stack([rho, rho * u, rho * v, rho * w, E], 1)


def write_msh3d(path, mesh, mixed_zones=(), crlf=False):
    """Fluent ASCII 3D .msh: zones with a fixed face node count, or, for the
    zone indices in mixed_zones, a mixed zone (node count 0 in the header,
    each line led by its node count)."""
    nl = "\r\n" if crlf else "\n"
    xyz, faces, fc, zones = mesh["node_xyz"], mesh["faces"], mesh["face_cells"], mesh["zones"]
    nN, nF, nC = len(xyz), len(faces), int(mesh["n_cells"])
    out = ['(0 "mstcfd meshgen 3D")', "(2 3)",
           f"(10 (0 1 {nN:x} 0 3))", f"(10 (1 1 {nN:x} 1 3)", "("]
    out += [f"{x!r} {y!r} {z!r}" for x, y, z in xyz.tolist()]
    out += ["))", f"(12 (0 1 {nC:x} 0 0))", f"(12 (2 1 {nC:x} 1 0))",
            f"(13 (0 1 {nF:x} 0 0))"]
    for zi, (zid, st, en, ty) in enumerate(zones.tolist()):
        k = len(faces[st - 1])
        mixed = zi in mixed_zones
        out.append(f'(0 "zone {zi}")')
        out.append(f"(13 ({zid + 2:x} {st:x} {en:x} {ty:x} {0 if mixed else k:x})(")
        for f in range(st - 1, en):
            ids = " ".join(f"{v + 1:x}" for v in faces[f])
            c0, c1 = fc[f] + 1
            lead = f"{len(faces[f]):x} " if mixed else ""
            out.append(f"{lead}{ids} {c0:x} {c1 if c1 > 0 else 0:x}")
        out.append("))")
    with open(path, "w", newline="") as fh:
        fh.write(nl.join(out) + nl)


# ---------------------------------------------------------------------------
# initial states
# ---------------------------------------------------------------------------
def reference_inlet():
    """CONST.h:70-83 as the macros expand: (1, 0, 0, 1/286.32*715.8)."""
    return np.array([1.0, 1.0 * 0, 1.0 * 0, 1 * (1 / 286.32 * 715.8 + 0.5 * (0 * 0 + 0 * 0))])


def sod_state(cell_ctr, x0=0.5):
    """Time::initialization (time/Time.cpp:13-53): the reference state, with
    rho scaled by 0.125 and E by 0.1 where the cell centre x > x0."""
    q = np.tile(reference_inlet(), (len(cell_ctr), 1))
    right = cell_ctr[:, 0] > x0
    q[right, 0] *= 0.125
    q[right, 3] *= 0.1
    return q


def primitive_to_q(rho, u, v, p):
    return np.stack([rho, rho * u, rho * v, p / (GAMMA - 1) + 0.5 * rho * (u * u + v * v)], -1)


def q_to_primitive(q):
    rho = q[..., 0]
    u, v = q[..., 1] / rho, q[..., 2] / rho
    p = (GAMMA - 1) * (q[..., 3] - 0.5 * rho * (u * u + v * v))
    return rho, u, v, p


def isentropic_vortex(xy, t=0.0, length=10.0, beta=5.0, mach=0.5, x0=None):
    """Isentropic vortex of strength beta convected along +x at the given
    Mach number (free stream rho = p = 1) on the periodic square [0,L)^2,
    as the sum over the nearest periodic images."""
    x0 = np.array([length / 2, length / 2]) if x0 is None else np.asarray(x0)
    ainf = np.sqrt(GAMMA)
    uinf = mach * ainf
    c = x0 + np.array([uinf * t, 0.0])
    du = np.zeros(len(xy))
    dv = np.zeros(len(xy))
    dT = np.zeros(len(xy))
    for ix in (-1, 0, 1):
        for iy in (-1, 0, 1):
            cx = (c[0] % length) + ix * length
            cy = (c[1] % length) + iy * length
            dx, dy = xy[:, 0] - cx, xy[:, 1] - cy
            r2 = dx * dx + dy * dy
            e = np.exp(0.5 * (1 - r2))
            du += -beta / (2 * np.pi) * dy * e
            dv += beta / (2 * np.pi) * dx * e
            dT += -(GAMMA - 1) * beta ** 2 / (8 * GAMMA * np.pi ** 2) * e * e
    T = 1.0 + dT
    rho = T ** (1 / (GAMMA - 1))
    p = rho * T
    return primitive_to_q(rho, uinf + du, dv, p)


def random_state(n, seed=0, umax=2.0):
    """Random physical states: rho, p in [0.5, 1.5], |u|,|v| <= umax."""
    r = np.random.default_rng(seed)
    return primitive_to_q(r.uniform(0.5, 1.5, n), r.uniform(-umax, umax, n),
                          r.uniform(-umax, umax, n), r.uniform(0.5, 1.5, n))


def smooth_state(xy, amp=0.2, umax=0.8):
    """Smooth, physical, non-uniform state (for 2nd-order parity cases)."""
    x, y = xy[:, 0], xy[:, 1]
    rho = 1 + amp * np.sin(3.1 * x + 0.7) * np.cos(2.3 * y + 0.2)
    u = umax * np.cos(1.7 * x - 0.4) * np.sin(2.9 * y + 1.1)
    v = umax * np.sin(2.2 * x + 0.3) * np.cos(1.3 * y - 0.5)
    p = 1 + amp * np.cos(2.7 * x - 1.0) * np.sin(1.9 * y + 0.4)
    return primitive_to_q(rho, u, v, p)
