"""Seeded synthetic workloads.

``contact_pairs`` builds the contact-kernel microbenchmark: candidate pairs of
the four types (point-point, point-edge, point-triangle, edge-edge) with their
own vertices placed uniformly in the unit cube, a separation drawn log-uniform
in [1e-6, 1e-2] along the pair's normal, and per-vertex displacements drawn
from N(0, (0.5 sep)^2) per component.  Pairs are grouped by type.
"""
import numpy as np

PP, PE, PT, EE = 0, 1, 2, 3
NV = {PP: 2, PE: 3, PT: 4, EE: 4}


def _unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _perp_unit(rng, d):
    """Random unit vectors perpendicular to rows of d."""
    r = rng.standard_normal(d.shape)
    dn = _unit(d)
    r = r - (r * dn).sum(1, keepdims=True) * dn
    return _unit(r)


def contact_pairs(n_pairs, seed=0, mix=(0.1, 0.1, 0.4, 0.4), sep_range=(1e-6, 1e-2), disp_scale=0.5):
    """Returns dict(type u8[n], idx i32[n,4], x f64[nv,3], dx f64[nv,3], sep f64[n]).

    mix gives the fractions of (PP, PE, PT, EE); types are laid out in the order
    PT, EE, PE, PP so that the dominant types come first.
    """
    rng = np.random.default_rng(seed)
    counts = {t: int(round(n_pairs * f)) for t, f in zip((PP, PE, PT, EE), mix)}
    counts[EE] += n_pairs - sum(counts.values())
    order = (PT, EE, PE, PP)
    nv_total = sum(counts[t] * NV[t] for t in order)
    x = np.empty((nv_total, 3))
    types = np.empty(n_pairs, np.uint8)
    idx = np.full((n_pairs, 4), -1, np.int32)
    seps = np.empty(n_pairs)
    off_p, off_v = 0, 0
    for t in order:
        m = counts[t]
        if m == 0:
            continue
        sep = 10.0 ** rng.uniform(np.log10(sep_range[0]), np.log10(sep_range[1]), m)
        sgn = np.where(rng.random(m) < 0.5, -1.0, 1.0)[:, None]
        if t == PT:
            t0, t1, t2 = rng.random((m, 3)), rng.random((m, 3)), rng.random((m, 3))
            n = _unit(np.cross(t1 - t0, t2 - t0))
            u, v = rng.random(m), rng.random(m)
            flip = u + v > 1
            u[flip], v[flip] = 1 - u[flip], 1 - v[flip]
            foot = t0 + u[:, None] * (t1 - t0) + v[:, None] * (t2 - t0)
            p = foot + sgn * sep[:, None] * n
            verts = [p, t0, t1, t2]
        elif t == EE:
            ea0, ea1 = rng.random((m, 3)), rng.random((m, 3))
            ea = ea1 - ea0
            s = rng.uniform(0.1, 0.9, m)
            pa = ea0 + s[:, None] * ea
            n = _perp_unit(rng, ea)
            pb = pa + sgn * sep[:, None] * n
            db = _perp_unit(rng, n)
            L = rng.uniform(0.2, 1.0, m)
            tt = rng.uniform(0.1, 0.9, m)
            eb0 = pb - (tt * L)[:, None] * db
            eb1 = pb + ((1 - tt) * L)[:, None] * db
            verts = [ea0, ea1, eb0, eb1]
        elif t == PE:
            e0, e1 = rng.random((m, 3)), rng.random((m, 3))
            s = rng.uniform(0.1, 0.9, m)
            foot = e0 + s[:, None] * (e1 - e0)
            n = _perp_unit(rng, e1 - e0)
            p = foot + sep[:, None] * n
            verts = [p, e0, e1]
        else:
            p0 = rng.random((m, 3))
            d = _unit(rng.standard_normal((m, 3)))
            verts = [p0, p0 + sep[:, None] * d]
        k = NV[t]
        base = off_v + np.arange(m) * k
        for j in range(k):
            x[base + j] = verts[j]
            idx[off_p:off_p + m, j] = base + j
        types[off_p:off_p + m] = t
        seps[off_p:off_p + m] = sep
        off_p += m
        off_v += m * k
    # per-vertex displacement ~ N(0, (disp_scale * sep of its pair)^2)
    vsep = np.empty(nv_total)
    off_p, off_v = 0, 0
    for t in order:
        m, k = counts[t], NV[t]
        vsep[off_v:off_v + m * k] = np.repeat(seps[off_p:off_p + m], k)
        off_p += m
        off_v += m * k
    dx = rng.standard_normal((nv_total, 3)) * (disp_scale * vsep)[:, None]
    return dict(type=types, idx=idx, x=x, dx=dx, sep=seps)


def pair_bytes(types, fp64_hessian=False):
    """Algorithmic bytes of the CCD pass and the barrier pass over these pairs.

    CCD: 16 B (type + 4 indices, 17 B counted as 16 + 1) + nv * 48 B (x and dx) + 8 B toc + 1 B hit.
    Barrier: 17 B + nv * 24 B (x) [+ 96 B rest positions for EE] + 8 B energy + nv*3*8 B gradient
    + (3nv)(3nv+1)/2 Hessian entries (4 or 8 B).
    """
    nv = np.array([2, 3, 4, 4])[types.astype(np.int64)]
    ccd = (17 + nv * 48 + 9).sum()
    m = 3 * nv
    hb = 8 if fp64_hessian else 4
    bar = (17 + nv * 24 + np.where(types == EE, 96, 0) + 8 + nv * 24 + m * (m + 1) // 2 * hb).sum()
    return int(ccd), int(bar)


# ---------------------------------------------------------------------------
# Shell scenes
# ---------------------------------------------------------------------------
def cloth_grid(n, m, size_x, size_z, y=0.0, origin=(0.0, 0.0)):
    """n x m vertex grid in the plane y = const with the connectivity of the
    reference's mat_gen.py: quad (i, j) -> triangles (i,j)(i+1,j)(i,j+1) and
    (i+1,j+1)(i,j+1)(i+1,j), vertex index i*m + j."""
    i, j = np.meshgrid(np.arange(n), np.arange(m), indexing="ij")
    X = np.stack([origin[0] + i.ravel() * size_x / (n - 1), np.full(n * m, float(y)),
                  origin[1] + j.ravel() * size_z / (m - 1)], 1)
    idx = lambda r, c: r * m + c
    ii, jj = np.meshgrid(np.arange(n - 1), np.arange(m - 1), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    t1 = np.stack([idx(ii, jj), idx(ii + 1, jj), idx(ii, jj + 1)], 1)
    t2 = np.stack([idx(ii + 1, jj + 1), idx(ii, jj + 1), idx(ii + 1, jj)], 1)
    T = np.stack([t1, t2], 1).reshape(-1, 3)
    return X, T.astype(np.int32)


def box_shell(size, center, nsub=2):
    """Closed box surface (edge length `size`) with each face split into
    nsub x nsub quads, two triangles each, outward normals."""
    c = np.asarray(center, float)
    h = size / 2.0
    verts = {}
    tris = []

    def vid(p):
        key = tuple(np.round(p, 12))
        if key not in verts:
            verts[key] = len(verts)
        return verts[key]

    for axis in range(3):
        for sgn in (-1.0, 1.0):
            u_ax, v_ax = [a for a in range(3) if a != axis]
            for a in range(nsub):
                for b in range(nsub):
                    q = []
                    for (da, db) in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        p = np.zeros(3)
                        p[axis] = sgn * h
                        p[u_ax] = -h + (a + da) * size / nsub
                        p[v_ax] = -h + (b + db) * size / nsub
                        q.append(vid(p + c))
                    # orientation so that the normal points outward
                    flip = (sgn > 0) == ((axis + 1) % 3 == u_ax)
                    if flip:
                        tris += [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
                    else:
                        tris += [[q[0], q[2], q[1]], [q[0], q[3], q[2]]]
    X = np.zeros((len(verts), 3))
    for k, i in verts.items():
        X[i] = k
    return X, np.array(tris, np.int32)


def icosphere(radius, center, subdiv=3):
    """Geodesic sphere from a subdivided icosahedron (outward normals)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    V = [np.array(v, float) / np.linalg.norm(v) for v in V]
    F = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
         [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11],
         [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    for _ in range(subdiv):
        mid = {}

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                p = V[a] + V[b]
                V.append(p / np.linalg.norm(p))
                mid[k] = len(V) - 1
            return mid[k]

        nf = []
        for a, b, c in F:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        F = nf
    X = np.array(V) * radius + np.asarray(center, float)
    return X, np.array(F, np.int32)


def rotate_y(P, center, angle):
    """Rotates points P about the vertical axis through `center` by `angle`."""
    c, s = np.cos(angle), np.sin(angle)
    Q = np.asarray(P, float) - center
    return np.stack([c * Q[:, 0] + s * Q[:, 2], Q[:, 1], -s * Q[:, 0] + c * Q[:, 2]], 1) + center


def cloth_on_sphere(n=200, size=2.0, radius=0.5, gap=0.01, subdiv=4):
    """Cloth n x n (size x size) centred above a sphere (fixed centre, Dirichlet
    vertices) whose top is `gap` below the cloth.  Returns X, T, dbc indices and
    the sphere centre."""
    center = np.zeros(3)
    cl = cloth_grid(n, n, size, size, y=radius + gap, origin=(-size / 2, -size / 2))
    sp = icosphere(radius, center, subdiv)
    X, T, offs = merge_meshes(cl, sp)
    dbc = np.arange(offs[1], X.shape[0], dtype=np.int32)
    return X, T, dbc, center


def cloth_on_box(n=40, size=1.0, box=0.3, height=0.1, nsub=4):
    """Cloth n x n (size x size) `height` above a fixed box shell (Dirichlet)."""
    cl = cloth_grid(n, n, size, size, y=0.0, origin=(-size / 2, -size / 2))
    bx = box_shell(box, (0.0, -height - box / 2, 0.0), nsub)
    X, T, offs = merge_meshes(cl, bx)
    dbc = np.arange(offs[1], X.shape[0], dtype=np.int32)
    return X, T, dbc


def merge_meshes(*meshes):
    """Concatenates (X, T) meshes; returns X, T and the vertex offset of each."""
    Xs, Ts, offs = [], [], []
    o = 0
    for X, T in meshes:
        Xs.append(X)
        Ts.append(T + o)
        offs.append(o)
        o += X.shape[0]
    return np.concatenate(Xs), np.concatenate(Ts).astype(np.int32), offs


def rods_particles_on_cloth(n_rods=1000, seg_per_rod=100, rod_len=0.5, n_particles=20000, cloth_n=120,
                            cloth_size=1.0, layer_gap=2.5e-3, particle_gap=8e-3, lift=0.02, seed=0,
                            rods_per_layer=1, rod_spacing=5e-3, particles_per_row=None):
    """Mixed codimensional scene: straight rods of `seg_per_rod` segments and length
    `rod_len` in horizontal layers `layer_gap` apart, `rods_per_layer` parallel rods
    `rod_spacing` apart in a layer, each layer with a seeded random in-plane
    direction and (single-rod layers) a seeded random centre over the cloth;
    particles on a grid (`particle_gap` apart, `particles_per_row` per row, default
    a tall column) above the rods; a cloth_n x cloth_n cloth (cloth_size square,
    y = 0) pinned at its four corners.

    Returns X, T (cloth triangles), segments (n_rods*seg_per_rod, 2),
    particles (indices), dbc (the 4 cloth corners)."""
    rng = np.random.default_rng(seed)
    Xc, Tc = cloth_grid(cloth_n, cloth_n, cloth_size, cloth_size, y=0.0, origin=(-cloth_size / 2, -cloth_size / 2))
    nc = Xc.shape[0]
    corners = np.array([0, cloth_n - 1, nc - cloth_n, nc - 1], np.int32)
    pts = [Xc]
    segs = []
    o = nc
    half = 0.5 * (cloth_size - rod_len) * 0.9
    n_layers = (n_rods + rods_per_layer - 1) // rods_per_layer
    t = np.linspace(-0.5, 0.5, seg_per_rod + 1)[:, None] * rod_len
    r = 0
    for layer in range(n_layers):
        th = rng.uniform(0, 2 * np.pi)
        d = np.array([np.cos(th), 0.0, np.sin(th)])
        nrm = np.array([-d[2], 0.0, d[0]])
        y = lift + layer * layer_gap
        if rods_per_layer == 1:
            centres = [np.array([rng.uniform(-half, half), y, rng.uniform(-half, half)])]
        else:
            k = min(rods_per_layer, n_rods - r)
            off = (np.arange(k) - (k - 1) / 2) * rod_spacing
            shift = rng.uniform(-0.25, 0.25) * rod_spacing
            centres = [np.array([0.0, y, 0.0]) + (q + shift) * nrm for q in off]
        for c in centres:
            pts.append(c[None, :] + t * d[None, :])
            segs.append(np.column_stack([np.arange(seg_per_rod), np.arange(1, seg_per_rod + 1)]) + o)
            o += seg_per_rod + 1
            r += 1
    top = lift + n_layers * layer_gap + particle_gap
    if particles_per_row is None:
        side = int(np.ceil(np.sqrt(max(n_particles, 1) / 50.0)))
        nx = max(1, min(side, int(cloth_size * 0.8 / particle_gap)))
    else:
        nx = int(particles_per_row)
    P = []
    for k in range(n_particles):
        i, j, l = k % nx, (k // nx) % nx, k // (nx * nx)
        P.append([(i - (nx - 1) / 2) * particle_gap, top + l * particle_gap, (j - (nx - 1) / 2) * particle_gap])
    if n_particles:
        pts.append(np.array(P))
    particles = np.arange(o, o + n_particles, dtype=np.int32)
    X = np.concatenate(pts)
    S = np.concatenate(segs).astype(np.int32) if segs else np.zeros((0, 2), np.int32)
    return X, Tc.astype(np.int32), S, particles, corners


def rods_particles_on_cloth_full(seed=0):
    """The mixed codimensional scene at full size: 1000 rods x 100 segments (0.5 m)
    in 5 layers of 200 parallel rods 5 mm apart (seeded layer directions, layers
    2.5 mm apart, the lowest 1.5 mm above the cloth, i.e. in contact range from
    the start: rods and cloth fall together, so contact develops only where they
    already touch), 20000 particles in two 100 x 100 layers 5 mm apart, on a
    120 x 120 cloth (1 m) pinned at its corners; 135,400 vertices."""
    return rods_particles_on_cloth(n_rods=1000, seg_per_rod=100, rod_len=0.5, n_particles=20000, cloth_n=120,
                                   cloth_size=1.0, layer_gap=2.5e-3, particle_gap=5e-3, lift=1.5e-3, seed=seed,
                                   rods_per_layer=200, rod_spacing=5e-3, particles_per_row=100)


def stacked_shells(n=180, layers=8, size=1.0, gap=5e-3, jitter=1e-3, plate_n=21, plate_margin=0.1, seed=0):
    """`layers` cloths of n x n vertices (size x size) stacked `gap` apart, every
    vertex moved in-plane by a seeded uniform jitter in [-jitter, jitter] (rest
    shape = jittered shape), between a fixed ground plate `gap` below the lowest
    layer and a top plate `gap` above the highest (plates: plate_n x plate_n
    grids, `plate_margin` wider than the cloth on each side, Dirichlet).

    Returns X, T, dbc (all plate vertices), top (the top plate's vertices, which
    the scene moves down)."""
    rng = np.random.default_rng(seed)
    meshes = []
    for l in range(layers):
        Xl, Tl = cloth_grid(n, n, size, size, y=l * gap, origin=(-size / 2, -size / 2))
        J = rng.uniform(-jitter, jitter, size=(Xl.shape[0], 2))
        Xl[:, 0] += J[:, 0]
        Xl[:, 2] += J[:, 1]
        meshes.append((Xl, Tl))
    ps = size + 2 * plate_margin
    meshes.append(cloth_grid(plate_n, plate_n, ps, ps, y=-gap, origin=(-ps / 2, -ps / 2)))
    meshes.append(cloth_grid(plate_n, plate_n, ps, ps, y=layers * gap, origin=(-ps / 2, -ps / 2)))
    X, T, offs = merge_meshes(*meshes)
    dbc = np.arange(offs[layers], X.shape[0], dtype=np.int32)
    top = np.arange(offs[layers + 1], X.shape[0], dtype=np.int32)
    return X, T, dbc, top


def tet_box(n=3, size=0.1, center=(0.0, 0.0, 0.0)):
    """Cube (edge `size`) of n^3 cells, each split into 6 tetrahedra around its
    main diagonal (Kuhn subdivision, conforming across cells), all positively
    oriented.  Returns X ((n+1)^3, 3) and tets (6 n^3, 4)."""
    import itertools
    c = np.asarray(center, float)
    h = size / n
    idx = lambda i, j, k: (i * (n + 1) + j) * (n + 1) + k
    X = np.array([[i * h, j * h, k * h] for i in range(n + 1) for j in range(n + 1) for k in range(n + 1)])
    X += c - size / 2
    tets = []
    for i, j, k in itertools.product(range(n), range(n), range(n)):
        for perm in itertools.permutations(range(3)):
            p = [i, j, k]
            v = [idx(*p)]
            for ax in perm:
                p[ax] += 1
                v.append(idx(*p))
            a, b, cc, d = (X[q] for q in v)
            if np.linalg.det(np.column_stack([b - a, cc - a, d - a])) < 0:
                v[1], v[2] = v[2], v[1]
            tets.append(v)
    return X, np.array(tets, np.int32)
