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
