"""Seeded synthetic Newton systems in the learned preconditioner's layout.

A small cloth grid gives the vertex graph; every triangle edge adds a random
PSD coupling [[S, -S], [-S, S]] (S = R R^T), every vertex a mass term, and a
few random contact constraints add PSD blocks over 2-4 vertices.  The result
is SPD and stored as the GPU stores a Newton system: elastic blocks in ELL
form (block k of row i at k*nv + i, padded with the row's own column and zero
blocks), the contact part of the diagonal blocks, and the contact blocks as
packed upper triangles (78 per constraint).
"""
import numpy as np

import workloads as W


def _packed(Hc):
    m = Hc.shape[0]
    out = np.zeros(78, np.float32)
    w = 0
    for p in range(m):
        for q in range(p, m):
            out[w] = Hc[p, q]
            w += 1
    return out


def synthetic_system(n=6, ncon=6, seed=0, ndbc=0):
    rng = np.random.default_rng(seed)
    X, T = W.cloth_grid(n, n, 1.0, 1.0)
    nv = X.shape[0]
    blocks = {}

    def add(i, j, B):
        blocks[(i, j)] = blocks.get((i, j), np.zeros((3, 3))) + B

    edges = set()
    for t in T:
        for a in range(3):
            i, j = int(t[a]), int(t[(a + 1) % 3])
            edges.add((min(i, j), max(i, j)))
    for i in range(nv):
        add(i, i, np.eye(3) * rng.uniform(0.5, 2.0))
    for (i, j) in sorted(edges):
        R = rng.standard_normal((3, 3)) * rng.uniform(0.3, 3.0)
        S = R @ R.T
        add(i, i, S)
        add(j, j, S)
        add(i, j, -S)
        add(j, i, -S)
    proj = np.zeros(nv, np.uint8)
    dbc = rng.choice(nv, size=ndbc, replace=False) if ndbc else np.zeros(0, int)
    proj[dbc] = 1
    # Dirichlet rows and columns removed, identity diagonal
    for key in list(blocks):
        i, j = key
        if proj[i] or proj[j]:
            blocks[key] = np.zeros((3, 3))
    for i in dbc:
        blocks[(int(i), int(i))] = np.eye(3)
    rows = [sorted(j for (i, j) in blocks if i == r) for r in range(nv)]
    K = max(len(r) for r in rows)
    col = np.zeros((K, nv), np.int32)
    val = np.zeros((K, nv, 9), np.float32)
    for i in range(nv):
        for k in range(K):
            if k < len(rows[i]):
                col[k, i] = rows[i][k]
                val[k, i] = blocks[(i, rows[i][k])].reshape(9)
            else:
                col[k, i] = i
    kinds = rng.integers(0, 4, size=ncon).astype(np.int32)
    cverts = np.full((ncon, 4), -1, np.int32)
    chess = np.zeros((ncon, 78), np.float32)
    cdiag = np.zeros((nv, 9), np.float32)
    free = np.flatnonzero(proj == 0)
    for c in range(ncon):
        nvc = 2 if kinds[c] == 0 else (3 if kinds[c] == 1 else 4)
        vs = rng.choice(free, size=nvc, replace=False)
        cverts[c, :nvc] = vs
        R = rng.standard_normal((3 * nvc, 2)) * rng.uniform(1.0, 30.0)
        Hc = R @ R.T
        chess[c] = _packed(Hc)
        for q in range(nvc):
            cdiag[vs[q]] += Hc[3 * q:3 * q + 3, 3 * q:3 * q + 3].reshape(9)
    return dict(col=col, val=val, cdiag=cdiag, proj=proj, ckind=kinds, cverts=cverts, chess=chess)


def dense_matrix(s):
    """The full 3nv x 3nv matrix of a synthetic system (for checks)."""
    col, val = s["col"], s["val"]
    K, nv = col.shape
    A = np.zeros((3 * nv, 3 * nv))
    for k in range(K):
        for i in range(nv):
            j = col[k, i]
            A[3 * i:3 * i + 3, 3 * j:3 * j + 3] += val[k, i].reshape(3, 3)
    for c in range(s["ckind"].shape[0]):
        nvc = 2 if s["ckind"][c] == 0 else (3 if s["ckind"][c] == 1 else 4)
        m = 3 * nvc
        Hc = np.zeros((m, m))
        w = 0
        for p in range(m):
            for q in range(p, m):
                Hc[p, q] = Hc[q, p] = s["chess"][c, w]
                w += 1
        idx = np.concatenate([np.arange(3 * v, 3 * v + 3) for v in s["cverts"][c, :nvc]])
        A[np.ix_(idx, idx)] += Hc
    return A
