"""Seeded synthetic matrices and orderings for the SSIDS factor/solve path.

All matrices are returned as the lower triangle in compressed sparse column
form with 0-based indices: ``ptr`` (int64, n+1), ``row`` (int32), ``val``
(float64).  This is the input format of ``ssids_analyse``/``ssids_factor``
(src/ssids/ssids.f90:148,767) with the Fortran 1-based offsets removed.

The reference orders with METIS (src/metis5_wrapper.F90), which is not part of
the GPU path; here grid problems use a geometric nested dissection and general
problems a minimum-degree ordering (see ``spral_gb300.ssids.order_mindeg``).
"""
import numpy as np


def _coo_to_lower_csc(n, r, c, v):
    """Lower-triangle CSC from COO triplets (r >= c); duplicates summed."""
    r = np.asarray(r, dtype=np.int64)
    c = np.asarray(c, dtype=np.int64)
    v = np.asarray(v, dtype=np.float64)
    lo = np.maximum(r, c)
    hi = np.minimum(r, c)
    key = hi * n + lo
    order = np.argsort(key, kind="stable")
    key = key[order]
    v = v[order]
    uniq, start = np.unique(key, return_index=True)
    vals = np.add.reduceat(v, start) if len(v) else v
    cols = uniq // n
    rows = uniq % n
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ptr, cols + 1, 1)
    ptr = np.cumsum(ptr)
    return ptr, rows.astype(np.int32), vals


def laplacian_2d(nx, ny, shift=0.0):
    """5-point Laplacian on an nx x ny grid, diagonal 4+shift, off-diagonal -1."""
    idx = np.arange(nx * ny).reshape(ny, nx)
    r = [idx.ravel()]
    c = [idx.ravel()]
    v = [np.full(nx * ny, 4.0 + shift)]
    r.append(idx[:, 1:].ravel()); c.append(idx[:, :-1].ravel()); v.append(-np.ones((nx - 1) * ny))
    r.append(idx[1:, :].ravel()); c.append(idx[:-1, :].ravel()); v.append(-np.ones(nx * (ny - 1)))
    return _coo_to_lower_csc(nx * ny, np.concatenate(r), np.concatenate(c), np.concatenate(v))


def laplacian_3d(nx, ny=None, nz=None, shift=0.0):
    """7-point Laplacian on an nx x ny x nz grid, diagonal 6+shift, off-diagonal -1."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n = nx * ny * nz
    idx = np.arange(n).reshape(nz, ny, nx)
    r = [idx.ravel()]
    c = [idx.ravel()]
    v = [np.full(n, 6.0 + shift)]
    for a, b in ((idx[:, :, 1:], idx[:, :, :-1]), (idx[:, 1:, :], idx[:, :-1, :]),
                 (idx[1:, :, :], idx[:-1, :, :])):
        r.append(a.ravel()); c.append(b.ravel()); v.append(-np.ones(a.size))
    return _coo_to_lower_csc(n, np.concatenate(r), np.concatenate(c), np.concatenate(v))


def laplacian_eig_count_2d(nx, ny, shift):
    """Exact number of negative eigenvalues of the shifted 2D Laplacian."""
    lx = 2 - 2 * np.cos(np.pi * np.arange(1, nx + 1) / (nx + 1))
    ly = 2 - 2 * np.cos(np.pi * np.arange(1, ny + 1) / (ny + 1))
    ev = lx[None, :] + ly[:, None] + shift
    return int((ev < 0).sum()), int((ev == 0).sum()), float(np.abs(ev).min())


def laplacian_eig_count_3d(nx, ny, nz, shift):
    """Exact number of negative eigenvalues of the shifted 3D Laplacian."""
    l = [2 - 2 * np.cos(np.pi * np.arange(1, k + 1) / (k + 1)) for k in (nx, ny, nz)]
    ev = l[0][None, None, :] + l[1][None, :, None] + l[2][:, None, None] + shift
    return int((ev < 0).sum()), int((ev == 0).sum()), float(np.abs(ev).min())


def nd_order_grid(nx, ny, nz=1, leaf=8):
    """Geometric nested dissection of a structured grid.

    Returns ``order`` with order[i] = pivot position of vertex i (0-based):
    the two halves first, their separating plane last, recursively.
    """
    n = nx * ny * nz
    seq = np.empty(n, dtype=np.int64)
    pos = 0
    stack = [((0, nx), (0, ny), (0, nz), 0)]
    # iterative post-order: (box, state); state 0 = split, 1 = emit separator
    out = []

    def emit(box):
        (x0, x1), (y0, y1), (z0, z1) = box
        zz, yy, xx = np.meshgrid(np.arange(z0, z1), np.arange(y0, y1), np.arange(x0, x1),
                                 indexing="ij")
        return (xx + nx * (yy + ny * zz)).ravel()

    def rec(box):
        nonlocal pos
        (x0, x1), (y0, y1), (z0, z1) = box
        dims = [x1 - x0, y1 - y0, z1 - z0]
        if max(dims) <= leaf or dims[0] * dims[1] * dims[2] <= leaf ** 2:
            ids = emit(box)
            seq[pos:pos + len(ids)] = ids
            pos += len(ids)
            return
        d = int(np.argmax(dims))
        lo, hi = box[d]
        mid = (lo + hi) // 2
        left = list(box); left[d] = (lo, mid)
        right = list(box); right[d] = (mid + 1, hi)
        sep = list(box); sep[d] = (mid, mid + 1)
        if mid > lo:
            rec(tuple(left))
        if hi > mid + 1:
            rec(tuple(right))
        ids = emit_sep(tuple(sep), box)
        seq[pos:pos + len(ids)] = ids
        pos += len(ids)

    def emit_sep(sep, box):
        # separator vertices with a neighbour outside the box are ordered
        # last, so that the rest of the separator is a fundamental chain
        (x0, x1), (y0, y1), (z0, z1) = sep
        zz, yy, xx = np.meshgrid(np.arange(z0, z1), np.arange(y0, y1), np.arange(x0, x1),
                                 indexing="ij")
        edge = np.zeros(xx.shape, dtype=bool)
        for c, (lo, hi), full in ((xx, box[0], nx), (yy, box[1], ny), (zz, box[2], nz)):
            if lo > 0:
                edge |= c == lo
            if hi < full:
                edge |= c == hi - 1
        ids = (xx + nx * (yy + ny * zz)).ravel()
        e = edge.ravel()
        return np.concatenate([ids[~e], ids[e]])

    import sys
    sys.setrecursionlimit(10000)
    rec(((0, nx), (0, ny), (0, nz)))
    assert pos == n
    order = np.empty(n, dtype=np.int32)
    order[seq] = np.arange(n, dtype=np.int32)
    return order


def kkt(nh, na, h_nnz_row=7, a_nnz_row=4, reg=1e-8, seed=0):
    """KKT saddle point [[H, A^T], [A, -reg I]].

    H is nh x nh SPD: random symmetric pattern with about h_nnz_row entries
    per row, N(0,1) off-diagonals, diagonal = row abs-sum + 1.  A is na x nh
    with a_nnz_row N(0,1) entries per row at uniform columns.
    """
    rng = np.random.default_rng(seed)
    k = max((h_nnz_row - 1) // 2, 1)
    hr = rng.integers(0, nh, size=nh * k)
    hc = np.repeat(np.arange(nh), k)
    keep = hr != hc
    hr, hc = hr[keep], hc[keep]
    hv = rng.standard_normal(len(hr))
    ptr, row, val = _coo_to_lower_csc(nh, hr, hc, hv)
    cols = np.repeat(np.arange(nh), np.diff(ptr))
    absum = np.zeros(nh)
    np.add.at(absum, row, np.abs(val))
    np.add.at(absum, cols, np.abs(val))
    n = nh + na
    r = [row.astype(np.int64), np.arange(nh)]
    c = [cols, np.arange(nh)]
    v = [val, absum + 1.0]
    ar = np.repeat(np.arange(na), a_nnz_row) + nh
    ac = rng.integers(0, nh, size=na * a_nnz_row)
    av = rng.standard_normal(na * a_nnz_row)
    r += [ar, np.arange(nh, n)]
    c += [ac, np.arange(nh, n)]
    v += [av, np.full(na, -reg)]
    return _coo_to_lower_csc(n, np.concatenate(r), np.concatenate(c), np.concatenate(v))


def random_indef(n, density=0.01, seed=0, diag_scale=0.1):
    """Random sparse symmetric indefinite matrix: Unif[-1,1] entries, small
    diagonal so that 2x2 pivots and delays occur."""
    rng = np.random.default_rng(seed)
    nnz = max(int(density * n * n / 2), n)
    r = rng.integers(0, n, size=nnz)
    c = rng.integers(0, n, size=nnz)
    v = rng.uniform(-1, 1, size=nnz)
    r = np.concatenate([r, np.arange(n)])
    c = np.concatenate([c, np.arange(n)])
    v = np.concatenate([v, diag_scale * rng.uniform(-1, 1, size=n)])
    return _coo_to_lower_csc(n, r, c, v)


def sym_matvec(ptr, row, val, x):
    """y = A x for A given by its lower triangle (x may be 1-D or n x nrhs)."""
    n = len(ptr) - 1
    cols = np.repeat(np.arange(n), np.diff(ptr))
    x = np.asarray(x)
    y = np.zeros_like(x, dtype=np.float64)
    if x.ndim == 1:
        np.add.at(y, row, val * x[cols])
        off = row != cols
        np.add.at(y, cols[off], val[off] * x[row[off]])
    else:
        np.add.at(y, row, val[:, None] * x[cols])
        off = row != cols
        np.add.at(y, cols[off], val[off][:, None] * x[row[off]])
    return y


def scaled_bwd_error(ptr, row, val, x, b):
    """max_i |b - A x|_i / (||A||_inf ||x||_inf + ||b||_inf), per right-hand side
    (tests/ssids/ssids.f90:1762-1810)."""
    n = len(ptr) - 1
    cols = np.repeat(np.arange(n), np.diff(ptr))
    rs = np.zeros(n)
    np.add.at(rs, row, np.abs(val))
    off = row != cols
    np.add.at(rs, cols[off], np.abs(val[off]))
    anorm = rs.max() if n else 0.0
    x2 = x if x.ndim == 2 else x[:, None]
    b2 = b if b.ndim == 2 else b[:, None]
    r = b2 - sym_matvec(ptr, row, val, x2)
    return np.abs(r).max(axis=0) / (anorm * np.abs(x2).max(axis=0) + np.abs(b2).max(axis=0))


def equilibrate(ptr, row, val, iters=3):
    """Symmetric equilibration scaling s (S A S with unit inf-norm rows, a few
    Ruiz-style sweeps), for tests of scaled factorisations."""
    n = len(ptr) - 1
    cols = np.repeat(np.arange(n), np.diff(ptr))
    s = np.ones(n)
    for _ in range(iters):
        a = np.abs(val) * s[row] * s[cols]
        m = np.zeros(n)
        np.maximum.at(m, row, a)
        np.maximum.at(m, cols, a)
        m[m == 0] = 1.0
        s /= np.sqrt(m)
    return s
