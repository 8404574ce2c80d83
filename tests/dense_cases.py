"""Dense front test matrices in the style of the reference's kernel tests
(tests/ssids/kernels/ldlt_app.cxx:81-270): random symmetric Unif[-1,1]
entries, optionally with oversized rows/entries that force delayed pivots
and a dependent column that makes the matrix singular.  Seeded numpy RNG."""
import numpy as np


def gen_sym_indef(m, rng):
    a = rng.uniform(-1.0, 1.0, (m, m))
    return np.tril(a) + np.tril(a, -1).T


def cause_delays(a, rng, block=32):
    m = a.shape[0]
    for i in range(max(m // 8, 1)):
        idx = int(m * rng.random())
        if i == 0 and m > block and idx < block:
            idx += block
        idx = min(idx, m - 1)
        a[idx, :] *= 1000.0
        a[:, idx] *= 1000.0
        a[idx, idx] /= 1000.0
        r, c = int(m * rng.random()) % m, int(m * rng.random()) % m
        a[r, c] *= 1000.0
        if r != c:
            a[c, r] *= 1000.0


def make_singular(a, c1, c2):
    scal = a[c2, c1] / a[c1, c1]
    col = scal * a[:, c1]
    a[:, c2] = col
    a[c2, :] = col
    a[c2, c2] = scal * col[c1]


def full_solve(m, q1, l, d, perm, b):
    """Solve with the two-stage factors: columns [0, q1) from the first call,
    [q1, m) from the second (perm maps positions to original indices)."""
    L = np.tril(l, -1) + np.eye(m)
    x = b[perm].copy()
    x = np.linalg.solve(L, x)
    Dm = np.zeros((m, m))
    i = 0
    while i < m:
        if i + 1 < m and np.isinf(d[2 * i + 2]):
            blk = np.array([[d[2 * i], d[2 * i + 1]], [d[2 * i + 1], d[2 * i + 3]]])
            Dm[i:i + 2, i:i + 2] = blk
            i += 2
        else:
            Dm[i, i] = d[2 * i]
            i += 1
    x = Dm @ x
    x = np.linalg.solve(L.T, x)
    out = np.empty_like(x)
    out[perm] = x
    return out


def backward_error(a, x, b):
    """||b - Ax||_inf / (||A||_inf ||x||_inf + ||b||_inf) (framework.cxx:74)."""
    r = b - a @ x
    return np.abs(r).max() / (np.abs(a).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())
