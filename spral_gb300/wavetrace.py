"""Summary of a wavefront-solve trace.

With the environment variable SPRAL_GB300_WAVE_TRACE set to a path prefix,
the library runs its solve passes without CUDA graphs and, after each pass,
writes the item list and per-item global-timer stamps of the persistent
forward and backward launches:

    <prefix>.items   int32 pairs (front, item code), forward items first
    <prefix>.trace   uint64 quadruples per item: taken, last wait over,
                     finished (ns), SM
    <prefix>.meta    "nfwd nbwd", then per front "level m nelim"

Item codes: [0, 0x10000) pivot block, [0x10000, 0x20000) forward
contribution row block, [0x20000, 0x30000) gather chunk, 0x30000 a small
front whole, >= 0x100000 backward L21^T partial.

    python -m spral_gb300.wavetrace <prefix>
"""
import sys

import numpy as np

KINDS = "SGTPC"


def kind_of(codes):
    codes = np.asarray(codes)
    return np.where(codes >= 0x100000, "T",
                    np.where(codes >= 0x30000, "S",
                             np.where(codes >= 0x20000, "G",
                                      np.where(codes >= 0x10000, "C", "P"))))


def load(prefix):
    items = np.fromfile(prefix + ".items", dtype=np.int32).reshape(-1, 2)
    stamps = np.fromfile(prefix + ".trace", dtype=np.uint64).reshape(-1, 4).astype(np.int64)
    lines = open(prefix + ".meta").read().split("\n")
    nfwd, nbwd = map(int, lines[0].split())
    fronts = np.array([list(map(int, l.split())) for l in lines[1:] if l.strip()])
    return items, stamps, nfwd, nbwd, fronts


def summary(prefix, out=sys.stdout):
    items, stamps, nfwd, nbwd, fronts = load(prefix)
    level, m, nelim = fronts[:, 0], fronts[:, 1], fronts[:, 2]
    for name, sl in (("forward", slice(0, nfwd)), ("backward", slice(nfwd, nfwd + nbwd))):
        it, t = items[sl], stamps[sl]
        if len(it) == 0:
            continue
        t0 = t[:, 0].min()
        taken, ready, done = ((t[:, k] - t0) / 1e3 for k in range(3))
        k = kind_of(it[:, 1])
        print(f"{name}: {len(it)} items, span {done.max():.1f} us", file=out)
        for kk in KINDS:
            s = k == kk
            if s.any():
                print(f"  {kk}: {s.sum():5d} items, wait {np.mean(ready[s] - taken[s]):6.2f} us "
                      f"mean, work after the last wait {np.mean(done[s] - ready[s]):6.2f} us mean "
                      f"({np.max(done[s] - ready[s]):6.2f} max)", file=out)
        lv = level[it[:, 0]]
        for l in sorted(set(lv.tolist())):
            s = lv == l
            print(f"  level {l:2d}: {s.sum():5d} items, {taken[s].min():8.1f} .. {done[s].max():8.1f}"
                  f" us, largest front m {m[it[s, 0]].max()}, nelim {nelim[it[s, 0]].max()}",
                  file=out)
        piv = k == "P"
        if piv.any():
            f = it[piv, 0][np.argmax(nelim[it[piv, 0]])]
            s = piv & (it[:, 0] == f)
            ends = np.sort(done[s])
            gaps = np.diff(ends)
            print(f"  widest front ({m[f]} x {nelim[f]} eliminated): {s.sum()} pivot blocks, "
                  f"chain step median {np.median(gaps):.2f} us", file=out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python -m spral_gb300.wavetrace <prefix>")
    summary(sys.argv[1])
