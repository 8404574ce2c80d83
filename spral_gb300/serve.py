"""A request loop that serves factor and solve requests of mixed sizes on one
GPU with continuous admission.

Requests arrive over time.  A request is admitted as soon as a worker slot
is free and the device memory it needs fits in the budget; requests that
arrive while others are on the GPU are admitted as slots and memory free up,
so their work overlaps on the device (every numeric handle runs on its own
CUDA stream and the library calls release the interpreter lock).  Factors
stay resident on the device for later requests on the same matrix
(same-pattern refactorisations and repeated solves) and are evicted least
recently used when memory is needed.  Each request's result depends only on
its own inputs: the kernels of one handle never read another handle's data.

Request kinds:
  "factor"    a new matrix (pattern, values, pivot order) under a key, then
              the solve of its right-hand sides (refined in FP64 to the
              options' backward-error target)
  "refactor"  new values for the matrix under a key (same pattern), then the
              solve of its right-hand sides: a same-pattern refactorisation
              of the resident factors, or a fresh factorisation of the
              analysed pattern if they were evicted
"""
import collections
import dataclasses
import threading
import time

import numpy as np

from . import ssids


@dataclasses.dataclass
class Request:
    rid: int
    kind: str             # "factor" or "refactor"
    key: str              # matrix identity (same pattern under one key)
    val: np.ndarray       # values, lower CSC order
    b: np.ndarray         # right-hand sides, n x nrhs
    arrival: float = 0.0  # seconds from the start of the stream
    ptr: np.ndarray = None
    row: np.ndarray = None
    order: np.ndarray = None


@dataclasses.dataclass
class Result:
    rid: int
    x: np.ndarray = None
    flag: int = 0
    num_neg: int = 0
    error: str = None
    arrival: float = 0.0
    admitted: float = 0.0
    done: float = 0.0

    @property
    def latency(self):
        return self.done - self.arrival


def estimate_bytes(akeep, precision=ssids.PRECISION_FP64, nrhs=1):
    """Device memory a resident factorisation of `akeep` needs: factors,
    contribution blocks, workspaces and solve vectors, with slack for
    delayed pivots."""
    nrow, ncol = akeep.front_sizes()
    cm = nrow - ncol
    s = 4 if precision == ssids.PRECISION_MIXED else 8
    factors = 1.25 * (nrow * ncol).sum() * s
    contrib = (cm * cm).sum() * s
    work = (nrow.max() * 160 + 16 * nrow.sum()) * s + akeep.nnz * 8 * 3
    solve = 4 * akeep.n * max(nrhs, 16) * 8
    return int(factors + contrib + work + solve + (192 << 20))


class _Resident:
    def __init__(self, fk, nbytes):
        self.fk = fk
        self.nbytes = nbytes
        self.lock = threading.Lock()
        self.busy = 0
        self.last = time.perf_counter()


class Server:
    """Serves a list of requests; see the module docstring."""

    def __init__(self, slots=4, mem_budget=None, options=None):
        self.slots = max(1, int(slots))
        if mem_budget is None:
            import ctypes
            from . import _native
            free = ctypes.c_size_t(0)
            total = ctypes.c_size_t(0)
            if _native.lib().spral_ssids_gpu_mem_info(ctypes.byref(free), ctypes.byref(total)) != 0:
                raise RuntimeError("spral_gb300: no CUDA device")
            mem_budget = int(0.8 * free.value)
        self.budget = int(mem_budget)
        self.options = options or ssids.Options()
        self.resident = collections.OrderedDict()  # key -> _Resident, least recent first
        self.used = 0          # reserved device bytes
        self.active = 0        # requests on the GPU
        self.inflight = collections.Counter()  # key -> requests on the GPU
        self.cv = threading.Condition()
        self.akeeps = {}

    def _estimate(self, req):
        return estimate_bytes(self.akeeps[req.key], self.options.precision, req.b.shape[1])

    def _reserve(self, need):
        """Reserve `need` bytes, evicting idle resident factorisations least
        recently used first; False if they do not fit (called under cv)."""
        for key in list(self.resident):
            if self.used + need <= self.budget:
                break
            r = self.resident[key]
            if r.busy == 0:
                r.fk.free()
                self.used -= r.nbytes
                del self.resident[key]
        if self.used + need <= self.budget:
            self.used += need
            return True
        return False

    def _execute(self, req, need, pinned, res):
        """Run one request on a worker thread (no lock held during GPU work).
        `pinned` is the resident factorisation a refactorisation uses, or
        None when the request builds a new one with its reserved `need`."""
        r, kept = pinned, False
        try:
            if pinned is None:
                with self.cv:
                    old = self.resident.pop(req.key, None)
                    if old is not None:  # replaced by a new matrix under the same key
                        old.fk.free()
                        self.used -= old.nbytes
                fk = ssids.Fkeep(self.akeeps[req.key], req.val, self.options)
                r = _Resident(fk, need)
                r.busy = 1
                with self.cv:
                    self.resident[req.key] = r
                kept = True
                res.flag = fk.inform.flag
            else:
                res.flag = r.fk.refactor(req.val)
            res.num_neg = r.fk.inform.num_neg
            # solve plus FP64 refinement to the options' backward-error target
            res.x = r.fk.solve_refined(req.b) if res.flag >= 0 else None
        except Exception as e:  # reported per request, the loop goes on
            res.error = f"{type(e).__name__}: {e}"
        finally:
            with self.cv:
                if r is not None:
                    r.busy -= 1
                    r.last = time.perf_counter()
                if pinned is None and not kept:
                    self.used -= need  # no resident factorisation took the reservation
                self.active -= 1
                self.inflight[req.key] -= 1
                self.cv.notify_all()

    def run(self, requests, realtime=True):
        """Serve `requests` (their `arrival` offsets are honoured when
        realtime); returns the results in request order."""
        for req in requests:
            if req.kind == "factor":
                self.akeeps[req.key] = ssids.analyse(req.ptr, req.row, req.order)
        pending = collections.deque(sorted(requests, key=lambda q: q.arrival))
        results = {q.rid: Result(q.rid, arrival=q.arrival) for q in requests}
        threads = []
        t0 = time.perf_counter()
        with self.cv:
            while pending or self.active > 0:
                now = time.perf_counter() - t0
                progressed = False
                req = pending[0] if pending else None
                # admission in arrival order; a request waits while another
                # request on the same matrix is on the GPU
                if (req is not None and self.active < self.slots
                        and (not realtime or req.arrival <= now)
                        and self.inflight[req.key] == 0):
                    res = results[req.rid]
                    if req.key not in self.akeeps:
                        res.error = f"KeyError: no matrix under key {req.key!r}"
                        res.done = now
                        pending.popleft()
                        progressed = True
                    else:
                        pinned = self.resident.get(req.key) if req.kind == "refactor" else None
                        need = 0 if pinned is not None else self._estimate(req)
                        if pinned is not None:
                            pinned.busy += 1  # not evictable while in use
                        if self._reserve(need):
                            pending.popleft()
                            if pinned is not None:
                                self.resident.move_to_end(req.key)
                            if not realtime:
                                res.arrival = now
                            res.admitted = now
                            self.active += 1
                            self.inflight[req.key] += 1
                            th = threading.Thread(target=self._timed,
                                                  args=(req, need, pinned, res, t0))
                            threads.append(th)
                            th.start()
                            progressed = True
                        else:
                            if pinned is not None:
                                pinned.busy -= 1
                            if self.active == 0:
                                # nothing runs and every idle factorisation is
                                # evicted: it can never fit
                                res.error = "request does not fit in the memory budget"
                                res.done = now
                                pending.popleft()
                                progressed = True
                if not progressed:
                    wait = 0.05
                    if realtime and req is not None and req.arrival > now:
                        wait = min(wait, req.arrival - now)
                    self.cv.wait(timeout=max(wait, 1e-4))
        for th in threads:
            th.join()
        return [results[q.rid] for q in requests]

    def _timed(self, req, need, pinned, res, t0):
        self._execute(req, need, pinned, res)
        res.done = time.perf_counter() - t0

    def close(self):
        with self.cv:
            for r in self.resident.values():
                r.fk.free()
            self.resident.clear()
            self.used = 0


def poisson_stream(count, rate, seed=0, nmin=1000, nmax=200000, refactor_share=0.5,
                   nrhs_max=64):
    """A seeded request stream: 3D 7-point Laplacians with n log-uniform in
    [nmin, nmax] (shift uniform in [-0.5, 0]) and same-pattern
    refactorisations of earlier matrices (diagonal rescaled by a factor
    uniform in [0.5, 2]); nrhs uniform in [1, nrhs_max]; exponential
    inter-arrival times with the given rate (requests per second)."""
    from . import matrices as M
    rng = np.random.default_rng(seed)
    reqs, keys, t = [], [], 0.0
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        nrhs = int(rng.integers(1, nrhs_max + 1))
        if keys and rng.uniform() < refactor_share:
            key = keys[int(rng.integers(len(keys)))]
            base = key[1]
            val = base["val"].copy()
            val[base["diag"]] *= rng.uniform(0.5, 2.0)
            reqs.append(Request(rid, "refactor", key[0], val,
                                rng.standard_normal((base["n"], nrhs)), t))
        else:
            n = float(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
            k = max(4, int(round(n ** (1.0 / 3.0))))
            shift = float(rng.uniform(-0.5, 0.0))
            p, r, v = M.laplacian_3d(k, shift=shift)
            diag = p[:-1]  # the diagonal is the first entry of each lower-CSC column
            key = f"m{rid}"
            keys.append((key, {"val": v, "diag": diag, "n": k ** 3}))
            reqs.append(Request(rid, "factor", key, v, rng.standard_normal((k ** 3, nrhs)), t,
                                p, r, M.nd_order_grid(k, k, k)))
    return reqs
