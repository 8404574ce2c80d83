"""Admission logic of the request loop, on the CPU with a stand-in for the
GPU numeric handle (the real one is exercised by the GPU tests)."""
import threading
import time

import numpy as np

from spral_gb300 import serve, ssids, matrices as M


class FakeFkeep:
    live = 0
    peak = 0
    lock = threading.Lock()

    def __init__(self, akeep, val, options=None):
        self.akeep = akeep
        self.val = np.asarray(val)
        self.inform = ssids.Inform(flag=0, num_neg=int((self.val < 0).sum()))

    def _busy(self):
        with FakeFkeep.lock:
            FakeFkeep.live += 1
            FakeFkeep.peak = max(FakeFkeep.peak, FakeFkeep.live)
        time.sleep(0.02)
        with FakeFkeep.lock:
            FakeFkeep.live -= 1

    def solve(self, b):
        self._busy()
        return 2.0 * np.asarray(b) + self.val[0]

    solve_refined = solve

    def refactor(self, val):
        self.val = np.asarray(val)
        self.inform = ssids.Inform(flag=0, num_neg=int((self.val < 0).sum()))
        return 0

    def free(self):
        pass


def _stream(count=20, seed=1):
    return serve.poisson_stream(count, rate=400.0, seed=seed, nmin=64, nmax=1000, nrhs_max=4)


def test_serve_overlaps_and_respects_slots(monkeypatch):
    monkeypatch.setattr(ssids, "Fkeep", FakeFkeep)
    FakeFkeep.peak = 0
    reqs = _stream()
    srv = serve.Server(slots=3, mem_budget=1 << 40)
    res = srv.run(reqs, realtime=True)
    assert all(r.error is None for r in res)
    assert 1 < FakeFkeep.peak <= 3
    # same key: a refactorisation is served after the factorisation it needs
    first_done = {}
    for q, r in zip(reqs, res):
        if q.kind == "factor":
            first_done[q.key] = r.done
        else:
            assert r.admitted >= first_done[q.key] - 1e-9


def test_serve_memory_budget_and_eviction(monkeypatch):
    monkeypatch.setattr(ssids, "Fkeep", FakeFkeep)
    reqs = _stream(count=30, seed=2)
    srv = serve.Server(slots=4, mem_budget=0)
    need = max(serve.estimate_bytes(ssids.analyse(q.ptr, q.row, q.order), ssids.PRECISION_FP64,
                                    q.b.shape[1]) for q in reqs if q.kind == "factor")
    srv.budget = 2 * need  # room for about two resident factorisations
    seen = []
    orig = serve.Server._reserve

    def spy(self, n):
        ok = orig(self, n)
        seen.append(self.used)
        return ok

    monkeypatch.setattr(serve.Server, "_reserve", spy)
    res = srv.run(reqs, realtime=False)
    assert all(r.error is None for r in res), [r.error for r in res if r.error]
    assert max(seen) <= srv.budget
    # the results are those of each request alone
    alone = serve.Server(slots=1, mem_budget=1 << 40)
    monkeypatch.setattr(serve.Server, "_reserve", orig)
    ref = alone.run(reqs, realtime=False)
    for a, b in zip(res, ref):
        assert np.array_equal(a.x, b.x) and a.num_neg == b.num_neg
