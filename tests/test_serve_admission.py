"""The serving loop's admission on the host (CPU only): queries start in
arrival order, never before they arrive, never above the byte budget or the
slot count, and every one finishes; a query larger than the budget is
refused.  The query itself is a stand-in that sleeps and returns its id."""
import time

import numpy as np
import pytest

from vertexsurge_gb300 import serve


class FakeServer(serve.Server):
    def __init__(self, budget, slots, sizes, work_s):
        super().__init__(dg=None, budget_bytes=budget, slots=slots, make_stream=lambda: None)
        self.sizes, self.work_s = sizes, work_s
        self.live, self.max_live, self.max_bytes, self.used = 0, 0, 0, 0
        import threading
        self.mu = threading.Lock()

    def footprint(self, r):
        return self.sizes[r.rid]

    def run_query(self, r, stream):
        with self.mu:
            self.live += 1
            self.used += r.bytes
            self.max_live = max(self.max_live, self.live)
            self.max_bytes = max(self.max_bytes, self.used)
        time.sleep(self.work_s)
        with self.mu:
            self.live -= 1
            self.used -= r.bytes
        return (r.rid,)


def trace(n, gap_s):
    return [serve.Request(i, i * gap_s, np.zeros(1, np.uint32), 2, np.zeros(1, np.uint32),
                          np.zeros(1, np.uint32)) for i in range(n)]


@pytest.mark.parametrize("slots,budget", [(4, 100), (2, 1000), (8, 35)])
def test_admission_limits_and_order(slots, budget):
    rng = np.random.default_rng(slots)
    n = 40
    sizes = [int(x) for x in rng.integers(5, 30, n)]
    srv = FakeServer(budget, slots, sizes, work_s=0.01)
    tr = trace(n, 0.002)
    rep = srv.serve(tr)
    assert rep["queries"] == n and all(r.result == (r.rid,) for r in tr)
    assert srv.max_live <= slots and rep["peak_concurrent"] <= slots
    assert srv.max_bytes <= budget and rep["peak_bytes"] <= budget
    starts = [r.start for r in sorted(tr, key=lambda r: r.arrival)]
    assert all(a <= b + 1e-3 for a, b in zip(starts, starts[1:]))  # admitted in arrival order
    assert all(r.start + 1e-3 >= r.arrival for r in tr)            # never before arrival
    assert rep["p99_ms"] >= rep["p50_ms"] > 0


def test_oversized_request_is_refused():
    srv = FakeServer(50, 2, [10, 60, 10], work_s=0.0)
    with pytest.raises(ValueError):
        srv.serve(trace(3, 0.0))
