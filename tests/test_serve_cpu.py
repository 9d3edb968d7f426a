"""The request loop's scheduling on the host (a fake executor stands in for the GPU):
the seeded Poisson stream, in-order admission under the memory budget, every request
answered once, resident states freed, latencies from arrival to completion."""
import numpy as np
import pytest

from qtnh_gb300 import serve


def test_request_stream_shape():
    reqs = serve.request_stream(300, rate=400.0, seed=3)
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0)
    assert 0.5 < t[-1] < 1.1                      # ~300 / 400 s
    ns = np.array([r.circuit.n for r in reqs])
    assert ns.min() >= 12 and ns.max() <= 26
    assert np.mean(ns < 19) > 0.5                 # log-uniform: the small half of [12, 26] is denser
    for r in reqs[:20]:
        d = len(r.circuit.layers)
        assert 10 <= d <= 60
        assert all(len(layer.gates) == r.circuit.n // 2 for layer in r.circuit.layers)
        assert r.kind in ("amps", "rdm")
        if r.kind == "amps":
            assert len(r.query) == 256 and int(r.query.max()) < 2 ** r.circuit.n
        else:
            assert len(set(int(x) for x in r.query)) == 4
        for i, layer in enumerate(r.circuit.layers):
            assert (layer.phases is not None) == ((i + 1) % 4 == 0)
            assert (layer.ptup is not None) == ((i + 1) % 8 == 0)
            if layer.ptup is not None:
                # the redistribution of the headline workload: the top 3 indices exchanged
                # with 3 distinct local ones, three disjoint qubit exchanges
                sw = serve.swaps_of(layer)
                assert len(sw) == 3 and sorted(a for a, _ in sw) == [0, 1, 2] and all(b >= 3 for _, b in sw)


class FakeExecutor:
    def __init__(self):
        self.resident = {}
        self.peak = 0
        self.steps = []
        self.admitted = []

    def bytes_of(self, req):
        return 16 * 2 ** req.circuit.n

    def admit(self, req):
        self.admitted.append(req.rid)
        self.resident[req.rid] = self.bytes_of(req)
        self.peak = max(self.peak, sum(self.resident.values()))
        return req.rid

    def step(self, items):
        self.steps.append([(st, li) for st, _, li in items])

    def renorm(self, items):
        pass

    def answer(self, st, req):
        self.resident.pop(req.rid)
        return ("answer", req.rid)

    def sync(self):
        pass

    def fetch(self, out):
        return out


def test_serve_schedule_on_host():
    reqs = serve.request_stream(60, rate=400.0, seed=4, qubits=(12, 20), depth=(10, 20))
    ex = FakeExecutor()
    budget = 32 * 2 ** 20  # 32 MiB: a few small states at a time
    lat, results, stats = serve.serve(reqs, ex, budget_bytes=budget, realtime=False)
    assert stats["requests"] == len(reqs) == len(results)
    assert all(results[r.rid] == ("answer", r.rid) for r in reqs)
    assert ex.peak <= budget and not ex.resident
    assert ex.admitted == sorted(ex.admitted)          # in arrival order
    assert all(v >= 0 for v in lat.values())
    # every request's layers were applied in order, once each
    seen = {}
    for step in ex.steps:
        for rid, li in step:
            assert seen.get(rid, -1) == li - 1
            seen[rid] = li
    assert all(seen[r.rid] == len(r.circuit.layers) - 1 for r in reqs)
    assert stats["gate_layers"] == sum(len(r.circuit.layers) for r in reqs)


def test_serve_rejects_request_beyond_budget():
    reqs = serve.request_stream(2, rate=400.0, seed=5, qubits=(20, 20), depth=(10, 10))
    with pytest.raises(ValueError):
        serve.serve(reqs, FakeExecutor(), budget_bytes=1024, realtime=False)
