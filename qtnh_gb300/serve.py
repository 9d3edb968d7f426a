"""Request loop for circuit-simulation requests on one GPU.

Requests arrive as a seeded Poisson stream; each is a layered circuit in the shape of
the headline workload (Haar two-qubit SymmTensor gates on a random pairing per layer, a
phase DiagTensor layer every 4th layer, every 8th layer the redistribution of the top 3
indices: a permutation exchanging them with 3 random local indices, i.e. three disjoint
qubit exchanges) and asks for 256 amplitudes or the reduced density matrix of 4 qubits.
The loop admits arrived requests in order while their states fit an HBM budget, keeps
every admitted state resident, and advances all of them together in work-balanced steps:
the largest active request advances one layer per step, and every other one as many
layers as fit in the same amplitude-pass budget (2^n x gates per layer), each round of
layers one grouped call (qtnh_group_layer) over the requests still taking layers;
complex64 states are renormalised in FP64 every 8 layers, and finished requests are
answered (qtnh_gather / qtnh_rdm4, FP64 sums) and freed. Latency is arrival to completion on the
wall clock, the GPU work of a step synchronised before completions are stamped.

The executor is a parameter (GpuExecutor drives the C ABI), so the scheduling logic can
run against a fake one on the host."""
import collections
import math
import time
from dataclasses import dataclass

import numpy as np

from . import workload as wl

C128, C64 = 0, 1


@dataclass
class Request:
    rid: int
    arrival: float        # seconds after the stream starts
    circuit: object       # workload.Circuit
    kind: str             # "amps" or "rdm"
    query: np.ndarray     # 256 amplitude indices, or 4 qubits
    seed: int             # initial state seed


def request_stream(count, rate=400.0, seed=2026, qubits=(12, 26), depth=(10, 60), amps=256):
    """`count` requests with exponential inter-arrival times (mean 1/rate), qubit counts
    log-uniform in [qubits], depth uniform in [depth], outputs 256 amplitudes or a 4-qubit
    reduced density matrix with equal probability."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(count):
        t += float(rng.exponential(1.0 / rate))
        n = int(round(math.exp(rng.uniform(math.log(qubits[0]), math.log(qubits[1])))))
        dep = int(rng.integers(depth[0], depth[1] + 1))
        us = wl.haar_unitaries(rng, dep * (n // 2), 4)
        c = wl.Circuit(n)
        k = 0
        for layer in range(dep):
            order = rng.permutation(n)
            pairs = [(int(order[2 * j]), int(order[2 * j + 1])) for j in range(n // 2)]
            gates = [np.ascontiguousarray(us[k + j].T).reshape(-1) for j in range(len(pairs))]
            k += len(pairs)
            L = wl.Layer(pairs, gates)
            if (layer + 1) % 4 == 0:
                L.phases = rng.uniform(0.0, 2.0 * math.pi, n)
            if (layer + 1) % 8 == 0:
                local = rng.choice(np.arange(3, n), size=3, replace=False)
                ptup = list(range(n))
                for k3 in range(3):
                    ptup[k3], ptup[int(local[k3])] = int(local[k3]), k3
                L.ptup = ptup
            c.layers.append(L)
        if rng.random() < 0.5:
            query = rng.integers(0, 2 ** n, size=amps, dtype=np.uint64)
            kind = "amps"
        else:
            query = np.sort(rng.choice(n, size=4, replace=False)).astype(np.uint16)
            kind = "rdm"
        out.append(Request(i, t, c, kind, query, seed + 1 + i))
    return out


def swaps_of(layer):
    """The layer's permutation as disjoint qubit exchanges [(a, b), ...] (empty when none)."""
    if layer.ptup is None:
        return []
    out, seen = [], set()
    for i, p in enumerate(layer.ptup):
        if p == i or i in seen:
            continue
        if layer.ptup[p] != i:
            raise ValueError("a layer's permutation must be disjoint qubit exchanges")
        out.append((i, p))
        seen.update((i, p))
    return out


class GpuExecutor:
    """Resident states and grouped layer steps through the C ABI."""

    def __init__(self, precision):
        import torch
        import qtnh_gb300 as q
        self.torch, self.q, self.precision = torch, q, precision
        self.dtype = torch.complex128 if precision == C128 else torch.complex64

    def bytes_of(self, req):
        return (16 if self.precision == C128 else 8) * 2 ** req.circuit.n

    def admit(self, req):
        torch = self.torch
        g = torch.Generator(device="cuda")
        g.manual_seed(req.seed)
        psi = torch.randn(2 ** req.circuit.n, dtype=torch.complex128, device="cuda", generator=g)
        psi /= torch.linalg.vector_norm(psi)
        if self.precision == C128:
            return psi
        st = torch.empty(2 ** req.circuit.n, dtype=torch.complex64, device="cuda")
        self.q.state_convert(C64, psi, st)
        return st

    def step(self, items):
        """items: [(state, circuit, layer index)] -> applies that layer to each state: one
        grouped call for the gates, phases and first qubit exchange, one more grouped call
        (exchanges only) for each further exchange of a redistribution."""
        sw = [swaps_of(c.layers[li]) for _, c, li in items]
        self.q.group_layer(self.precision, [(st, c.n, c.layers[li].pairs, c.layers[li].gates, c.layers[li].phases,
                                             s[0] if s else None) for (st, c, li), s in zip(items, sw)])
        for k in range(1, max((len(s) for s in sw), default=0)):
            more = [(st, c.n, [], [], None, s[k]) for (st, c, _), s in zip(items, sw) if len(s) > k]
            self.q.group_layer(self.precision, more)

    def renorm(self, items):
        self.q.group_renorm(self.precision, [(st, c.n) for st, c in items])

    def answer(self, st, req):
        if req.kind == "amps":
            return self.q.gather(self.precision, st, req.circuit.n, req.query)
        return self.q.rdm4(self.precision, st, req.circuit.n, req.query)

    def sync(self):
        self.torch.cuda.synchronize()

    def fetch(self, out):
        return out.cpu().numpy()


def serve(requests, executor, budget_bytes=150e9, renorm_every=8, realtime=True, clock=time.perf_counter):
    """Runs the request loop. Returns (per-request latency s, results by rid, stats)."""
    pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
    active = []  # [request, state, next layer]
    used = 0
    lat, results = {}, {}
    layers_done = 0
    steps = 0
    t0 = clock()
    vclock = 0.0  # virtual time when not in real time: the stream advances with the steps
    while pending or active:
        now = (clock() - t0) if realtime else vclock
        while pending and pending[0].arrival <= now and used + executor.bytes_of(pending[0]) <= budget_bytes:
            r = pending.popleft()
            active.append([r, executor.admit(r), 0])
            used += executor.bytes_of(r)
        if pending and executor.bytes_of(pending[0]) > budget_bytes:
            raise ValueError("request %d does not fit the memory budget" % pending[0].rid)
        if not active:
            if realtime:
                time.sleep(max(0.0, pending[0].arrival - (clock() - t0)))
            else:
                vclock = pending[0].arrival
            continue
        # layers per request this step: the largest per-layer work sets the step's budget
        work = [2 ** r.circuit.n * max(1, r.circuit.n // 2) for r, _, _ in active]
        budget = max(work)
        take = [max(1, min(budget // w, len(a[0].circuit.layers) - a[2])) for a, w in zip(active, work)]
        for j in range(max(take)):
            part = [a for a, k in zip(active, take) if k > j]
            executor.step([(st, r.circuit, li) for r, st, li in part])
            layers_done += len(part)
            for a in part:
                a[2] += 1
            if renorm_every:
                due = [(st, r.circuit) for r, st, li in part if li % renorm_every == 0 and li < len(r.circuit.layers)]
                if due:
                    executor.renorm(due)
        steps += 1
        finished = [a for a in active if a[2] == len(a[0].circuit.layers)]
        outs = [(a[0], executor.answer(a[1], a[0])) for a in finished]
        executor.sync()
        t_done = (clock() - t0) if realtime else vclock
        for r, out in outs:
            lat[r.rid] = t_done - r.arrival
            results[r.rid] = executor.fetch(out)
            used -= executor.bytes_of(r)
        if not realtime:
            vclock += 1e-3
        active = [a for a in active if a[2] < len(a[0].circuit.layers)]
    makespan = ((clock() - t0) if realtime else vclock)
    v = np.array(list(lat.values())) if lat else np.zeros(1)
    stats = {"requests": len(lat), "makespan_s": makespan, "steps": steps, "gate_layers": layers_done,
             "p50_ms": float(np.percentile(v, 50) * 1e3), "p99_ms": float(np.percentile(v, 99) * 1e3),
             "mean_ms": float(v.mean() * 1e3), "requests_per_s": len(lat) / makespan if makespan else 0.0,
             "gate_layers_per_s": layers_done / makespan if makespan else 0.0}
    return lat, results, stats
