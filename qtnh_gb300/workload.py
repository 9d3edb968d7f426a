"""Seeded synthetic workloads in the shapes of the benchmark configurations.

``random_circuit`` builds the layered random circuit used for gate-layers/s:
n qubits, every layer a seeded random pairing of the qubits with one Haar-random
two-qubit SymmTensor gate per pair; every 4th layer also a layer of per-qubit
phase DiagTensors (phases uniform in [0, 2pi)); every 8th layer also a
redistribution: the top 3 indices are made distributed (rescatter +3), exchanged
with 3 seeded random local indices by a permutation (the single-GPU form of the
reference's mixed distributed/local swap, src/tensor/dense.cpp:220-257), and
gathered back (rescatter -3).

Gates follow the SymmTensor element layout [in_0, in_1, out_0, out_1]
(include/tensor/symm.hpp:22-45): contraction sums over the inputs, so a unitary
U acting as psi' = U psi is stored as els[in, out] = U[out, in].
Haar sampling: QR of a complex Gaussian matrix with the phase fix
Q diag(R_ii / |R_ii|) (Mezzadri, "How to generate random matrices from the
classical compact groups", 2007).
"""
import math
from dataclasses import dataclass, field

import numpy as np


def haar_unitary(rng, d):
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / math.sqrt(2.0)
    qm, r = np.linalg.qr(z)
    dr = np.diag(r)
    return qm * (dr / np.abs(dr))


def gate_elements(u):
    """SymmTensor elements of a k-qubit unitary (els[in, out] = U[out, in])."""
    return np.ascontiguousarray(u.T).reshape(-1).astype(np.complex128)


@dataclass
class Layer:
    pairs: list                  # [(q_a, q_b)] — gate g acts with input 0 on q_a, input 1 on q_b
    gates: list                  # SymmTensor elements (16 complex each)
    phases: np.ndarray = None    # per-qubit phases for the diagonal layer, or None
    ptup: list = None            # permutation after the layer, or None


@dataclass
class Circuit:
    n: int
    layers: list = field(default_factory=list)

    @property
    def dims(self):
        return [2] * self.n

    def gate_count(self):
        return sum(len(l.gates) for l in self.layers)


def random_circuit(n, depth, seed=2026, diag_every=4, perm_every=8, n_dis=3):
    rng = np.random.default_rng(seed)
    c = Circuit(n)
    for l in range(depth):
        order = rng.permutation(n)
        pairs = [(int(order[2 * j]), int(order[2 * j + 1])) for j in range(n // 2)]
        gates = [gate_elements(haar_unitary(rng, 4)) for _ in pairs]
        layer = Layer(pairs, gates)
        if diag_every and (l + 1) % diag_every == 0:
            layer.phases = rng.uniform(0.0, 2.0 * math.pi, n)
        if perm_every and (l + 1) % perm_every == 0:
            local = rng.choice(np.arange(n_dis, n), size=n_dis, replace=False)
            ptup = list(range(n))
            for k in range(n_dis):
                ptup[k], ptup[int(local[k])] = int(local[k]), k
            layer.ptup = ptup
        c.layers.append(layer)
    return c


def phase_factors(phases):
    """Concatenated per-qubit diagonals (1, e^{i phi}) for a diagonal layer."""
    return np.stack([np.ones_like(phases), np.exp(1j * phases)], axis=1).reshape(-1).astype(np.complex128)


def inverse_circuit(c):
    """The circuit that undoes ``c`` (layers reversed, U -> U^dagger, phases negated,
    permutations inverted)."""
    inv = Circuit(c.n)
    for layer in reversed(c.layers):
        # A layer runs gates, then phases, then the permutation; undo them in reverse.
        if layer.ptup is not None:
            ptup_inv = [0] * c.n
            for i, p in enumerate(layer.ptup):
                ptup_inv[p] = i
            inv.layers.append(Layer([], [], None, ptup_inv))
        if layer.phases is not None:
            inv.layers.append(Layer([], [], -layer.phases, None))
        gates = []
        for els in reversed(layer.gates):
            u = els.reshape(4, 4).T          # U[out, in]
            gates.append(gate_elements(u.conj().T))
        inv.layers.append(Layer(list(reversed(layer.pairs)), gates))
    return inv


def random_state(n, seed=7):
    """i.i.d. complex Gaussian amplitudes normalised to unit L2 (numpy, host)."""
    rng = np.random.default_rng(seed)
    psi = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    psi /= np.linalg.norm(psi)
    return psi


# ---- dense contraction pairs (the precision study of the dense GEMM) ------------------

DENSE_DIMS = (2, 4, 16, 32, 64)


def dense_pair(rng, max_elems=2 ** 26, mnk_range=(256, 16384), max_mnk=None):
    """One DenseTensor pair: ranks 4-6, dims from {2, 4, 16, 32, 64}, 2-3 shared indices at
    random positions, at most max_elems elements per tensor, M, N, K within mnk_range
    (and M*N*K <= max_mnk when given). Returns (dims1, dims2, wires, M, N, K)."""
    lo, hi = mnk_range
    while True:
        r1, r2 = int(rng.integers(4, 7)), int(rng.integers(4, 7))
        ns = int(rng.integers(2, 4))
        shared = [int(rng.choice(DENSE_DIMS)) for _ in range(ns)]
        o1 = [int(rng.choice(DENSE_DIMS)) for _ in range(r1 - ns)]
        o2 = [int(rng.choice(DENSE_DIMS)) for _ in range(r2 - ns)]
        M, N, K = int(np.prod(o1)), int(np.prod(o2)), int(np.prod(shared))
        if not (lo <= M <= hi and lo <= N <= hi and lo <= K <= hi):
            continue
        if M * K > max_elems or K * N > max_elems or (max_mnk and M * N * K > max_mnk):
            continue
        p1, p2 = [int(x) for x in rng.permutation(r1)], [int(x) for x in rng.permutation(r2)]
        d1, d2 = [0] * r1, [0] * r2
        for i, dim in enumerate(o1 + shared):
            d1[p1[i]] = dim
        for i, dim in enumerate(shared + o2):
            d2[p2[i]] = dim
        wires = [(p1[len(o1) + j], p2[j]) for j in range(ns)]
        return d1, d2, wires, M, N, K


# ---- batched uneven circuits (many independent circuits, mixed precision) -------------

def haar_unitaries(rng, count, d):
    """`count` Haar-random d x d unitaries at once (stacked QR with the phase fix)."""
    z = (rng.standard_normal((count, d, d)) + 1j * rng.standard_normal((count, d, d))) / math.sqrt(2.0)
    qm, r = np.linalg.qr(z)
    dr = np.diagonal(r, axis1=1, axis2=2)
    return qm * (dr / np.abs(dr))[:, None, :]


def batch_circuits(count, seed=2026, qubits=(10, 22), depth=(8, 32), diag_every=4, swap_prob=0.25, queries=64):
    """`count` independent circuits: qubits uniform in [qubits], depth uniform in [depth];
    every layer a seeded random pairing with one Haar two-qubit gate per pair, every
    `diag_every`-th layer per-qubit phases, and with probability `swap_prob` a SwapTensor
    exchange of two random qubits (as a permutation). Returns [(Circuit, query indices)]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(qubits[0], qubits[1] + 1))
        dep = int(rng.integers(depth[0], depth[1] + 1))
        us = haar_unitaries(rng, dep * (n // 2), 4)
        c = Circuit(n)
        k = 0
        for l in range(dep):
            order = rng.permutation(n)
            pairs = [(int(order[2 * j]), int(order[2 * j + 1])) for j in range(n // 2)]
            gates = [np.ascontiguousarray(us[k + j].T).reshape(-1).astype(np.complex128) for j in range(len(pairs))]
            k += len(pairs)
            layer = Layer(pairs, gates)
            if diag_every and (l + 1) % diag_every == 0:
                layer.phases = rng.uniform(0.0, 2.0 * math.pi, n)
            if rng.random() < swap_prob:
                a, b = (int(x) for x in rng.choice(n, size=2, replace=False))
                ptup = list(range(n))
                ptup[a], ptup[b] = b, a
                layer.ptup = ptup
            c.layers.append(layer)
        out.append((c, rng.integers(0, 2 ** n, size=queries, dtype=np.uint64)))
    return out


def write_api_circuit(path, circuit, psi=None, seed=None, n_dis=3):
    """Input file of the C++ API driver's circuit mode (qtnh_gb300/drivers/api_bench.cpp):
    the circuit, and either the initial state or the seed of one the driver draws."""
    import struct
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", circuit.n, len(circuit.layers)))
        if psi is not None:
            f.write(struct.pack("<i", 1))
            f.write(np.ascontiguousarray(psi, dtype=np.complex128).tobytes())
        else:
            f.write(struct.pack("<iQ", 0, int(seed or 0)))
        for layer in circuit.layers:
            f.write(struct.pack("<i", len(layer.gates)))
            for (a, b), els in zip(layer.pairs, layer.gates):
                f.write(struct.pack("<HH", a, b))
                f.write(np.ascontiguousarray(els, dtype=np.complex128).tobytes())
            if layer.phases is not None:
                f.write(struct.pack("<i", 1))
                f.write(np.asarray(layer.phases, dtype="<f8").tobytes())
            else:
                f.write(struct.pack("<i", 0))
            if layer.ptup is not None:
                f.write(struct.pack("<i", 1))
                f.write(np.asarray(layer.ptup, dtype="<u2").tobytes())
            else:
                f.write(struct.pack("<i", 0))
            f.write(struct.pack("<i", n_dis))


def run_api_driver(args, timeout=1800):
    """Runs the C++ API driver; returns its JSON line (dict)."""
    import json
    import subprocess
    from .build import DRIVER_BIN
    r = subprocess.run([DRIVER_BIN] + [str(a) for a in args], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("api_bench failed (%d): %s%s" % (r.returncode, r.stdout, r.stderr))
    return json.loads(r.stdout.strip().splitlines()[-1])
