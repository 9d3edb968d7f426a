"""Batched uneven circuits in mixed precision (qtnh_batch_*: complex64 states, grouped
persistent kernels under one CUDA graph, FP64 renormalisation every 8 layers, complex128
amplitude queries) against the oracle's complex128 circuit runner (the reference's
contraction sequence) and against the GPU's plain FP64 path for a larger circuit.

Error bar of the mixed-precision method: every pass over a state rounds each amplitude
to complex64 once (~6e-8 relative), so a circuit of G passes drifts like sqrt(G) * 6e-8;
asserted at 5e-6 relative L2 per circuit (queries and full states). The plain form of the
same schedule (complex128 states, FP64 math) is held to the contraction bar, 1e-12."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q
from oracle import oracle as orc
from qtnh_gb300 import workload as wl

pytestmark = pytest.mark.gpu
BAR = 5e-6


@pytest.fixture(scope="module", autouse=True)
def _setup():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    orc.build()
    q.lib()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128).reshape(-1)).cuda()


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def small_batch():
    circuits = wl.batch_circuits(12, seed=77, qubits=(10, 14), depth=(8, 20))
    b = q.Batch([c.n for c, _ in circuits])
    states = []
    for i, (c, qi) in enumerate(circuits):
        psi = wl.random_state(c.n, seed=100 + i)
        states.append(psi)
        b.set_state(i, dev(psi))
        b.add_circuit(i, c, qi)
    b.compile(renorm_every=8, autotune=True)
    b.run()
    res = b.results().cpu().numpy()
    refs = [orc.run_circuit(psi, c) for psi, (c, _) in zip(states, circuits)]
    return circuits, b, res, refs


def test_batch_queries_match_oracle(small_batch):
    circuits, b, res, refs = small_batch
    k = 0
    for (c, qi), ref in zip(circuits, refs):
        got = res[k:k + len(qi)]
        k += len(qi)
        assert rel(got, ref[qi.astype(np.int64)]) < BAR, c.n
    info = b.info()
    assert info["gate_threads"] in (128, 256, 512) and info["gate_chunk"] in (64, 256, 1024)  # pair kernel
    assert info["launches_per_run"] >= info["rounds"]


def test_batch_full_states_and_norm(small_batch):
    circuits, b, _, refs = small_batch
    for i in (0, 5, 11):
        st = b.state(i).cpu().numpy()
        assert rel(st, refs[i]) < BAR
        assert abs(np.linalg.norm(st) - 1.0) < 1e-6


def test_batch_graph_replay(small_batch):
    circuits, b, res, _ = small_batch
    b.run()  # the graph starts from the stored initial states every time
    again = b.results().cpu().numpy()
    assert rel(again, res) < 1e-12


def test_batch_large_circuit_vs_fp64_engine():
    from qtnh_gb300.circuit import DeviceCircuit
    (c, qi), = wl.batch_circuits(1, seed=5, qubits=(20, 20), depth=(12, 12))
    psi = wl.random_state(c.n, seed=6)
    b = q.Batch([c.n])
    b.set_state(0, dev(psi))
    b.add_circuit(0, c, qi)
    b.compile(renorm_every=8, autotune=False)
    b.run()
    got = b.state(0).cpu().numpy()
    old = q.get_arithmetic()
    q.set_arithmetic(q.ARITH_FP64)
    try:
        st = dev(psi)
        out = DeviceCircuit(c).run(st, torch.empty_like(st))
        torch.cuda.synchronize()
        ref = out.cpu().numpy()
    finally:
        q.set_arithmetic(old)
    assert rel(got, ref) < BAR
    assert rel(b.results().cpu().numpy(), ref[qi.astype(np.int64)]) < BAR


def test_plain_batch_matches_oracle():
    # the plain method on the same schedule: complex128 states, FP64 math, no renormalisation
    circuits = wl.batch_circuits(10, seed=78, qubits=(10, 14), depth=(8, 20))
    b = q.Batch([c.n for c, _ in circuits], precision=q.STATE_C128)
    states = []
    for i, (c, qi) in enumerate(circuits):
        psi = wl.random_state(c.n, seed=300 + i)
        states.append(psi)
        b.set_state(i, dev(psi))
        b.add_circuit(i, c, qi)
    b.compile(renorm_every=0, autotune=True)
    b.run()
    res = b.results().cpu().numpy()
    k = 0
    for i, ((c, qi), psi) in enumerate(zip(circuits, states)):
        ref = orc.run_circuit(psi, c)
        assert rel(res[k:k + len(qi)], ref[qi.astype(np.int64)]) < 1e-12
        k += len(qi)
        if i % 3 == 0:
            assert rel(b.state(i).cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("precision,bar", [(None, BAR), (q.STATE_C128, 1e-12)], ids=["mixed", "plain"])
def test_batch_overlapping_gates_in_a_layer(precision, bar):
    # gates of a layer that share a qubit are not fused: (0,1) then (1,2) run as single
    # passes, (1,2) and (3,4) as a pair, (5,6) alone; targets include the lowest and the
    # highest qubit, and a 5-qubit circuit (odd) sits beside them
    rng = np.random.default_rng(31)
    circuits = []
    for n in (12, 5):
        c = wl.Circuit(n)
        for layer in range(3):
            pairs = [(0, 1), (1, 2), (3, 4)] + ([(5, 6), (n - 1, 7)] if n > 8 else [])
            us = wl.haar_unitaries(rng, len(pairs), 4)
            c.layers.append(wl.Layer(pairs, [np.ascontiguousarray(u.T).reshape(-1) for u in us]))
        circuits.append(c)
    b = q.Batch([c.n for c in circuits], precision=precision)
    states = [wl.random_state(c.n, seed=40 + i) for i, c in enumerate(circuits)]
    for i, c in enumerate(circuits):
        b.set_state(i, dev(states[i]))
        b.add_circuit(i, c)
    b.compile(renorm_every=0, autotune=False)
    b.run()
    for i, c in enumerate(circuits):
        assert rel(b.state(i).cpu().numpy(), orc.run_circuit(states[i], c)) < bar


def test_batch_deep_circuits_within_1e6():
    # the mixed-precision bar of the batched form: 1e-6 relative L2 against the FP64 oracle
    # on circuits of ~320 gates per amplitude (depth 40 at 16 qubits): the gates sum their
    # products exactly in 64-bit integers, so each pass over a state rounds once
    circuits = wl.batch_circuits(3, seed=91, qubits=(15, 16), depth=(40, 40))
    b = q.Batch([c.n for c, _ in circuits])
    states = []
    for i, (c, qi) in enumerate(circuits):
        psi = wl.random_state(c.n, seed=500 + i)
        states.append(psi)
        b.set_state(i, dev(psi))
        b.add_circuit(i, c, qi)
    b.compile(renorm_every=8, autotune=False)
    b.run()
    for i, (c, _) in enumerate(circuits):
        ref = orc.run_circuit(states[i], c)
        got = b.state(i).cpu().numpy()
        assert rel(got, ref) < 1e-6, (c.n, rel(got, ref))
        fid = abs(np.vdot(ref, got)) ** 2 / (np.vdot(ref, ref).real * np.vdot(got, got).real)
        assert fid > 1 - 1e-9


def test_batch_rejects_invalid_operations():
    b = q.Batch([10, 12])
    eye = np.eye(4, dtype=np.complex128).reshape(-1)
    c = wl.Circuit(10)
    c.layers.append(wl.Layer([(0, 1)], [eye]))
    with pytest.raises(q.QtnhError):
        b.add_circuit(2, c)  # no circuit 2
    c = wl.Circuit(10)
    c.layers.append(wl.Layer([(3, 3)], [eye]))
    with pytest.raises(q.QtnhError):
        b.add_circuit(0, c)  # a gate on one qubit twice
    with pytest.raises(q.QtnhError):
        b.add_circuit(1, wl.Circuit(12), queries=[2 ** 12])
    with pytest.raises(q.QtnhError):
        q.Batch([10], precision=7)  # no such state precision


def test_plain_batch_float_float_gates_match_oracle(small_batch, monkeypatch):
    # the plain complex128 schedule with float-float gate arithmetic (QTNH_BATCH_GATES=f32x2,
    # the grouped pair and single-gate kernels in compensated FP32): every final state within
    # the contraction bar of the oracle
    circuits, _, _, refs = small_batch
    monkeypatch.setenv("QTNH_BATCH_GATES", "f32x2")
    b = q.Batch([c.n for c, _ in circuits], precision=q.STATE_C128)
    for i, (c, qi) in enumerate(circuits):
        b.set_state(i, dev(wl.random_state(c.n, seed=100 + i)))
        b.add_circuit(i, c, qi)
    b.compile(renorm_every=0, autotune=True)
    monkeypatch.delenv("QTNH_BATCH_GATES")
    b.run()
    for i, ref in enumerate(refs):
        assert rel(b.state(i).cpu().numpy(), ref) < 1e-12
    assert q.take_device_errors() == 0
