"""The circuit runner's call plan (qtnh_gb300/circuit.py), checked on the host: the phase
layers folded into the gates before them, every stretch of gate layers and redistributions
between two diagonal layers one qtnh_apply_gate_runs call, and the plan replayed with the
oracle's contractions equal to the circuit applied one Tensor::contract at a time
(oracle.run_circuit). No GPU: the plan is built on CPU tensors and never launched."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as orc
from qtnh_gb300 import workload as wl
from qtnh_gb300.circuit import DeviceCircuit


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    orc.build()


def replay(dc, psi):
    """Applies the plan's calls with the oracle: gates (SymmTensor layout, read from the
    runner's gate buffer at the plan's pointers), permutations between runs, diagonal
    layers."""
    n = dc.n
    base = dc.gates.data_ptr()
    gates = dc.gates.numpy()
    cur = orc.Tensor(orc.DENSE, [], [2] * n, psi)
    for kind, args in dc.steps:
        if kind == "runs":
            nr, counts, ks, tg, ptrs, pts, nperm = args
            assert nperm == nr.value - 1
            counts = list(counts)[:nr.value]
            tg, ptrs, pts = list(tg), list(ptrs), list(pts)
            g = 0
            for r, c in enumerate(counts):
                for _ in range(c):
                    assert ks[g] == 2
                    j = (ptrs[g] - base) // (16 * 16)
                    els = gates[16 * j:16 * (j + 1)]
                    cur, _, _ = orc.contract(cur, orc.Tensor(orc.SYMM, [], [2, 2, 2, 2], els),
                                             [(tg[2 * g], 0), (tg[2 * g + 1], 1)])
                    g += 1
                if r + 1 < nr.value:
                    pt = pts[n * r:n * (r + 1)]
                    cur = orc.Tensor(orc.DENSE, [], [2] * n, orc.permute(cur.els.reshape([2] * n), pt).reshape(-1))
        else:
            nf, axes, f = args
            f = f.numpy()
            for k, ax in enumerate(list(axes)[:nf.value]):
                cur, _, _ = orc.contract(cur, orc.Tensor(orc.DIAG, [], [2, 2], f[2 * k:2 * k + 2]), [(ax, 0)])
    return cur.els


def test_even_circuit_is_one_call():
    # every qubit is covered by a gate in every layer: all phase layers fold, and the two
    # redistributions sit inside the one call (three runs, the last one empty)
    n, depth = 8, 16
    c = wl.random_circuit(n, depth, seed=11)
    dc = DeviceCircuit(c, device="cpu")
    assert [k for k, _ in dc.steps] == ["runs"]
    nr, counts, *_, nperm = dc.steps[0][1]
    assert nr.value == 3 and list(counts)[:3] == [32, 32, 0] and nperm == 2
    psi = wl.random_state(n, seed=12)
    assert np.linalg.norm(replay(dc, psi) - orc.run_circuit(psi, c)) < 1e-12 * np.linalg.norm(psi)


def test_odd_circuit_keeps_a_diagonal_layer_per_phase_layer():
    # one qubit per layer has no gate: its phase stays a diagonal layer, which ends a call
    n, depth = 7, 12
    c = wl.random_circuit(n, depth, seed=21)
    dc = DeviceCircuit(c, device="cpu")
    kinds = [k for k, _ in dc.steps]
    assert kinds == ["runs", "diag", "runs", "diag", "runs", "diag"]
    assert all(args[0].value == 1 for k, args in dc.steps if k == "diag")  # one leftover qubit each
    psi = wl.random_state(n, seed=22)
    assert np.linalg.norm(replay(dc, psi) - orc.run_circuit(psi, c)) < 1e-12 * np.linalg.norm(psi)


def test_folded_gate_is_the_gate_then_its_phases():
    # the gate buffer holds (D_a (x) D_b) U for the gates of a phase layer
    n = 6
    c = wl.random_circuit(n, 4, seed=31, perm_every=0)
    dc = DeviceCircuit(c, device="cpu")
    layer = c.layers[3]
    first = sum(len(L.gates) for L in c.layers[:3])
    for j, ((a, b), els) in enumerate(zip(layer.pairs, layer.gates)):
        u = np.asarray(els).reshape(4, 4).T  # u[out, in]
        da = np.array([1.0, np.exp(1j * layer.phases[a])])
        db = np.array([1.0, np.exp(1j * layer.phases[b])])
        want = (np.kron(np.diag(da), np.diag(db)) @ u).T.reshape(-1)
        got = dc.gates.numpy()[16 * (first + j):16 * (first + j + 1)]
        assert np.allclose(got, want, rtol=0, atol=1e-15)
