"""QFT on 16 qubits (the reference's QFT example/test workload, examples/qft.cpp:53-149,
tests/gen/qft.hpp:49-142) on a random state, as the sequence of Tensor::contract calls
a qtnh user makes: a Hadamard SymmTensor per qubit, a controlled-phase DiagTensor
(phases pi / 2^(j-i)) per qubit pair, then SwapTensor reversals. With dq distributed
qubits (the reference run with 2^dq ranks), every gate on a distributed qubit is first
wrapped in the "DIST" identity tensors of the reference QFT network (IdenTensor with one
distributed and one local index: DIST(1) on the gate input, DIST(0) on its output),
then contracted with the state.

The GPU engine (C ABI) and the oracle run the same calls: every step returns the same
dimension replacements and dis/loc split; every swap moves data bit-exactly (its result
holds exactly its input's values; a swap of two local qubits equals the exchange of the
two axes of its own input); the final state agrees with the oracle and with the discrete
Fourier transform within 1e-12 relative L2."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

N_QUBITS = 16
S = 2 ** -0.5
HADAMARD = np.array([S, S, S, -S], dtype=np.complex128)


@pytest.fixture(scope="module", autouse=True)
def _setup():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    orc.build()
    q.lib()


class OracleEngine:
    def tensor(self, kind, dis, loc, els=None, n_dis_in=0):
        kinds = {q.DENSE: orc.DENSE, q.SYMM: orc.SYMM, q.SWAP: orc.SWAP, q.IDEN: orc.IDEN, q.DIAG: orc.DIAG}
        return orc.Tensor(kinds[kind], dis, loc, els, n_dis_in)

    def contract(self, t1, t2, wires):
        return orc.contract(t1, t2, wires)

    def host(self, t):
        return t.els

    def split(self, t):
        return list(t.dis), list(t.loc)


class GpuEngine:
    def tensor(self, kind, dis, loc, els=None, n_dis_in=0):
        data = None
        if els is not None:
            data = torch.from_numpy(np.ascontiguousarray(els, dtype=np.complex128).reshape(-1)).cuda()
        return q.Tensor(kind, dis, loc, data, n_dis_in)

    def contract(self, t1, t2, wires):
        res, r1, r2, _ = q.contract(t1, t2, wires)
        return res, r1, r2

    def host(self, t):
        torch.cuda.synchronize()
        return t.data.cpu().numpy()

    def split(self, t):
        return list(t.dis), list(t.loc)


def run_qft(eng, psi, n, dq, trace):
    """Applies the QFT; trace(kind, before, after, wires, pos) sees every contraction."""
    st = eng.tensor(q.DENSE, [2] * dq, [2] * (n - dq), psi)
    pos = list(range(n))  # axis of the state holding qubit q

    def gate(st, pos, g, qubits, kind):
        k = len(qubits)
        gin, gout = list(range(k)), list(range(k, 2 * k))
        for m, qb in enumerate(qubits):
            if qb < dq:
                g, r1, r2 = eng.contract(eng.tensor(q.IDEN, [2], [2], None, 1), g, [(1, gin[m])])
                trace("dist-in", None, g, None, None)
                gin, gout = [r2[x] for x in gin], [r2[x] for x in gout]
                gin[m] = r1[0]
                g, r1, r2 = eng.contract(g, eng.tensor(q.IDEN, [2], [2], None, 0), [(gout[m], 1)])
                trace("dist-out", None, g, None, None)
                gin, gout = [r1[x] for x in gin], [r1[x] for x in gout]
                gout[m] = r2[0]
        wires = [(pos[qb], gin[m]) for m, qb in enumerate(qubits)]
        out, r1, r2 = eng.contract(st, g, wires)
        pos = [r1[p] for p in pos]
        for m, qb in enumerate(qubits):
            pos[qb] = r2[gout[m]]
        trace(kind, st, out, wires, pos)
        return out, pos

    for i in range(n):
        st, pos = gate(st, pos, eng.tensor(q.SYMM, [], [2, 2], HADAMARD), [i], "h")
        for j in range(i + 1, n):
            d = np.array([1, 1, 1, np.exp(1j * math.pi / 2 ** (j - i))], dtype=np.complex128)
            st, pos = gate(st, pos, eng.tensor(q.DIAG, [], [2, 2, 2, 2], d), [i, j], "cp")
    for k in range(n // 2):
        st, pos = gate(st, pos, eng.tensor(q.SWAP, [], [2] * 4), [k, n - 1 - k], "swap")
    return st, pos


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(params=[q.ARITH_BF16X6, q.ARITH_F32X2, q.ARITH_FP64], ids=["bf16x6", "f32x2", "fp64"])
def arith(request):
    old = q.get_arithmetic()
    q.set_arithmetic(request.param)
    yield request.param
    q.set_arithmetic(old)


@pytest.mark.parametrize("dq", [0, 1, 2])
def test_qft16_matches_oracle_and_dft(dq, arith):
    n = N_QUBITS
    rng = np.random.default_rng(1600 + dq)
    psi = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    psi /= np.linalg.norm(psi)

    steps = {"oracle": [], "gpu": []}
    oracle, gpu = OracleEngine(), GpuEngine()
    swaps = []

    def trace_for(name, eng):
        def trace(kind, before, after, wires, pos):
            steps[name].append((kind, eng.split(after), None if pos is None else list(pos)))
            if name == "gpu" and kind == "swap":
                swaps.append((eng.host(before), eng.split(before), eng.host(after), eng.split(after), wires))
        return trace

    ref, ref_pos = run_qft(oracle, psi, n, dq, trace_for("oracle", oracle))
    out, out_pos = run_qft(gpu, psi, n, dq, trace_for("gpu", gpu))

    # same dimension replacements and dis/loc splits at every step
    assert steps["gpu"] == steps["oracle"]
    assert out_pos == ref_pos
    # every swap moves data bit-exactly: the result holds exactly its input's values, and
    # a swap of two local qubits is the exchange of their two axes
    assert len(swaps) == n // 2
    direct = 0
    for before, (bd, bl), after, (ad, al), wires in swaps:
        assert np.array_equal(np.sort(after), np.sort(before))
        (x, _), (y, _) = wires
        if (bd, bl) == (ad, al) and x >= len(bd) and y >= len(bd):
            want = np.swapaxes(before.reshape(bd + bl), x, y).reshape(-1)
            assert np.array_equal(after, want)
            direct += 1
    assert direct >= n // 2 - 2 * dq
    # final amplitudes
    out_h = gpu.host(out)
    assert rel_l2(out_h, oracle.host(ref)) < 1e-12
    dft = np.fft.ifft(psi) * math.sqrt(2 ** n)
    in_qubit_order = out_h.reshape([2] * n).transpose(out_pos).reshape(-1)
    assert rel_l2(in_qubit_order, dft) < 1e-12
