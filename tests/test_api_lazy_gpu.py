"""The drop-in path: workloads written against the qtnh C++ API (include/qtnh.hpp), run by
qtnh_gb300/drivers/api_bench.cpp.

* The random layered circuit with one Tensor::contract per gate and per phase diagonal
  (the in-place rule, src/tensor/contract.cpp:250-289) and rescatter / permute /
  rescatter redistributions: the C++ API queues the in-place contractions and applies them
  as fused layers, so the result must equal the batched C ABI runner (DeviceCircuit, which
  fuses the same gates, though the C++ queue spans several layers, so its fixed-point
  chains are longer) within 1e-12 and the oracle within 1e-12 relative L2.
* The QFT (configs of the reference's example: Hadamard SymmTensors, controlled-phase
  DiagTensors, SwapTensor reversals, "DIST" identities for distributed qubits) as a
  TensorNetwork contracted with contractAll(order): the same dims and, within 1e-12
  relative L2, the same amplitudes as the oracle's run of the same contractions, and the
  discrete Fourier transform of the input.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q
from oracle import oracle as orc
from qtnh_gb300 import workload as wl
from qtnh_gb300.circuit import DeviceCircuit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _setup():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from qtnh_gb300 import build
    build.build()
    orc.build()


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_api_circuit_matches_batched_runner_and_oracle(tmp_path):
    n, depth = 16, 16
    c = wl.random_circuit(n, depth, seed=771)
    psi = wl.random_state(n, seed=772)
    fin, fout = str(tmp_path / "c.bin"), str(tmp_path / "c.out")
    wl.write_api_circuit(fin, c, psi=psi)
    line = wl.run_api_driver(["circuit", fin, fout, 0, 1])
    assert line["contractions_per_run"] == c.gate_count() + n * (depth // 4)
    out = np.fromfile(fout, dtype=np.complex128)
    state = torch.from_numpy(psi.copy()).cuda()
    dev = DeviceCircuit(c).run(state, torch.empty_like(state)).cpu().numpy()
    assert rel_l2(out, dev) < 1e-12
    assert rel_l2(out, orc.run_circuit(psi, c)) < 1e-12
    assert q.take_device_errors() == 0


@pytest.mark.parametrize("dq", [0, 1])
def test_api_qft_network_matches_oracle_and_dft(tmp_path, dq):
    from tests.test_qft_gpu import OracleEngine, run_qft
    n = 16
    rng = np.random.default_rng(1700 + dq)
    psi = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    psi /= np.linalg.norm(psi)
    fin, fout = str(tmp_path / "q.bin"), str(tmp_path / "q.out")
    psi.astype(np.complex128).tofile(fin)
    line = wl.run_api_driver(["qft", n, dq, fin, fout, 0, 1])
    out = np.fromfile(fout, dtype=np.complex128)
    ref, pos = run_qft(OracleEngine(), psi, n, dq, lambda *a: None)
    assert line["dims"] == list(ref.dis) + list(ref.loc) and line["ndis"] == len(ref.dis)
    assert rel_l2(out, ref.els) < 1e-12
    dft = np.fft.ifft(psi) * math.sqrt(2 ** n)
    assert rel_l2(out.reshape([2] * n).transpose(pos).reshape(-1), dft) < 1e-12
