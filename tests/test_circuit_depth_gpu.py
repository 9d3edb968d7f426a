"""The headline circuit family at its full depth against the oracle.

The benchmark workload is the random layered circuit: every layer one Haar two-qubit
SymmTensor gate per pair of a seeded pairing, every 4th layer a phase DiagTensor on
every qubit, every 8th layer a rescatter of the top 3 indices with a permutation
exchanging them with 3 local ones. Here it runs at n = 20 for all 40 layers (400 gates,
10 phase layers, 5 redistributions) through the engine's C ABI (DeviceCircuit) in each
arithmetic mode, and through the oracle's Tensor::contract per gate
(src/tensor/contract.cpp:250-289, the in-place rule), on the same seeded input.

For each mode the test reports and bounds:
  * relative L2 error of the final state, ||out - ref|| / ||ref|| <= 1e-12;
  * max amplitude error relative to the largest amplitude,
    max |out - ref| / max |ref| <= 1e-12;
  * infidelity 1 - |<ref|out>|^2 / (<ref|ref> <out|out>) <= 1e-20 (it is the squared
    norm of the error component orthogonal to ref, so it sits far below the L2 error).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q
from oracle import oracle as orc
from qtnh_gb300 import workload as wl
from qtnh_gb300.circuit import DeviceCircuit

pytestmark = pytest.mark.gpu

QUBITS = 20
DEPTH = 40
REL_L2_TOL = 1e-12
MAX_ABS_TOL = 1e-12
INFIDELITY_TOL = 1e-20


def state_errors(out, ref):
    """(relative L2, max amplitude error / largest amplitude, infidelity) of out vs ref."""
    d = out - ref
    rel = np.linalg.norm(d) / np.linalg.norm(ref)
    mx = np.max(np.abs(d)) / np.max(np.abs(ref))
    # 1 - |<ref|out>|^2 / (<ref|ref> <out|out>) = |out_perp|^2 / |out|^2, out_perp the part of
    # out orthogonal to ref (no cancellation, unlike 1 minus a fidelity near 1)
    perp = out - (np.vdot(ref, out) / np.vdot(ref, ref).real) * ref
    return rel, mx, np.vdot(perp, perp).real / np.vdot(out, out).real


@pytest.fixture(scope="module")
def reference():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    c = wl.random_circuit(QUBITS, DEPTH, seed=4031)
    psi = wl.random_state(QUBITS, seed=4032)
    return c, psi, orc.run_circuit(psi, c)


@pytest.mark.parametrize("mode", ["bf16x6", "f32x2", "fp64"])
def test_full_depth_circuit_matches_oracle(reference, mode):
    c, psi, ref = reference
    assert c.gate_count() == DEPTH * QUBITS // 2
    old = q.get_arithmetic()
    q.set_arithmetic(q.ARITH_NAMES[mode])
    try:
        dc = DeviceCircuit(c)
        state = torch.from_numpy(psi.copy()).cuda()
        scratch = torch.empty_like(state)
        out = dc.run(state, scratch).cpu().numpy()
    finally:
        q.set_arithmetic(old)
    assert q.take_device_errors() == 0
    rel, mx, infid = state_errors(out, ref)
    print("n=%d depth=%d %s: rel L2 %.3e, max |err| / max |amp| %.3e, 1 - fidelity %.3e"
          % (QUBITS, DEPTH, mode, rel, mx, infid))
    assert rel <= REL_L2_TOL
    assert mx <= MAX_ABS_TOL
    assert infid <= INFIDELITY_TOL
