"""The request loop on the GPU (grouped layer steps over resident states, FP64
renormalisation, amplitude and reduced-density-matrix answers) in plain complex128 and
mixed complex64, against the oracle's complex128 contraction sequence of every
request: plain within 1e-12 relative, mixed within the batched-circuit bar 5e-6; and a
request's answer served alone against the same request served in a mix of others."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q
from oracle import oracle as orc
from qtnh_gb300 import serve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _setup():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    orc.build()
    q.lib()


def reference(req):
    g = torch.Generator(device="cuda")
    g.manual_seed(req.seed)
    psi = torch.randn(2 ** req.circuit.n, dtype=torch.complex128, device="cuda", generator=g)
    psi = (psi / torch.linalg.vector_norm(psi)).cpu().numpy()
    fin = orc.run_circuit(psi, req.circuit)
    n = req.circuit.n
    if req.kind == "amps":
        return fin[req.query.astype(np.int64)]
    qs = [int(x) for x in req.query]
    rest = [i for i in range(n) if i not in qs]
    m = fin.reshape([2] * n).transpose(qs + rest).reshape(16, -1)
    return m @ m.conj().T


@pytest.mark.parametrize("precision,bar", [(serve.C128, 1e-12), (serve.C64, 5e-6)], ids=["plain", "mixed"])
def test_serve_answers_match_oracle(precision, bar):
    reqs = serve.request_stream(14, rate=4000.0, seed=11, qubits=(10, 14), depth=(10, 18))
    ex = serve.GpuExecutor(precision)
    lat, results, stats = serve.serve(reqs, ex, budget_bytes=4 * 2 ** 20,
                                      renorm_every=8 if precision == serve.C64 else 0, realtime=False)
    assert stats["requests"] == len(reqs)
    for r in reqs:
        got, ref = np.asarray(results[r.rid]), reference(r)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < bar, (r.rid, r.kind, r.circuit.n, err)
    assert q.take_device_errors() == 0


def test_serve_plain_float_float_gates_match_oracle(monkeypatch):
    # complex128 states with the grouped gates in float-float (QTNH_BATCH_GATES=f32x2, read
    # at every grouped call): the plain bar of 1e-12 against the oracle still holds
    monkeypatch.setenv("QTNH_BATCH_GATES", "f32x2")
    reqs = serve.request_stream(10, rate=4000.0, seed=31, qubits=(10, 14), depth=(16, 24))
    lat, results, stats = serve.serve(reqs, serve.GpuExecutor(serve.C128), budget_bytes=4 * 2 ** 20,
                                      renorm_every=0, realtime=False)
    assert stats["requests"] == len(reqs)
    for r in reqs:
        got, ref = np.asarray(results[r.rid]), reference(r)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-12, (r.rid, r.kind, r.circuit.n, err)
    assert q.take_device_errors() == 0


@pytest.mark.parametrize("precision,bar", [(serve.C128, 1e-13), (serve.C64, 1e-6)], ids=["plain", "mixed"])
def test_serve_result_same_alone_and_in_mix(precision, bar):
    # a request's answer does not depend on what else is on the GPU: served in a mix of
    # requests of other sizes and depths (grouped launches, work-balanced steps, several
    # layers per step) and served alone, the answers agree within the stated tolerance
    # (FP64 atomics in norms and RDM sums make the two runs differ in the last bits only)
    reqs = serve.request_stream(12, rate=4000.0, seed=21, qubits=(10, 15), depth=(10, 24))
    renorm = 8 if precision == serve.C64 else 0
    _, mix, _ = serve.serve(reqs, serve.GpuExecutor(precision), budget_bytes=8 * 2 ** 20, renorm_every=renorm,
                            realtime=False)
    for r in reqs[::3]:
        _, alone, _ = serve.serve([r], serve.GpuExecutor(precision), budget_bytes=8 * 2 ** 20, renorm_every=renorm,
                                  realtime=False)
        a, m = np.asarray(alone[r.rid]), np.asarray(mix[r.rid])
        assert np.linalg.norm(a - m) / np.linalg.norm(a) < bar, (r.rid, r.kind, r.circuit.n)
    assert q.take_device_errors() == 0
