"""The bounded-wait error path of the tcgen05 gate-pair kernel, exercised without faulting
the GPU: the test hook qtnh_debug_expire_exchange_wait makes the first exponent exchange of
every CTA wait on a shared-memory barrier that nothing completes, with a ~2^20-cycle limit.
That wait comes before any MMA, tensor-memory load or bulk copy of the CTA is issued. The
launch must end by itself, raise error bit 2 (qtnh_take_device_errors), free its tensor
memory and leave the state as it was; the next launch with the hook off must be correct."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_expired_exchange_wait_is_reported_and_recovered():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = np.random.default_rng(5150)
    n = 13  # 512 groups of 16: four 128-group tiles, the tcgen05 kernel
    psi = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)

    def haar():
        z = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
        u, r = np.linalg.qr(z)
        return (u * (np.diag(r) / np.abs(np.diag(r)))).T.reshape(-1)

    gates = [([3, 9], haar()), ([0, 12], haar())]
    old = q.get_arithmetic()
    q.set_arithmetic(q.ARITH_BF16X6)
    q.take_device_errors()
    st = torch.from_numpy(psi.copy()).cuda()
    L = q.lib()
    try:
        q.check(L.qtnh_debug_expire_exchange_wait(ctypes.c_int(1)))
        q.apply_gate_layer(st, [2] * n, [(t, torch.from_numpy(g).cuda()) for t, g in gates])
        flags = q.take_device_errors()  # synchronizes: the launch has ended
    finally:
        q.check(L.qtnh_debug_expire_exchange_wait(ctypes.c_int(0)))
    try:
        assert flags & 4, flags
        assert np.array_equal(st.cpu().numpy(), psi)  # nothing was written
        # the context is usable and the tensor memory free: a normal launch is correct
        q.apply_gate_layer(st, [2] * n, [(t, torch.from_numpy(g).cuda()) for t, g in gates])
        out = st.cpu().numpy()
        assert q.take_device_errors() == 0
    finally:
        q.set_arithmetic(old)
    ref = orc.Tensor(orc.DENSE, [], [2] * n, psi)
    for t, g in gates:
        ref, _, _ = orc.contract(ref, orc.Tensor(orc.SYMM, [], [2, 2, 2, 2], g), [(t[0], 0), (t[1], 1)])
    assert np.linalg.norm(out - ref.els) / np.linalg.norm(ref.els) < 1e-12
