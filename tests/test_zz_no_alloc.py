"""qtnh_contract_dense_noalloc: the contraction entry point for callers that cannot
allocate device memory while they run (their device memory belongs to a host
framework's own allocator or a fixed budget, or a cudaMalloc would stall a
latency-critical loop). Its scratch is a fixed 16 MiB array inside the library.

Checked through the C ABI against qtnh_contract_dense on two calls in a row (the
second call reuses the scratch left by the first), within the contraction tolerance of
the other GPU tests; across those calls the library takes no scratch buffer and the
device's stream-ordered pool holds no more bytes than before (qtnh_workspace_stats);
an oversized contraction must be refused before any work. Runs alone in a fresh process
as well as after the other tests."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q

pytestmark = pytest.mark.gpu
REL_TOL = 1e-12


def _call(fn, a, da, b, db, wires, pos_a, pos_b, c):
    w = (ctypes.c_uint16 * max(1, 2 * len(wires)))(*[x for p in wires for x in p])
    return fn(ctypes.c_void_p(a.data_ptr()), ctypes.c_int32(len(da)), q._u64(da), ctypes.c_void_p(b.data_ptr()),
              ctypes.c_int32(len(db)), q._u64(db), ctypes.c_int32(len(wires)), w, q._u16(pos_a), q._u16(pos_b),
              ctypes.c_void_p(c.data_ptr()), q._stream())


def _stats():
    allocs, used = ctypes.c_uint64(0), ctypes.c_uint64(0)
    q.check(q.lib().qtnh_workspace_stats(ctypes.byref(allocs), ctypes.byref(used)))
    return allocs.value, used.value


def _case(rng, da, db, wires, pos_a, pos_b):
    a = torch.from_numpy(rng.standard_normal(int(np.prod(da))) + 1j * rng.standard_normal(int(np.prod(da)))).cuda()
    b = torch.from_numpy(rng.standard_normal(int(np.prod(db))) + 1j * rng.standard_normal(int(np.prod(db)))).cuda()
    n_out = 1
    for i, d in enumerate(da):
        if pos_a[i] != q.X:
            n_out *= d
    for i, d in enumerate(db):
        if pos_b[i] != q.X:
            n_out *= d
    ref = torch.empty(n_out, dtype=torch.complex128, device="cuda")
    out = torch.full((n_out,), complex(float("nan"), 0.0), dtype=torch.complex128, device="cuda")
    q.check(_call(q.lib().qtnh_contract_dense, a, da, b, db, wires, pos_a, pos_b, ref))
    torch.cuda.synchronize()
    before = _stats()
    q.check(_call(q.lib().qtnh_contract_dense_noalloc, a, da, b, db, wires, pos_a, pos_b, out))
    torch.cuda.synchronize()
    after = _stats()
    assert after == before, "the allocation-free path allocated: %s -> %s" % (before, after)
    r, o = ref.cpu().numpy(), out.cpu().numpy()
    return np.linalg.norm(o - r) / np.linalg.norm(r)


def test_noalloc_matches_allocating_path_twice():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = np.random.default_rng(2024)
    X = q.X
    # A[i,k,j,l] B[l,m,k]: both operands and the result need a permutation (scratch)
    da, db = [8, 16, 4, 6], [6, 12, 16]
    wires = [(1, 2), (3, 0)]
    pos_a, pos_b = [2, X, 0, X], [X, 1, X]
    assert _case(rng, da, db, wires, pos_a, pos_b) < REL_TOL
    # second call in a row, different shapes: the scratch holds the first call's data
    da2, db2 = [4, 32, 8], [8, 4, 10]
    assert _case(rng, da2, db2, [(2, 0), (0, 1)], [X, 1, X], [X, X, 0]) < REL_TOL


def test_noalloc_refuses_oversized():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    X = q.X
    da, db = [1025, 1024], [1025, 8]   # the permuted copy of A alone exceeds 2^20 elements
    a = torch.zeros(1025 * 1024, dtype=torch.complex128, device="cuda")
    b = torch.zeros(1025 * 8, dtype=torch.complex128, device="cuda")
    c = torch.zeros(1024 * 8, dtype=torch.complex128, device="cuda")
    rc = _call(q.lib().qtnh_contract_dense_noalloc, a, da, b, db, [(0, 0)], [X, 0], [X, 1], c)
    assert rc == 6  # QTNH_ERR_UNSUPPORTED
    assert b"scratch" in q.lib().qtnh_last_error()
