"""C ABI checks that need no GPU: the library loads, exports every declared entry
point, and its host-side contraction planning (Tensor::contract metadata,
src/tensor/contract.cpp:204-289) agrees with the oracle."""
import ctypes
import itertools
import json
import os
import random

import numpy as np
import pytest

import qtnh_gb300 as q
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
RT = json.load(open(os.path.join(HERE, "golden", "random_tensors.json")))["groups"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    orc.build()
    q.lib()


def test_exports_every_declared_symbol():
    names = q.declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(q.lib(), n), n


def test_abi_version_and_no_device():
    assert q.lib().qtnh_abi_version() == 1
    n = ctypes.c_int(-1)
    q.check(q.lib().qtnh_device_count(ctypes.byref(n)))
    assert n.value >= 0


def _orc_kind(kind):
    return {q.DENSE: orc.DENSE, q.SYMM: orc.SYMM, q.SWAP: orc.SWAP, q.IDEN: orc.IDEN, q.DIAG: orc.DIAG}[kind]


def _oracle_meta(kind1, dis1, loc1, kind2, dis2, loc2, ndi2, wires, repls=None):
    def mk(kind, dis, loc, ndi):
        dims = dis + loc
        if kind in (orc.DENSE, orc.SYMM):
            els = np.zeros(int(np.prod(dims)) if dims else 1, dtype=np.complex128)
        elif kind == orc.DIAG:
            t = orc.Tensor(kind, dis, loc, None, ndi)
            nin = int(np.prod(dis[:ndi] + loc[:len(loc) // 2 - ndi])) if (dis[:ndi] + loc[:len(loc) // 2 - ndi]) else 1
            els = np.zeros(nin, dtype=np.complex128)
        else:
            els = None
        return orc.Tensor(kind, dis, loc, els, ndi)
    t1 = mk(_orc_kind(kind1), dis1, loc1, 0)
    t2 = mk(_orc_kind(kind2), dis2, loc2, ndi2)
    res, r1, r2 = orc.contract(t1, t2, wires, repls)
    return res.dis, res.loc, r1, r2, res.bc[0]


def _both(kind1, dis1, loc1, kind2, dis2, loc2, ndi2, wires, repls=None):
    exc_o = exc_q = None
    try:
        o = _oracle_meta(kind1, dis1, loc1, kind2, dis2, loc2, ndi2, wires, repls)
    except (ValueError, IndexError, RuntimeError) as e:
        exc_o = type(e)
    try:
        g = q.contract_plan(q.Tensor(kind1, dis1, loc1), q.Tensor(kind2, dis2, loc2, None, ndi2), wires, repls)
    except (ValueError, IndexError, RuntimeError) as e:
        exc_q = type(e)
    if exc_o or exc_q:
        assert exc_o is not None and exc_q is not None, (exc_o, exc_q)
        assert issubclass(exc_q, exc_o) or issubclass(exc_o, ValueError) == issubclass(exc_q, ValueError)
        return None
    assert list(o[0]) == g[0] and list(o[1]) == g[1]
    assert list(o[2]) == g[2] and list(o[3]) == g[3]
    assert o[4] == g[4]
    return g


@pytest.mark.parametrize("group,s1,s2", [("dense_vals", 0, 0), ("mpi2r_vals", 1, 0), ("mpi4r_vals", 1, 1),
                                         ("mpi8r_vals", 2, 1)])
def test_plan_matches_oracle_on_goldens(group, s1, s2):
    for cv in RT[group]:
        d1, d2 = cv["t1"]["dims"], cv["t2"]["dims"]
        g = _both(q.DENSE, d1[:s1], d1[s1:], q.DENSE, d2[:s2], d2[s2:], 0, [tuple(w) for w in cv["wires"]])
        assert g is not None and g[0] + g[1] == cv["t3"]["dims"]


def test_plan_symmetric_and_delta_kinds():
    rng = random.Random(11)
    for _ in range(300):
        r1 = rng.randint(1, 5)
        d = rng.choice([2, 3])
        loc1 = [d] * r1
        nd1 = rng.randint(0, min(2, r1))
        dis1, loc1 = loc1[:nd1], loc1[nd1:]
        kind2 = rng.choice([q.SYMM, q.SWAP, q.IDEN, q.DIAG])
        if kind2 == q.SWAP:
            dis2, loc2, ndi2 = [], [d] * 4, 0
        else:
            k = rng.randint(1, 2)
            dis2, loc2, ndi2 = [], [d] * (2 * k), 0
        tot2 = len(dis2) + len(loc2)
        nw = rng.randint(0, min(len(loc1), tot2))
        a = rng.sample(range(nd1, nd1 + len(loc1)), nw)
        b = rng.sample(range(tot2), nw)
        _both(q.DENSE, dis1, loc1, kind2, dis2, loc2, ndi2, list(zip(a, b)))


def test_plan_distributed_wires_and_errors():
    rng = random.Random(5)
    for _ in range(300):
        dis1 = [rng.choice([2, 3]) for _ in range(rng.randint(0, 2))]
        loc1 = [rng.choice([2, 3]) for _ in range(rng.randint(0, 3))]
        dis2 = [rng.choice([2, 3]) for _ in range(rng.randint(0, 2))]
        loc2 = [rng.choice([2, 3]) for _ in range(rng.randint(0, 3))]
        r1, r2 = len(dis1) + len(loc1), len(dis2) + len(loc2)
        nw = rng.randint(0, min(r1, r2))
        wires = list(zip(rng.sample(range(r1), nw), rng.sample(range(r2), nw))) if nw else []
        _both(q.DENSE, dis1, loc1, q.DENSE, dis2, loc2, 0, wires)


def test_plan_custom_replacements():
    # README.md:153-165 example: wire (1, 0), dimRepls1 = {0, X, 2}, dimRepls2 = {X, 1}
    g = _both(q.DENSE, [], [2, 2, 2], q.DENSE, [], [2, 2], 0, [(1, 0)], ([0, q.X, 2], [q.X, 1]))
    assert g[2] == [0, q.X, 2] and g[3] == [q.X, 1]
    # a repeated position is refused by both
    _both(q.DENSE, [], [2, 2, 2], q.DENSE, [], [2, 2], 0, [(1, 0)], ([0, q.X, 1], [q.X, 1]))


def test_plan_rejects_like_reference():
    with pytest.raises(ValueError):  # contract.cpp:209-211
        q.contract_plan(q.Tensor(q.DENSE, [], [2, 2]), q.Tensor(q.DENSE, [], [3]), [(0, 0)])
    with pytest.raises(ValueError):  # contract.cpp:212-214
        q.contract_plan(q.Tensor(q.DENSE, [2], [2]), q.Tensor(q.DENSE, [], [2]), [(0, 0)])


def test_gate_runs_argument_checks_before_any_launch():
    # qtnh_apply_gate_runs checks every argument on the host before the first launch, so
    # these fail here without a GPU (the device pointers are never touched)
    L = q.lib()
    n = 6
    dims = q._u64([2] * n)
    state, scratch = ctypes.c_void_p(0x1000), ctypes.c_void_p(0x2000)
    gates = (ctypes.c_void_p * 4)(0x3000, 0x3100, 0x3200, 0x3300)
    ks = (ctypes.c_int32 * 4)(2, 2, 2, 2)

    def call(nruns, per_run, targets, ptups, st=state, sc=scratch, rank=n):
        return L.qtnh_apply_gate_runs(st, sc, ctypes.c_int32(rank), dims, ctypes.c_int32(nruns),
                                      (ctypes.c_int32 * max(1, len(per_run)))(*per_run), ks, q._u16(targets), gates,
                                      q._u16(ptups), None)

    ident = list(range(n))
    good_t = [0, 1, 2, 3, 4, 5, 0, 2]
    assert call(0, [], good_t, []) == 1                                      # no run
    assert call(2, [2, 2], good_t, ident, sc=None) == 1                       # no scratch
    assert call(2, [2, 2], good_t, ident, sc=state) == 1                      # scratch is the state
    assert call(2, [2, 2], good_t, [0, 1, 2, 3, 4, 4]) == 1                   # not a permutation
    assert call(2, [2, 2], [0, 1, 2, 3, 4, 6, 0, 2], ident) == 3              # target out of range
    assert call(2, [2, 2], [0, 1, 2, 3, 4, 5, 1, 1], ident) == 1              # target repeated
    assert call(2, [2, -1], good_t, ident) == 1                               # negative gate count
    assert call(1, [2], good_t, [], rank=65) == 1                             # rank beyond QTNH_MAX_RANK


def test_gemm_slice_setting_and_gate_timing_on_the_host():
    L = q.lib()
    assert q.get_gemm_slice() == 32
    for bad in (0, -3, 4097):
        assert L.qtnh_set_gemm_slice(ctypes.c_int(bad)) == 1
    assert q.get_gemm_slice() == 32
    q.set_gemm_slice(64)
    assert q.get_gemm_slice() == 64
    q.set_gemm_slice(32)
    # nothing recorded: zero time, zero launches (no device needed)
    assert q.gate_timing(False) == (0.0, 0)
