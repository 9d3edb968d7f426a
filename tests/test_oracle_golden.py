"""Pin the oracle against the reference's own golden vectors.

Mirrors the reference's tests: tests/c2-tensor.cpp:141-214 (dense-dense,
dense-swap, invalid swaps, dense-identity), tests/c2-mpi.cpp:80-214
(contractions of rescattered tensors on 2..8 ranks; here every slab is resident,
so the whole global result is compared), tests/c2-network.cpp:16-199 (networks
and QFT amplitude).
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests.qft_network import build_qft

HERE = os.path.dirname(os.path.abspath(__file__))
RT = json.load(open(os.path.join(HERE, "golden", "random_tensors.json")))["groups"]
TN = json.load(open(os.path.join(HERE, "golden", "random_tn.json")))["groups"]


def _els(info):
    a = np.array(info["els"], dtype=np.float64)
    return (a[:, 0] + 1j * a[:, 1]).astype(np.complex128)


def _equal(a, b, tol):
    # utils::equal (src/core/utils.cpp:69-72): |a - b| < tol elementwise
    return np.all(np.abs(np.asarray(a).reshape(-1) - np.asarray(b).reshape(-1)) < tol)


@pytest.fixture(scope="module", autouse=True)
def _built():
    orc.build()


@pytest.mark.parametrize("i", range(20))
def test_dense_dense(i):
    cv = RT["dense_vals"][i]
    t1 = orc.Tensor(orc.DENSE, [], cv["t1"]["dims"], _els(cv["t1"]))
    t2 = orc.Tensor(orc.DENSE, [], cv["t2"]["dims"], _els(cv["t2"]))
    t3, _, _ = orc.contract(t1, t2, [tuple(w) for w in cv["wires"]])
    assert t3.dims == cv["t3"]["dims"]
    assert _equal(t3.els, _els(cv["t3"]), 1e-5)


def test_dense_invalid_dims():
    t1 = orc.Tensor(orc.DENSE, [], [2, 2], np.arange(4))
    t2 = orc.Tensor(orc.DENSE, [], [3], np.arange(3))
    with pytest.raises(ValueError):
        orc.contract(t1, t2, [(0, 0)])


@pytest.mark.parametrize("i", range(10))
def test_dense_swap(i):
    cv = RT["swap_vals"][i]
    n = cv["t2"]["dims"][0]
    t1 = orc.Tensor(orc.DENSE, [], cv["t1"]["dims"], _els(cv["t1"]))
    t2 = orc.Tensor(orc.SWAP, [], [n] * 4, None, 0)
    t3, _, _ = orc.contract(t1, t2, [tuple(w) for w in cv["wires"]])
    assert t3.dims == cv["t3"]["dims"]
    assert _equal(t3.els, _els(cv["t3"]), 1e-5)


@pytest.mark.parametrize("i", range(5))
def test_invalid_swaps(i):
    cv = RT["invalid_swaps"][i]
    n = cv["t2"]["dims"][0]
    t1 = orc.Tensor(orc.DENSE, [], cv["t1"]["dims"], _els(cv["t1"]))
    t2 = orc.Tensor(orc.SWAP, [], [n] * 4, None, 0)
    with pytest.raises((ValueError, RuntimeError)):
        orc.contract(t1, t2, [tuple(w) for w in cv["wires"]])


@pytest.mark.parametrize("i", range(10))
def test_dense_identity(i):
    cv = RT["id_vals"][i]
    t1 = orc.Tensor(orc.DENSE, [], cv["t1"]["dims"], _els(cv["t1"]))
    t2 = orc.Tensor(orc.IDEN, [], cv["t2"]["dims"], None, 0)
    t3, _, _ = orc.contract(t1, t2, [tuple(w) for w in cv["wires"]])
    assert t3.dims == cv["t3"]["dims"]
    assert _equal(t3.els, _els(cv["t3"]), 1e-5)


# tests/c2-mpi.cpp:80-214: (group, leading dims moved to the distributed prefix of t1, of t2)
MPI_CASES = [("mpi2r_vals", 1, 0), ("mpi3r_vals", 1, 0), ("mpi4r_vals", 1, 1), ("mpi6r_vals", 1, 1),
             ("mpi8r_vals", 2, 1)]


@pytest.mark.parametrize("group,s1,s2", MPI_CASES)
@pytest.mark.parametrize("i", range(5))
def test_distributed_contraction(group, s1, s2, i):
    cv = RT[group][i]
    d1, d2 = cv["t1"]["dims"], cv["t2"]["dims"]
    # DenseTensor::make(env, {}, dims, els) followed by Tensor::rescatter(tp, s): the first
    # s local dims become distributed; global order is unchanged (dense.cpp:123-150).
    t1 = orc.Tensor(orc.DENSE, d1[:s1], d1[s1:], _els(cv["t1"]))
    t2 = orc.Tensor(orc.DENSE, d2[:s2], d2[s2:], _els(cv["t2"]))
    t3, _, _ = orc.contract(t1, t2, [tuple(w) for w in cv["wires"]])
    assert t3.dims == cv["t3"]["dims"]
    assert len(t3.dis) == s1 + s2
    assert _equal(t3.els, _els(cv["t3"]), 1e-5)


def _make_net(tnv):
    net = orc.Network()
    ids = [net.insert(orc.Tensor(orc.DENSE, [], t["dims"], _els(t))) for t in tnv["tensors"]]
    bids = [net.add_bond(ids[b["t1"]], ids[b["t2"]], [tuple(w) for w in b["wires"]]) for b in tnv["bonds"]]
    return net, bids


@pytest.mark.parametrize("i", range(5))
def test_network_two_tensors(i):
    tnv = TN["tn2_vals"][i]
    net, _ = _make_net(tnv)
    res = net.get(net.contract_all())
    assert res.dims == tnv["result"]["dims"]
    assert _equal(res.els, _els(tnv["result"]), 1e-5)


@pytest.mark.parametrize("i", range(5))
def test_network_circular_ordered(i):
    tnv = TN["tn4c_vals"][i]
    net, bids = _make_net(tnv)
    res = net.get(net.contract_all(bids))
    assert res.dims == tnv["result"]["dims"]
    assert _equal(res.els, _els(tnv["result"]), 1e-2)


@pytest.mark.parametrize("group", ["tn3_vals", "tn4_vals"])
@pytest.mark.parametrize("i", range(5))
def test_network_chains_ordered(group, i):
    # The reference's "3-tensors"/"4-tensors" sections iterate tn2_vals
    # (tests/c2-network.cpp:49,90), so these goldens were never exercised there. With the
    # bonds contracted in listed order, the result index order is the einsum order.
    tnv = TN[group][i]
    net, bids = _make_net(tnv)
    res = net.get(net.contract_all(bids))
    assert res.dims == tnv["result"]["dims"]
    assert _equal(res.els, _els(tnv["result"]), 1e-2)


class _OrcNet:
    def __init__(self):
        self.net = orc.Network()

    def make(self, kind, dis, loc, els, n_dis_in):
        return self.net.insert(orc.Tensor(kind, dis, loc, els, n_dis_in))

    def add_bond(self, a, b, wires):
        return self.net.add_bond(a, b, wires)


@pytest.mark.parametrize("nq,dq", [(2, 0), (3, 0), (4, 0), (5, 0), (5, 2), (6, 2), (7, 3)])
def test_qft_amplitude(nq, dq):
    # tests/c2-network.cpp:155-199 and tests/c2-mpi.cpp:241-303: amplitude 0 equals 1.
    w = _OrcNet()
    order = build_qft(w, nq, dq)
    res = w.net.get(w.net.contract_all(order))
    assert len(res.dims) == nq
    assert abs(res.els[0] - 1.0) < 1e-4
    # |+...+> maps to |0...0>: every other amplitude vanishes.
    assert np.max(np.abs(res.els[1:])) < 1e-12


def test_permute_matches_numpy_transpose():
    rng = np.random.default_rng(7)
    for rank in range(1, 6):
        dims = list(rng.integers(1, 4, size=rank))
        a = rng.standard_normal(dims) + 1j * rng.standard_normal(dims)
        ptup = list(rng.permutation(rank))
        out = orc.permute(a, ptup)
        # new axis ptup[i] is old axis i  =>  numpy axes: new axis j takes old axis inv[j]
        inv = np.argsort(ptup)
        assert np.array_equal(out, np.transpose(a, inv))


def test_swap_asymmetric_throws():
    with pytest.raises(RuntimeError):
        orc.swap(np.zeros((2, 3), dtype=np.complex128), 0, 1)


def test_diag_equals_expanded_symmetric():
    rng = np.random.default_rng(3)
    psi = rng.standard_normal(16) + 1j * rng.standard_normal(16)
    d = np.exp(1j * rng.uniform(0, 2 * np.pi, 4))
    state = orc.Tensor(orc.DENSE, [], [2, 2, 2, 2], psi)
    diag = orc.Tensor(orc.DIAG, [], [2, 2, 2, 2], d, 0)
    full = orc.Tensor(orc.SYMM, [], [2, 2, 2, 2], np.diag(d).reshape(-1), 0)
    a, r1a, r2a = orc.contract(state, diag, [(3, 0), (1, 1)])
    b, r1b, r2b = orc.contract(state, full, [(3, 0), (1, 1)])
    assert a.dims == b.dims and r1a == r1b and r2a == r2b
    assert np.array_equal(a.els, b.els)
