"""The oracle restatement against the reference's own code (oracle/_ref: the reference
checkout's src/core and src/tensor compiled with a single-process MPI subset), at world
size 1, on the CPU. Skipped where the reference checkout is absent (the library is built
from it).

* the reference itself reproduces its golden vectors (dense_vals, swap_vals, id_vals;
  tests/gen/random-tensors.hpp of the reference) through this build;
* random dense contractions (ranks 1-5, 1-3 wires at random positions, default and
  custom replacements), SymmTensor gates in place, SwapTensor and IdenTensor relabellings:
  the oracle gives the same result dims and replacements and bit-identical elements;
* Tensor::permute (the reference's derived-datatype Alltoallv path) and Tensor::swap on
  random tensors: bit-identical; a non-identity permute at world size 1 is pinned by no
  reference test, so this is its pin; asymmetric swaps throw in both.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from oracle import reference as ref

HERE = os.path.dirname(os.path.abspath(__file__))

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference checkout (oracle/_ref) not available")


def crandn(rng, n):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def _golden():
    with open(os.path.join(HERE, "golden", "random_tensors.json")) as f:
        return json.load(f)["groups"]


def _els(info):
    a = np.array(info["els"], dtype=np.float64)
    return (a[:, 0] + 1j * a[:, 1]).astype(np.complex128)


@pytest.mark.parametrize("group,kind2", [("dense_vals", ref.DENSE), ("swap_vals", ref.SWAP), ("id_vals", ref.IDEN)])
def test_reference_build_reproduces_its_goldens(group, kind2):
    cases = _golden()[group]
    assert cases
    for c in cases:
        t1, t2, t3 = c["t1"], c["t2"], c["t3"]
        d2 = [t2["dims"][0]] * 4 if kind2 == ref.SWAP else t2["dims"]
        e2 = _els(t2) if kind2 == ref.DENSE else None
        dims, out, _, _ = ref.contract((ref.DENSE, t1["dims"], 0, _els(t1)), (kind2, d2, 0, e2),
                                       [tuple(w) for w in c["wires"]])
        assert dims == t3["dims"]
        assert np.all(np.abs(out - _els(t3)) < 1e-5)  # utils::equal, the reference tests' 1e-5


def _random_case(rng):
    r1, r2 = int(rng.integers(1, 5)), int(rng.integers(1, 5))
    d1 = [int(x) for x in rng.integers(1, 5, size=r1)]
    d2 = [int(x) for x in rng.integers(1, 5, size=r2)]
    nw = int(rng.integers(1, min(r1, r2) + 1))
    i1 = [int(x) for x in rng.choice(r1, size=nw, replace=False)]
    i2 = [int(x) for x in rng.choice(r2, size=nw, replace=False)]
    for a, b in zip(i1, i2):
        d2[b] = d1[a]
    return d1, d2, list(zip(i1, i2))


@pytest.mark.parametrize("seed", range(40))
def test_oracle_matches_reference_dense(seed):
    rng = np.random.default_rng(7000 + seed)
    d1, d2, wires = _random_case(rng)
    a, b = crandn(rng, int(np.prod(d1))), crandn(rng, int(np.prod(d2)))
    dims, out, r1, r2 = ref.contract((ref.DENSE, d1, 0, a), (ref.DENSE, d2, 0, b), wires)
    o, q1, q2 = orc.contract(orc.Tensor(orc.DENSE, [], d1, a), orc.Tensor(orc.DENSE, [], d2, b), wires)
    assert o.dis + o.loc == dims and q1 == r1 and q2 == r2
    assert np.array_equal(o.els, out)


@pytest.mark.parametrize("seed", range(10))
def test_oracle_matches_reference_custom_replacements(seed):
    rng = np.random.default_rng(7100 + seed)
    d1, d2, wires = _random_case(rng)
    a, b = crandn(rng, int(np.prod(d1))), crandn(rng, int(np.prod(d2)))
    open1 = [i for i in range(len(d1)) if i not in [w[0] for w in wires]]
    open2 = [i for i in range(len(d2)) if i not in [w[1] for w in wires]]
    pos = [int(x) for x in rng.permutation(len(open1) + len(open2))]
    rp1, rp2 = [ref.X] * len(d1), [ref.X] * len(d2)
    for k, i in enumerate(open1):
        rp1[i] = pos[k]
    for k, i in enumerate(open2):
        rp2[i] = pos[len(open1) + k]
    dims, out, _, _ = ref.contract((ref.DENSE, d1, 0, a), (ref.DENSE, d2, 0, b), wires, repls=(rp1, rp2))
    o, _, _ = orc.contract(orc.Tensor(orc.DENSE, [], d1, a), orc.Tensor(orc.DENSE, [], d2, b), wires, repls=(rp1, rp2))
    assert o.dis + o.loc == dims
    assert np.array_equal(o.els, out)


@pytest.mark.parametrize("k,seed", [(1, 0), (1, 1), (2, 0), (2, 1), (3, 0)])
def test_oracle_matches_reference_symm_gate(k, seed):
    rng = np.random.default_rng(7200 + 10 * k + seed)
    n = 7
    psi = crandn(rng, 2 ** n)
    g = crandn(rng, 4 ** k)
    tg = [int(x) for x in rng.choice(n, size=k, replace=False)]
    wires = [(t, j) for j, t in enumerate(tg)]
    dims, out, r1, r2 = ref.contract((ref.DENSE, [2] * n, 0, psi), (ref.SYMM, [2] * (2 * k), 0, g), wires)
    o, q1, q2 = orc.contract(orc.Tensor(orc.DENSE, [], [2] * n, psi), orc.Tensor(orc.SYMM, [], [2] * (2 * k), g), wires)
    assert o.dis + o.loc == dims and q1 == r1 and q2 == r2
    assert np.array_equal(o.els, out)


@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_reference_swap_and_identity_tensors(seed):
    rng = np.random.default_rng(7300 + seed)
    n = 6
    psi = crandn(rng, 2 ** n)
    x, y = [int(v) for v in rng.choice(n, size=2, replace=False)]
    dims, out, r1, r2 = ref.contract((ref.DENSE, [2] * n, 0, psi), (ref.SWAP, [2] * 4, 0, None), [(x, 0), (y, 1)])
    o, q1, q2 = orc.contract(orc.Tensor(orc.DENSE, [], [2] * n, psi), orc.Tensor(orc.SWAP, [], [2] * 4), [(x, 0), (y, 1)])
    assert o.dis + o.loc == dims and q1 == r1 and q2 == r2
    assert np.array_equal(o.els, out)
    dims, out, r1, r2 = ref.contract((ref.DENSE, [2] * n, 0, psi), (ref.IDEN, [2, 2], 0, None), [(x, 0)])
    o, q1, q2 = orc.contract(orc.Tensor(orc.DENSE, [], [2] * n, psi), orc.Tensor(orc.IDEN, [], [2, 2], None, 0),
                             [(x, 0)])
    assert o.dis + o.loc == dims and q1 == r1 and q2 == r2
    assert np.array_equal(o.els, out)


@pytest.mark.parametrize("seed", range(30))
def test_oracle_matches_reference_permute_and_swap(seed):
    rng = np.random.default_rng(7400 + seed)
    r = int(rng.integers(2, 7))
    dims = [int(x) for x in rng.integers(1, 5, size=r)]
    a = crandn(rng, int(np.prod(dims)))
    ptup = [int(x) for x in rng.permutation(r)]
    nd, out = ref.permute(dims, a, ptup)
    mine = orc.permute(a.reshape(dims), ptup)
    assert list(mine.shape) == nd
    assert np.array_equal(mine.reshape(-1), out)
    i1, i2 = [int(x) for x in rng.choice(r, size=2, replace=False)]
    if dims[i1] == dims[i2]:
        nd, out = ref.swap(dims, a, i1, i2)
        assert np.array_equal(orc.swap(a.reshape(dims), i1, i2).reshape(-1), out)
    else:
        with pytest.raises(RuntimeError):
            ref.swap(dims, a, i1, i2)
        with pytest.raises(RuntimeError):
            orc.swap(a.reshape(dims), i1, i2)
