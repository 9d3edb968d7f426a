"""GPU parity of the C ABI against the oracle (and the reference's golden vectors).

Data movement (permute, swap, delta contractions) must be bit-exact; contractions
within 1e-12 relative L2 (the plain complex128 bar), goldens within the
reference's own 1e-5 (tests/c2-tensor.cpp:157)."""
import ctypes
import json
import math
import os
import random

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
RT = json.load(open(os.path.join(HERE, "golden", "random_tensors.json")))["groups"]
REL_TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _setup():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    orc.build()
    q.lib()


@pytest.fixture(params=[q.ARITH_F32X2, q.ARITH_FP64, q.ARITH_BF16X6], ids=["f32x2", "fp64", "bf16x6"])
def arith(request):
    old = q.get_arithmetic()
    q.set_arithmetic(request.param)
    yield request.param
    q.set_arithmetic(old)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128).reshape(-1)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def rel_l2(a, b):
    a, b = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
    scale = max(np.max(np.abs(b)) if b.size else 0.0, 1e-300)
    a, b = a / scale, b / scale
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def crandn(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _els(info):
    a = np.array(info["els"], dtype=np.float64)
    return (a[:, 0] + 1j * a[:, 1]).astype(np.complex128)


# ---- permute / swap -----------------------------------------------------------------

def _perm_cases():
    rng = random.Random(1)
    cases = []
    for _ in range(40):
        r = rng.randint(1, 6)
        dims = [rng.choice([1, 2, 3, 4, 5, 7, 16, 33, 64]) for _ in range(r)]
        while np.prod(dims) > 2 ** 20:
            dims[rng.randrange(r)] = 2
        p = list(range(r))
        rng.shuffle(p)
        cases.append((dims, p))
    for n in (10, 14, 20):  # qubit tensors
        for _ in range(4):
            p = list(range(n))
            rng.shuffle(p)
            cases.append(([2] * n, p))
        p = list(range(n))
        for k in range(3):  # exchange 3 top axes with 3 low axes
            p[k], p[n - 1 - 2 * k] = p[n - 1 - 2 * k], p[k]
        cases.append(([2] * n, p))
    cases.append(([2] * 20, [1, 0, 2] + list(range(3, 20))))  # run copy
    cases.append(([4096, 3], [1, 0]))                           # huge axis split for the tile
    # small innermost axes next to a large merged axis: the merged axis is split so the
    # tile takes only its inner part (top 3 <-> bottom 3 axes, the Tensor::swap of the
    # outermost and innermost axes, non-power-of-two splits, several tiles per step)
    n = 20
    cases.append(([2] * n, [n - 3, n - 2, n - 1] + list(range(3, n - 3)) + [0, 1, 2]))
    cases.append(([2] * n, [n - 1] + list(range(1, n - 1)) + [0]))
    cases.append(([3, 1000, 7], [2, 1, 0]))
    cases.append(([5, 6000], [1, 0]))
    cases.append(([7, 1009], [1, 0]))                           # prime axis: whole-axis tile
    cases.append(([3, 4099], [1, 0]))                           # gather fallback (no tile fits)
    return cases


@pytest.mark.parametrize("dims,ptup", _perm_cases())
def test_permute_bit_exact(dims, ptup):
    rng = np.random.default_rng(len(dims) * 7 + sum(ptup))
    a = crandn(rng, dims)
    ref = orc.permute(a, ptup)
    out = host(q.permute(dev(a), dims, ptup))
    assert np.array_equal(out.view(np.uint64), ref.reshape(-1).view(np.uint64))


def test_swap_bit_exact_and_asymmetric():
    rng = np.random.default_rng(2)
    dims = [3, 2, 3, 4]
    a = crandn(rng, dims)
    out = host(q.swap(dev(a), dims, 0, 2))
    assert np.array_equal(out, orc.swap(a, 0, 2).reshape(-1))
    with pytest.raises(q.QtnhError):
        q.swap(dev(a), dims, 0, 1)


# ---- contractions on the reference's golden vectors ----------------------------------

def _run_contract(t1, t2, wires):
    o1 = orc.Tensor({q.DENSE: orc.DENSE, q.SYMM: orc.SYMM, q.SWAP: orc.SWAP, q.IDEN: orc.IDEN, q.DIAG: orc.DIAG}[t1[0]],
                    t1[1], t1[2], t1[3], t1[4])
    o2 = orc.Tensor({q.DENSE: orc.DENSE, q.SYMM: orc.SYMM, q.SWAP: orc.SWAP, q.IDEN: orc.IDEN, q.DIAG: orc.DIAG}[t2[0]],
                    t2[1], t2[2], t2[3], t2[4])
    ref, r1, r2 = orc.contract(o1, o2, wires)
    g1 = q.Tensor(t1[0], t1[1], t1[2], dev(t1[3]) if t1[3] is not None else None, t1[4])
    g2 = q.Tensor(t2[0], t2[1], t2[2], dev(t2[3]) if t2[3] is not None else None, t2[4])
    res, q1, q2, st = q.contract(g1, g2, wires)
    assert res.dis == ref.dis and res.loc == ref.loc
    assert q1 == r1 and q2 == r2 and st == ref.bc[0]
    return host(res.data), ref.els


@pytest.mark.parametrize("i", range(20))
def test_golden_dense(i):
    cv = RT["dense_vals"][i]
    out, ref = _run_contract((q.DENSE, [], cv["t1"]["dims"], _els(cv["t1"]), 0),
                             (q.DENSE, [], cv["t2"]["dims"], _els(cv["t2"]), 0), [tuple(w) for w in cv["wires"]])
    assert np.all(np.abs(out - _els(cv["t3"])) < 1e-5)
    assert rel_l2(out, ref) < REL_TOL


@pytest.mark.parametrize("i", range(10))
def test_golden_swap_bit_exact(i):
    cv = RT["swap_vals"][i]
    n = cv["t2"]["dims"][0]
    out, ref = _run_contract((q.DENSE, [], cv["t1"]["dims"], _els(cv["t1"]), 0), (q.SWAP, [], [n] * 4, None, 0),
                             [tuple(w) for w in cv["wires"]])
    assert np.all(np.abs(out - _els(cv["t3"])) < 1e-5)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("i", range(10))
def test_golden_identity_bit_exact(i):
    cv = RT["id_vals"][i]
    out, ref = _run_contract((q.DENSE, [], cv["t1"]["dims"], _els(cv["t1"]), 0),
                             (q.IDEN, [], cv["t2"]["dims"], None, 0), [tuple(w) for w in cv["wires"]])
    assert np.all(np.abs(out - _els(cv["t3"])) < 1e-5)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("i", range(5))
def test_golden_invalid_swaps(i):
    cv = RT["invalid_swaps"][i]
    n = cv["t2"]["dims"][0]
    with pytest.raises(q.QtnhError):
        q.contract(q.Tensor(q.DENSE, [], cv["t1"]["dims"], dev(_els(cv["t1"]))), q.Tensor(q.SWAP, [], [n] * 4),
                   [tuple(w) for w in cv["wires"]])


@pytest.mark.parametrize("group,s1,s2", [("mpi2r_vals", 1, 0), ("mpi3r_vals", 1, 0), ("mpi4r_vals", 1, 1),
                                         ("mpi6r_vals", 1, 1), ("mpi8r_vals", 2, 1)])
def test_golden_distributed(group, s1, s2):
    for cv in RT[group]:
        d1, d2 = cv["t1"]["dims"], cv["t2"]["dims"]
        out, ref = _run_contract((q.DENSE, d1[:s1], d1[s1:], _els(cv["t1"]), 0),
                                 (q.DENSE, d2[:s2], d2[s2:], _els(cv["t2"]), 0), [tuple(w) for w in cv["wires"]])
        assert np.all(np.abs(out - _els(cv["t3"])) < 1e-5)
        assert rel_l2(out, ref) < REL_TOL


# ---- seeded random contractions against the oracle -----------------------------------

def test_random_dense_contractions():
    rng = random.Random(3)
    nrng = np.random.default_rng(3)
    for _ in range(60):
        dis1 = [rng.choice([2, 3, 4]) for _ in range(rng.randint(0, 2))]
        loc1 = [rng.choice([2, 3, 4, 5]) for _ in range(rng.randint(0, 4))]
        dis2 = [rng.choice([2, 3, 4]) for _ in range(rng.randint(0, 2))]
        loc2 = [rng.choice([2, 3, 4, 5]) for _ in range(rng.randint(0, 4))]
        wires = []
        for i in range(len(dis1)):  # some distributed wires (the reference's "reduced" indices)
            cands = [j for j in range(len(dis2)) if dis2[j] == dis1[i] and j not in [w[1] for w in wires]]
            if cands and rng.random() < 0.5:
                wires.append((i, rng.choice(cands)))
        for i in range(len(loc1)):
            cands = [j for j in range(len(loc2)) if loc2[j] == loc1[i] and len(dis2) + j not in [w[1] for w in wires]]
            if cands and rng.random() < 0.6:
                wires.append((len(dis1) + i, len(dis2) + rng.choice(cands)))
        a = crandn(nrng, dis1 + loc1)
        b = crandn(nrng, dis2 + loc2)
        out, ref = _run_contract((q.DENSE, dis1, loc1, a, 0), (q.DENSE, dis2, loc2, b, 0), wires)
        assert rel_l2(out, ref) < REL_TOL


def test_large_gemm_contraction():
    nrng = np.random.default_rng(9)
    a = crandn(nrng, [16, 32, 64, 4])
    b = crandn(nrng, [64, 8, 16, 3])
    out, ref = _run_contract((q.DENSE, [], [16, 32, 64, 4], a, 0), (q.DENSE, [], [64, 8, 16, 3], b, 0), [(2, 0), (0, 2)])
    assert rel_l2(out, ref) < REL_TOL


def haar(rng, d):
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / math.sqrt(2)
    qm, r = np.linalg.qr(z)
    return qm * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_symmetric_gate_in_place(k, arith):
    nrng = np.random.default_rng(20 + k)
    n = 12
    psi = crandn(nrng, [2] * n)
    u = haar(nrng, 2 ** k)
    els = u.T.reshape(-1)  # SymmTensor layout [in..., out...]: els[in, out] = U[out, in]
    targets = list(nrng.choice(n, size=k, replace=False))
    wires = [(int(t), j) for j, t in enumerate(targets)]
    out, ref = _run_contract((q.DENSE, [], [2] * n, psi, 0), (q.SYMM, [], [2] * (2 * k), els, 0), wires)
    assert rel_l2(out, ref) < REL_TOL


def test_gate_kernel_direct_matches_oracle(arith):
    nrng = np.random.default_rng(4)
    n = 16
    psi = crandn(nrng, [2] * n)
    u = haar(nrng, 4)
    els = u.T.reshape(-1)
    st = dev(psi)
    q.apply_gate(st, [2] * n, [3, 15], dev(els))
    ref, _, _ = orc.contract(orc.Tensor(orc.DENSE, [], [2] * n, psi), orc.Tensor(orc.SYMM, [], [2] * 4, els),
                             [(3, 0), (15, 1)])
    assert rel_l2(host(st), ref.els) < REL_TOL


def test_diagonal_in_place_and_layer(arith):
    nrng = np.random.default_rng(6)
    n = 14
    psi = crandn(nrng, [2] * n)
    d = np.exp(1j * nrng.uniform(0, 2 * np.pi, 4))
    out, ref = _run_contract((q.DENSE, [], [2] * n, psi, 0), (q.DIAG, [], [2] * 4, d, 0), [(5, 0), (2, 1)])
    assert rel_l2(out, ref) < REL_TOL
    # a whole layer of single-qubit phases equals n successive rank-2 diagonal contractions
    phases = nrng.uniform(0, 2 * np.pi, n)
    factors = np.stack([np.ones(n), np.exp(1j * phases)], axis=1).reshape(-1)
    st = dev(psi)
    q.apply_diag_layer(st, [2] * n, list(range(n)), dev(factors))
    cur = orc.Tensor(orc.DENSE, [], [2] * n, psi)
    for j in range(n):
        cur, _, _ = orc.contract(cur, orc.Tensor(orc.DIAG, [], [2, 2], factors[2 * j:2 * j + 2]), [(j, 0)])
    assert rel_l2(host(st), cur.els) < REL_TOL


@pytest.mark.parametrize("tdims,p", [([2, 2], 0), ([2, 2], 1), ([3], 0), ([2, 3, 2], 1)])
def test_symm_diag_product(tdims, p):
    # out[in, o] = gate[in, o] * diag[o_p]: the gate then the diagonal on its p-th target,
    # as one gate (what the C++ queue folds); also in place
    rng = np.random.default_rng(60 + p + len(tdims))
    D = int(np.prod(tdims))
    g = crandn(rng, [D * D]).reshape(-1)
    d = crandn(rng, [tdims[p]]).reshape(-1)
    odig = (np.arange(D) // int(np.prod(tdims[p + 1:]))) % tdims[p]
    want = (g.reshape(D, D) * d[odig][None, :]).reshape(-1)
    gd, dd, od = dev(g), dev(d), dev(np.zeros_like(g))
    td = (ctypes.c_uint64 * len(tdims))(*tdims)
    for out in (od, gd):
        q.check(q.lib().qtnh_symm_diag_product(q._ptr(gd), len(tdims), td, p, q._ptr(dd), q._ptr(out), q._stream()))
        assert np.max(np.abs(host(out) - want)) <= 1e-15 * np.max(np.abs(want))  # one complex product each
    with pytest.raises(q.InvalidArgument):
        q.check(q.lib().qtnh_symm_diag_product(q._ptr(gd), len(tdims), td, len(tdims), q._ptr(dd), q._ptr(od),
                                                q._stream()))


def test_diagonals_default_mode_out_of_range(bf16x6):
    # the default mode's diagonal kernels mix FP64 elements, float-float elements and the
    # FP64 fallback of a warp whose float-float elements are out of range: tiny, huge,
    # zero and subnormal regions, each compared on its own scale
    nrng = np.random.default_rng(17)
    n = 13
    psi = crandn(nrng, [2] * n).reshape(-1)
    psi[:1024] *= 1e-200
    psi[1024:2048] *= 1e200
    psi[2048:2304] = 0.0
    psi[2304] = 5e-324
    regions = (slice(0, 1024), slice(1024, 2048), slice(2048, 1 << n))
    d = np.exp(1j * nrng.uniform(0, 2 * np.pi, 4)) * np.array([1.0, 1e-40, 1.0, 3.0])
    out, ref = _run_contract((q.DENSE, [], [2] * n, psi, 0), (q.DIAG, [], [2] * 4, d, 0), [(n - 1, 0), (3, 1)])
    for sl in regions:
        assert rel_l2(np.asarray(out).reshape(-1)[sl], np.asarray(ref).reshape(-1)[sl]) < REL_TOL
    factors = np.stack([np.ones(n), np.exp(1j * nrng.uniform(0, 2 * np.pi, n))], axis=1).reshape(-1)
    st = dev(psi)
    q.apply_diag_layer(st, [2] * n, list(range(n)), dev(factors))
    cur = orc.Tensor(orc.DENSE, [], [2] * n, psi)
    for j in range(n):
        cur, _, _ = orc.contract(cur, orc.Tensor(orc.DIAG, [], [2, 2], factors[2 * j:2 * j + 2]), [(j, 0)])
    got = host(st)
    for sl in regions:
        assert rel_l2(got[sl], cur.els[sl]) < REL_TOL


def test_norm2():
    # against the correctly rounded sum of the squares; half of the elements are squared
    # in float-float, so also with amplitudes outside that range (FP64 there), zeros and
    # a length that is not a multiple of the kernel's step
    nrng = np.random.default_rng(8)
    for n, scale_blocks in ((1 << 18, False), ((1 << 18) + 77, True)):
        a = crandn(nrng, [n])
        if scale_blocks:
            a[:4096] *= 1e-40
            a[4096:8192] *= 1e40
            a[8192:9000] = 0.0
        sq = np.concatenate([a.real ** 2, a.imag ** 2])
        ref = math.fsum(sq.tolist())
        assert abs(q.norm2(dev(a)) - ref) < 1e-13 * ref


def test_distributed_identity_moves_index():
    # IdenTensor with one distributed and one local index ("DIST" in the reference's QFT):
    # contracting a state index with its local index moves it into the distributed prefix.
    nrng = np.random.default_rng(10)
    psi = crandn(nrng, [2, 2, 2])
    out, ref = _run_contract((q.DENSE, [], [2, 2, 2], psi, 0), (q.IDEN, [2], [2], None, 0), [(1, 1)])
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("targets", [[2, 9], [2, 9, 4], [2, 9, 4, 6]], ids=["D4", "D8", "D16"])
def test_f32x2_falls_back_to_fp64_out_of_range(targets):
    # tiny and huge magnitudes, zeros and subnormals in one state: groups outside the
    # split range take the FP64 path, the rest the float-float path; all within tolerance
    # (D = 4: per warp in the register-blocked kernel; D = 8, 16: per batch of groups in
    # the shared-memory kernel)
    old = q.get_arithmetic()
    q.set_arithmetic(q.ARITH_F32X2)
    try:
        nrng = np.random.default_rng(12)
        n = 10
        psi = crandn(nrng, [2] * n).reshape(-1)
        psi[:64] *= 1e-200
        psi[64:128] *= 1e200
        psi[128:160] = 0.0
        psi[160] = 5e-324
        k = len(targets)
        u = haar(nrng, 2 ** k)
        els = u.T.reshape(-1)
        st = dev(psi)
        q.apply_gate(st, [2] * n, targets, dev(els))
        ref, _, _ = orc.contract(orc.Tensor(orc.DENSE, [], [2] * n, psi), orc.Tensor(orc.SYMM, [], [2] * (2 * k), els),
                                 [(t, j) for j, t in enumerate(targets)])
        out = host(st)
        for sl in (slice(0, 64), slice(64, 128), slice(128, 1024)):
            assert rel_l2(out[sl], ref.els[sl]) < REL_TOL
    finally:
        q.set_arithmetic(old)


def test_circuit_inverse_returns_state(arith):
    # size-independent property: circuit followed by its inverse is the identity
    from qtnh_gb300 import workload as wl
    from qtnh_gb300.circuit import DeviceCircuit
    n = 20
    c = wl.random_circuit(n, 16, seed=5)
    psi = wl.random_state(n, seed=6)
    st = dev(psi)
    scratch = torch.empty_like(st)
    out = DeviceCircuit(c).run(st, scratch)
    other = scratch if out is st else st
    back = DeviceCircuit(wl.inverse_circuit(c)).run(out, other)
    assert rel_l2(host(back), psi) < 1e-12


def test_circuit_matches_oracle(arith):
    from qtnh_gb300 import workload as wl
    from qtnh_gb300.circuit import DeviceCircuit
    n = 14
    c = wl.random_circuit(n, 16, seed=8)
    psi = wl.random_state(n, seed=9)
    st = dev(psi)
    out = DeviceCircuit(c).run(st, torch.empty_like(st))
    ref = orc.run_circuit(psi, c)
    assert rel_l2(host(out), ref) < 1e-12


@pytest.mark.parametrize("k", [1, 2])
def test_symmetric_gate_qutrits(k, arith):
    # non-power-of-two dimensions take the general index decode and the D=3 / D=9 kernels
    nrng = np.random.default_rng(30 + k)
    dims = [3, 2, 3, 3, 2, 3]
    psi = crandn(nrng, dims)
    u = haar(nrng, 3 ** k)
    els = u.T.reshape(-1)
    targets = [0, 3] if k == 2 else [5]
    wires = [(t, j) for j, t in enumerate(targets)]
    out, ref = _run_contract((q.DENSE, [], dims, psi, 0), (q.SYMM, [], [3] * (2 * k), els, 0), wires)
    assert rel_l2(out, ref) < REL_TOL


# ---- tensor-core (bf16 slice) gate pairs --------------------------------------------

def _oracle_layer(psi, n, gates):
    cur = orc.Tensor(orc.DENSE, [], [2] * n, psi)
    for targets, els in gates:
        k = len(targets)
        cur, _, _ = orc.contract(cur, orc.Tensor(orc.SYMM, [], [2] * (2 * k), els), [(t, j) for j, t in enumerate(targets)])
    return cur.els


@pytest.fixture
def bf16x6():
    old = q.get_arithmetic()
    q.set_arithmetic(q.ARITH_BF16X6)
    q.take_device_errors()
    yield
    q.set_arithmetic(old)
    assert q.take_device_errors() == 0  # no bounded wait of the tcgen05 kernel expired


@pytest.mark.parametrize("seed", range(6))
def test_gate_pairs_tensor_core_match_oracle(seed, bf16x6):
    # disjoint two-qubit pairs, targets anywhere (low bits included), fused on the tensor cores
    nrng = np.random.default_rng(100 + seed)
    n = 12
    psi = crandn(nrng, [2] * n)
    perm = [int(x) for x in nrng.permutation(n)]
    if seed == 0:
        perm = [0, 1, 2, 3, 11, 10, 9, 8] + perm[8:]  # bits 0..3 and the top bits
    gates = [(perm[2 * j:2 * j + 2], haar(nrng, 4).T.reshape(-1)) for j in range(n // 2)]
    st = dev(psi)
    before = q.launches()
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    assert q.launches() - before == 3  # six gates, three fused launches
    assert rel_l2(host(st), _oracle_layer(psi, n, gates)) < REL_TOL


@pytest.mark.parametrize("n", [8, 10, 18, 22])
def test_gate_pairs_tensor_core_sizes(n, bf16x6):
    # n < 11: the mma.sync kernel (fewer than one 128-group tile); n = 18: the tcgen05
    # kernel with one tile per CTA; n = 22: 2048 tiles, 13-14 per CTA, so both teams and
    # both phases of every barrier are used several times
    nrng = np.random.default_rng(200 + n)
    psi = crandn(nrng, [2] * n)
    perm = [int(x) for x in nrng.permutation(n)]
    gates = [(perm[2 * j:2 * j + 2], haar(nrng, 4).T.reshape(-1)) for j in range(4)]
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    assert rel_l2(host(st), _oracle_layer(psi, n, gates)) < REL_TOL


def test_gate_pairs_tensor_core_fall_back_many_tiles(bf16x6):
    # FP64 groups scattered through a state of many tiles per CTA: every 37th block of
    # 4096 amplitudes is scaled to 1e-250 (the targets are bits 2, 5, 9, 11, so each group
    # lies inside one block); each region is compared on its own scale
    nrng = np.random.default_rng(15)
    n = 21
    psi = crandn(nrng, [2] * n).reshape(-1)
    blocks = psi.reshape(-1, 4096)
    tiny = np.zeros(blocks.shape[0], dtype=bool)
    tiny[::37] = True
    blocks[tiny] *= 1e-250
    gates = [([n - 1 - 2, n - 1 - 9], haar(nrng, 4).T.reshape(-1)),
             ([n - 1 - 5, n - 1 - 11], haar(nrng, 4).T.reshape(-1))]
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    out, ref = host(st).reshape(-1, 4096), _oracle_layer(psi, n, gates).reshape(-1, 4096)
    assert rel_l2(out[tiny], ref[tiny]) < REL_TOL
    assert rel_l2(out[~tiny], ref[~tiny]) < REL_TOL


def test_gate_layer_tensor_core_mixed(bf16x6):
    # odd gate counts, one-qubit gates and overlapping pairs are applied unfused, in order
    nrng = np.random.default_rng(7)
    n = 10
    psi = crandn(nrng, [2] * n)
    gates = [([0, 5], haar(nrng, 4)), ([5, 1], haar(nrng, 4)), ([2, 3], haar(nrng, 4)), ([7], haar(nrng, 2)),
             ([8, 9], haar(nrng, 4)), ([4, 6], haar(nrng, 4)), ([9, 2], haar(nrng, 4))]
    gates = [(t, u.T.reshape(-1)) for t, u in gates]
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    assert rel_l2(host(st), _oracle_layer(psi, n, gates)) < REL_TOL


def test_gate_pairs_tensor_core_fall_back_out_of_range(bf16x6):
    # groups with tiny, huge, zero or subnormal amplitudes take FP64 (per warp of 8
    # groups); each region is compared on its own scale
    nrng = np.random.default_rng(13)
    n = 12
    psi = crandn(nrng, [2] * n).reshape(-1)
    psi[:1024] *= 1e-250        # the targets (bits 0, 1, 3, 7) keep every group inside one region
    psi[1024:2048] *= 1e250
    psi[2048:2560] = 0.0
    psi[2560] = 5e-324
    psi[3000] *= 1e-70          # small but in range inside an ordinary group
    gates = [([10, 11], haar(nrng, 4).T.reshape(-1)), ([4, 8], haar(nrng, 4).T.reshape(-1))]
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    out, ref = host(st), _oracle_layer(psi, n, gates)
    for sl in (slice(0, 1024), slice(1024, 2048), slice(2048, 4096)):
        assert rel_l2(out[sl], ref[sl]) < REL_TOL


@pytest.mark.parametrize("dims,targets,scale", [
    ([2] * 14, [0, 1], 1.0),              # targets on the two top axes: identity on axes 2, 3
    ([2] * 14, [13, 6], 1.0),             # innermost target: identity on axes 0, 1
    ([2] * 8, [5, 2], 1.0),               # 16 groups: the mma.sync kernel
    ([4, 2, 8, 2, 2, 2, 2, 2, 2, 2], [3, 9], 1.0),  # identity skips the size-4 and size-8 axes
    ([2] * 12, [4, 7], 1e250),            # entries out of the digit range: FP64 groups
    ([3, 2, 2, 2, 2, 2, 2, 2, 2], [1, 5], 1.0),     # not a power of two: float-float kernel
    ([2] * 13, [12, 3, 7], 1.0),          # three-qubit gate (x) I2
    ([2] * 8, [0, 7, 2], 1.0),            # three-qubit gate, mma.sync kernel
    ([2] * 13, [5, 0, 12, 9], 1.0),       # four-qubit gate as the 16x16 operator itself
    ([2, 4, 2, 2, 8, 2, 2, 2], [0, 2, 3, 7], 1.0),  # four-qubit gate, mixed power-of-two dims
    ([2] * 11, [1, 6, 2, 10], 1e-250),    # four-qubit gate out of the digit range: FP64 groups
], ids=["top", "inner", "small", "mixed-radix", "huge-gate", "qutrit-axis", "3q", "3q-small", "4q",
        "4q-mixed-radix", "4q-tiny-gate"])
def test_lone_gate_on_tensor_cores(dims, targets, scale, bf16x6):
    # a single gate on 2, 3 or 4 qubits runs on the tensor cores as one 16x16 operator
    # (gate (x) I4, gate (x) I2, or the gate itself)
    k = len(targets)
    nrng = np.random.default_rng(len(dims) * 7 + targets[0] + 100 * k)
    psi = crandn(nrng, dims)
    els = crandn(nrng, [4 ** k]) * scale
    st = dev(psi)
    before = q.launches()
    q.apply_gate(st, dims, targets, dev(els))
    if 3 not in dims:
        assert q.launches() - before == 1
    ref, _, _ = orc.contract(orc.Tensor(orc.DENSE, [], dims, psi), orc.Tensor(orc.SYMM, [], [2] * (2 * k), els),
                             [(t, j) for j, t in enumerate(targets)])
    assert rel_l2(host(st), ref.els) < REL_TOL


def test_gate_pairs_tensor_core_general_gate_and_fallback(bf16x6):
    # non-unitary gates: rows of very different scale; a gate with huge entries runs FP64
    nrng = np.random.default_rng(14)
    n = 11
    psi = crandn(nrng, [2] * n)
    ga = crandn(nrng, [16]) * np.array([1e-3] * 4 + [1.0] * 4 + [1e5] * 4 + [2.0] * 4)
    gb = crandn(nrng, [16])
    gates = [([1, 9], ga), ([4, 6], gb)]
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    assert rel_l2(host(st), _oracle_layer(psi, n, gates)) < REL_TOL
    gates = [([1, 9], ga * 1e250), ([4, 6], gb)]
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    assert rel_l2(host(st), _oracle_layer(psi, n, gates)) < REL_TOL


def _disjoint_pairs(nrng, n, npairs):
    """2 * npairs two-qubit gates; each consecutive pair of gates on four distinct qubits."""
    gates = []
    for _ in range(npairs):
        q4 = [int(x) for x in nrng.choice(n, size=4, replace=False)]
        gates.append((q4[:2], haar(nrng, 4).T.reshape(-1)))
        gates.append((q4[2:], haar(nrng, 4).T.reshape(-1)))
    return gates


@pytest.mark.parametrize("n,npairs", [(16, 2), (16, 3), (17, 7), (22, 4)])
def test_gate_layer_fixed_point_chain_matches_oracle(n, npairs, bf16x6):
    # a run of fused pairs: the first pass in doubles, the next ones carry the state as
    # 64-bit fixed point at one scale, the last writes doubles
    nrng = np.random.default_rng(900 + 10 * n + npairs)
    psi = crandn(nrng, [2] * n).reshape(-1)
    psi /= np.linalg.norm(psi)
    gates = _disjoint_pairs(nrng, n, npairs)
    st = dev(psi)
    before = q.launches()
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    assert q.launches() - before == npairs
    out, ref = host(st), _oracle_layer(psi, n, gates)
    assert rel_l2(out, ref) < REL_TOL
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < REL_TOL


def test_gate_layer_chain_keeps_regions_of_very_different_scale(bf16x6):
    # a region 2^-40 below the rest: the chain does not start (every nonzero half group
    # must lie within 2^6 of the largest magnitude), so each region keeps its own accuracy
    nrng = np.random.default_rng(31)
    n = 14
    psi = crandn(nrng, [2] * n).reshape(-1)
    psi[:4096] *= 2.0 ** -40  # the targets (the four lowest bits) keep groups inside a region
    gates = [([n - 1, n - 2], haar(nrng, 4).T.reshape(-1)), ([n - 3, n - 4], haar(nrng, 4).T.reshape(-1)),
             ([n - 1, n - 3], haar(nrng, 4).T.reshape(-1)), ([n - 2, n - 4], haar(nrng, 4).T.reshape(-1)),
             ([n - 4, n - 1], haar(nrng, 4).T.reshape(-1)), ([n - 3, n - 2], haar(nrng, 4).T.reshape(-1))]
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    out, ref = host(st), _oracle_layer(psi, n, gates)
    assert rel_l2(out[:4096], ref[:4096]) < REL_TOL
    assert rel_l2(out[4096:], ref[4096:]) < REL_TOL


@pytest.mark.parametrize("rows", [[8.0, 8.0, 8.0, 8.0], [1.0, 2.0 ** -9, 2.0 ** 4, 0.75]], ids=["scaled", "rows_apart"])
def test_gate_layer_chain_non_unitary_gates(rows, bf16x6):
    # non-unitary gates: scaled by 8 (the rows of the fused operator stay within 2 bits of
    # each other: the chain passes cut every row's digits at one scale, no output shift), or
    # with rows 2^-9 .. 2^4 (each row has its own scale and its outputs are shifted to the
    # common one)
    nrng = np.random.default_rng(40 + int(rows[1] < 1))
    n = 16
    psi = crandn(nrng, [2] * n).reshape(-1)
    psi /= np.linalg.norm(psi)
    rows = np.array(rows)
    gates = [(t, (rows[:, None] * g.reshape(4, 4).T).T.reshape(-1)) for t, g in _disjoint_pairs(nrng, n, 4)]
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    out, ref = host(st), _oracle_layer(psi, n, gates)
    assert rel_l2(out, ref) < REL_TOL
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < REL_TOL
    assert q.take_device_errors() == 0


def test_gate_layer_chain_zero_state_and_nonfinite_gate(bf16x6):
    nrng = np.random.default_rng(32)
    n = 13
    gates = _disjoint_pairs(nrng, n, 3)
    # a zero state stays exactly zero through the chain
    st = dev(np.zeros(2 ** n, dtype=np.complex128))
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in gates])
    assert np.all(host(st) == 0)
    # a gate of the second pair with entries beyond the digit range (1e70 ~ 2^232): that
    # pass runs every group in FP64 from the fixed-point input and writes doubles, the next
    # ones (the state now ~1e70) stay in FP64
    psi = crandn(nrng, [2] * n).reshape(-1)
    big = [(t, g.copy()) for t, g in gates]
    big[2] = (big[2][0], big[2][1] * 1e70)
    st = dev(psi)
    q.apply_gate_layer(st, [2] * n, [(t, dev(g)) for t, g in big])
    assert rel_l2(host(st), _oracle_layer(psi, n, big)) < REL_TOL


# ---- runs of gates separated by permutations (qtnh_apply_gate_runs) -----------------


def _oracle_runs(psi, dims, runs):
    """runs: list of (gates, ptup); the oracle's contractions, then Tensor::permute."""
    cur = np.asarray(psi, dtype=np.complex128).reshape(-1)
    dims = list(dims)
    for gates, pt in runs:
        t = orc.Tensor(orc.DENSE, [], dims, cur)
        for targets, els in gates:
            tdims = [dims[x] for x in targets]
            t, _, _ = orc.contract(t, orc.Tensor(orc.SYMM, [], tdims * 2, els), [(x, j) for j, x in enumerate(targets)])
        cur = t.els
        if pt is not None:
            cur = orc.permute(cur.reshape(dims), pt).reshape(-1)
            nd = [0] * len(dims)
            for i, p in enumerate(pt):
                nd[p] = dims[i]
            dims = nd
    return cur


@pytest.mark.parametrize("counts", [[2, 4, 4], [6, 4], [3, 4], [4, 0, 6]], ids=["first", "fixed", "lone", "empty"])
def test_gate_runs_chain_across_permutations(counts, bf16x6):
    # the fixed-point chain continues across the permutations: after the first pass (a
    # permutation of doubles), after a later pass (of 64-bit fixed point), around a lone
    # gate that ends a run, and across an empty run (two permutations in a row)
    nrng = np.random.default_rng(50 + len(counts) + counts[0])
    n = 16
    psi = crandn(nrng, [2] * n).reshape(-1)
    psi /= np.linalg.norm(psi)
    runs = []
    for j, c in enumerate(counts):
        gates = _disjoint_pairs(nrng, n, (c + 1) // 2)[:c]
        pt = [int(x) for x in nrng.permutation(n)] if j + 1 < len(counts) else None
        runs.append((gates, pt))
    st, sc = dev(psi), dev(np.zeros_like(psi))
    res = q.apply_gate_runs(st, sc, [2] * n, [([(t, dev(g)) for t, g in gl], pt) for gl, pt in runs])
    assert res is (sc if (len(counts) - 1) % 2 else st)
    out, ref = host(res), _oracle_runs(psi, [2] * n, runs)
    assert rel_l2(out, ref) < REL_TOL
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < REL_TOL
    # the same sequence as separate calls (each layer its own chain) agrees to the same level
    st2, sc2 = dev(psi), dev(np.zeros_like(psi))
    cur, oth = st2, sc2
    for gl, pt in runs:
        if gl:
            q.apply_gate_layer(cur, [2] * n, [(t, dev(g)) for t, g in gl])
        if pt is not None:
            q.permute(cur, [2] * n, pt, out=oth)
            cur, oth = oth, cur
    assert rel_l2(out, host(cur)) < REL_TOL


def test_gate_runs_mixed_dims(arith):
    # non-power-of-two dims (general gate kernels, permutations change the dims)
    nrng = np.random.default_rng(60)
    dims = [3, 2, 4, 2, 3, 2]
    psi = crandn(nrng, dims).reshape(-1)
    pt0 = [2, 0, 5, 1, 3, 4]
    d1 = [0] * 6
    for i, p in enumerate(pt0):
        d1[p] = dims[i]
    runs = [([([0, 1], haar(nrng, 6).T.reshape(-1)), ([2], haar(nrng, 4).T.reshape(-1))], pt0),
            ([([d1.index(3), d1.index(4)], haar(nrng, 12).T.reshape(-1))], None)]
    st, sc = dev(psi), dev(np.zeros_like(psi))
    res = q.apply_gate_runs(st, sc, dims, [([(t, dev(g)) for t, g in gl], pt) for gl, pt in runs])
    assert res is sc
    assert rel_l2(host(res), _oracle_runs(psi, dims, runs)) < REL_TOL


def test_gate_runs_checks_before_launch(bf16x6):
    nrng = np.random.default_rng(61)
    n = 12
    psi = crandn(nrng, [2] * n).reshape(-1)
    gates = [(t, dev(g)) for t, g in _disjoint_pairs(nrng, n, 2)]
    st, sc = dev(psi), dev(np.zeros_like(psi))
    bad_perm = list(range(n))
    bad_perm[3] = 4  # not a permutation
    with pytest.raises(q.InvalidArgument):
        q.apply_gate_runs(st, sc, [2] * n, [(gates, bad_perm), (gates, None)])
    with pytest.raises(q.OutOfRange):
        q.apply_gate_runs(st, sc, [2] * n, [(gates, list(range(n))), ([([0, n], gates[0][1])], None)])
    with pytest.raises(q.InvalidArgument):
        q.apply_gate_runs(st, st, [2] * n, [(gates, list(range(n))), (gates, None)])
    # nothing was launched: the state is unchanged
    assert np.array_equal(host(st), psi)


@pytest.mark.parametrize("dims,targets", [([3, 2, 3, 2, 2], [0, 1]), ([2, 3, 4, 2], [3, 1, 2]), ([2] * 9, [1, 3, 4, 6, 8]),
                                          ([5, 3, 2], [0])],
                         ids=["D6", "D24", "D32", "D5"])
def test_symmetric_gate_general_sizes(dims, targets, arith):
    # gate sizes outside the register-blocked kernels (D = 6, 24, 32, 5) take the general kernel
    nrng = np.random.default_rng(70 + len(targets))
    psi = crandn(nrng, dims).reshape(-1)
    D = int(np.prod([dims[t] for t in targets]))
    els = haar(nrng, D).T.reshape(-1)
    st = dev(psi)
    q.apply_gate(st, dims, targets, dev(els))
    ref, _, _ = orc.contract(orc.Tensor(orc.DENSE, [], dims, psi),
                             orc.Tensor(orc.SYMM, [], [dims[t] for t in targets] * 2, els),
                             [(t, j) for j, t in enumerate(targets)])
    assert rel_l2(host(st), ref.els) < REL_TOL


def test_gate_timing_counts_fused_passes():
    # qtnh_gate_timing: one timed launch per fused pair pass (the first pass of the chain
    # and the chain passes), none for permutations; recording off afterwards
    old = q.get_arithmetic()
    q.set_arithmetic(q.ARITH_BF16X6)
    try:
        nrng = np.random.default_rng(62)
        n = 14
        psi = crandn(nrng, [2] * n).reshape(-1)
        gates = [(t, dev(g)) for t, g in _disjoint_pairs(nrng, n, 5)]  # 10 gates: 5 pair passes
        st, sc = dev(psi), dev(np.zeros_like(psi))
        q.gate_timing(False)
        q.gate_timing(True)
        q.apply_gate_runs(st, sc, [2] * n, [(gates[:4], list(range(n))[::-1]), (gates[4:], None)])
        ms, launches = q.gate_timing(False)
        assert launches == 5 and ms > 0
        q.apply_gate_layer(st, [2] * n, gates[:2])
        assert q.gate_timing(False) == (0.0, 0)
    finally:
        q.set_arithmetic(old)
