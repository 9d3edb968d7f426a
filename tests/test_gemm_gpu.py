"""Split-precision dense contractions (QTNH_GEMM_BF16X3: the complex GEMM of
_contract_dense, src/tensor/contract.cpp:12-201, as three-piece bf16 products with FP32
accumulation on the tcgen05 tensor cores) against the plain FP64 path, which is itself
parity-tested against the oracle. The bar is the split method's own, FP32-level: the
pieces hold 24 bits of every real, the dominant piece product accumulates apart from the
others, and K is accumulated in slices of 512 reals that are summed with compensated
additions; asserted at 2e-6 relative L2 and 2e-5 of the largest magnitude for K up to
16384."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _setup():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    q.lib()


@pytest.fixture
def bf16x3():
    old = q.get_gemm_precision()
    q.take_device_errors()
    q.set_gemm_precision(q.GEMM_BF16X3)
    yield
    q.set_gemm_precision(old)
    assert q.take_device_errors() == 0  # no bounded wait of the tcgen05 GEMM expired


def crandn(rng, shape, scale=1.0):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * scale


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128).reshape(-1)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def errors(out, ref):
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    mx = np.max(np.abs(out - ref)) / np.max(np.abs(ref))
    return rel, mx


@pytest.mark.parametrize("M,N,K", [(3, 5, 7), (64, 256, 8), (100, 300, 77), (256, 512, 1024), (1000, 130, 513),
                                   (129, 257, 2048), (64, 64, 16384)])
def test_split_gemm_matrix(M, N, K, bf16x3):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    a = crandn(rng, (M, K), 1 / np.sqrt(K))
    b = crandn(rng, (K, N))
    res, _, _, _ = q.contract(q.Tensor(q.DENSE, [], [M, K], dev(a)), q.Tensor(q.DENSE, [], [K, N], dev(b)), [(1, 0)])
    out = host(res.data).reshape(M, N)
    rel, mx = errors(out, a @ b)
    assert rel < 2e-6 and mx < 2e-5, (rel, mx)


def test_split_gemm_special_values(bf16x3):
    # zeros, a zero row and column, magnitudes far apart, values outside the float-float
    # split range (FP64 piece path); this mode's range is FP32's (|C| < 3.4e38)
    rng = np.random.default_rng(5)
    M, N, K = 64, 300, 40
    a = crandn(rng, (M, K))
    b = crandn(rng, (K, N))
    a[3, :] = 0
    b[:, 7] = 0
    a[5, 2] = 1e-30   # below the float-float split range: FP64 piece path
    a[6, :] *= 1e28   # above it (products stay inside the FP32 range of the accumulators)
    res, _, _, _ = q.contract(q.Tensor(q.DENSE, [], [M, K], dev(a)), q.Tensor(q.DENSE, [], [K, N], dev(b)), [(1, 0)])
    out = host(res.data).reshape(M, N)
    ref = a @ b
    assert np.all(out[3, :] == 0) and np.all(out[:, 7] == 0)
    for rows in (slice(0, 6), slice(6, 7), slice(7, M)):
        rel, mx = errors(out[rows], ref[rows])
        assert rel < 2e-6, (rows, rel)


def _pair(rng):
    # a dense pair as in the precision study: ranks 4-6, dims from {2, 4, 16, 32, 64},
    # 2-3 shared indices at random positions
    dims_pool = [2, 4, 16, 32, 64]
    while True:
        r1, r2 = int(rng.integers(4, 7)), int(rng.integers(4, 7))
        ns = int(rng.integers(2, 4))
        shared = [int(rng.choice(dims_pool)) for _ in range(ns)]
        d1 = [int(rng.choice(dims_pool)) for _ in range(r1 - ns)] + shared
        d2 = shared + [int(rng.choice(dims_pool)) for _ in range(r2 - ns)]
        if np.prod(d1) <= 2 ** 20 and np.prod(d2) <= 2 ** 20:
            break
    p1, p2 = [int(x) for x in rng.permutation(r1)], [int(x) for x in rng.permutation(r2)]
    # axis i of the unpermuted tensor sits at p[i]
    dd1, dd2 = [0] * r1, [0] * r2
    for i, pos in enumerate(p1):
        dd1[pos] = d1[i]
    for i, pos in enumerate(p2):
        dd2[pos] = d2[i]
    wires = [(p1[r1 - ns + j], p2[j]) for j in range(ns)]
    return dd1, dd2, wires, int(np.prod(shared))


@pytest.mark.parametrize("seed", range(6))
def test_split_contraction_vs_fp64(seed, bf16x3):
    rng = np.random.default_rng(900 + seed)
    d1, d2, wires, ksize = _pair(rng)
    a = crandn(rng, d1, 1 / np.sqrt(ksize))
    b = crandn(rng, d2)
    t1, t2 = q.Tensor(q.DENSE, [], d1, dev(a)), q.Tensor(q.DENSE, [], d2, dev(b))
    split, _, _, _ = q.contract(t1, t2, wires)
    q.set_gemm_precision(q.GEMM_FP64)
    plain, _, _, _ = q.contract(t1, t2, wires)
    q.set_gemm_precision(q.GEMM_BF16X3)
    assert split.dis == plain.dis and split.loc == plain.loc
    rel, mx = errors(host(split.data), host(plain.data))
    assert rel < 2e-6 and mx < 2e-5, (d1, d2, wires, rel, mx)


@pytest.mark.parametrize("d1,d2,wires", [
    ([3, 5, 7], [2, 3, 4], [(0, 1)]),                  # small K, A permuted (tile)
    ([4099, 3], [4099, 5], [(0, 0)]),                  # prime K: A through the gather form
    ([6, 10], [7, 10, 3], [(1, 1)]),                   # B permuted, K = 10 (padding inside a K-core)
    ([5, 9, 4, 7], [7, 3, 9, 2], [(1, 2), (3, 0)]),    # two wires, both operands permuted
    ([64, 2, 33, 16], [16, 33, 5], [(3, 0), (2, 1)]),  # power-of-two and odd axes mixed
])
def test_split_fused_permutes(d1, d2, wires, bf16x3):
    # operand permutes fused into the piece splits (tiled and gather forms, padding of
    # rows and of K) against the FP64 plain path
    rng = np.random.default_rng(sum(d1) + 3 * sum(d2))
    ksize = int(np.prod([d1[a] for a, _ in wires]))
    a = crandn(rng, d1, 1 / np.sqrt(ksize))
    b = crandn(rng, d2)
    t1, t2 = q.Tensor(q.DENSE, [], d1, dev(a)), q.Tensor(q.DENSE, [], d2, dev(b))
    split, _, _, _ = q.contract(t1, t2, wires)
    q.set_gemm_precision(q.GEMM_FP64)
    plain, _, _, _ = q.contract(t1, t2, wires)
    q.set_gemm_precision(q.GEMM_BF16X3)
    rel, mx = errors(host(split.data), host(plain.data))
    assert rel < 2e-6 and mx < 2e-5, (d1, d2, wires, rel, mx)


@pytest.mark.parametrize("d1,d2,wires", [
    ([4, 2], [2, 4, 3], [(1, 0), (0, 1)]),      # A fully wired and permuted: M = 1
    ([3, 5, 2], [2, 5], [(2, 0), (1, 1)]),      # B fully wired: N = 1
    ([1, 6, 1, 3], [3, 1, 7], [(3, 0)]),        # size-1 axes on both sides
    ([5, 1, 4], [1, 9], [(1, 0)]),              # K = 1 (one wire of size 1)
    ([2, 2, 2, 2, 2, 2], [2, 2, 2, 2], [(5, 0), (0, 3)]),  # qubit tensors, wires at both ends
])
def test_split_fused_edge_shapes(d1, d2, wires, bf16x3):
    # degenerate shapes through the fused permute-split and padding kernels
    rng = np.random.default_rng(7 * len(d1) + len(d2))
    a = crandn(rng, d1)
    b = crandn(rng, d2)
    t1, t2 = q.Tensor(q.DENSE, [], d1, dev(a)), q.Tensor(q.DENSE, [], d2, dev(b))
    split, _, _, _ = q.contract(t1, t2, wires)
    q.set_gemm_precision(q.GEMM_FP64)
    plain, _, _, _ = q.contract(t1, t2, wires)
    q.set_gemm_precision(q.GEMM_BF16X3)
    rel, mx = errors(host(split.data), host(plain.data))
    assert rel < 2e-6 and mx < 2e-5, (d1, d2, wires, rel, mx)


SLICE_MAX = 4096  # QTNH_GEMM_SLICE_MAX


@pytest.mark.parametrize("slice_steps,bound", [(1, 1.5e-7), (16, 5e-7), (64, 2e-6), (SLICE_MAX, 3e-5)])
def test_split_gemm_slice_length(slice_steps, bound, bf16x3):
    # K = 4096 complex = 512 K-steps: 512, 32, 8 and 1 slices; the error grows with the
    # slice length (the tensor core's FP32 accumulation loses up to an ulp per K-step)
    old = q.get_gemm_slice()
    assert old == 32
    q.set_gemm_slice(slice_steps)
    try:
        rng = np.random.default_rng(90)
        M, N, K = 256, 512, 4096
        a = crandn(rng, (M, K), 1 / np.sqrt(K))
        b = crandn(rng, (K, N))
        res, _, _, _ = q.contract(q.Tensor(q.DENSE, [], [M, K], dev(a)), q.Tensor(q.DENSE, [], [K, N], dev(b)),
                                  [(1, 0)])
        rel, _ = errors(host(res.data).reshape(M, N), a @ b)
        assert rel < bound, (slice_steps, rel)
    finally:
        q.set_gemm_slice(old)
    with pytest.raises(q.InvalidArgument):
        q.set_gemm_slice(0)
    with pytest.raises(q.InvalidArgument):
        q.set_gemm_slice(SLICE_MAX + 1)
    assert q.get_gemm_slice() == old
