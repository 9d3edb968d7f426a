"""The plain dense contraction's GEMM on the tensor cores (QTNH_GEMM_OZ6, the default):
the complex GEMM of _contract_dense (src/tensor/contract.cpp:133-162 sums complex<double>
products over the closed indices) as exact products of six balanced 8-bit digits per
real, level sums exact in FP32 over chunks of 128 reals of K, chunks accumulated exactly.

Checked against numpy's complex128 GEMM (FP64) on matrices from the smallest shape the
mode takes (2^18 complex multiply-adds) to K = 16384 (128 chunks; split K over the SMs),
padded edges (M, N, K not multiples of the tiles), rows and columns of very different
scale, zero rows and columns, infinities and NaNs (recomputed in FP64), and through
Tensor::contract with the operand permutes against the oracle. The bar is the plain
method's: 1e-12 relative L2 and 1e-12 of the largest magnitude (measured ~1e-14)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import qtnh_gb300 as q
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
REL_TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _setup():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    q.lib()


@pytest.fixture
def oz6():
    old = q.get_gemm_precision()
    q.take_device_errors()
    q.set_gemm_precision(q.GEMM_OZ6)
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


def gemm(a, b):
    M, K = a.shape
    N = b.shape[1]
    res, _, _, _ = q.contract(q.Tensor(q.DENSE, [], [M, K], dev(a)), q.Tensor(q.DENSE, [], [K, N], dev(b)), [(1, 0)])
    return host(res.data).reshape(M, N)


def errors(out, ref):
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    mx = np.max(np.abs(out - ref)) / np.max(np.abs(ref))
    return rel, mx


@pytest.mark.parametrize("M,N,K", [(64, 64, 64), (100, 300, 77), (256, 512, 1024), (1000, 130, 513),
                                   (129, 257, 2048), (64, 64, 16384), (700, 33, 4096), (2048, 2048, 64)])
def test_oz6_gemm_matrix(M, N, K, oz6):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    a = crandn(rng, (M, K), 1 / np.sqrt(K))
    b = crandn(rng, (K, N))
    rel, mx = errors(gemm(a, b), a @ b)
    assert rel < REL_TOL and mx < REL_TOL, (rel, mx)


def test_oz6_gemm_scales_and_zeros(oz6):
    rng = np.random.default_rng(11)
    M, N, K = 200, 150, 300
    a = crandn(rng, (M, K)) * np.exp2(rng.integers(-300, 300, size=(M, 1)))
    b = crandn(rng, (K, N)) * np.exp2(rng.integers(-300, 300, size=(1, N)))
    a[7, :] = 0
    b[:, 9] = 0
    a[11, 5] *= 1e-12  # one element far below the rest of its row
    out, ref = gemm(a, b), a @ b
    # every element within 1e-12 of the largest product magnitude of its row and column
    mag = np.abs(a) @ np.abs(b)
    worst = np.max(np.abs(out - ref) / np.where(mag > 0, mag, 1.0))
    assert worst < 1e-13, worst
    assert np.all(out[7, :] == 0) and np.all(out[:, 9] == 0)


def test_oz6_gemm_infinities_and_nans(oz6):
    rng = np.random.default_rng(12)
    M, N, K = 96, 80, 128
    a = crandn(rng, (M, K))
    b = crandn(rng, (K, N))
    a[3, 10] = np.inf
    b[20, 5] = complex(np.nan, 0.0)
    out = gemm(a, b)
    ref = a @ b
    special = np.zeros((M, N), dtype=bool)
    special[3, :] = True
    special[:, 5] = True
    assert np.all(np.isnan(out[:, 5]))
    assert np.all(~np.isfinite(out[3, :]))
    rel, _ = errors(out[~special], ref[~special])
    assert rel < REL_TOL


@pytest.mark.parametrize("seed", range(4))
def test_oz6_contraction_with_permutes_matches_oracle(seed, oz6):
    # rank-4 x rank-3 operands, two wires at random positions: permute to [open | wired],
    # digit GEMM, permute to the reference's output order
    rng = np.random.default_rng(300 + seed)
    d1 = [int(x) for x in rng.choice([4, 8, 16], size=4)]
    d2 = [int(x) for x in rng.choice([4, 8, 16], size=3)]
    i1 = rng.choice(4, size=2, replace=False)
    i2 = rng.choice(3, size=2, replace=False)
    for x, y in zip(i1, i2):
        d2[y] = d1[x]
    wires = [(int(x), int(y)) for x, y in zip(i1, i2)]
    a = crandn(rng, d1)
    b = crandn(rng, d2)
    M = int(np.prod(d1)) // int(np.prod([d1[x] for x in i1]))
    N = int(np.prod(d2)) // int(np.prod([d2[y] for y in i2]))
    K = int(np.prod([d1[x] for x in i1]))
    res, _, _, _ = q.contract(q.Tensor(q.DENSE, [], d1, dev(a)), q.Tensor(q.DENSE, [], d2, dev(b)), wires)
    ref, _, _ = orc.contract(orc.Tensor(orc.DENSE, [], d1, a.reshape(-1)), orc.Tensor(orc.DENSE, [], d2, b.reshape(-1)),
                             wires)
    assert res.dis + res.loc == ref.dis + ref.loc
    out = host(res.data)
    rel, mx = errors(out, ref.els)
    assert rel < REL_TOL and mx < REL_TOL, (rel, mx)


def test_oz6_is_the_default_plain_gemm():
    assert q.get_gemm_precision() in (q.GEMM_OZ6, q.GEMM_FP64, q.GEMM_BF16X3)
    import os
    if os.environ.get("QTNH_GEMM") in (None, "", "oz6"):
        assert q.get_gemm_precision() == q.GEMM_OZ6
