"""Python binding of the GB300 tensor-contraction engine (``libqtnh_cuda.so``).

The engine's boundary is the C ABI in ``include/qtnh_cuda.h``; this module binds
it with ctypes so tests and benchmarks can drive the same entry points a C or C++
caller uses. PyTorch only supplies device memory and streams: tensors passed in
are ``torch.complex128`` CUDA tensors (global row-major order over
``dis_dims + loc_dims``) and results come back the same way.

There is no CPU fallback: every call goes through the CUDA library, and loading
fails loudly when it has not been built (``python -m qtnh_gb300.build``).
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "lib", "libqtnh_cuda.so")
HEADER = os.path.join(ROOT, "include", "qtnh_cuda.h")

X = 0xFFFF
DENSE, SYMM, SWAP, IDEN, DIAG = 0, 1, 2, 3, 4
STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "RUNTIME", 3: "OUT_OF_RANGE", 4: "CUDA", 5: "NO_MEMORY",
          6: "UNSUPPORTED", 7: "CAPACITY"}


class QtnhError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class InvalidArgument(QtnhError, ValueError):
    pass


class OutOfRange(QtnhError, IndexError):
    pass


_EXC = {1: InvalidArgument, 3: OutOfRange}


class TensorDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("ndis", ctypes.c_int32), ("nloc", ctypes.c_int32),
                ("n_dis_in", ctypes.c_int32), ("dims", ctypes.POINTER(ctypes.c_uint64)), ("data", ctypes.c_void_p)]


_lib = None


def lib():
    """Load ``libqtnh_cuda.so`` (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libqtnh_cuda.so is not built; run `python -m qtnh_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        L.qtnh_last_error.restype = ctypes.c_char_p
        L.qtnh_kernel_launch_count.restype = ctypes.c_uint64
        _lib = L
    return _lib


def declared_functions():
    """Names of the entry points declared in include/qtnh_cuda.h."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qtnh_\w+)\s*\(", src)))


def check(rc):
    if rc != 0:
        msg = lib().qtnh_last_error().decode()
        raise _EXC.get(rc, QtnhError)(rc, msg)


def launches():
    """Kernels launched by the library since it was loaded."""
    return int(lib().qtnh_kernel_launch_count())


def _u64(vals):
    vals = [int(v) for v in vals]
    return (ctypes.c_uint64 * max(1, len(vals)))(*vals)


def _u16(vals):
    vals = [int(v) for v in vals]
    return (ctypes.c_uint16 * max(1, len(vals)))(*vals)


def _stream(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _check_c128(t):
    import torch
    if t.dtype != torch.complex128 or not t.is_cuda or not t.is_contiguous():
        raise TypeError("expected a contiguous complex128 CUDA tensor")


class Tensor:
    """A tensor as the engine sees it: kind, dis/loc dims, input count, device data."""

    def __init__(self, kind, dis, loc, data=None, n_dis_in=0):
        self.kind = kind
        self.dis = [int(d) for d in dis]
        self.loc = [int(d) for d in loc]
        self.n_dis_in = int(n_dis_in)
        self.data = data
        if data is not None:
            _check_c128(data)

    @property
    def dims(self):
        return self.dis + self.loc

    def desc(self):
        self._dims = _u64(self.dims)
        return TensorDesc(self.kind, len(self.dis), len(self.loc), self.n_dis_in,
                          ctypes.cast(self._dims, ctypes.POINTER(ctypes.c_uint64)),
                          ctypes.c_void_p(self.data.data_ptr() if self.data is not None else 0))


def contract_plan(t1, t2, wires, repls=None):
    """Tensor::contract metadata (host only). Returns (dis, loc, repls1, repls2, str)."""
    r1, r2 = len(t1.dims), len(t2.dims)
    w = _u16([x for p in wires for x in p])
    rep1 = (ctypes.c_uint16 * max(1, r1))(*(repls[0] if repls else [X] * r1))
    rep2 = (ctypes.c_uint16 * max(1, r2))(*(repls[1] if repls else [X] * r2))
    ndis, nloc, st = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint64()
    out_dims = (ctypes.c_uint64 * max(1, r1 + r2))()
    d1, d2 = t1.desc(), t2.desc()
    check(lib().qtnh_contract_plan(ctypes.byref(d1), ctypes.byref(d2), ctypes.c_int32(len(wires)), w,
                                   ctypes.c_int32(0 if repls else 1), rep1, rep2, ctypes.byref(ndis),
                                   ctypes.byref(nloc), out_dims, ctypes.byref(st)))
    dims = [int(out_dims[i]) for i in range(ndis.value + nloc.value)]
    return (dims[:ndis.value], dims[ndis.value:], [rep1[i] for i in range(r1)], [rep2[i] for i in range(r2)],
            int(st.value))


def contract(t1, t2, wires, repls=None, out=None, stream=None):
    """Tensor::contract on the device. Returns (Tensor result, repls1, repls2, str)."""
    import torch
    dis, loc, rep1, rep2, st = contract_plan(t1, t2, wires, repls)
    n = 1
    for d in dis + loc:
        n *= d
    if out is None:
        out = torch.empty(n, dtype=torch.complex128, device="cuda")
    r1, r2 = len(t1.dims), len(t2.dims)
    w = _u16([x for p in wires for x in p])
    a1 = (ctypes.c_uint16 * max(1, r1))(*rep1)
    a2 = (ctypes.c_uint16 * max(1, r2))(*rep2)
    ndis, nloc, stv = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint64()
    out_dims = (ctypes.c_uint64 * max(1, r1 + r2))()
    d1, d2 = t1.desc(), t2.desc()
    check(lib().qtnh_contract(ctypes.byref(d1), ctypes.byref(d2), ctypes.c_int32(len(wires)), w, ctypes.c_int32(0),
                              a1, a2, ctypes.byref(ndis), ctypes.byref(nloc), out_dims, ctypes.byref(stv), _ptr(out),
                              ctypes.c_uint64(out.numel()), _stream(stream)))
    return Tensor(DENSE, dis, loc, out.reshape(-1)), rep1, rep2, st


def permute(x, dims, ptup, out=None, stream=None):
    import torch
    _check_c128(x)
    new = [0] * len(dims)
    for i, p in enumerate(ptup):
        new[p] = dims[i]
    if out is None:
        out = torch.empty(x.numel(), dtype=torch.complex128, device=x.device)
    check(lib().qtnh_permute(_ptr(x), _ptr(out), ctypes.c_int32(len(dims)), _u64(dims), _u16(ptup), _stream(stream)))
    return out


def swap(x, dims, i1, i2, out=None, stream=None):
    import torch
    _check_c128(x)
    if out is None:
        out = torch.empty(x.numel(), dtype=torch.complex128, device=x.device)
    check(lib().qtnh_swap(_ptr(x), _ptr(out), ctypes.c_int32(len(dims)), _u64(dims), ctypes.c_int32(i1),
                          ctypes.c_int32(i2), _stream(stream)))
    return out


def apply_gate(state, dims, targets, gate, stream=None):
    _check_c128(state)
    _check_c128(gate)
    check(lib().qtnh_apply_gate(_ptr(state), ctypes.c_int32(len(dims)), _u64(dims), ctypes.c_int32(len(targets)),
                                _u16(targets), _ptr(gate), _stream(stream)))
    return state


def apply_gate_layer(state, dims, gates, stream=None):
    """gates: list of (targets, device gate tensor)."""
    _check_c128(state)
    ks = (ctypes.c_int32 * max(1, len(gates)))(*[len(t) for t, _ in gates])
    tg = _u16([x for t, _ in gates for x in t])
    ptrs = (ctypes.c_void_p * max(1, len(gates)))(*[g.data_ptr() for _, g in gates])
    check(lib().qtnh_apply_gate_layer(_ptr(state), ctypes.c_int32(len(dims)), _u64(dims), ctypes.c_int32(len(gates)),
                                      ks, tg, ptrs, _stream(stream)))
    return state


def apply_gate_runs(state, scratch, dims, runs, stream=None):
    """runs: list of (gates, ptup) -- gates a list of (targets, device gate tensor) as in
    apply_gate_layer, ptup the permutation after the run (None for the last run). Returns
    the buffer holding the result (scratch after an odd number of permutations)."""
    _check_c128(state)
    if len(runs) > 1:
        _check_c128(scratch)
    for j, (_, pt) in enumerate(runs):
        if (pt is None) != (j + 1 == len(runs)):
            raise ValueError("every run but the last is followed by a permutation")
    gates = [g for gl, _ in runs for g in gl]
    ng = (ctypes.c_int32 * len(runs))(*[len(gl) for gl, _ in runs])
    ks = (ctypes.c_int32 * max(1, len(gates)))(*[len(t) for t, _ in gates])
    tg = _u16([x for t, _ in gates for x in t])
    ptrs = (ctypes.c_void_p * max(1, len(gates)))(*[g.data_ptr() for _, g in gates])
    pts = _u16([x for _, pt in runs[:-1] for x in pt])
    check(lib().qtnh_apply_gate_runs(_ptr(state), _ptr(scratch),
                                     ctypes.c_int32(len(dims)), _u64(dims), ctypes.c_int32(len(runs)), ng, ks, tg,
                                     ptrs, pts, _stream(stream)))
    return scratch if (len(runs) - 1) % 2 else state


def apply_diag(state, dims, targets, diag, stream=None):
    _check_c128(state)
    _check_c128(diag)
    check(lib().qtnh_apply_diag(_ptr(state), ctypes.c_int32(len(dims)), _u64(dims), ctypes.c_int32(len(targets)),
                                _u16(targets), _ptr(diag), _stream(stream)))
    return state


def apply_diag_layer(state, dims, axes, factors, stream=None):
    """factors: concatenated per-axis diagonals (device complex128)."""
    _check_c128(state)
    _check_c128(factors)
    check(lib().qtnh_apply_diag_layer(_ptr(state), ctypes.c_int32(len(dims)), _u64(dims), ctypes.c_int32(len(axes)),
                                      _u16(axes), _ptr(factors), _stream(stream)))
    return state


def take_device_errors():
    """Device error flags raised since the last call (0: none); synchronizes."""
    f = ctypes.c_uint32()
    check(lib().qtnh_take_device_errors(ctypes.byref(f)))
    return int(f.value)


def norm2(x, stream=None):
    _check_c128(x)
    r = ctypes.c_double()
    check(lib().qtnh_norm2(_ptr(x), ctypes.c_uint64(x.numel()), ctypes.byref(r), _stream(stream)))
    return r.value


ARITH_FP64, ARITH_F32X2, ARITH_BF16X6 = 0, 1, 2
ARITH_NAMES = {"fp64": ARITH_FP64, "f32x2": ARITH_F32X2, "bf16x6": ARITH_BF16X6}


def set_arithmetic(mode):
    """QTNH_ARITH_FP64 (0), QTNH_ARITH_F32X2 (1) or QTNH_ARITH_BF16X6 (2) for the
    gate/diagonal kernels."""
    check(lib().qtnh_set_arithmetic(ctypes.c_int(mode)))


def get_arithmetic():
    return int(lib().qtnh_get_arithmetic())


GEMM_FP64, GEMM_BF16X3, GEMM_OZ6 = 0, 1, 2


def set_gemm_precision(mode):
    """QTNH_GEMM_OZ6 (2, default: FP64-accurate digit products on tcgen05), QTNH_GEMM_FP64
    (0, FP64 fused multiply-adds) or QTNH_GEMM_BF16X3 (1, split precision on tcgen05)."""
    check(lib().qtnh_set_gemm_precision(ctypes.c_int(mode)))


def get_gemm_precision():
    return int(lib().qtnh_get_gemm_precision())


def set_gemm_slice(k_steps):
    """K-steps per split-K slice of the BF16x3 GEMM (default 32): longer slices are faster
    and less accurate (error in proportion to the length)."""
    check(lib().qtnh_set_gemm_slice(ctypes.c_int(k_steps)))


def get_gemm_slice():
    return int(lib().qtnh_get_gemm_slice())


def gemm_timing(enable):
    """(ms, launches) of the tcgen05 GEMM kernel since the last call; then (dis)arm recording."""
    ms, n = ctypes.c_double(), ctypes.c_uint64()
    check(lib().qtnh_gemm_timing(ctypes.c_int(1 if enable else 0), ctypes.byref(ms), ctypes.byref(n)))
    return ms.value, int(n.value)


def gate_timing(enable):
    """(ms, launches) of the fused gate-pair passes since the last call; then (dis)arm recording."""
    ms, n = ctypes.c_double(), ctypes.c_uint64()
    check(lib().qtnh_gate_timing(ctypes.c_int(1 if enable else 0), ctypes.byref(ms), ctypes.byref(n)))
    return ms.value, int(n.value)


class Batch:
    """Batched circuits on the C ABI's qtnh_batch_* entry points: add circuits, compile
    once (rounds of grouped kernels, autotuning, CUDA graph capture), run and read the
    queries. precision STATE_C64 (default): mixed precision, complex64 states with FP64
    renormalisation and complex128 queries; STATE_C128: the plain method, complex128
    states and FP64 math on the same schedule."""

    def __init__(self, nqubits, precision=None):
        self._b = ctypes.c_void_p()
        self.precision = STATE_C64 if precision is None else int(precision)
        arr = (ctypes.c_int32 * len(nqubits))(*[int(x) for x in nqubits])
        check(lib().qtnh_batch_create_typed(ctypes.byref(self._b), ctypes.c_int32(len(nqubits)), arr,
                                            ctypes.c_int32(self.precision)))
        self.nq = [int(x) for x in nqubits]
        self.nqueries = 0

    def __del__(self):
        try:
            if self._b:
                lib().qtnh_batch_destroy(self._b)
        except Exception:
            pass

    def set_state(self, c, psi, stream=None):
        _check_c128(psi)
        check(lib().qtnh_batch_set_state(self._b, ctypes.c_int32(c), _ptr(psi), _stream(stream)))

    def add_circuit(self, c, circuit, queries=()):
        """Registers a workload.Circuit (gates, phase layers, qubit-swap permutations)."""
        import numpy as np
        L = lib()
        for li, layer in enumerate(circuit.layers):
            for (qa, qb), els in zip(layer.pairs, layer.gates):
                e = np.ascontiguousarray(els, dtype=np.complex128)
                check(L.qtnh_batch_add_gate(self._b, ctypes.c_int32(c), ctypes.c_int32(li), ctypes.c_uint16(qa),
                                            ctypes.c_uint16(qb), ctypes.c_void_p(e.ctypes.data)))
            if layer.phases is not None:
                ph = np.ascontiguousarray(layer.phases, dtype=np.float64)
                check(L.qtnh_batch_add_phases(self._b, ctypes.c_int32(c), ctypes.c_int32(li),
                                              ph.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
            if layer.ptup is not None:
                moved = [i for i, p in enumerate(layer.ptup) if p != i]
                if len(moved) != 2 or layer.ptup[moved[0]] != moved[1]:
                    raise ValueError("only two-qubit swaps are supported as permutations")
                check(L.qtnh_batch_add_swap(self._b, ctypes.c_int32(c), ctypes.c_int32(li), ctypes.c_uint16(moved[0]),
                                            ctypes.c_uint16(moved[1])))
        if len(queries):
            idx = np.ascontiguousarray(queries, dtype=np.uint64)
            check(L.qtnh_batch_add_queries(self._b, ctypes.c_int32(c), ctypes.c_int32(len(idx)),
                                           idx.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
            self.nqueries += len(idx)

    def compile(self, renorm_every=8, autotune=True):
        check(lib().qtnh_batch_compile(self._b, ctypes.c_int32(renorm_every), ctypes.c_int32(1 if autotune else 0)))

    def run(self, stream=None):
        check(lib().qtnh_batch_run(self._b, _stream(stream)))

    def results(self, out=None, stream=None):
        import torch
        if out is None:
            out = torch.empty(max(1, self.nqueries), dtype=torch.complex128, device="cuda")
        check(lib().qtnh_batch_results(self._b, _ptr(out), ctypes.c_uint64(out.numel()), _stream(stream)))
        return out[:self.nqueries]

    def state(self, c, stream=None):
        import torch
        out = torch.empty(2 ** self.nq[c], dtype=torch.complex128, device="cuda")
        check(lib().qtnh_batch_state(self._b, ctypes.c_int32(c), _ptr(out), _stream(stream)))
        return out

    def info(self):
        amps, rounds, lpr, chunk = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        th = ctypes.c_int32()
        check(lib().qtnh_batch_info(self._b, ctypes.byref(amps), ctypes.byref(rounds), ctypes.byref(lpr),
                                    ctypes.byref(th), ctypes.byref(chunk)))
        return {"amplitudes": amps.value, "rounds": rounds.value, "launches_per_run": lpr.value,
                "gate_threads": th.value, "gate_chunk": chunk.value}


# ---- grouped operations on many resident states (request loops) ------------------------

STATE_C128, STATE_C64 = 0, 1


def _check_state(t, precision):
    import torch
    want = torch.complex128 if precision == STATE_C128 else torch.complex64
    if t.dtype != want or not t.is_cuda or not t.is_contiguous():
        raise TypeError("expected a contiguous %s CUDA tensor" % want)


def state_convert(to_precision, src, dst, stream=None):
    """complex128 -> complex64 (to_precision STATE_C64) or back, n = src.numel()."""
    check(lib().qtnh_state_convert(ctypes.c_int32(to_precision), _ptr(src), _ptr(dst), ctypes.c_uint64(src.numel()),
                                   _stream(stream)))
    return dst


def group_layer(precision, items, stream=None):
    """items: [(state, n, pairs, gates, phases or None, swap (qa, qb) or None)] -> the layer
    applied to every state in grouped launches (qtnh_group_layer)."""
    import numpy as np
    ns = len(items)
    if ns == 0:
        return
    for it in items:
        _check_state(it[0], precision)
    states = (ctypes.c_void_p * ns)(*[it[0].data_ptr() for it in items])
    nq = (ctypes.c_int32 * ns)(*[int(it[1]) for it in items])
    ng = (ctypes.c_int32 * ns)(*[len(it[2]) for it in items])
    pairs = _u16([x for it in items for p in it[2] for x in p])
    gl = [np.asarray(g, dtype=np.complex128).reshape(16) for it in items for g in it[3]]
    gates = np.ascontiguousarray(np.concatenate(gl) if gl else np.zeros(16, np.complex128))
    hp = (ctypes.c_uint8 * ns)(*[0 if it[4] is None else 1 for it in items])
    pl = [np.asarray(it[4], dtype=np.float64) for it in items if it[4] is not None]
    phases = np.ascontiguousarray(np.concatenate(pl) if pl else np.zeros(1))
    sw = _u16([x for it in items for x in (it[5] if it[5] is not None else (0xFFFF, 0xFFFF))])
    check(lib().qtnh_group_layer(ctypes.c_int32(precision), ctypes.c_int32(ns), states, nq, ng, pairs,
                                 ctypes.c_void_p(gates.ctypes.data), hp,
                                 phases.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), sw, _stream(stream)))


def group_renorm(precision, items, stream=None):
    """items: [(state, n)] -> every state scaled to unit L2 norm (FP64 norms)."""
    ns = len(items)
    if ns == 0:
        return
    states = (ctypes.c_void_p * ns)(*[it[0].data_ptr() for it in items])
    nq = (ctypes.c_int32 * ns)(*[int(it[1]) for it in items])
    check(lib().qtnh_group_renorm(ctypes.c_int32(precision), ctypes.c_int32(ns), states, nq, _stream(stream)))


def gather(precision, state, n, idx, stream=None):
    """Amplitudes state[idx] as a complex128 CUDA tensor."""
    import numpy as np
    import torch
    _check_state(state, precision)
    ix = np.ascontiguousarray(idx, dtype=np.uint64)
    out = torch.empty(max(1, len(ix)), dtype=torch.complex128, device="cuda")
    check(lib().qtnh_gather(ctypes.c_int32(precision), _ptr(state), ctypes.c_int32(n), ctypes.c_int32(len(ix)),
                            ix.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), _ptr(out), _stream(stream)))
    return out[:len(ix)]


def rdm4(precision, state, n, qubits, stream=None):
    """16 x 16 reduced density matrix of 4 qubits (complex128 CUDA tensor, FP64 sums)."""
    import torch
    _check_state(state, precision)
    out = torch.empty(256, dtype=torch.complex128, device="cuda")
    check(lib().qtnh_rdm4(ctypes.c_int32(precision), _ptr(state), ctypes.c_int32(n), _u16(qubits), _ptr(out),
                          _stream(stream)))
    return out.reshape(16, 16)
