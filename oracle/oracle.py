"""ORACLE — test infrastructure only.

ctypes wrapper around ``oracle/_build/liboracle.so`` (built from
``oracle/qtnh_oracle.cpp`` by :func:`build`). Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module, and only as the checker or as the timed CPU baseline. The product
(``qtnh_gb300``) never imports it.

All element arrays are numpy ``complex128`` in global row-major order over
``dis_dims + loc_dims`` (every slab resident, rank order).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SRC = os.path.join(HERE, "qtnh_oracle.cpp")

DENSE, SYMM, SWAP, IDEN, DIAG = 0, 1, 2, 3, 4
X = 0xFFFF

ERRORS = {1: ValueError, 2: RuntimeError, 3: IndexError, 5: RuntimeError}


def build(force=False):
    """Compile the oracle with g++ (-O2, scalar, no fast-math)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", LIB_PATH, SRC]
    subprocess.check_call(cmd)
    return LIB_PATH


class _OrcTensor(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("ndis", ctypes.c_int32),
        ("nloc", ctypes.c_int32),
        ("n_dis_in", ctypes.c_int32),
        ("dims", ctypes.POINTER(ctypes.c_uint64)),
        ("els", ctypes.POINTER(ctypes.c_double)),
        ("str_", ctypes.c_uint32),
        ("cyc", ctypes.c_uint32),
        ("off", ctypes.c_uint32),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = LIB_PATH if os.path.exists(LIB_PATH) else build()
        L = ctypes.CDLL(path)
        L.orc_last_error.restype = ctypes.c_char_p
        for name in ("orc_permute", "orc_swap", "orc_contract", "orc_dense_of", "orc_tn_insert",
                     "orc_tn_add_bond", "orc_tn_contract_bond", "orc_tn_contract_all", "orc_tn_get"):
            getattr(L, name).restype = ctypes.c_int32
        L.orc_tn_new.restype = ctypes.c_void_p
        L.orc_tn_free.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise ERRORS.get(rc, RuntimeError)(lib().orc_last_error().decode())


class Tensor:
    """A global tensor: kind, dis/loc dims, symmetric input count and elements."""

    def __init__(self, kind, dis, loc, els=None, n_dis_in=0, bc=(1, 1, 0)):
        self.kind = kind
        self.dis = [int(d) for d in dis]
        self.loc = [int(d) for d in loc]
        self.n_dis_in = int(n_dis_in)
        self.els = None if els is None else np.ascontiguousarray(els, dtype=np.complex128).reshape(-1)
        self.bc = tuple(bc)

    @property
    def dims(self):
        return self.dis + self.loc

    def _desc(self):
        self._dims_arr = (ctypes.c_uint64 * max(1, len(self.dims)))(*self.dims)
        d = _OrcTensor()
        d.kind, d.ndis, d.nloc, d.n_dis_in = self.kind, len(self.dis), len(self.loc), self.n_dis_in
        d.dims = ctypes.cast(self._dims_arr, ctypes.POINTER(ctypes.c_uint64))
        if self.els is not None:
            d.els = self.els.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.str_, d.cyc, d.off = self.bc
        return d

    def dense(self):
        """Dense elements (reshaped to the total dims)."""
        if self.kind in (DENSE, SYMM):
            return self.els.reshape(self.dims)
        n = int(np.prod(self.dims)) if self.dims else 1
        out = np.empty(n, dtype=np.complex128)
        _check(lib().orc_dense_of(ctypes.byref(self._desc()), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  ctypes.c_uint64(n)))
        return out.reshape(self.dims)


def permute(a, ptup):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    dims = (ctypes.c_uint64 * a.ndim)(*a.shape)
    pt = (ctypes.c_uint16 * a.ndim)(*ptup)
    new_shape = [0] * a.ndim
    for i, p in enumerate(ptup):
        new_shape[p] = a.shape[i]
    out = np.empty(new_shape, dtype=np.complex128)
    _check(lib().orc_permute(a.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p),
                             ctypes.c_int32(a.ndim), dims, pt))
    return out


def swap(a, i1, i2):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    dims = (ctypes.c_uint64 * a.ndim)(*a.shape)
    out = np.empty_like(a)
    _check(lib().orc_swap(a.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p),
                          ctypes.c_int32(a.ndim), dims, ctypes.c_int32(i1), ctypes.c_int32(i2)))
    return out


def contract(t1, t2, wires, repls=None):
    """Tensor::contract. Returns (Tensor result, repls1, repls2)."""
    L = lib()
    r1, r2 = len(t1.dims), len(t2.dims)
    nw = len(wires)
    w = (ctypes.c_uint16 * max(1, 2 * nw))(*[x for p in wires for x in p])
    rep1 = (ctypes.c_uint16 * max(1, r1))()
    rep2 = (ctypes.c_uint16 * max(1, r2))()
    use_def = 1
    if repls is not None:
        use_def = 0
        for i, v in enumerate(repls[0]):
            rep1[i] = v
        for i, v in enumerate(repls[1]):
            rep2[i] = v
    ndis, nloc = ctypes.c_int32(), ctypes.c_int32()
    out_dims = (ctypes.c_uint64 * max(1, r1 + r2))()
    bc = (ctypes.c_uint32 * 3)()
    d1, d2 = t1._desc(), t2._desc()
    args = [ctypes.byref(d1), ctypes.byref(d2), ctypes.c_int32(nw), w, ctypes.c_int32(use_def), rep1, rep2,
            ctypes.byref(ndis), ctypes.byref(nloc), out_dims, bc]
    rc = L.orc_contract(*args, None, ctypes.c_uint64(0))
    if rc != 4:
        _check(rc)
    dims = [int(out_dims[i]) for i in range(ndis.value + nloc.value)]
    n = int(np.prod(dims)) if dims else 1
    out = np.empty(n, dtype=np.complex128)
    _check(L.orc_contract(*args, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_uint64(n)))
    res = Tensor(DENSE, dims[:ndis.value], dims[ndis.value:], out, bc=(bc[0], bc[1], bc[2]))
    return res, [rep1[i] for i in range(r1)], [rep2[i] for i in range(r2)]


class Network:
    """TensorNetwork with the reference's contraction / rewiring rules."""

    def __init__(self):
        self._h = ctypes.c_void_p(lib().orc_tn_new())
        self._keep = []

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_tn_free(self._h)
            self._h = None

    def insert(self, t):
        tid = ctypes.c_uint32()
        d = t._desc()
        self._keep.append(t)
        _check(lib().orc_tn_insert(self._h, ctypes.byref(d), ctypes.byref(tid)))
        return tid.value

    def add_bond(self, a, b, wires):
        bid = ctypes.c_uint32()
        w = (ctypes.c_uint16 * max(1, 2 * len(wires)))(*[x for p in wires for x in p])
        _check(lib().orc_tn_add_bond(self._h, ctypes.c_uint32(a), ctypes.c_uint32(b), ctypes.c_int32(len(wires)), w,
                                     ctypes.byref(bid)))
        return bid.value

    def contract_bond(self, bid):
        tid = ctypes.c_uint32()
        _check(lib().orc_tn_contract_bond(self._h, ctypes.c_uint32(bid), ctypes.byref(tid)))
        return tid.value

    def contract_all(self, order=None):
        tid = ctypes.c_uint32()
        if order is None:
            _check(lib().orc_tn_contract_all(self._h, ctypes.c_int32(-1), None, ctypes.byref(tid)))
        else:
            o = (ctypes.c_uint32 * max(1, len(order)))(*order)
            _check(lib().orc_tn_contract_all(self._h, ctypes.c_int32(len(order)), o, ctypes.byref(tid)))
        return tid.value

    def get(self, tid):
        ndis, nloc = ctypes.c_int32(), ctypes.c_int32()
        dims = (ctypes.c_uint64 * 64)()
        bc = (ctypes.c_uint32 * 3)()
        rc = lib().orc_tn_get(self._h, ctypes.c_uint32(tid), ctypes.byref(ndis), ctypes.byref(nloc), dims, bc, None,
                              ctypes.c_uint64(0))
        if rc != 4:
            _check(rc)
        d = [int(dims[i]) for i in range(ndis.value + nloc.value)]
        n = int(np.prod(d)) if d else 1
        out = np.empty(n, dtype=np.complex128)
        _check(lib().orc_tn_get(self._h, ctypes.c_uint32(tid), ctypes.byref(ndis), ctypes.byref(nloc), dims, bc,
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_uint64(n)))
        return Tensor(DENSE, d[:ndis.value], d[ndis.value:], out, bc=(bc[0], bc[1], bc[2]))


def run_circuit(psi, circuit, layers=None):
    """Apply a layered circuit (qtnh_gb300.workload.Circuit) the way a qtnh user would:
    one Tensor::contract per gate (SymmTensor, in-place rule), one per single-qubit
    DiagTensor, and Tensor::permute for a redistribution. Returns the final state."""
    n = circuit.n
    cur = Tensor(DENSE, [], [2] * n, psi)
    for layer in circuit.layers[:layers]:
        for (a, b), els in zip(layer.pairs, layer.gates):
            cur, _, _ = contract(cur, Tensor(SYMM, [], [2, 2, 2, 2], els), [(a, 0), (b, 1)])
        if layer.phases is not None:
            for qb in range(n):
                d = np.array([1.0, np.exp(1j * layer.phases[qb])], dtype=np.complex128)
                cur, _, _ = contract(cur, Tensor(DIAG, [], [2, 2], d), [(qb, 0)])
        if layer.ptup is not None:
            cur = Tensor(DENSE, [], [2] * n, permute(cur.els.reshape([2] * n), layer.ptup))
    return cur.els
