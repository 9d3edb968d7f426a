"""The reference's own code at world size 1 — test infrastructure only.

ctypes wrapper around ``oracle/_ref/libqtnh_ref.so`` (built by ``oracle/ref_build.py``
from the reference checkout's sources and the single-process MPI subset). Only tests
import it, to pin the oracle restatement (``oracle/qtnh_oracle.cpp``) to the real code;
it is absent wherever the reference checkout is (e.g. on a GPU machine), and then
``available()`` is False.
"""
import ctypes
import os

import numpy as np

from . import ref_build

DENSE, SYMM, SWAP, IDEN = 0, 1, 2, 3
X = 0xFFFF
_lib = None


def available():
    return lib() is not None


def lib():
    global _lib
    if _lib is None:
        path = ref_build.LIB_PATH if os.path.exists(ref_build.LIB_PATH) else ref_build.build()
        if path is None or not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        L.ref_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _u64(v):
    return (ctypes.c_uint64 * max(1, len(v)))(*[int(x) for x in v])


def _u16(v):
    return (ctypes.c_uint16 * max(1, len(v)))(*[int(x) for x in v])


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _check(rc):
    if rc != 0:
        raise {1: ValueError, 3: IndexError}.get(rc, RuntimeError)(lib().ref_last_error().decode())


def _arr(els, n):
    if els is None:
        return None
    a = np.ascontiguousarray(np.asarray(els, dtype=np.complex128).reshape(-1))
    assert a.size == n
    return a


def contract(t1, t2, wires, repls=None):
    """Tensor::contract of (kind, dims, n_in, els) tensors without distributed indices.
    Returns (dims, elements, repls1, repls2)."""
    (k1, d1, n1, e1), (k2, d2, n2, e2) = t1, t2
    a1, a2 = _arr(e1, int(np.prod(d1))), _arr(e2, int(np.prod(d2)))
    r1 = _u16(repls[0] if repls else [X] * len(d1))
    r2 = _u16(repls[1] if repls else [X] * len(d2))
    cap = int(np.prod(d1)) * int(np.prod(d2))
    out = np.zeros(cap, dtype=np.complex128)
    od = (ctypes.c_uint64 * (len(d1) + len(d2) + 1))()
    rank = ctypes.c_int32()
    w = _u16([x for p in wires for x in p])
    _check(lib().ref_contract(k1, len(d1), n1, _u64(d1), _dptr(a1), k2, len(d2), n2, _u64(d2), _dptr(a2), len(wires), w,
                              0 if repls else 1, r1, r2, ctypes.byref(rank), od, _dptr(out), ctypes.c_uint64(cap)))
    dims = [int(od[i]) for i in range(rank.value)]
    return dims, out[:int(np.prod(dims)) if dims else 1].copy(), list(r1)[:len(d1)], list(r2)[:len(d2)]


def permute(dims, els, ptup):
    a = _arr(els, int(np.prod(dims)))
    out = np.zeros_like(a)
    od = (ctypes.c_uint64 * len(dims))()
    _check(lib().ref_permute(len(dims), _u64(dims), _dptr(a), _u16(ptup), od, _dptr(out)))
    return [int(x) for x in od], out


def swap(dims, els, i1, i2):
    a = _arr(els, int(np.prod(dims)))
    out = np.zeros_like(a)
    od = (ctypes.c_uint64 * len(dims))()
    _check(lib().ref_swap(len(dims), _u64(dims), _dptr(a), i1, i2, od, _dptr(out)))
    return [int(x) for x in od], out


def gate_layers(psi, n, pairs, gates):
    """One Tensor::contract per two-qubit SymmTensor gate, in order; returns the state."""
    st = np.ascontiguousarray(psi, dtype=np.complex128).copy()
    g = np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=np.complex128).reshape(-1) for x in gates]))
    _check(lib().ref_gate_layers(n, _dptr(st), len(pairs), _u16([x for p in pairs for x in p]), _dptr(g)))
    return st
