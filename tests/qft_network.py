"""QFT tensor network in the layout the reference's QFT test builds.

The network follows the structure of the reference's QFT fixture
(tests/gen/qft.hpp:49-142 and examples/qft.cpp:53-149): every qubit starts as
|+>, ``dq`` leading qubits are moved to distributed indices with identity
"DIST" tensors (IdenTensor with one distributed and one local index), each
qubit gets a Hadamard SymmTensor and controlled-phase SymmTensors with phase
pi / 2^(j-i) towards every later qubit, and the bonds are listed in the order
they must be contracted. The QFT of |+...+> is |0...0>, so amplitude 0 is 1.

``net`` is any object with ``make(kind, dis, loc, els, n_dis_in)`` returning a
tensor id and ``add_bond(t1, t2, wires)`` returning a bond id, so the same
builder drives the oracle and the GPU engine.
"""
import math

import numpy as np

DENSE, SYMM, SWAP, IDEN, DIAG = 0, 1, 2, 3, 4

S = 2 ** -0.5
PLUS = np.array([S, S], dtype=np.complex128)
HADAMARD = np.array([S, S, S, -S], dtype=np.complex128)


def cphase(p):
    e = np.zeros(16, dtype=np.complex128)
    e[0] = e[5] = e[10] = 1.0
    e[15] = np.exp(1j * p)
    return e


def build_qft(net, nq, dq):
    order = []
    qid = [0] * nq
    qidx = [0] * nq

    def dist(n_dis_in):
        return net.make(IDEN, [2], [2], None, n_dis_in)

    for i in range(nq):
        qid[i] = net.make(DENSE, [], [2], PLUS, 0)
        qidx[i] = 0
        if i < dq:
            t = dist(0)
            order.append(net.add_bond(qid[i], t, [(0, 1)]))
            qid[i] = t
            qidx[i] = 0
        if i > 0:
            order.append(net.add_bond(qid[i - 1], qid[i], []))

    for i in range(nq):
        h = net.make(SYMM, [], [2, 2], HADAMARD, 0)
        t_in, t_out, out_idx = h, h, 1
        if i < dq:
            t_in = dist(1)
            order.append(net.add_bond(t_in, h, [(1, 0)]))
            t_out = dist(0)
            order.append(net.add_bond(h, t_out, [(1, 1)]))
            out_idx = 0
        order.append(net.add_bond(qid[i], t_in, [(qidx[i], 0)]))
        qid[i], qidx[i] = t_out, out_idx

        for j in range(i + 1, nq):
            cp = net.make(SYMM, [], [2, 2, 2, 2], cphase(math.pi / 2 ** (j - i)), 0)
            a_in, b_in, a_out, b_out = cp, cp, cp, cp
            ia_in, ib_in, ia_out, ib_out = 0, 1, 2, 3
            if i < dq:
                a_in = dist(1)
                order.append(net.add_bond(a_in, cp, [(1, 0)]))
                ia_in = 0
                a_out = dist(0)
                order.append(net.add_bond(cp, a_out, [(2, 1)]))
                ia_out = 0
            if j < dq:
                b_in = dist(1)
                order.append(net.add_bond(b_in, cp, [(1, 1)]))
                ib_in = 0
                b_out = dist(0)
                order.append(net.add_bond(cp, b_out, [(3, 1)]))
                ib_out = 0
            order.append(net.add_bond(qid[i], a_in, [(qidx[i], ia_in)]))
            order.append(net.add_bond(qid[j], b_in, [(qidx[j], ib_in)]))
            qid[i], qidx[i] = a_out, ia_out
            qid[j], qidx[j] = b_out, ib_out
    return order
