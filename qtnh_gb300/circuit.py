"""Run a layered circuit on a device-resident state through the C ABI.

Each layer is the sequence of contractions a qtnh user would write:
``Tensor::contract(state, gate, {{q_a, 0}, {q_b, 1}})`` for every gate (in-place
rule, src/tensor/contract.cpp:250-289), one rank-2 DiagTensor contraction per
qubit for a phase layer, and ``Tensor::rescatter`` / ``Tensor::permute`` /
``Tensor::rescatter`` for a redistribution. The runner issues them as the
batched entry points of the C ABI (qtnh_apply_gate_runs, qtnh_apply_diag_layer);
rescatter is metadata-only with all slabs resident. The gates of consecutive layers go
into one call (in order), as the C++ API's queue of in-place contractions does, with
the permutations between them: qtnh_apply_gate_runs applies runs of gates separated by
permutations, so the fused passes on both sides of a permutation form one fixed-point
chain. Only a diagonal layer ends such a call.
A phase layer directly after a layer's gates is folded into those gates: the diagonal
on the qubits (a, b) of gate U follows it, so (D_a (x) D_b) U replaces U (elementwise,
exact up to one rounding of each product); qubits that no gate of the layer covers keep
a diagonal layer of their own. The phases then cost no pass over the state, and the gate
runs on both sides of them form one chain.
All argument arrays are built once so the timed loop is only library calls.
"""
import ctypes

import numpy as np

from . import (_stream, _u16, _u64, check, lib)
from .workload import phase_factors


class DeviceCircuit:
    def __init__(self, circuit, device="cuda"):
        import torch
        self.n = circuit.n
        self.dims = _u64(circuit.dims)
        self.rank = ctypes.c_int32(circuit.n)
        all_gates = []
        residual = []  # per layer: the qubits whose phases stay a diagonal layer
        for layer in circuit.layers:
            gates = [np.asarray(g, dtype=np.complex128) for g in layer.gates]
            rest = []
            if layer.phases is not None:
                covered = set()
                for j, (a, b) in enumerate(layer.pairs):
                    da, db = np.exp(1j * layer.phases[a]), np.exp(1j * layer.phases[b])
                    # els[in * 4 + out] = U[out][in], out = 2 o_a + o_b: scale output o by d_a(o_a) d_b(o_b)
                    scale = np.array([1.0, db, da, da * db], dtype=np.complex128)
                    gates[j] = (gates[j].reshape(4, 4) * scale[None, :]).reshape(-1)
                    covered.update((a, b))
                rest = [qb for qb in range(circuit.n) if qb not in covered]
            residual.append(rest)
            all_gates.extend(gates)
        self.gates = torch.from_numpy(np.concatenate(all_gates) if all_gates else np.zeros(1, np.complex128)).to(device)
        base = self.gates.data_ptr()
        self.steps = []
        gi = 0
        runs = []  # the open qtnh_apply_gate_runs call: [targets, gate indices, ptup] per run

        def close():
            if len(runs) > 1 or (runs and runs[0][1]):
                ks = [2] * sum(len(ix) for _, ix, _ in runs)
                ptrs = [base + 16 * 16 * j for _, ix, _ in runs for j in ix]
                pts = [x for _, _, pt in runs[:-1] for x in pt]
                self.steps.append(("runs", (ctypes.c_int32(len(runs)),
                                            (ctypes.c_int32 * len(runs))(*[len(ix) for _, ix, _ in runs]),
                                            (ctypes.c_int32 * max(1, len(ks)))(*ks),
                                            _u16([x for tg, _, _ in runs for x in tg]),
                                            (ctypes.c_void_p * max(1, len(ptrs)))(*ptrs), _u16(pts), len(runs) - 1)))
            runs.clear()

        for layer, rest in zip(circuit.layers, residual):
            if not runs:
                runs.append([[], [], None])
            for j, pr in enumerate(layer.pairs):
                runs[-1][0].extend(pr)
                runs[-1][1].append(gi + j)
            gi += len(layer.gates)
            if rest:
                close()
                f = torch.from_numpy(phase_factors(np.asarray(layer.phases)[rest])).to(device)
                self.steps.append(("diag", (ctypes.c_int32(len(rest)), _u16(rest), f)))
            if layer.ptup is not None:
                if not runs:
                    runs.append([[], [], None])
                runs[-1][2] = list(layer.ptup)
                runs.append([[], [], None])
        close()
        self.layers = len(circuit.layers)
        self.gate_count = gi

    def run(self, state, scratch, stream=None, events=None):
        """Apply the circuit; returns the buffer holding the result (state or scratch).

        events: optional dict of kind -> list of (start, end) CUDA event pairs recorded
        around every library call on the launch stream (for per-kernel timing)."""
        L = lib()
        st = _stream(stream)
        cur, other = state, scratch
        for kind, args in self.steps:
            ev = None
            if events is not None:
                import torch
                ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                ev[0].record(stream)
            if kind == "runs":
                nr, counts, ks, tg, ptrs, pts, nperm = args
                check(L.qtnh_apply_gate_runs(ctypes.c_void_p(cur.data_ptr()), ctypes.c_void_p(other.data_ptr()),
                                             self.rank, self.dims, nr, counts, ks, tg, ptrs, pts, st))
                if nperm % 2:
                    cur, other = other, cur
            else:
                nf, axes, f = args
                check(L.qtnh_apply_diag_layer(ctypes.c_void_p(cur.data_ptr()), self.rank, self.dims, nf, axes,
                                              ctypes.c_void_p(f.data_ptr()), st))
            if ev is not None:
                ev[1].record(stream)
                events.setdefault(kind, []).append(ev)
        return cur
