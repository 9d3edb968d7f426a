#!/usr/bin/env python
"""Gate-layers/s of the complex128 contraction engine on the random layered circuit.

Workload (the configuration the headline metric is quoted on): n = 28 qubits
(2^28 complex128 amplitudes, 4 GiB), depth 40; every layer 14 Haar-random
two-qubit SymmTensor gates on a seeded random pairing; every 4th layer a layer of
per-qubit phase DiagTensors; every 8th layer a rescatter of the top 3 indices and a
seeded permutation exchanging them with 3 local indices. A step is one pass of the
whole circuit over the state. Inputs (4 GiB) are far larger than L2 (129 MB), so no
L2 flush is needed between steps.

value : gate-layers/s with the state resident in HBM (CUDA events on the launch stream).
e2e   : the same through the C ABI with host buffers: every step copies the initial
        state from pinned host memory to the device and the result back, on two copy
        streams with two device state buffers, so that the next step's input copy and
        this step's result copy overlap the circuit.
arith : default bf16x6: each layer's gates applied as fused pairs (two disjoint
        two-qubit gates = one 16x16 unitary) on the bf16 tensor cores with error-free
        8-bit digits (complex128 in and out, ~1e-14 relative error per pair);
        `--arith f32x2|fp64` times the per-gate float-float / native FP64 kernels.
roofline: the dominant kernel (the fused gate-pair kernel; with f32x2/fp64 the
        two-qubit gate kernel), algorithmic bytes 32 * 2^n per launch (the state read
        and written once) over its event-timed average duration, against the measured
        HBM copy bandwidth.
cpu_baseline: the oracle port of the reference's contraction path on one host core,
        on a bounded sample (n = 20, 4 layers), extrapolated to n = 28.

`--impl reference` times that CPU port with every host core (one replica per core,
the reference's slab-per-rank parallelism without communication) and prints the
same metric.
Multi-GPU (torchrun): independent replicas, one per GPU ("replicas only").
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "gate-layers/s"
UNIT = "gate-layers/s"
CPU_SAMPLE_N = 20
CPU_SAMPLE_LAYERS = 4


def max_over_ranks(ms, dist, device):
    """The slowest rank's time (every rank gets it); ms unchanged without a process group."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=28)
    p.add_argument("--depth", type=int, default=40)
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--arith", default="bf16x6", choices=["bf16x6", "f32x2", "fp64"],
                   help="arithmetic of the gate/diagonal kernels (storage is complex128 either way)")
    p.add_argument("--no-arith-check", action="store_true")
    p.add_argument("--workload", default="circuit",
                   choices=["circuit", "contract", "batch", "serve", "kernels", "qft", "api"],
                   help="circuit: the n=28 random layered circuit (headline); contract: 64 seeded dense "
                        "contraction pairs, split-precision BF16x3 GEMM vs FP64 plain (precision study); batch: "
                        "2048 uneven circuits in mixed precision under one CUDA graph; serve: a Poisson request "
                        "stream through the request loop, plain complex128 vs mixed complex64; kernels: the "
                        "plain path's permute, diag, gate and norm kernels one by one (HBM fractions); qft: the "
                        "16-qubit QFT network through the C++ API's TensorNetwork::contractAll; api: the headline "
                        "circuit through the C++ API, one Tensor::contract per gate")
    p.add_argument("--requests", type=int, default=400)
    p.add_argument("--circuits", type=int, default=2048)
    p.add_argument("--pairs", type=int, default=64)
    p.add_argument("--max-elems", type=int, default=2 ** 26,
                   help="contract workload: largest tensor of a pair, in elements (smaller for profiling captures)")
    return p.parse_args()


def _config(a, cpu_cores=None):
    return {
        "workload": "random layered circuit, n=%d qubits, depth %d, %d Haar 2-qubit SymmTensor gates/layer, "
                    "phase DiagTensor layer every 4th, rescatter+permute of top 3 indices every 8th"
                    % (a.n, a.depth, a.n // 2),
        "qubits": a.n,
        "depth": a.depth,
        "gates_per_layer": a.n // 2,
        "element": "complex128",
        "state_bytes": 16 * (2 ** a.n),
        "l2_flush": "not needed: the %s state is larger than the 129 MB L2" % (
            "%d GiB" % (2 ** a.n // 2 ** 26) if a.n >= 26 else "%d MiB" % (2 ** a.n // 2 ** 16)),
        "execution": "the gates of consecutive layers between redistributions as fused pairs in one fixed-point chain; "
                     "each phase layer folded into the gates just before it ((D_a x D_b) U per gate on qubits a, b)",
        "parallelism": "replicas" if a.gpus > 1 else "single GPU",
    }


def _peaks(key="hbm_gbs"):
    """Measured peak (MEASURED_PEAKS.json: hbm_gbs or bf16_tflops), else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d[key]), "measured"
    except Exception:
        return (6800.0 if key == "hbm_gbs" else 1900.0), "fallback"


def _traffic(kernel, n):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, scaled to 2^n."""
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            d = json.load(f)
        e = d[kernel]
        return float(e["bytes_per_launch"]) * (2 ** n) / float(e["elements"])
    except Exception:
        return None


def _host_link(host, dev):
    """This machine's host link: a copy of `host` (pinned) to `dev` and one back, each alone on
    its own stream after an untimed copy in the same direction (the first large copy after
    idle runs slower), timed with CUDA events (GB/s); the e2e number depends on it."""
    import torch
    s = torch.cuda.Stream()
    out = {}
    for name in ("h2d", "d2h"):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            for timed in (False, True):
                if timed:
                    e0.record(s)
                if name == "h2d":
                    dev.copy_(host, non_blocking=True)
                else:
                    host.copy_(dev, non_blocking=True)
        e1.record(s)
        torch.cuda.synchronize()
        out[name] = host.numel() * host.element_size() / (e0.elapsed_time(e1) * 1e-3) / 1e9
    return out


class _Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "qtnh_clocks_%d.csv" % os.getpid())

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        loaded = sorted(sm)[len(sm) // 4:] if sm else []
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def _device_state_errors(out, ref):
    """Device tensors -> (relative L2, max |out - ref| / max |ref|, 1 - fidelity). The
    infidelity 1 - |<ref|out>|^2 / (<ref|ref> <out|out>) is computed as the squared norm of
    out's component orthogonal to ref over |out|^2, which keeps its digits far below 1e-16."""
    import torch
    d = out - ref
    rel = (torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref)).item()
    mx = (d.abs().max() / ref.abs().max()).item()
    perp = out - (torch.vdot(ref, out) / torch.vdot(ref, ref)) * ref
    infid = (torch.vdot(perp, perp).real / torch.vdot(out, out).real).item()
    return rel, mx, infid


def _cpu_sample(n, layers, seed, reps=1):
    """Oracle port on one core: seconds per gate-layer at n qubits over `layers` layers."""
    from oracle import oracle as orc
    from qtnh_gb300 import workload as wl
    orc.build()
    c = wl.random_circuit(n, layers, seed=seed)
    psi = wl.random_state(n, seed=seed + 1)
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.run_circuit(psi, c)
    return (time.perf_counter() - t0) / (layers * reps)


def _extrapolate(sec_per_layer, n_sample, n_target):
    # work per layer ~ gates_per_layer * 2^n
    return sec_per_layer * (2.0 ** (n_target - n_sample)) * ((n_target // 2) / (n_sample // 2))


def _sample_desc(n_target, cores):
    return ("oracle port of the reference's Tensor::contract path (scalar C++), %d layer(s) of the same circuit family "
            "at n=%d on %d core(s), extrapolated to n=%d by 2^%d x gates/layer" %
            (CPU_SAMPLE_LAYERS, CPU_SAMPLE_N, cores, n_target, n_target - CPU_SAMPLE_N))


def _worker(args):
    n, layers, seed = args
    return _cpu_sample(n, layers, seed)


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import oracle as orc
    orc.build()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(cores) as pool:
        for step in range(a.warmup + a.steps):
            t0 = time.perf_counter()
            pool.map(_worker, [(CPU_SAMPLE_N, CPU_SAMPLE_LAYERS, a.seed)] * cores)
            dt = time.perf_counter() - t0
            if step >= a.warmup:
                times.append(dt)
    sec_per_layer_sample = statistics.median(times) / (CPU_SAMPLE_LAYERS * cores)
    value = 1.0 / _extrapolate(sec_per_layer_sample, CPU_SAMPLE_N, a.n)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": statistics.median(times) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)", "config": _config(a),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": _sample_desc(a.n, cores) + "; one independent replica per core"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- the drop-in path: workloads through the C++ API (qtnh_gb300/drivers/api_bench.cpp) ----

QFT_METRIC = "QFT networks/s (n=16, TensorNetwork::contractAll through the C++ API)"
API_METRIC = "gate-layers/s through the C++ API (one Tensor::contract per gate)"


def _qft_config(n):
    return {"workload": "QFT on n=%d qubits as a TensorNetwork (random complex Gaussian state, Hadamard SymmTensors, "
                        "controlled-phase DiagTensors, SwapTensor reversals; DIST identities for distributed qubits), "
                        "TensorNetwork::contractAll(order)" % n,
            "qubits": n, "element": "complex128", "l2_flush": "not needed: every run copies its state in and out",
            "parallelism": "single GPU"}


def _qft_oracle_seconds(n, dq, seed):
    """One QFT run of the oracle port (the same contractions, one core)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_qft_gpu import OracleEngine, run_qft
    from oracle import oracle as orc
    orc.build()
    rng = np.random.default_rng(seed)
    psi = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    psi /= np.linalg.norm(psi)
    t0 = time.perf_counter()
    run_qft(OracleEngine(), psi, n, dq, lambda *x: None)
    return time.perf_counter() - t0


def main_qft(a):
    """The reference example's QFT network on n=16 through the C++ API; every run copies the state in
    (DenseTensor::make) and the result out, so value and e2e are the same measurement."""
    import numpy as np
    from qtnh_gb300 import build as bld
    from qtnh_gb300 import workload as wl
    n = 16 if a.n == 28 else a.n
    bld.build()
    if a.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        times = [_qft_oracle_seconds(n, 0, a.seed) for _ in range(a.warmup + a.steps)][a.warmup:]
        sec = statistics.median(times)
        line = {"metric": QFT_METRIC, "value": 1.0 / sec, "unit": "QFT/s", "impl": "reference", "n_gpus": a.gpus,
                "steps": a.steps, "warmup": a.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)",
                "config": _qft_config(n),
                "cpu_baseline": {"value": 1.0 / sec, "unit": "QFT/s", "cores": 1, "kind": "port",
                                 "sample": "one full QFT run (dq = 0) of the oracle port per step"},
                "e2e": {"value": 1.0 / sec, "unit": "QFT/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    cpu = None
    if not a.no_cpu_baseline:
        s0, s1 = _qft_oracle_seconds(n, 0, a.seed), _qft_oracle_seconds(n, 1, a.seed)
        cpu = {"value": 1.0 / s0, "unit": "QFT/s", "cores": 1, "kind": "port",
               "sample": "one full QFT run of the oracle port (dq = 0; dq = 1: %.3f QFT/s)" % (1.0 / s1)}
    rng = np.random.default_rng(a.seed)
    psi = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    psi /= np.linalg.norm(psi)
    tmp = tempfile.mkdtemp(prefix="qtnh_qft_")
    fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    psi.astype(np.complex128).tofile(fin)
    runs = {}
    clocks = _Clocks(0)
    clocks.start()
    for dq in (1, 0):
        runs[dq] = wl.run_api_driver(["qft", n, dq, fin, fout, a.warmup, a.steps])
    ck = clocks.stop()
    # dq = 0 ran last: every gate in place and the swaps reverse the qubits, so the result in
    # its own index order is the discrete Fourier transform of the input
    out = np.fromfile(fout, dtype=np.complex128)
    dft = np.fft.ifft(psi) * math.sqrt(2 ** n)
    err = float(np.linalg.norm(out - dft) / np.linalg.norm(dft))
    v = 1e3 / runs[0]["ms_per_run"]
    line = {"metric": QFT_METRIC, "value": v, "unit": "QFT/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": runs[0]["ms_per_run"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic (seeded state)", "config": _qft_config(n),
            "timing": "host clock around the stream (the C++ API path); every run includes DenseTensor::make's copy "
                      "in and the result's copy out",
            "contractions_per_run": runs[0]["contractions_per_run"],
            "dq1": {"value": 1e3 / runs[1]["ms_per_run"], "ms_per_run": runs[1]["ms_per_run"],
                    "contractions_per_run": runs[1]["contractions_per_run"]},
            "result_check": {"rel_l2_vs_dft": err},
            "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": "QFT/s", "h2d_bytes_per_step": 16 * 2 ** n, "d2h_bytes_per_step": 16 * 2 ** n},
            "clocks": ck, "gpu_launches": None}
    print(json.dumps(line), flush=True)


def main_api(a):
    """The headline circuit through the C++ API: one Tensor::contract per gate and per phase
    diagonal, rescatter/permute/rescatter every 8th layer; the state is made once (seeded)."""
    from qtnh_gb300 import build as bld
    from qtnh_gb300 import workload as wl
    bld.build()
    circ = wl.random_circuit(a.n, a.depth, seed=a.seed)
    tmp = tempfile.mkdtemp(prefix="qtnh_api_")
    fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    wl.write_api_circuit(fin, circ, seed=a.seed + 1)
    clocks = _Clocks(0)
    clocks.start()
    r = wl.run_api_driver(["circuit", fin, fout, a.warmup, a.steps])
    ck = clocks.stop()
    os.remove(fout)
    v = a.depth / (r["ms_per_run"] * 1e-3)
    line = {"metric": API_METRIC, "value": v, "unit": "gate-layers/s", "n_gpus": 1, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": r["ms_per_run"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "arith": a.arith, "data": "synthetic (seeded circuit and state)",
            "config": _config(a),
            "timing": "host clock around the stream; every step applies the circuit through per-gate "
                      "Tensor::contract calls (queued in-place contractions applied as fused layers) and ends with "
                      "Tensor::copy",
            "contractions_per_step": r["contractions_per_run"], "clocks": ck}
    print(json.dumps(line), flush=True)


# ---- dense contraction pairs: split-precision GEMM vs FP64 plain ---------------------

CONTRACT_METRIC = "contraction TFLOP/s (BF16x3 split precision, FP32 accumulation) vs FP64 plain at stated error"
CPU_GEMM_SAMPLE = (128, 128, 128)


def _contract_config(a, pairs, slice_steps=None):
    mnk = [(M, N, K) for _, _, _, M, N, K in pairs]
    return {
        "workload": "%d seeded DenseTensor pairs: ranks 4-6, dims from {2,4,16,32,64}, 2-3 shared indices at random "
                    "positions, <= 2^26 elements per tensor, M,N,K in [256,16384]; entries complex Gaussian, A scaled "
                    "1/sqrt(K)" % len(pairs),
        "pairs": len(pairs),
        "flop_per_step": float(sum(8.0 * M * N * K for M, N, K in mnk)),
        "max_mnk": [int(x) for x in max(mnk, key=lambda t: t[0] * t[1] * t[2])],
        "element": "complex128 in and out",
        "streams": "pairs alternately on two streams (independent contractions)",
        "split_k_slice_steps": slice_steps,
        "l2_flush": "not needed: the operands of a step (GBs) are far larger than the 129 MB L2",
        "parallelism": "replicas" if a.gpus > 1 else "single GPU",
    }


def _cpu_gemm_sample():
    """Oracle port on one core: seconds for one complex contraction of CPU_GEMM_SAMPLE."""
    import numpy as np
    from oracle import oracle as orc
    orc.build()
    M, N, K = CPU_GEMM_SAMPLE
    rng = np.random.default_rng(1)
    t1 = orc.Tensor(orc.DENSE, [], [M, K], rng.standard_normal(M * K) + 1j * rng.standard_normal(M * K))
    t2 = orc.Tensor(orc.DENSE, [], [K, N], rng.standard_normal(K * N) + 1j * rng.standard_normal(K * N))
    t0 = time.perf_counter()
    orc.contract(t1, t2, [(1, 0)])
    return time.perf_counter() - t0


def _gemm_worker(_):
    return _cpu_gemm_sample()


def run_reference_contract(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    M, N, K = CPU_GEMM_SAMPLE
    times = []
    with ctx.Pool(cores) as pool:
        for step in range(a.warmup + a.steps):
            t0 = time.perf_counter()
            pool.map(_gemm_worker, range(cores))
            if step >= a.warmup:
                times.append(time.perf_counter() - t0)
    value = cores * 8.0 * M * N * K / statistics.median(times) / 1e12
    line = {
        "metric": CONTRACT_METRIC, "value": value, "unit": "TFLOP/s", "impl": "reference", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": statistics.median(times) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)",
        "config": {"workload": "complex128 contraction %dx%dx%d, one per host core (the reference's triple loop, "
                               "oracle port)" % (M, N, K)},
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                         "sample": "oracle port of _contract_dense, one %dx%dx%d contraction per core" % (M, N, K)},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main_contract(a):
    import numpy as np
    import torch
    import qtnh_gb300 as q
    from qtnh_gb300 import workload as wl

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        sec = min(_cpu_gemm_sample() for _ in range(2))
        M, N, K = CPU_GEMM_SAMPLE
        cpu = {"value": 8.0 * M * N * K / sec / 1e12, "unit": "TFLOP/s", "cores": 1, "kind": "port",
               "sample": "oracle port of _contract_dense, one %dx%dx%d complex contraction on one core" % (M, N, K)}

    rng = np.random.default_rng(a.seed)
    pairs = [wl.dense_pair(rng, max_elems=a.max_elems) for _ in range(a.pairs)]
    g = torch.Generator(device=dev)
    g.manual_seed(a.seed + 1)
    tens = []
    max_out = 0
    for d1, d2, wires, M, N, K in pairs:
        A = torch.randn(int(np.prod(d1)), dtype=torch.complex128, device=dev, generator=g) / math.sqrt(K)
        B = torch.randn(int(np.prod(d2)), dtype=torch.complex128, device=dev, generator=g)
        tens.append((q.Tensor(q.DENSE, [], d1, A), q.Tensor(q.DENSE, [], d2, B), wires))
        max_out = max(max_out, M * N)
    out = torch.empty(max_out, dtype=torch.complex128, device=dev)
    ref = torch.empty(max_out, dtype=torch.complex128, device=dev)
    flops = sum(8.0 * M * N * K for _, _, _, M, N, K in pairs)
    tensor_flops = sum(48.0 * M * N * K for _, _, _, M, N, K in pairs)  # 6 piece pairs x real form
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()

    # the pairs are independent: they go alternately to two streams (each with its own
    # output buffer), so that one pair's memory-bound kernels (operand splits, split-K
    # reduction) run beside the other's tensor-core GEMM
    side = torch.cuda.Stream()
    out2 = torch.empty_like(out)

    def step(buf, two=True):
        fork = torch.cuda.Event()
        fork.record(stream)
        side.wait_event(fork)
        for i, ((t1, t2, wires), (_, _, _, M, N, _)) in enumerate(zip(tens, pairs)):
            if two and i % 2:
                q.contract(t1, t2, wires, out=out2[:M * N], stream=side)
            else:
                q.contract(t1, t2, wires, out=buf[:M * N], stream=stream)
        join = torch.cuda.Event()
        join.record(side)
        stream.wait_event(join)

    # FP64 plain: one timed pass (the reference numbers of the study) and the errors
    q.set_gemm_precision(q.GEMM_FP64)
    step(out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    step(out)
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)

    # plain on the tensor cores (QTNH_GEMM_OZ6, the default): exact digit products,
    # FP64-level results; timed over the same steps, errors against the FP64 FMA arm
    q.set_gemm_precision(q.GEMM_OZ6)
    q.take_device_errors()
    step(out)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(a.steps):
        step(out)
    e1.record(stream)
    torch.cuda.synchronize()
    oz_ms = e0.elapsed_time(e1) / a.steps
    oz_rels, oz_maxs = [], []
    for (t1, t2, wires), (_, _, _, M, N, _) in zip(tens, pairs):
        q.set_gemm_precision(q.GEMM_FP64)
        q.contract(t1, t2, wires, out=ref[:M * N])
        q.set_gemm_precision(q.GEMM_OZ6)
        q.contract(t1, t2, wires, out=out[:M * N])
        d = out[:M * N] - ref[:M * N]
        oz_rels.append((torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref[:M * N])).item())
        oz_maxs.append((d.abs().max() / ref[:M * N].abs().max()).item())
    oz_errors = q.take_device_errors()

    q.set_gemm_precision(q.GEMM_BF16X3)
    q.take_device_errors()
    rels, maxs = [], []
    for (t1, t2, wires), (_, _, _, M, N, _) in zip(tens, pairs):
        q.set_gemm_precision(q.GEMM_FP64)
        q.contract(t1, t2, wires, out=ref[:M * N])
        q.set_gemm_precision(q.GEMM_BF16X3)
        q.contract(t1, t2, wires, out=out[:M * N])
        d = out[:M * N] - ref[:M * N]
        rels.append((torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref[:M * N])).item())
        maxs.append((d.abs().max() / ref[:M * N].abs().max()).item())

    # split precision: warm-up, then the timed steps
    for _ in range(a.warmup):
        step(out)
    torch.cuda.synchronize()
    clocks = _Clocks(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    q.gemm_timing(True)
    l0 = q.launches()
    e0.record(stream)
    for _ in range(a.steps):
        step(out)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ck = clocks.stop()
    q.gemm_timing(False)
    launches = q.launches() - l0
    ms = e0.elapsed_time(e1)
    # the GEMM kernel's own rate: in the two-stream timed region its launches overlap the
    # other stream's kernels (a launch's events then span time it shares with them), so it
    # is timed on its own in one single-stream pass of the same step right after
    q.gemm_timing(True)
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    step(out, two=False)
    s1.record(stream)
    torch.cuda.synchronize()
    gemm_ms, gemm_launches = q.gemm_timing(False)
    single_ms = s0.elapsed_time(s1)
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * flops * a.steps / (ms * 1e-3) / 1e12
    errors = q.take_device_errors()

    # e2e: host operands copied in, results copied out, every contraction
    hosts = [(t1.data.cpu().pin_memory(), t2.data.cpu().pin_memory()) for t1, t2, _ in tens]
    host_out = torch.empty(max_out, dtype=torch.complex128, pin_memory=True)
    h2d = sum(16 * (t1.data.numel() + t2.data.numel()) for t1, t2, _ in tens)
    d2h = sum(16 * M * N for _, _, _, M, N, _ in pairs)
    # copies on two copy streams: the operands of the pairs LOOK ahead go in while this pair
    # contracts (the host link, not the contractions, is the bound of this arm), results come
    # out of NOUT output buffers in rotation (one copy stream for both directions, as the
    # circuit arm uses, measured 33.7 against 65-70 TFLOP/s here)
    LOOK, NOUT = 8, 4
    h2d_s, d2h_s = torch.cuda.Stream(), torch.cuda.Stream()
    outs = [out] + [torch.empty_like(out) for _ in range(NOUT - 1)]
    in_ev = [torch.cuda.Event() for _ in tens]
    done_ev = [torch.cuda.Event() for _ in tens]
    free_out = [torch.cuda.Event() for _ in range(NOUT)]

    def copy_in(j):
        t1, t2, _ = tens[j]
        ha, hb = hosts[j]
        h2d_s.wait_event(done_ev[j])  # the pair's previous contraction has read its operands
        with torch.cuda.stream(h2d_s):
            t1.data.copy_(ha, non_blocking=True)
            t2.data.copy_(hb, non_blocking=True)
        in_ev[j].record(h2d_s)

    def e2e_run(steps):
        for e in done_ev + free_out:
            e.record(stream)
        barrier()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        h2d_s.wait_event(f0)
        P = len(tens)
        total = steps * P
        look = max(1, min(LOOK, P - 1))  # never ahead of the pair's own previous contraction
        for f in range(min(look, total)):
            copy_in(f % P)
        for f in range(total):
            j = f % P
            (t1, t2, wires), (_, _, _, M, N, _) = tens[j], pairs[j]
            o = outs[f % NOUT]
            stream.wait_event(in_ev[j])
            stream.wait_event(free_out[f % NOUT])
            q.contract(t1, t2, wires, out=o[:M * N])
            done_ev[j].record(stream)
            # pair f + look: its previous contraction (f + look - P < f, or f itself) is queued
            if f + look < total:
                copy_in((f + look) % P)
            d2h_s.wait_event(done_ev[j])
            with torch.cuda.stream(d2h_s):
                host_out[:M * N].copy_(o[:M * N], non_blocking=True)
            free_out[f % NOUT].record(d2h_s)
        stream.wait_stream(d2h_s)
        f1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return f0.elapsed_time(f1)

    e2e_run(1)  # warm-up of the copy path (the first large host copies after idle run slower)
    ems = e2e_run(a.steps)
    if dist is not None:
        t = torch.tensor([ems], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ems = float(t.item())
    e2e = world * flops * a.steps / (ems * 1e-3) / 1e12

    if rank == 0:
        peak, peak_kind = _peaks("bf16_tflops")
        achieved = tensor_flops / (gemm_ms * 1e-3) / 1e12 if gemm_ms else None
        line = {
            "metric": CONTRACT_METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128 (bf16x3 pieces, fp32 accumulation)",
            "data": "synthetic (seeded dense pairs, complex Gaussian entries)", "config": _contract_config(a, pairs, q.get_gemm_slice()),
            "plain_fp64": {"tflops": flops / (plain_ms * 1e-3) / 1e12, "ms_per_step": plain_ms,
                           "speedup_of_split": (flops / (ms / a.steps * 1e-3)) / (flops / (plain_ms * 1e-3))},
            "plain_oz6": {"tflops": flops / (oz_ms * 1e-3) / 1e12, "ms_per_step": oz_ms,
                          "speedup_over_fp64_fma": plain_ms / oz_ms,
                          "error_vs_fp64_fma": {"rel_l2_median": statistics.median(oz_rels), "rel_l2_max": max(oz_rels),
                                                "max_abs_over_max_max": max(oz_maxs)},
                          "device_errors": oz_errors},
            "error_vs_fp64": {"rel_l2_median": statistics.median(rels), "rel_l2_max": max(rels),
                              "max_abs_over_max_median": statistics.median(maxs), "max_abs_over_max_max": max(maxs)},
            "roofline": {"bound": "tensor", "kernel": "gemm_bf16x3_umma_kernel", "achieved": achieved, "peak": peak,
                         "peak_source": peak_kind, "unit": "TFLOP/s",
                         "frac": (achieved / peak) if achieved and peak else None, "traffic": None,
                         "alg_flop_per_step": tensor_flops, "kernel_ms_per_step": gemm_ms,
                         "kernel_launches_per_step": gemm_launches,
                         "kernel_share_of_step": gemm_ms / single_ms if single_ms else None,
                         "timed": "one single-stream pass of the step after the timed region (%.2f ms; "
                                  "the two-stream timed step: %.2f ms)" % (single_ms, ms / a.steps)},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "clocks": ck,
            "gpu_launches": launches,
            "device_errors": errors,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ---- batched uneven circuits in mixed precision -------------------------------------

BATCH_METRIC = "batched gate-layers/s (2048 uneven circuits, complex64, FP64 renormalisation and queries)"


def _batch_bytes(circuits, amp_bytes=8):
    """HBM bytes of one batch run, three ways (complex64 amplitudes of `amp_bytes`):
    per_gate -- the per-kernel algorithmic figure (a gate reads and writes the state,
    2 * amp_bytes per amplitude) summed over every gate, phase layer (the same), swap
    (half the state) and renormalisation (norm read + scale read/write); moved -- what the
    schedule's passes move (two disjoint gates of a layer share one pass, greedy
    consecutive pairing as the executor does), plus the reset copy of the initial states;
    layer -- one read and one write of the state per circuit layer."""
    per_gate = moved = layer = 0
    for c, _ in circuits:
        S = amp_bytes * 2 ** c.n
        moved += 2 * S  # reset from the initial states
        for li, L in enumerate(c.layers):
            g = len(L.gates)
            per_gate += 2 * S * g
            k, passes = 0, 0
            while k < g:
                a, b = L.pairs[k], L.pairs[k + 1] if k + 1 < g else None
                k += 2 if b is not None and not (set(a) & set(b)) else 1
                passes += 1
            moved += 2 * S * passes
            extra = 0
            if L.phases is not None:
                extra += 2 * S
            if L.ptup is not None:
                extra += S
            if (li + 1) % 8 == 0:
                extra += 3 * S  # norm + scale
            per_gate += extra
            moved += extra
            layer += 2 * S
    return {"per_gate": per_gate, "moved": moved, "layer": layer}


def _state_errors(got, ref):
    """Relative L2, largest amplitude error (relative to the largest amplitude) and fidelity
    |<ref|got>|^2 / (|ref|^2 |got|^2) of a state against its FP64 reference."""
    import numpy as np
    nr, ng = np.vdot(ref, ref).real, np.vdot(got, got).real
    # 1 - fidelity as |got_perp|^2 / |got|^2 (got_perp: got's component orthogonal to ref)
    perp = got - (np.vdot(ref, got) / nr) * ref
    infid = float(np.vdot(perp, perp).real / ng)
    return {"rel_l2": float(np.linalg.norm(got - ref) / np.sqrt(nr)),
            "max_abs": float(np.max(np.abs(got - ref)) / np.max(np.abs(ref))),
            "fidelity": 1.0 - infid, "infidelity": infid}


def _worst_state_errors(errs):
    if not errs:
        return None
    return {"rel_l2_max": max(e["rel_l2"] for e in errs), "max_abs_max": max(e["max_abs"] for e in errs),
            "fidelity_min": min(e["fidelity"] for e in errs), "one_minus_fidelity_max":
            max(e["infidelity"] for e in errs)}


def main_batch(a):
    import numpy as np
    import torch
    import qtnh_gb300 as q
    from qtnh_gb300 import workload as wl

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        spl = _cpu_sample(CPU_SAMPLE_N, CPU_SAMPLE_LAYERS, a.seed)
        cpu = {"value": 1.0 / _extrapolate(spl, CPU_SAMPLE_N, 16), "unit": "gate-layers/s", "cores": 1, "kind": "port",
               "sample": "oracle port (scalar C++), %d layers of a random circuit at n=%d on one core, scaled to the "
                         "batch's amplitude-weighted mean circuit (~n=16)" % (CPU_SAMPLE_LAYERS, CPU_SAMPLE_N)}

    t_gen = time.perf_counter()
    circuits = wl.batch_circuits(a.circuits, seed=a.seed)
    b = q.Batch([c.n for c, _ in circuits])
    g = torch.Generator(device=dev)
    g.manual_seed(a.seed + 1)
    for i, (c, qi) in enumerate(circuits):
        psi = torch.randn(2 ** c.n, dtype=torch.complex128, device=dev, generator=g)
        psi /= torch.linalg.vector_norm(psi)
        b.set_state(i, psi)
        b.add_circuit(i, c, qi)
    b.compile(renorm_every=8, autotune=True)
    t_gen = time.perf_counter() - t_gen
    info = b.info()
    layers = sum(len(c.layers) for c, _ in circuits)
    gates = sum(c.gate_count() for c, _ in circuits)
    stream = torch.cuda.current_stream()

    for _ in range(a.warmup):
        b.run()
    torch.cuda.synchronize()
    clocks = _Clocks(local)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = q.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        b.run()
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    launches = q.launches() - l0
    ms = e0.elapsed_time(e1)
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    sec = ms / a.steps * 1e-3
    value = world * layers / sec
    res = b.results().cpu().numpy()

    # error against FP64 on the smaller circuits (oracle port, host)
    errs, state_errs = [], []
    if rank == 0:
        from oracle import oracle as orc
        orc.build()
        off = np.cumsum([0] + [len(qi) for _, qi in circuits])
        small = sorted(range(len(circuits)), key=lambda i: (circuits[i][0].n, len(circuits[i][0].layers)))[:12]
        g2 = torch.Generator(device=dev)  # the same seeded initial states
        g2.manual_seed(a.seed + 1)
        inits = {}
        for i, (c, _) in enumerate(circuits):
            psi = torch.randn(2 ** c.n, dtype=torch.complex128, device=dev, generator=g2)
            if i in small:
                inits[i] = (psi / torch.linalg.vector_norm(psi)).cpu().numpy()
        for i in small:
            c, qi = circuits[i]
            full = orc.run_circuit(inits[i], c)
            ref = full[qi.astype(np.int64)]
            got = res[off[i]:off[i + 1]]
            errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
            st = b.state(i).cpu().numpy()
            state_errs.append(_state_errors(st, full))

    # e2e: initial states from pinned host memory (complex128), results back to the host
    # (one pinned host block; the next step's states are copied into a device staging block
    # on a copy stream while the current step's graph runs, then converted in place)
    offs = np.cumsum([0] + [2 ** c.n for c, _ in circuits]).tolist()
    host_all = torch.empty(offs[-1], dtype=torch.complex128, pin_memory=True)
    g3 = torch.Generator(device=dev)
    g3.manual_seed(a.seed + 1)
    for i, (c, _) in enumerate(circuits):
        psi = torch.randn(2 ** c.n, dtype=torch.complex128, device=dev, generator=g3)
        host_all[offs[i]:offs[i + 1]].copy_((psi / torch.linalg.vector_norm(psi)).cpu())
    dev_stage = torch.empty(offs[-1], dtype=torch.complex128, device=dev)
    host_res = torch.empty(max(1, b.nqueries), dtype=torch.complex128, pin_memory=True)
    dres = torch.empty(max(1, b.nqueries), dtype=torch.complex128, device=dev)
    h2d_s = torch.cuda.Stream()
    in_ev, free_ev = torch.cuda.Event(), torch.cuda.Event()
    free_ev.record(stream)

    def copy_in():
        h2d_s.wait_event(free_ev)  # the previous states were converted into the batch
        with torch.cuda.stream(h2d_s):
            dev_stage.copy_(host_all, non_blocking=True)
        in_ev.record(h2d_s)

    def e2e_run(steps):
        free_ev.record(stream)
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        h2d_s.wait_event(f0)
        copy_in()
        for st in range(steps):
            stream.wait_event(in_ev)
            for i in range(len(circuits)):
                b.set_state(i, dev_stage[offs[i]:offs[i + 1]])
            free_ev.record(stream)
            if st + 1 < steps:
                copy_in()
            b.run()
            b.results(out=dres)
            host_res.copy_(dres, non_blocking=True)
        f1.record(stream)
        torch.cuda.synchronize()
        return f0.elapsed_time(f1)

    e2e_run(1)  # warm-up of the copy path (the first large host copy after idle runs slower)
    ems = e2e_run(a.steps)
    e2e = world * layers / (ems / a.steps * 1e-3)
    h2d = 16 * offs[-1]
    del dev_stage

    # the plain method on the same circuits and schedule (complex128 states, FP64 math, no
    # renormalisation): the reference point of the mixed-precision speed-up, and the FP64
    # states the mixed states are compared with (all queries; full states of the largest
    # circuits). One warm-up and one timed run: it is several times slower.
    bp = q.Batch([c.n for c, _ in circuits], precision=q.STATE_C128)
    g4 = torch.Generator(device=dev)
    g4.manual_seed(a.seed + 1)
    for i, (c, qi) in enumerate(circuits):
        psi = torch.randn(2 ** c.n, dtype=torch.complex128, device=dev, generator=g4)
        bp.set_state(i, psi / torch.linalg.vector_norm(psi))
        bp.add_circuit(i, c, qi)
    bp.compile(renorm_every=0, autotune=True)
    bp.run()
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    bp.run()
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1)
    if dist is not None:
        t = torch.tensor([plain_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        plain_ms = float(t.item())
    plain_value = world * layers / (plain_ms * 1e-3)
    pres = bp.results().cpu().numpy()
    offq = np.cumsum([0] + [len(qi) for _, qi in circuits])
    q_vs_plain = [float(np.linalg.norm(res[offq[i]:offq[i + 1]] - pres[offq[i]:offq[i + 1]]) /
                        np.linalg.norm(pres[offq[i]:offq[i + 1]])) for i in range(len(circuits))]
    largest = sorted(range(len(circuits)), key=lambda i: -circuits[i][0].n)[:8]
    plain_states = {i: bp.state(i).cpu().numpy() for i in largest}
    s_vs_plain = [_state_errors(b.state(i).cpu().numpy(), plain_states[i]) for i in largest]
    del bp

    # the plain method with the fastest plain arithmetic the grouped kernels have: complex128
    # states, gates in float-float (QTNH_BATCH_GATES=f32x2: FP64-level results at FP32
    # speed); the reference point of the speed-up beside the FP64 one
    os.environ["QTNH_BATCH_GATES"] = "f32x2"
    bq = q.Batch([c.n for c, _ in circuits], precision=q.STATE_C128)
    g6 = torch.Generator(device=dev)
    g6.manual_seed(a.seed + 1)
    for i, (c, qi) in enumerate(circuits):
        psi = torch.randn(2 ** c.n, dtype=torch.complex128, device=dev, generator=g6)
        bq.set_state(i, psi / torch.linalg.vector_norm(psi))
        bq.add_circuit(i, c, qi)
    bq.compile(renorm_every=0, autotune=True)
    del os.environ["QTNH_BATCH_GATES"]
    bq.run()
    torch.cuda.synchronize()
    p0.record(stream)
    for _ in range(a.steps):
        bq.run()
    p1.record(stream)
    torch.cuda.synchronize()
    ff_ms = p0.elapsed_time(p1) / a.steps
    ffres = bq.results().cpu().numpy()
    ff_vs_fp64 = max(float(np.linalg.norm(ffres[offq[i]:offq[i + 1]] - pres[offq[i]:offq[i + 1]]) /
                           np.linalg.norm(pres[offq[i]:offq[i + 1]])) for i in range(len(circuits)))
    del bq

    # the same complex64 batch with FP32 gate sums (QTNH_BATCH_GATES=fp32): the faster,
    # less accurate point of the trade-off
    os.environ["QTNH_BATCH_GATES"] = "fp32"
    bf = q.Batch([c.n for c, _ in circuits])
    g5 = torch.Generator(device=dev)
    g5.manual_seed(a.seed + 1)
    for i, (c, qi) in enumerate(circuits):
        psi = torch.randn(2 ** c.n, dtype=torch.complex128, device=dev, generator=g5)
        bf.set_state(i, psi / torch.linalg.vector_norm(psi))
        bf.add_circuit(i, c, qi)
    bf.compile(renorm_every=8, autotune=True)
    del os.environ["QTNH_BATCH_GATES"]
    bf.run()
    torch.cuda.synchronize()
    p0.record(stream)
    for _ in range(a.steps):
        bf.run()
    p1.record(stream)
    torch.cuda.synchronize()
    fp32_ms = p0.elapsed_time(p1) / a.steps
    fres = bf.results().cpu().numpy()
    f_vs_plain = [float(np.linalg.norm(fres[offq[i]:offq[i + 1]] - pres[offq[i]:offq[i + 1]]) /
                        np.linalg.norm(pres[offq[i]:offq[i + 1]])) for i in range(len(circuits))]
    fs_vs_plain = [_state_errors(bf.state(i).cpu().numpy(), plain_states[i]) for i in largest]
    del bf, plain_states

    if rank == 0:
        byts = _batch_bytes(circuits)
        peak, peak_kind = _peaks()
        achieved = byts["per_gate"] / sec / 1e9
        line = {
            "metric": BATCH_METRIC, "value": value, "unit": "gate-layers/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 (gates: exact 64-bit fixed-point sums; FP64 renormalisation every 8 "
                                             "layers, complex128 queries)",
            "data": "synthetic (seeded circuits and states)",
            "config": {"workload": "%d independent circuits, qubits U{10..22}, depth U{8..32}, Haar two-qubit gates on "
                                   "random pairings, phase layer every 4th layer, a SwapTensor with probability 1/4 "
                                   "per layer, 64 seeded amplitude queries each" % len(circuits),
                       "circuits": len(circuits), "layers": layers, "gates": gates,
                       "amplitudes": info["amplitudes"], "rounds": info["rounds"],
                       "graph_launches_per_step": info["launches_per_run"],
                       "autotuned": {"gate_threads": info["gate_threads"], "gate_chunk_groups": info["gate_chunk"]},
                       "host_build_s": t_gen, "l2_flush": "not needed: states total GBs, far beyond the 129 MB L2",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "circuits_per_s": world * len(circuits) / sec,
            "error_vs_fp64": {"circuits_checked": len(errs), "queries_rel_l2_max": max(errs) if errs else None,
                              "queries_rel_l2_median": statistics.median(errs) if errs else None,
                              "states": _worst_state_errors(state_errs)},
            "plain_c128": {"value": plain_value, "unit": "gate-layers/s", "ms_per_step": plain_ms, "steps": 1,
                           "dtype": "c128 (FP64 math, same rounds and graph)",
                           "speedup_of_mixed": value / plain_value,
                           "mixed_vs_plain": {"queries_rel_l2_max": max(q_vs_plain),
                                              "queries_rel_l2_median": statistics.median(q_vs_plain),
                                              "largest_states": _worst_state_errors(s_vs_plain),
                                              "states_checked": len(s_vs_plain)}},
            "plain_c128_f32x2": {"value": world * layers / (ff_ms * 1e-3), "unit": "gate-layers/s", "ms_per_step": ff_ms,
                                 "dtype": "c128 (gates in float-float, same rounds and graph)",
                                 "speedup_of_mixed": value / (world * layers / (ff_ms * 1e-3)),
                                 "queries_rel_l2_max_vs_fp64": ff_vs_fp64},
            "fp32_gates": {"value": world * layers / (fp32_ms * 1e-3), "unit": "gate-layers/s", "ms_per_step": fp32_ms,
                           "speedup_of_plain": (world * layers / (fp32_ms * 1e-3)) / plain_value,
                           "vs_plain": {"queries_rel_l2_max": max(f_vs_plain),
                                        "queries_rel_l2_median": statistics.median(f_vs_plain),
                                        "largest_states": _worst_state_errors(fs_vs_plain)}},
            "roofline": {"bound": "hbm", "kernel": "whole graph (grouped pair kernel dominant)", "achieved": achieved,
                         "peak": peak, "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "alg_bytes_per_step": byts["per_gate"],
                         "note": "algorithmic bytes per gate; two gates share one pass, so this can exceed 1",
                         "moved_bytes_per_step": byts["moved"],
                         "moved_frac": byts["moved"] / sec / 1e9 / peak,
                         "layer_bytes_per_step": byts["layer"],
                         "layer_frac": byts["layer"] / sec / 1e9 / peak},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": "gate-layers/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 16 * b.nqueries},
            "clocks": ck,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ---- request loop ---------------------------------------------------------------------

SERVE_METRIC = "serving p99 latency (mixed complex64; p50, throughput and plain complex128 beside it)"


def main_serve(a):
    import numpy as np
    import torch
    import qtnh_gb300 as q
    from qtnh_gb300 import serve

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    cpu = None
    if rank == 0 and not a.no_cpu_baseline:
        spl = _cpu_sample(CPU_SAMPLE_N, CPU_SAMPLE_LAYERS, a.seed)
        cpu = {"value": 1.0 / _extrapolate(spl, CPU_SAMPLE_N, 16), "unit": "gate-layers/s", "cores": 1, "kind": "port",
               "sample": "oracle port (scalar C++), %d layers of a random circuit at n=%d on one core, scaled to "
                         "n=16" % (CPU_SAMPLE_LAYERS, CPU_SAMPLE_N)}
    reqs = serve.request_stream(a.requests, rate=400.0, seed=a.seed)
    warm = serve.request_stream(4, rate=4000.0, seed=a.seed + 99, qubits=(12, 16), depth=(10, 12))
    out = {}
    # mixed: complex64 states; plain: complex128 states in FP64; plain_f32x2: complex128
    # states, gates in float-float (QTNH_BATCH_GATES=f32x2, the fastest plain arithmetic of
    # the grouped kernels)
    for name, prec in (("mixed", serve.C64), ("plain", serve.C128), ("plain_f32x2", serve.C128)):
        if name == "plain_f32x2":
            os.environ["QTNH_BATCH_GATES"] = "f32x2"
        ex = serve.GpuExecutor(prec)
        serve.serve(warm, ex, renorm_every=8 if prec == serve.C64 else 0)
        torch.cuda.synchronize()
        clocks = _Clocks(local)
        clocks.start()
        l0 = q.launches()
        lat, results, stats = serve.serve(reqs, ex, budget_bytes=150e9, renorm_every=8 if prec == serve.C64 else 0)
        stats["clocks"] = clocks.stop()
        stats["gpu_launches"] = q.launches() - l0
        out[name] = (stats, results)
        os.environ.pop("QTNH_BATCH_GATES", None)
    errs = []
    for r in reqs:
        a_, b_ = np.asarray(out["mixed"][1][r.rid]), np.asarray(out["plain"][1][r.rid])
        errs.append(float(np.linalg.norm(a_ - b_) / np.linalg.norm(b_)))
    ms, ps = out["mixed"][0], out["plain"][0]
    # the same stream at an arrival rate the mixed path sustains (3/4 of its measured
    # request throughput at 400/s): latency without the queueing of an overloaded stream
    sus_rate = 0.75 * ms["requests_per_s"]
    sus_reqs = serve.request_stream(a.requests, rate=sus_rate, seed=a.seed)
    ex = serve.GpuExecutor(serve.C64)
    _, _, sus = serve.serve(sus_reqs, ex, budget_bytes=150e9, renorm_every=8)
    if rank == 0:
        gate_bytes = sum(16 * 16 * len(layer.gates) for r in reqs for layer in r.circuit.layers)
        answer_bytes = sum(16 * (256 if r.kind == "amps" else 256) for r in reqs)
        line = {
            "metric": SERVE_METRIC, "value": ms["p99_ms"], "unit": "ms", "n_gpus": 1, "steps": ms["steps"],
            "warmup": 1, "ms_per_step": ms["makespan_s"] * 1e3 / max(1, ms["steps"]), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 (mixed) vs c128 (plain)",
            "data": "synthetic (seeded Poisson request stream, seeded circuits and states)",
            "config": {"workload": "%d requests, Poisson arrivals at 400/s, qubits log-uniform 12..26, depth 10..60, "
                                   "Haar two-qubit gates, phase layer every 4th, every 8th layer the top 3 indices "
                                   "exchanged with 3 random local ones, "
                                   "256 amplitudes or a 4-qubit reduced density matrix each; 150 GB admission budget; "
                                   "all active requests advance one layer per grouped step" % len(reqs),
                       "requests": len(reqs), "rate_per_s": 400.0, "budget_bytes": 150e9,
                       "parallelism": "single GPU"},
            "mixed": {k: ms[k] for k in ("p50_ms", "p99_ms", "mean_ms", "requests_per_s", "gate_layers_per_s",
                                         "makespan_s", "steps")},
            "plain": {k: ps[k] for k in ("p50_ms", "p99_ms", "mean_ms", "requests_per_s", "gate_layers_per_s",
                                         "makespan_s", "steps")},
            "plain_f32x2": dict({k: out["plain_f32x2"][0][k] for k in ("p50_ms", "p99_ms", "mean_ms", "requests_per_s",
                                                                       "gate_layers_per_s", "makespan_s")},
                                answers_rel_max_vs_fp64=max(
                                    float(np.linalg.norm(np.asarray(out["plain_f32x2"][1][r.rid]) -
                                                         np.asarray(out["plain"][1][r.rid])) /
                                          np.linalg.norm(np.asarray(out["plain"][1][r.rid]))) for r in reqs)),
            "error_mixed_vs_plain": {"rel_max": max(errs), "rel_median": statistics.median(errs)},
            "mixed_sustainable_load": dict({k: sus[k] for k in ("p50_ms", "p99_ms", "mean_ms", "requests_per_s",
                                                                "gate_layers_per_s", "makespan_s")},
                                           rate_per_s=sus_rate),
            "cpu_baseline": cpu,
            "e2e": {"value": ms["p99_ms"], "unit": "ms", "h2d_bytes_per_step": gate_bytes / max(1, ms["steps"]),
                    "d2h_bytes_per_step": answer_bytes / max(1, ms["steps"])},
            "clocks": ms["clocks"],
            "gpu_launches": ms["gpu_launches"],
        }
        print(json.dumps(line), flush=True)


KERNELS_METRIC = "plain complex128 kernels: achieved HBM GB/s per kernel (fraction of measured copy bandwidth)"


def main_kernels(a):
    """The plain path's data-movement and streaming kernels one by one on a 2^n-amplitude
    complex128 state (n = 28: 4 GiB, far beyond L2): permutes (rescatter-style index
    exchanges, a full reversal, Tensor::swap), DiagTensor contractions (the QFT's
    controlled phase, a per-qubit phase layer), one-, two- and four-qubit SymmTensor
    gates in each arithmetic, and the FP64-accurate norm. Each case: 3 warm-up launches, then `steps` launches timed with CUDA events;
    algorithmic bytes are the state read and written once (32 B per amplitude; the norm
    reads it, 16 B)."""
    import numpy as np
    import torch
    import qtnh_gb300 as q

    n = a.n
    N = 2 ** n
    dims = [2] * n
    reps = max(3, a.steps)
    peak, peak_kind = _peaks()

    cpu = None
    if not a.no_cpu_baseline:
        from oracle import oracle as orc
        orc.build()
        ns = 22
        xh = (np.random.default_rng(1).standard_normal(2 ** ns) + 0j).reshape([2] * ns)
        pt = list(range(ns))
        pt[0:3], pt[ns - 3:ns] = pt[ns - 3:ns], pt[0:3]
        t0 = time.perf_counter()
        for _ in range(3):
            orc.permute(xh, pt)
        sec = (time.perf_counter() - t0) / 3
        cpu = {"value": 32 * 2 ** ns / sec / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": "oracle port permute (scalar C++, one core) of a 2^22-element complex128 tensor, top 3 and "
                         "bottom 3 axes exchanged, 3 repetitions"}

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(a.seed)
    x = torch.randn(N, dtype=torch.complex128, device=dev, generator=g)
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(a.seed)
    theta = float(rng.uniform(0, 2 * math.pi))
    cphase = torch.tensor([1, 1, 1, complex(math.cos(theta), math.sin(theta))], dtype=torch.complex128, device=dev)
    ph = rng.uniform(0, 2 * math.pi, n)
    factors = torch.tensor(np.stack([np.ones(n), np.exp(1j * ph)], axis=1).reshape(-1), dtype=torch.complex128,
                           device=dev)
    m = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    u, _ = np.linalg.qr(m)
    gate = torch.tensor(np.ascontiguousarray(u.T).reshape(-1), dtype=torch.complex128, device=dev)
    m4 = rng.standard_normal((16, 16)) + 1j * rng.standard_normal((16, 16))
    u4, _ = np.linalg.qr(m4)
    gate4 = torch.tensor(np.ascontiguousarray(u4.T).reshape(-1), dtype=torch.complex128, device=dev)
    t4 = [2, 9, n - 12, n - 3]
    h1 = torch.tensor(np.array([1, 1, 1, -1]) / math.sqrt(2.0), dtype=torch.complex128, device=dev)  # Hadamard

    def top3_with(lo):
        pt = list(range(n))
        for i in range(3):
            pt[i], pt[lo + i] = lo + i, i
        return pt

    rev = [n - 1 - i for i in range(n)]
    cases = [
        ("permute: top 3 <-> axes %d..%d" % (n // 2, n // 2 + 2), "fp64", 32,
         lambda: q.permute(x, dims, top3_with(n // 2), out=y)),
        ("permute: top 3 <-> innermost 3", "fp64", 32, lambda: q.permute(x, dims, top3_with(n - 3), out=y)),
        ("permute: full reversal", "fp64", 32, lambda: q.permute(x, dims, rev, out=y)),
        ("swap: axes 0 <-> %d" % (n - 1), "fp64", 32, lambda: q.swap(x, dims, 0, n - 1, out=y)),
        ("diag: controlled phase on (3, %d)" % (n - 5), "fp64", 32, lambda: q.apply_diag(x, dims, [3, n - 5], cphase)),
        ("diag: controlled phase on (3, %d)" % (n - 5), "f32x2", 32,
         lambda: q.apply_diag(x, dims, [3, n - 5], cphase)),
        ("diag: controlled phase on (3, %d)" % (n - 5), "bf16x6", 32,
         lambda: q.apply_diag(x, dims, [3, n - 5], cphase)),
        ("diag layer: %d per-qubit phases" % n, "fp64", 32,
         lambda: q.apply_diag_layer(x, dims, list(range(n)), factors)),
        ("diag layer: %d per-qubit phases" % n, "f32x2", 32,
         lambda: q.apply_diag_layer(x, dims, list(range(n)), factors)),
        ("diag layer: %d per-qubit phases" % n, "bf16x6", 32,
         lambda: q.apply_diag_layer(x, dims, list(range(n)), factors)),
        ("gate: two-qubit SymmTensor on (4, %d)" % (n - 3), "fp64", 32, lambda: q.apply_gate(x, dims, [4, n - 3], gate)),
        ("gate: two-qubit SymmTensor on (4, %d)" % (n - 3), "f32x2", 32,
         lambda: q.apply_gate(x, dims, [4, n - 3], gate)),
        ("gate: two-qubit SymmTensor on (4, %d)" % (n - 3), "bf16x6", 32,
         lambda: q.apply_gate(x, dims, [4, n - 3], gate)),
        ("gate: one-qubit SymmTensor (Hadamard) on %d" % (n - 6), "fp64", 32,
         lambda: q.apply_gate(x, dims, [n - 6], h1)),
        ("gate: one-qubit SymmTensor (Hadamard) on %d" % (n - 6), "f32x2", 32,
         lambda: q.apply_gate(x, dims, [n - 6], h1)),
        ("gate: four-qubit SymmTensor on (%d, %d, %d, %d)" % tuple(t4), "f32x2", 32,
         lambda: q.apply_gate(x, dims, t4, gate4)),
        ("gate: four-qubit SymmTensor on (%d, %d, %d, %d)" % tuple(t4), "bf16x6", 32,
         lambda: q.apply_gate(x, dims, t4, gate4)),
        ("norm: sum of squares (FP64-accurate)", "bf16x6", 16, lambda: q.norm2(x)),
    ]
    old = q.get_arithmetic()
    out = {}
    clocks = _Clocks(0)
    torch.cuda.synchronize()
    clocks.start()
    l0 = q.launches()
    for name, arith, bpe, fn in cases:
        q.set_arithmetic(q.ARITH_NAMES[arith])
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        gbs = bpe * N / (ms * 1e-3) / 1e9
        label = {"fp64": "fp64", "f32x2": "f32x2",
                 "bf16x6": "default: tensor cores" if name.startswith("gate")
                 else "default: fp64 + f32x2"}[arith]
        out["%s [%s]" % (name, label)] = {"ms": ms, "gbs": gbs, "frac": gbs / peak, "bytes": bpe * N}
    launches = q.launches() - l0
    ck = clocks.stop()
    q.set_arithmetic(old)
    assert q.take_device_errors() == 0

    # e2e: a permute through the C ABI with host buffers (pinned), copies inside the timed region
    hx = x.cpu().pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    pt = top3_with(n // 2)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(reps):
        x.copy_(hx, non_blocking=True)
        q.permute(x, dims, pt, out=y)
        hy.copy_(y, non_blocking=True)
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = f0.elapsed_time(f1) / reps

    # the headline: permutes, the swap and the diagonals as the default arithmetic runs them;
    # the pure FP64 / float-float variants, the gate and the FP64 norm stay listed per kernel
    hbm_cases = {k: v for k, v in out.items()
                 if k.startswith(("permute", "swap")) or (k.startswith("diag") and "default" in k)}
    worst = min(hbm_cases, key=lambda k: hbm_cases[k]["frac"])
    line = {
        "metric": KERNELS_METRIC, "value": hbm_cases[worst]["frac"], "unit": "fraction of measured HBM (worst case)",
        "n_gpus": 1, "steps": reps, "warmup": 3, "ms_per_step": sum(v["ms"] for v in out.values()),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded state, gates and phases)",
        "config": {"workload": "plain-path kernels one by one on a 2^%d-amplitude complex128 state" % n,
                   "qubits": n, "state_bytes": 16 * N,
                   "l2_flush": "not needed: the %d MiB state is larger than the 129 MB L2" % (16 * N >> 20)},
        "kernels": out,
        "roofline": {"bound": "hbm", "kernel": worst, "achieved": hbm_cases[worst]["gbs"], "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": hbm_cases[worst]["frac"], "traffic": None},
        "cpu_baseline": cpu,
        "e2e": {"value": 32 * N / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s (permute with host copies)",
                "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 16 * N},
        "clocks": ck,
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


def main():
    a = _args()
    if a.workload == "kernels":
        if a.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the kernels workload has no reference arm: it "
                              "times this engine's kernels one by one"}))
        else:
            main_kernels(a)
        return
    if a.workload == "serve":
        if a.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the serving workload has no reference arm: the "
                              "reference has no request loop; its CPU gate-layer rate is the batch and circuit "
                              "workloads' reference arm"}))
        else:
            main_serve(a)
        return
    if a.workload == "batch":
        if a.impl == "reference":
            a.n = 16
            run_reference(a)
        else:
            main_batch(a)
        return
    if a.workload == "qft":
        main_qft(a)
        return
    if a.workload == "api":
        if a.impl == "reference":
            run_reference(a)
        else:
            main_api(a)
        return
    if a.workload == "contract":
        if a.impl == "reference":
            run_reference_contract(a)
        else:
            main_contract(a)
        return
    if a.impl == "reference":
        run_reference(a)
        return

    import torch
    import qtnh_gb300 as q
    from qtnh_gb300.circuit import DeviceCircuit
    from qtnh_gb300 import workload as wl

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    # CPU baseline first (before any GPU work, single core), rank 0 only.
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        spl = _cpu_sample(CPU_SAMPLE_N, CPU_SAMPLE_LAYERS, a.seed)
        cpu = {"value": 1.0 / _extrapolate(spl, CPU_SAMPLE_N, a.n), "unit": UNIT, "cores": 1, "kind": "port",
               "sample": _sample_desc(a.n, 1)}

    q.set_arithmetic(q.ARITH_NAMES[a.arith])
    circ = wl.random_circuit(a.n, a.depth, seed=a.seed)
    dc = DeviceCircuit(circ, device=dev)
    N = 2 ** a.n
    g = torch.Generator(device=dev)
    g.manual_seed(a.seed + 1)
    state = torch.randn(N, dtype=torch.complex128, device=dev, generator=g)
    state /= torch.linalg.vector_norm(state)
    scratch = torch.empty_like(state)
    host_in = torch.empty(N, dtype=torch.complex128, pin_memory=True)
    host_in.copy_(state)
    host_out = torch.empty(N, dtype=torch.complex128, pin_memory=True)
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()

    # warm-up
    cur, oth = state, scratch
    for _ in range(a.warmup):
        res = dc.run(cur, oth)
        if res is not cur:
            cur, oth = oth, cur
    torch.cuda.synchronize()

    # timed region: device-resident
    clocks = _Clocks(local)
    events = {}
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = q.launches()
    q.gate_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        res = dc.run(cur, oth, events=events)
        if res is not cur:
            cur, oth = oth, cur
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ck = clocks.stop()
    launches = q.launches() - l0
    pass_ms, pass_launches = q.gate_timing(False)
    ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    ms_per_step = ms / a.steps
    value = world * a.depth * a.steps / (ms / 1e3)

    # roofline of the dominant kernel (two-qubit gate kernel; with bf16x6 the fused
    # gate-pair passes, one launch per pair of gates: the first pass of a chain by the
    # pair kernel, the others by the fixed-point chain kernel). With bf16x6 the library
    # times every pass with CUDA events on the launch stream (qtnh_gate_timing); the
    # other arithmetics take the span of the gate calls over their gate count.
    runs_ms = sum(s.elapsed_time(e) for s, e in events.get("runs", []))
    diag_ms = sum(s.elapsed_time(e) for s, e in events.get("diag", []))
    kernel = {"f32x2": "gate_kernel_f32x2<4>", "fp64": "gate_kernel<4>",
              "bf16x6": "gate_pair_chain_kernel + gate_pair_umma_kernel"}[a.arith]
    if a.arith == "bf16x6" and pass_launches:
        gate_launch_ms = pass_ms / pass_launches
        gates_ms = pass_ms
    else:
        gate_launch_ms = runs_ms / (a.steps * dc.gate_count) if dc.gate_count else None
        gates_ms = runs_ms
    alg_bytes = 32.0 * N
    peak, peak_kind = _peaks()
    achieved = alg_bytes / (gate_launch_ms * 1e-3) / 1e9 if gate_launch_ms else None
    # perm: the rest of the gate-run calls (the permutations and the gaps between launches)
    share = {"gates": gates_ms / ms, "diag": diag_ms / ms, "perm": max(0.0, runs_ms - gates_ms) / ms}

    # e2e through the C ABI with host buffers: every step copies its input state from
    # pinned host memory and its result back, with three state buffers in rotation so that
    # step i-1's result copy and step i+1's input copy both run during step i. The copies go
    # one after the other on one copy stream: on these hosts a host-to-device copy that runs
    # beside a device-to-host one slows to a fraction of its speed alone (4 GiB each way:
    # 273 ms and 78 ms together against ~21 ms and ~22 ms one after the other)
    NB = 3
    h2d_s = torch.cuda.Stream()
    d2h_s = h2d_s
    bufs = [(cur, oth)] + [(torch.empty_like(cur), torch.empty_like(cur)) for _ in range(NB - 1)]
    in_ev = [torch.cuda.Event() for _ in range(NB)]
    free_ev = [torch.cuda.Event() for _ in range(NB)]
    done_ev = torch.cuda.Event()

    def copy_in(i):
        c = bufs[i % NB][0]
        h2d_s.wait_event(free_ev[i % NB])  # that buffer's previous result has been copied out
        q.check(q.lib().qtnh_memcpy_h2d(q._ptr(c), q._ptr(host_in), q.ctypes.c_size_t(16 * N), q._stream(h2d_s)))
        in_ev[i % NB].record(h2d_s)

    warm_ev = torch.cuda.Event()

    def e2e_run(steps):
        for e in free_ev:
            e.record(stream)
        barrier()
        torch.cuda.synchronize()
        # the host link idles while the ranks synchronize, and the first large copy after
        # an idle period runs several times slower: a 256 MiB copy just before the timed
        # region wakes it (untimed; every step's own copies are inside the region)
        w = min(N, 1 << 24)
        q.check(q.lib().qtnh_memcpy_h2d(q._ptr(bufs[0][1]), q._ptr(host_in), q.ctypes.c_size_t(16 * w),
                                        q._stream(h2d_s)))
        warm_ev.record(h2d_s)
        stream.wait_event(warm_ev)
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        h2d_s.wait_event(f0)
        copy_in(0)
        for i in range(steps):
            c, o = bufs[i % NB]
            stream.wait_event(in_ev[i % NB])
            res = dc.run(c, o)
            done_ev.record(stream)
            if i + 1 < steps:
                copy_in(i + 1)
            d2h_s.wait_event(done_ev)
            q.check(q.lib().qtnh_memcpy_d2h(q._ptr(host_out), q._ptr(res), q.ctypes.c_size_t(16 * N), q._stream(d2h_s)))
            free_ev[i % NB].record(d2h_s)
        stream.wait_stream(d2h_s)
        f1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return f0.elapsed_time(f1), res

    # warm-up of the copy path (the fresh state buffers and the pinned host buffers: the
    # first copy into a buffer runs several times slower), then the timed steps
    e2e_run(max(NB, min(a.warmup, 2 * NB)))
    ems, res = e2e_run(a.steps)
    last_c, last_o = bufs[(a.steps - 1) % NB]
    cur, oth = (res, last_o) if res is last_c else (res, last_c)
    del bufs
    if dist is not None:
        t = torch.tensor([ems], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ems = float(t.item())
    e2e = world * a.depth * a.steps / (ems / 1e3)
    norm = q.norm2(cur)
    link = _host_link(host_in, oth)  # (oth: a scratch state buffer)

    # circuit-level cross-check of the timed arithmetic against native FP64 on the same input
    arith_check = None
    if not a.no_arith_check:
        outs = {}
        mode = a.arith if a.arith != "fp64" else "f32x2"
        for m in (mode, "fp64"):
            q.set_arithmetic(q.ARITH_NAMES[m])
            cur.copy_(host_in)
            res = dc.run(cur, oth)
            outs[m] = res.clone()
        q.set_arithmetic(q.ARITH_NAMES[a.arith])
        rel, mx, infid = _device_state_errors(outs[mode], outs["fp64"])
        arith_check = {"circuit_rel_l2_%s_vs_fp64" % mode: rel,
                       "circuit_max_abs_rel_%s_vs_fp64" % mode: mx,
                       "circuit_infidelity_%s_vs_fp64" % mode: infid,
                       "gates": dc.gate_count, "qubits": a.n}
        del outs

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "arith": a.arith,
            "data": "synthetic (seeded circuit; state i.i.d. complex Gaussian, unit L2)",
            "config": _config(a),
            "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak,
                         "peak_source": peak_kind, "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                         "traffic": _traffic(kernel, a.n), "alg_bytes_per_launch": alg_bytes,
                         "launch_ms": gate_launch_ms, "time_share": share,
                         "layer_frac": value / world * 2 * 16 * N / (peak * 1e9)},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 16 * N,
                    "host_link_gbs": link},
            "clocks": ck,
            "gpu_launches": launches,
            "final_norm2": norm,
            "arith_check": arith_check,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
