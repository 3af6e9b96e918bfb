#!/usr/bin/env python
"""Benchmark: forward + adjoint backward of a depth-400 random circuit on 24 qubits.

Workload (synthetic, seeded): n_wires=24, bsz=16 (a 2 GiB complex64 state); 400 gates,
each a U3 on a uniform wire with probability 0.6 (angles ~U[-pi, pi) per sample) or a
uniform choice of CNOT / CZ / CRX(theta per sample) on a uniform ordered wire pair.
One step = |0..0> init, the 400 gates, the full probabilities [16, 2^24], the
expectation values of 8 random 24-site Pauli strings, and the gradient of their sum
with respect to every gate angle (adjoint method).  ``value`` is circuits/s
(bsz x steps / device time) with inputs resident in HBM; ``e2e`` is the same through
the public API with the angles copied from pinned host memory and the expvals and
gradients copied back every step.  The state (2 GiB) is larger than L2 (129 MB), so no
flush is needed between steps.

``--impl reference`` times upstream torchquantum itself (the offline install in
``baseline/_ref``: its gate functions, ``apply_unitary_bmm`` and torch autograd on the
host cores, every host thread) on a bounded sample of the same circuit, extrapolated to
circuits/s; without that install it times the oracle's numpy restatement instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+bwd circuits/s fused+adjoint vs plain at <=1e-5 vs FP64; HBM GB/s per gate"

# DRAM traffic (read + write bytes) of one tensor-core adjoint launch, measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum) on a smaller case of the same kernel
# (n_wires=22, bsz=8, per-row U); the kernel streams every amplitude of psi and lam once,
# so traffic scales with the amplitudes processed.
ADJ_TRAFFIC_CAPTURE = {"n": 22, "bsz": 8, "dram_bytes": 539.099648e6 + 477.703168e6}
ADJ_STORED_TRAFFIC_CAPTURE = {"n": 22, "bsz": 8, "dram_bytes": 539.404288e6 + 221.680896e6}
UNIT = "circuits/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--method", default="fused", choices=["plain", "fused"])
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain method for comparison")
    ap.add_argument("--n", type=int, default=24)
    ap.add_argument("--bsz", type=int, default=16)
    ap.add_argument("--depth", type=int, default=400)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations' summaries (c1, c3, c4, c5) in the headline line")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU time of the baseline sample")
    ap.add_argument("--fuse", default="auto", help="fused block width 1..6 or auto (autotuner)")
    ap.add_argument("--kernels", action="store_true",
                    help="only time the hot kernels alone at --n/--bsz (roofline table; for profiling)")
    ap.add_argument("--quick", action="store_true", help="skip e2e/roofline/baseline (profiling runs)")
    ap.add_argument("--workload", default="random", choices=["random", "c1", "c3", "c4", "c5"],
                    help="random: the headline circuit (default); c1: small encoder+U3+CNOT model (n=4, bsz=32); "
                         "c3: fused widths k=4..6 at n=26/28; c4: 256 uneven circuits in one persistent batch; "
                         "c5: differentiation workload (n=20, bsz=64)")
    return ap.parse_args()


def dist_env():
    from torchquantum_gb300.replicas import rank_env

    return rank_env()


# ------------------------------------------------------------------ CPU legs
def cpu_model() -> str:
    """CPU model of this host (x86 "model name", or the Arm implementer/part ids)."""
    info = {}
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if ":" in line:
                    k, v = line.split(":", 1)
                    info.setdefault(k.strip(), v.strip())
    except OSError:
        pass
    if "model name" in info:
        return info["model name"]
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    parts = [f"{k} {info[k]}" for k in ("CPU implementer", "CPU part") if k in info]
    return ", ".join(parts) or "unknown"


def cpu_sample(args, seconds: float):
    """Time the oracle's autograd-style fwd + reverse sweep on one circuit of the
    workload (bsz 1) over the first G gates, G sized to ~``seconds``; returns
    (circuits/s extrapolated to the full depth, description, threads)."""
    from oracle import statevec as O
    from torchquantum_gb300 import workloads as W

    gates, ncols = W.random_circuit(args.n, args.depth, seed=0)
    theta = W.random_params(1, ncols, seed=1)
    og = W.oracle_gates(gates, theta)

    cpu = {}

    def run(g):
        t0, c0 = time.perf_counter(), time.process_time()
        s, saved, mats = O.forward_saving(args.n, 1, og[:g], np.complex64)
        O.backward_sweep(args.n, og[:g], saved, mats, s.copy())
        wall = time.perf_counter() - t0
        cpu["cores"] = (time.process_time() - c0) / max(wall, 1e-9)
        return wall

    t1 = run(2) / 2
    g = int(max(2, min(args.depth, seconds / max(t1, 1e-6))))
    t = run(g)
    per_circuit = t / g * args.depth
    # cores actually used: process CPU time / wall time of the sample (numpy runs the
    # permute copies on one thread; BLAS may thread the matmuls)
    threads = round(cpu["cores"], 2)
    desc = (f"oracle (numpy complex64) fwd keeping per-gate states + reverse sweep, n={args.n}, 1 circuit, "
            f"first {g} of {args.depth} gates in {t:.1f} s, extrapolated to the full depth")
    return 1.0 / per_circuit, desc, threads, g, t


class UpstreamStep:
    """The headline step run by upstream torchquantum itself on the host cores.

    Gates go through upstream's own public path: ``tqf.u3 / cnot / cz / crx`` on an
    upstream ``QuantumDevice`` (``torchquantum/functional/gate_wrapper.py:324-446`` ->
    ``apply_unitary_bmm``, ``:96-140``), and torch autograd differentiates them with
    respect to the per-sample angles, as an upstream training step does.  The 8 Pauli
    expvals cannot use upstream's ``expval_joint_analytical`` at n = 24 (it builds a dense
    2^n x 2^n matrix, ``measurement/measurements.py:232-279``), so they use the same
    sum over amplitude pairs as the engine, written with torch ops on the host and
    differentiated by autograd; the probabilities are ``|psi|^2`` of the final state.
    A step of the sample is ``gates_per_step`` consecutive gates of the circuit (the
    window advances every step) forward + backward on a fresh device; the measurement
    (forward + backward) is timed once.  Circuits/s = bsz / (measurement time + depth x
    mean time per gate)."""

    def __init__(self, args):
        import torch

        from oracle import upstream as U
        from oracle import statevec as O
        from torchquantum_gb300 import workloads as W

        self.torch = torch
        self.tq = U.import_upstream()
        import torchquantum.functional as tqf  # upstream's gate functions

        self.fns = {"u3": tqf.u3, "cnot": tqf.cnot, "cz": tqf.cz, "crx": tqf.crx}
        self.n, self.bsz, self.depth = args.n, args.bsz, args.depth
        self.gates, ncols = W.random_circuit(args.n, args.depth, seed=0)
        self.theta = torch.tensor(W.random_params(args.bsz, ncols, seed=1))
        self.paulis = W.random_paulis(args.n, 8, seed=2)
        self.pw = torch.tensor(np.random.default_rng(3).normal(size=(1, 8)), dtype=torch.float32)
        self.masks = [O.pauli_masks(p, args.n) for p in self.paulis]
        self.pos = 0

    def gates_fwd_bwd(self, g: int) -> float:
        """Wall seconds of g consecutive gates (forward + autograd backward)."""
        torch = self.torch
        th = self.theta.clone().requires_grad_(True)
        t0 = time.perf_counter()
        q = self.tq.QuantumDevice(n_wires=self.n, bsz=self.bsz)
        # in the full circuit nearly every gate follows a parameterised one, so its
        # backward propagates the state cotangent: make the window's input differentiable
        q.states.requires_grad_(True)
        for k in range(g):
            gd = self.gates[(self.pos + k) % self.depth]
            p = th[:, gd["off"]:gd["off"] + gd["np"]] if gd["np"] else None
            self.fns[gd["name"]](q, wires=gd["wires"], params=p)
        s = q.get_states_1d()
        s[:, :1].abs().pow(2).sum().backward()
        dt = time.perf_counter() - t0
        self.pos = (self.pos + g) % self.depth
        del q, s, th
        return dt

    def _tables(self, strings):
        torch = self.torch
        idx = torch.arange(1 << self.n, dtype=torch.int64)
        out = []
        for j in strings:
            x, z, ny = self.masks[j]
            src = idx ^ x
            v, par = src & z, torch.zeros_like(idx)
            for b in range(self.n):
                par ^= (v >> b) & 1
            ph = (1j ** ny) * (1.0 - 2.0 * par.to(torch.float32))
            out.append((j, src, ph.to(torch.complex64)))
        return out

    def measurement_fwd_bwd(self, strings) -> float:
        """Wall seconds of probs + the given strings' expvals, forward + backward, on a
        normalised random state (the observables' index tables are built beforehand)."""
        torch = self.torch
        tabs = self._tables(strings)
        g = torch.Generator().manual_seed(4)
        s = torch.randn(self.bsz, 1 << self.n, dtype=torch.complex64, generator=g)
        s = (s / s.abs().pow(2).sum(1, keepdim=True).sqrt()).requires_grad_(True)
        t0 = time.perf_counter()
        pr = s.abs() ** 2
        ev = torch.stack([(s.conj() * ph * s[:, src]).sum(1).real for _, src, ph in tabs], 1)
        loss = (ev * self.pw[:, [j for j, _, _ in tabs]]).sum() + 0.0 * pr[:, 0].sum()
        loss.backward()
        dt = time.perf_counter() - t0
        del s, pr, ev, loss, tabs
        return dt


def upstream_cpu_baseline(args, seconds: float):
    """cpu_baseline of our arm: upstream on the host cores, a bounded sample (about
    ``seconds`` of gates plus one string's measurement, scaled to 8)."""
    import torch

    torch.set_num_threads(os.cpu_count() or 1)
    up = UpstreamStep(args)
    c0, w0 = time.process_time(), time.perf_counter()
    t1 = up.gates_fwd_bwd(1)
    g = int(max(1, min(8, seconds / max(t1, 1e-6))))
    tg = up.gates_fwd_bwd(g)
    tm = up.measurement_fwd_bwd([0]) * 8
    cores = round((time.process_time() - c0) / max(time.perf_counter() - w0, 1e-9), 2)
    value = args.bsz / (tm + args.depth * tg / g)
    desc = (f"upstream torchquantum 0.1.8 (torch CPU, complex64, autograd) on {os.cpu_count()} threads of "
            f"{cpu_model()}: {g} gates of the circuit fwd+bwd at n={args.n} bsz={args.bsz} in {tg:.1f} s, "
            f"1 of the 8 Pauli expvals fwd+bwd in {tm / 8:.1f} s (x8); circuits/s = bsz / (8 expvals + "
            f"{args.depth} x time per gate)")
    return value, desc, cores


def _peak_rss_reset() -> None:
    """Reset this process's peak resident set (VmHWM) so the next reading covers only
    what follows (Linux: writing 5 to /proc/self/clear_refs)."""
    try:
        with open("/proc/self/clear_refs", "w") as f:
            f.write("5")
    except OSError:
        pass


def _peak_rss_bytes() -> int:
    try:
        with open("/proc/self/status") as f:
            for line in f:
                if line.startswith("VmHWM:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def upstream_c1_baseline(steps: int = 30) -> dict:
    """Upstream's own CPU path for the n=4 model (GeneralEncoder + 2 x (Op1QAllLayer(U3) +
    Op2QAllLayer(CNOT, circular)), 4 x expval_joint_analytical, bsz 32), fwd + autograd bwd."""
    import torch

    from oracle import upstream as U

    torch.set_num_threads(os.cpu_count() or 1)
    tq = U.import_upstream()
    from torchquantum.measurement import expval_joint_analytical

    funcs = ["rx", "ry", "rz", "rx"]
    enc = tq.GeneralEncoder([{"input_idx": [4 * g + w], "func": funcs[g], "wires": [w]} for g in range(4)
                             for w in range(4)])
    layers = []
    for _ in range(2):
        layers += [tq.layer.Op1QAllLayer(op=tq.U3, n_wires=4, has_params=True, trainable=True),
                   tq.layer.Op2QAllLayer(op=tq.CNOT, n_wires=4, circular=True)]
    model = torch.nn.ModuleList([enc] + layers)
    x = torch.rand(32, 16, generator=torch.Generator().manual_seed(0)) * np.pi
    obs = ["".join("Z" if i == j else "I" for i in range(4)) for j in range(4)]

    def step():
        model.zero_grad(set_to_none=True)
        q = tq.QuantumDevice(n_wires=4, bsz=32)
        enc(q, x)
        for lay in layers:
            lay(q)
        torch.stack([expval_joint_analytical(q, o) for o in obs], -1).sum().backward()

    for _ in range(3):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = (time.perf_counter() - t0) / steps
    return {"value": 32 / dt, "unit": UNIT, "ms_per_step": dt * 1e3, "cores": os.cpu_count(),
            "kind": "reference", "cpu_model": cpu_model(),
            "sample": f"upstream torchquantum 0.1.8, the same model fwd+bwd, {steps} steps after 3 warm-up"}


def upstream_c4_baseline(specs, angles, seconds: float = 20.0) -> dict:
    """Upstream's CPU path for the 256 uneven circuits: a Python loop, one upstream
    QuantumDevice per circuit (RY, RZ per wire, CZ ladder per layer through tqf), <Z_0> by
    tq.expval (measurements.py:282-312).  Circuits are timed in a seeded random order
    until ``seconds`` have passed; the total is extrapolated by gate work (layers x gates
    per layer x 2^n)."""
    import torch

    from oracle import upstream as U

    torch.set_num_threads(os.cpu_count() or 1)
    tq = U.import_upstream()
    import torchquantum.functional as tqf

    def cost(i):
        n, L = specs[i]
        return L * (3 * n - 1) * (1 << n)

    order = np.random.default_rng(5).permutation(len(specs))
    done, spent, lat = [], 0.0, []
    with torch.no_grad():
        for i in order:
            (n, L), (ry, rz) = specs[i], angles[i]
            t0 = time.perf_counter()
            q = tq.QuantumDevice(n_wires=n, bsz=1)
            for l in range(L):
                for w in range(n):
                    tqf.ry(q, wires=w, params=float(ry[l, w]))
                    tqf.rz(q, wires=w, params=float(rz[l, w]))
                for w in range(n - 1):
                    tqf.cz(q, wires=[w, w + 1])
            tq.expval(q, 0, tq.PauliZ())
            dt = time.perf_counter() - t0
            done.append(int(i))
            lat.append(dt)
            spent += dt
            if spent > seconds:
                break
    rate = sum(cost(i) for i in done) / spent
    total = sum(cost(i) for i in range(len(specs))) / rate
    return {"value": len(specs) / total, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
            "cpu_model": cpu_model(),
            "sample": f"upstream torchquantum 0.1.8, {len(done)} of {len(specs)} circuits one at a time in "
                      f"{spent:.1f} s (forward, no grad), total extrapolated by gate work L x (3n - 1) x 2^n",
            "sample_latency_ms": {"p50": float(np.percentile(lat, 50)) * 1e3,
                                  "p99": float(np.percentile(lat, 99)) * 1e3}}


def upstream_c5_baseline(batches=(1, 4)) -> dict:
    """Upstream autograd for the differentiation workload (n=20, 10 layers of RY, RZ per
    wire + CZ ladder after the per-sample RY input layer, 400 shared angles, 50 weighted
    Pauli strings) at reduced bsz: upstream's tqf gates with torch autograd on the host;
    the 50 expvals as the torch sum over amplitude pairs (upstream's dense-kron
    expval_joint_analytical needs a 2^20 x 2^20 matrix).  Peak RSS per bsz."""
    import torch

    from oracle import upstream as U
    from oracle import statevec as O
    from torchquantum_gb300 import workloads as W

    torch.set_num_threads(os.cpu_count() or 1)
    tq = U.import_upstream()
    import torchquantum.functional as tqf

    n, layers, m = 20, 10, 50
    gates, ncols = W.hea_circuit(n, layers)
    rng = np.random.default_rng(7)
    theta0 = rng.uniform(-np.pi, np.pi, size=(1, ncols)).astype(np.float32)
    x = rng.uniform(0, np.pi, size=(64, n)).astype(np.float32)
    paulis = W.random_paulis(n, m, seed=8)
    w = torch.tensor(rng.normal(size=m).astype(np.float32))
    idx = torch.arange(1 << n, dtype=torch.int64)
    tabs = []
    for pstr in paulis:
        xm, zm, ny = O.pauli_masks(pstr, n)
        src = idx ^ xm
        v, par = src & zm, torch.zeros_like(idx)
        for b in range(n):
            par ^= (v >> b) & 1
        tabs.append((src, ((1j ** ny) * (1.0 - 2.0 * par.to(torch.float32))).to(torch.complex64)))
    fns = {"ry": tqf.ry, "rz": tqf.rz, "cz": tqf.cz}
    out = {}
    for bsz in batches:
        th = torch.tensor(theta0, requires_grad=True)
        xt = torch.tensor(x[:bsz])
        _peak_rss_reset()
        t0 = time.perf_counter()
        q = tq.QuantumDevice(n_wires=n, bsz=bsz)
        for wi in range(n):
            tqf.ry(q, wires=wi, params=xt[:, wi:wi + 1])
        for g in gates:
            p = th[:, g["off"]:g["off"] + g["np"]] if g["np"] else None
            fns[g["name"]](q, wires=g["wires"], params=p)
        s = q.get_states_1d()
        ev = torch.stack([(s.conj() * ph * s[:, src]).sum(1).real for src, ph in tabs], 1)
        (ev * w).sum().backward()
        dt = time.perf_counter() - t0
        out[f"bsz{bsz}"] = {"circuits_per_s": bsz / dt, "s_per_step": dt, "peak_rss_bytes": _peak_rss_bytes()}
        del q, s, ev, th
    best = max(v["circuits_per_s"] for v in out.values())
    return {"value": best, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference", "cpu_model": cpu_model(),
            "sample": "upstream torchquantum 0.1.8 autograd, one fwd+bwd step per bsz in "
                      f"{list(batches)} (bsz=64 would need ~317 GB of saved states); value = the better bsz",
            "per_bsz": out}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import torch

    torch.set_num_threads(os.cpu_count() or 1)
    from oracle import upstream as U

    c_start, t_run0 = time.process_time(), time.perf_counter()
    if U.available():
        up = UpstreamStep(args)
        t_meas = up.measurement_fwd_bwd(range(8))
        t1 = up.gates_fwd_bwd(1)
        # gates per step sized so warm-up + timed steps take about three minutes
        budget = 180.0 / max(1, args.steps + args.warmup)
        g = int(max(1, min(8, budget / max(t1, 1e-6))))
        for _ in range(args.warmup):
            up.gates_fwd_bwd(g)
        times = [up.gates_fwd_bwd(g) for _ in range(args.steps)]
        per_step = sum(times) / len(times)
        value = args.bsz / (t_meas + args.depth * per_step / g)
        method = ("upstream torchquantum 0.1.8 itself (baseline/_ref, imported with stand-ins for its absent "
                  "optional deps): tqf gates -> gate_wrapper -> apply_unitary_bmm with torch autograd, torch CPU, "
                  "complex64; Pauli expvals as a torch sum over amplitude pairs (upstream's dense-kron "
                  "expval_joint_analytical needs a 2^24 x 2^24 matrix)")
        sample = (f"each step: {g} consecutive gates of the circuit (window advancing) fwd+bwd at n={args.n} "
                  f"bsz={args.bsz}; probs + 8 expvals fwd+bwd timed once ({t_meas:.1f} s); circuits/s = bsz / "
                  f"(expvals + {args.depth} x mean time per gate)")
        kind = "reference"
    else:
        # upstream not installed: the oracle's restatement of its algorithm
        from oracle import statevec as O
        from torchquantum_gb300 import workloads as W

        gates, ncols = W.random_circuit(args.n, args.depth, seed=0)
        og = W.oracle_gates(gates, W.random_params(1, ncols, seed=1))

        def one(g):
            s, saved, mats = O.forward_saving(args.n, 1, og[:g], np.complex64)
            O.backward_sweep(args.n, og[:g], saved, mats, s.copy())

        t0 = time.perf_counter()
        one(1)
        t1 = time.perf_counter() - t0
        budget = 180.0 / max(1, args.steps + args.warmup)
        g = int(max(1, min(args.depth, budget / max(t1, 1e-6))))
        for _ in range(args.warmup):
            one(g)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            one(g)
            times.append(time.perf_counter() - t0)
        per_step = sum(times) / len(times)
        value = 1.0 / (per_step / g * args.depth)
        method = ("upstream algorithm restated on the host (numpy complex64, autograd-style forward keeping "
                  "per-gate states, then the reverse sweep); upstream itself not installed in baseline/_ref")
        sample = f"1 circuit, first {g} of {args.depth} gates fwd+bwd per step, extrapolated"
        kind = "port"
    threads = round((time.process_time() - c_start) / max(time.perf_counter() - t_run0, 1e-9), 2)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": _config(args), "impl": "reference", "method": method,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample,
                         "cpu_model": cpu_model(), "host_threads": os.cpu_count()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _config(args):
    """The workload (identical for both arms; the engine method is reported beside it)."""
    state_mb = args.bsz * (8 << args.n) / 2**20
    flush = (f"none needed: state {state_mb:.0f} MiB > L2 129 MB" if state_mb > 129 else
             f"not flushed: state {state_mb:.0f} MiB fits in L2 (129 MB)")
    return {"workload": f"random circuit n={args.n} bsz={args.bsz} depth={args.depth} "
                        "(U3 60%, CNOT/CZ/CRX 40%) + probs + 8 Pauli expvals, fwd + adjoint bwd",
            "n_wires": args.n, "global_batch": args.bsz, "depth": args.depth, "l2_flush": flush}


# ------------------------------------------------------------------ GPU leg
class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def run_ours(args):
    import torch

    from torchquantum_gb300 import replicas as R

    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        R.init("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import _lib
    from torchquantum_gb300 import workloads as W

    n, bsz = args.n, args.bsz
    gates, ncols = W.random_circuit(n, args.depth, seed=0)
    theta_host = W.random_params(bsz, ncols, seed=R.rank_seed(1, rank))
    paulis = W.random_paulis(n, 8, seed=2)
    pw = torch.tensor(np.random.default_rng(3).normal(size=(1, 8)), dtype=torch.float32, device=dev)
    theta_dev = torch.tensor(theta_host, device=dev)

    def step(theta, method=args.method, keep=False):
        q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
        if method == "plain_gate_by_gate":  # the plain method without staged low-qubit runs
            q.stage_low = False
        if method in ("fused", "fused_in_place"):
            q.method = "fused"
            q.fuse_wires = args.fuse if args.fuse == "auto" else int(args.fuse)
            if method == "fused_in_place":  # reverse sweep uncomputes in place: O(1) extra states
                q.checkpoint = False
        W.apply_circuit(q, gates, theta)
        pr = tq.probs(q)
        ev = tq.expval_joint_analytical_batch(q, paulis)
        (ev * pw).sum().backward()
        if keep:
            last["q"] = q
        return ev, pr

    last = {}

    barrier = R.barrier

    th = theta_dev.clone().requires_grad_(True)
    for w in range(args.warmup):
        th.grad = None
        step(th, keep=w == args.warmup - 1)  # the last warm-up step's plan describes the timed steps
    fusion_info = None
    if args.method == "fused":
        segs = last["q"]._tape
        fusion_info = {"width": [getattr(sg, "fuse_width", None) for sg in segs],
                       "passes": sum(len(sg.exec_ops) for sg in segs),
                       "tensor_core_passes": sum(1 for sg in segs for op in sg.exec_ops if getattr(op, "tc", False)),
                       # tensor-core blocks whose input state the forward kept for the backward
                       "stored_inputs": sum(1 for sg in segs for op in sg.exec_ops
                                            if getattr(op, "kept_input", False)),
                       "chosen_by": "autotuner (measured pass costs)" if args.fuse == "auto" else f"fixed k={args.fuse}"}
    last.clear()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.reset_peak_memory_stats(dev)
    mem0 = torch.cuda.memory_allocated(dev)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = _lib.LAUNCHES[0]
    # the dominant kernel's launches inside the timed steps, bracketed by CUDA events on
    # the stream they run on (the roofline's live duration)
    live = {"fused_adjoint_stored": AdjointTimer(stored=True), "fused_adjoint": AdjointTimer(stored=False)}
    _lib.SEGMENT_HOOKS["backward"] = lambda rec, after: [t(rec, after) for t in live.values()]
    try:
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(args.steps):
                th.grad = None
                ev_main, _ = step(th)
            e1.record(stream)
            torch.cuda.synchronize()
    finally:
        _lib.SEGMENT_HOOKS["backward"] = None
    launches = _lib.LAUNCHES[0] - launches0
    peak_states = (torch.cuda.max_memory_allocated(dev) - mem0) / (bsz * (8 << n))
    ms = R.max_over_ranks(e0.elapsed_time(e1), dev)
    value = R.job_throughput(bsz * args.steps, world, ms / 1e3)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic", "config": _config(args), "method": args.method,
            "clocks": clk.summary(), "gpu_launches": launches}
    if fusion_info:
        line["config"]["fusion"] = fusion_info
        line["peak_states"] = peak_states  # device memory of the timed steps, in states
    # gate applications per second (each circuit applies `depth` gates forward and
    # reverses them in the adjoint sweep)
    line["gate_applications_per_s"] = value * args.depth
    if world > 1:
        line["config"]["parallelism"] = f"replicas x{world} (batch sharding, no collective in the step)"

    _lib.check_status(dev)
    if args.method == "fused" and not args.quick and not args.no_plain:
        g_main, ev_main = th.grad.detach().clone(), ev_main.detach().clone()
        # ---------------- the same fused step with the in-place reverse sweep (O(1) extra
        # states), and the plain method: with staged low-qubit runs (its default) and
        # strictly gate by gate
        variant_out = {}
        for variant, key in (("fused_in_place", "fused_adjoint_in_place"), ("plain", "plain_method"),
                             ("plain_gate_by_gate", "plain_gate_by_gate")):
            for _ in range(2):
                th.grad = None
                step(th, variant)
            torch.cuda.synchronize()
            barrier()
            torch.cuda.reset_peak_memory_stats(dev)
            m0 = torch.cuda.memory_allocated(dev)
            e0.record(stream)
            for _ in range(args.steps):
                th.grad = None
                ev_v, _ = step(th, variant)
            e1.record(stream)
            torch.cuda.synchronize()
            variant_out[key] = (th.grad.detach().clone(), ev_v.detach().clone())
            ms_plain = R.max_over_ranks(e0.elapsed_time(e1), dev)
            v_plain = R.job_throughput(bsz * args.steps, world, ms_plain / 1e3)
            line[key] = {"value": v_plain, "unit": UNIT, "ms_per_step": ms_plain / args.steps,
                         "gate_applications_per_s": v_plain * args.depth,
                         "peak_states": (torch.cuda.max_memory_allocated(dev) - m0) / (bsz * (8 << n))}
        line["fused_speedup_vs_plain"] = value / line["plain_gate_by_gate"]["value"]
        line["fused_speedup_vs_plain_staged"] = value / line["plain_method"]["value"]
        line["fused_adjoint_in_place"]["speedup_vs_plain"] = \
            line["fused_adjoint_in_place"]["value"] / line["plain_gate_by_gate"]["value"]
        # the timed step's outputs against the plain gate-by-gate adjoint sweep on the same
        # angles (complex64 throughout; the complex128 central-difference check of the same
        # workload is a test, since it takes minutes)
        g_ref, ev_ref = variant_out["plain_gate_by_gate"]
        line["max_err"] = {"reference": "plain gate-by-gate adjoint sweep, same angles",
                           "grad_max_abs": float(g_ref.abs().max()),
                           "grad": float((g_main - g_ref).abs().max()),
                           "expval": float((ev_main - ev_ref).abs().max()),
                           "grad_fused_in_place": float((variant_out["fused_adjoint_in_place"][0] - g_ref).abs().max()),
                           "grad_plain_staged": float((variant_out["plain_method"][0] - g_ref).abs().max())}
    if not args.quick:
        # ---------------- end to end through the public API with host buffers
        pin_theta = torch.from_numpy(theta_host).pin_memory()
        out_ev = torch.empty(bsz, 8, dtype=torch.float32).pin_memory()
        out_g = torch.empty(bsz, ncols, dtype=torch.float32).pin_memory()
        torch.cuda.synchronize()
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            thd = pin_theta.to(dev, non_blocking=True).requires_grad_(True)
            ev, _ = step(thd)
            out_ev.copy_(ev.detach(), non_blocking=True)
            out_g.copy_(thd.grad, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_e2e = R.max_over_ranks(e0.elapsed_time(e1), dev)
        line["e2e"] = {"value": R.job_throughput(bsz * args.steps, world, ms_e2e / 1e3), "unit": UNIT,
                       "h2d_bytes_per_step": int(pin_theta.numel() * 4),
                       "d2h_bytes_per_step": int(out_ev.numel() * 4 + out_g.numel() * 4)}
        # ---------------- roofline of the dominant kernel (adjoint dense 1-wire step)
        line["roofline"], line["kernels"] = roofline(args, dev, bool(fusion_info and fusion_info["stored_inputs"]),
                                                     live)
        line["plain_gate_pass"] = line["kernels"]["dense1_fwd"]
        line["plain_gate_pass_summary"] = plain_pass_summary(line["kernels"], bsz * (8 << n),
                                                             line["roofline"]["peak"])
    if rank == 0 and world == 1 and not args.no_cpu_baseline and not args.quick:
        from oracle import upstream as U

        if U.available():
            v, desc, threads = upstream_cpu_baseline(args, args.cpu_seconds)
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "reference", "sample": desc,
                                    "cpu_model": cpu_model()}
        v, desc, threads, g, tcpu = cpu_sample(args, args.cpu_seconds / 2)
        port = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc, "cpu_model": cpu_model()}
        line.setdefault("cpu_baseline", port)
        if line["cpu_baseline"] is not port:
            line["cpu_baseline_port"] = port
    if rank == 0 and world == 1 and not args.quick and not args.no_configs:
        line["configs"] = other_configs(args)
    R.finish()
    if rank == 0:
        print(json.dumps(line), flush=True)


def upstream_forward_sample(n: int, bsz: int, depth: int, gates_timed: int = 3) -> dict:
    """Upstream's gate-by-gate forward of the random circuit (no grad) on the host:
    ``gates_timed`` gates timed after one warm-up gate, extrapolated to ``depth``."""
    import torch

    from oracle import upstream as U
    from torchquantum_gb300 import workloads as W

    torch.set_num_threads(os.cpu_count() or 1)
    tq = U.import_upstream()
    import torchquantum.functional as tqf

    fns = {"u3": tqf.u3, "cnot": tqf.cnot, "cz": tqf.cz, "crx": tqf.crx}
    gates, ncols = W.random_circuit(n, depth, seed=0)
    th = torch.tensor(W.random_params(bsz, ncols, seed=1))
    with torch.no_grad():
        q = tq.QuantumDevice(n_wires=n, bsz=bsz)
        times = []
        for g in gates[:gates_timed + 1]:
            t0 = time.perf_counter()
            fns[g["name"]](q, wires=g["wires"], params=th[:, g["off"]:g["off"] + g["np"]] if g["np"] else None)
            times.append(time.perf_counter() - t0)
        del q
    per_gate = sum(times[1:]) / gates_timed
    return {"value": bsz / (per_gate * depth), "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
            "cpu_model": cpu_model(),
            "sample": f"upstream torchquantum 0.1.8 forward gate by gate at n={n} bsz={bsz}: {gates_timed} gates "
                      f"timed ({per_gate:.2f} s per gate), extrapolated to {depth} gates"}


def other_configs(args) -> dict:
    """The other configurations measured in the same run (short: a few steps each), each
    with upstream's own CPU path timed on the host as its baseline (when upstream is
    installed)."""
    import copy

    import torch

    from oracle import upstream as U

    a = copy.copy(args)
    a.steps, a.warmup = min(args.steps, 10), 3
    have_up = U.available()
    out = {}

    def keep(d, keys):
        return {k: d[k] for k in keys if k in d}

    c1 = run_c1(a, emit=False)
    out["c1"] = keep(c1, ("value", "unit", "ms_per_step", "config", "p50_ms", "p99_ms"))
    if have_up:
        out["c1"]["cpu_baseline"] = upstream_c1_baseline()
    torch.cuda.empty_cache()
    c3 = run_c3(a, emit=False)
    out["c3"] = keep(c3, ("value", "unit", "ms_per_step", "config", "cases"))
    if have_up:
        out["c3"]["cpu_baseline"] = upstream_forward_sample(26, 8, args.depth)
    torch.cuda.empty_cache()
    c4 = run_c4(a, emit=False)
    out["c4"] = keep(c4, ("value", "unit", "ms_per_step", "config", "e2e", "latency_ms", "batch_kernel",
                          "default_launch_shape", "engine_one_circuit_at_a_time"))
    if have_up:
        specs, angles = c4_workload(np.random.default_rng(0))
        out["c4"]["cpu_baseline"] = upstream_c4_baseline(specs, angles)
    torch.cuda.empty_cache()
    c5 = run_c5(a, emit=False)
    out["c5"] = keep(c5, ("value", "unit", "ms_per_step", "config", "variants"))
    if have_up:
        out["c5"]["cpu_baseline"] = upstream_c5_baseline()
    torch.cuda.empty_cache()
    return out


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# gate mix of the random circuit: 60 % U3 (dense 1-wire), 40 % CNOT / CZ / CRX evenly
PLAIN_GATE_MIX = {"dense1_fwd": 0.6, "cnot_fwd": 0.4 / 3, "cz_fwd": 0.4 / 3, "crx_fwd": 0.4 / 3}


def plain_pass_summary(kernels: dict, state_bytes: int, peak: float) -> dict:
    """The plain method's HBM rate over the circuit's gate mix: algorithmic bytes of an
    average gate over its average kernel time (each kernel timed alone on the bench state),
    and the same time against a uniform 2 S per gate (the convention CPU numbers use)."""
    b = sum(w * kernels[k]["bytes"] for k, w in PLAIN_GATE_MIX.items())
    t = sum(w * kernels[k]["us"] for k, w in PLAIN_GATE_MIX.items()) / 1e6
    return {"GB/s": b / t / 1e9, "frac": b / t / 1e9 / peak, "us_per_gate": t * 1e6,
            "uniform_2S_GB/s": 2 * state_bytes / t / 1e9,
            "mix": "60% U3, 13.3% each CNOT / CZ / CRX; bytes 2 S / S / S/2 / S per pass"}


class AdjointTimer:
    """Segment-runner hook: brackets each reverse step of a tensor-core block (with a stored
    input, or uncomputed in place) by CUDA events on the current stream -- the stream the
    runner launches the kernel on."""

    def __init__(self, stored: bool):
        self.stored = stored
        self.events = []
        self._start = None

    def __call__(self, rec, after):
        import torch

        from torchquantum_gb300 import _lib

        if rec.kind != _lib.X_BLOCK_TC or rec.skip_reverse or bool(rec.stored) != self.stored:
            return
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        if after:
            self.events.append((self._start, ev))
        else:
            self._start = ev

    def mean_s(self):
        return sum(s.elapsed_time(e) for s, e in self.events) / len(self.events) / 1e3 if self.events else None


def roofline(args, dev, stored=True, live=None):
    """Time the engine's hot kernels alone (CUDA events on the launching stream) on the
    bench's state size; algorithmic bytes per launch from the touched amplitudes.
    ``stored``: the fused step's blocks kept their inputs, so its dominant kernel is the
    stored-input adjoint step.  ``live``: AdjointTimers of the tensor-core reverse steps over
    the timed steps; the roofline's achieved rate uses their average launch duration."""
    import torch

    from torchquantum_gb300 import _lib

    n, bsz = args.n, args.bsz
    S = bsz * (1 << n) * 8
    psi = torch.zeros(bsz, 1 << n, dtype=torch.complex64, device=dev)
    psi[:, 0] = 1
    lam = psi.clone()
    mat = torch.tensor(np.tile(np.eye(2), (bsz, 1, 1)), dtype=torch.complex64, device=dev)
    mat4 = torch.tensor(np.tile(np.eye(2), (bsz, 1, 1)), dtype=torch.complex64, device=dev)
    grad = torch.zeros(bsz * 8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    peak, peak_kind = _peaks()
    reps = 24
    res = {}

    def timeit(fn):
        for w in range(3):
            fn(w)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for i in range(reps):
            fn(i)
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps / 1e3

    wires = [int(w) for w in np.random.default_rng(0).integers(0, n, size=reps + 3)]
    pairs = [tuple(int(x) for x in np.random.default_rng(i).choice(n, 2, replace=False)) for i in range(reps + 3)]
    kernels = {
        "dense1_fwd": (lambda i: _lib.apply_matrix(psi, n, [wires[i]], mat, bsz), 2 * S),
        "dense1_adj": (lambda i: _lib.adjoint_matrix(psi, lam, n, [wires[i]], mat, bsz, grad), 4 * S),
        "crx_fwd": (lambda i: _lib.apply_controlled(psi, n, [pairs[i][0]], [pairs[i][1]], mat4, bsz), S),
        "cnot_fwd": (lambda i: _lib.apply_mcx(psi, n, [pairs[i][0]], 1, pairs[i][1]), S),
        "cz_fwd": (lambda i: _lib.apply_phase(psi, n, list(pairs[i]), mat[:, 0, 0].contiguous(), bsz), S // 2),
    }
    # a staged run of 8 dense one-qubit gates on the low wires: one pass (2S / 4S)
    sdescs = []
    for j in range(8):
        d = _lib.StagedOp()
        d.kind, d.nwires, d.batch, d.operand = _lib.S_DENSE1, 1, bsz, mat.data_ptr()
        d.wires[0] = n - 1 - j
        sdescs.append(d)
    gstage = torch.zeros(8, bsz * 8, dtype=torch.float64, device=dev)
    sdescs_g = []
    for j, d in enumerate(sdescs):
        e = _lib.StagedOp.from_buffer_copy(d)
        e.grad = gstage[j].data_ptr()
        sdescs_g.append(e)
    tb = min(n, _lib.STAGED_MAX_TILE_BITS)
    kernels["staged8_fwd"] = (lambda i: _lib.staged_apply(psi, n, sdescs, tb), 2 * S)
    kernels["staged8_adj"] = (lambda i: _lib.staged_adjoint(psi, lam, n, sdescs_g, tb), 4 * S)
    # the bench step's measurement kernels, at the algorithmic bytes of the unit: 8 Pauli
    # expvals fused in one pass read the state once (S); the backward seed
    # sum_j c_j P_j psi reads it and writes the result (2 S).  Strings with different
    # X-masks run as coset passes (partners read from shared memory): one pass per group
    from torchquantum_gb300.measurement import pauli_masks
    from torchquantum_gb300 import workloads as W

    strings = W.random_paulis(n, 8, seed=2)
    xs = [pauli_masks(o, n)[0] for o in strings]
    zs = [pauli_masks(o, n)[1] for o in strings]
    coef = torch.ones(bsz, 8, dtype=torch.float32, device=dev)
    kernels["expval8"] = (lambda i: _lib.pauli_expval(psi, n, xs, zs), S)
    kernels["apply_sum8"] = (lambda i: _lib.pauli_apply_sum(psi, n, xs, zs, coef), 2 * S)
    for name, (fn, nbytes) in kernels.items():
        t = timeit(fn)
        gbs = nbytes / t / 1e9
        res[name] = {"us": t * 1e6, "bytes": nbytes, "GB/s": gbs, "frac": gbs / peak}
    # CZ touches a quarter of the amplitudes; where one of its wires is among the two lowest
    # address bits, every touched 32-byte sector is only partly used (DRAM moves whole
    # sectors): the same pass on the bytes of the sectors it touches
    sec = np.mean([1.0 if max(bb) < 2 else (0.5 if min(bb) < 2 else 0.25)
                   for bb in ([n - 1 - w for w in pairs[i]] for i in range(reps))])
    res["cz_fwd"]["sector_bytes"] = int(2 * S * sec)
    res["cz_fwd"]["frac_sector_bytes"] = 2 * S * sec / (res["cz_fwd"]["us"] / 1e6) / 1e9 / peak
    for name in ("expval8", "apply_sum8"):
        res[name]["passes"] = _lib.expval_passes(xs, n) if name == "expval8" else len(_lib.coset_groups(xs, n))
        # shared-memory reads of the coset passes: own pair + one partner pair per string
        res[name]["smem_loads_GB/s"] = (9 if name == "expval8" else 8) * S / (res[name]["us"] / 1e6) / 1e9
    if n >= 13:
        # fused 6-wire block on the tensor cores: forward (2S) and adjoint step (4S) per launch
        rng = np.random.default_rng(0)
        z = rng.normal(size=(bsz, 64, 64)) + 1j * rng.normal(size=(bsz, 64, 64))
        u = torch.tensor(np.linalg.qr(z)[0], dtype=torch.complex128, device=dev)
        wsets = [[int(x) for x in np.random.default_rng(i).choice(n, 6, replace=False)] for i in range(reps + 3)]
        imgs = [_lib.fused_prepare(u, w) for w in wsets]
        imghs = [_lib.fused_prepare(u.conj().transpose(-1, -2).contiguous(), w) for w in wsets]
        mr = torch.zeros(bsz, 128, 128, dtype=torch.float64, device=dev)
        tiles = bsz * (1 << (n - 6)) // 128
        fl_apply = tiles * 24 * 128 * 128 * 16 * 2
        out = torch.empty_like(psi)
        extra = {
            "fused6_tc_fwd": (lambda i: _lib.fused_apply(psi, n, wsets[i], imgs[i], bsz), 2 * S, fl_apply),
            "fused6_tc_fwd_to": (lambda i: _lib.fused_apply_to(psi, out, n, wsets[i], imgs[i], bsz), 2 * S,
                                 fl_apply),
            "fused6_tc_adj": (lambda i: _lib.fused_adjoint(psi, lam, n, wsets[i], imghs[i], bsz, mr), 4 * S,
                              3 * fl_apply),
            # reads the block's stored input and lam, writes lam: 3 S
            "fused6_tc_adj_stored": (lambda i: _lib.fused_adjoint_stored(out, lam, n, wsets[i], imghs[i], bsz, mr),
                                     3 * S, 3 * fl_apply),
        }
        for name, (fn, nbytes, flops) in extra.items():
            t = timeit(fn)
            gbs = nbytes / t / 1e9
            res[name] = {"us": t * 1e6, "bytes": nbytes, "GB/s": gbs, "frac": gbs / peak,
                         "tensor_TFLOP/s": flops / t / 1e12}
        _lib.check_status(dev)
    traffic = None
    cap = None
    if args.method == "fused" and stored and "fused6_tc_adj_stored" in res:
        dom = res["fused6_tc_adj_stored"]
        kname = "tqk::tc::k_tc<true> (stored-input adjoint step of a fused 6-wire block, tcgen05 split-BF16)"
        cap = ADJ_STORED_TRAFFIC_CAPTURE
    elif args.method == "fused" and "fused6_tc_adj" in res:
        dom = res["fused6_tc_adj"]
        kname = "tqk::tc::k_tc<true> (adjoint step of a fused 6-wire block, tcgen05 split-BF16)"
        cap = ADJ_TRAFFIC_CAPTURE
    if cap is not None and cap.get("dram_bytes"):
        traffic = cap["dram_bytes"] * (bsz << n) / (cap["bsz"] << cap["n"])
    if cap is None:
        dom = res["dense1_adj"]
        kname = "k_dense_adj<2> (adjoint step of a dense 1-wire gate)"
    achieved, source = dom["GB/s"], "kernel timed alone (CUDA events, random wire sets)"
    entry = "fused_adjoint_stored" if cap is ADJ_STORED_TRAFFIC_CAPTURE else "fused_adjoint"
    if live and cap is not None and live[entry].events:
        t = live[entry].mean_s()
        achieved = dom["bytes"] / t / 1e9
        source = (f"average of its {len(live[entry].events)} launches inside the timed steps (CUDA events on the "
                  f"launching stream); alone: {dom['GB/s']:.0f} GB/s")
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "achieved_source": source,
            "traffic": traffic, "algorithmic_bytes": dom["bytes"], "kernel": kname,
            "peak_source": f"{peak_kind} hbm_gbs (burst copy)",
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum at n=22, bsz=8, scaled by amplitudes"
            if traffic is not None else None}
    return roof, res


# ------------------------------------------------------------------ other configurations
def _timed(fn, steps, warmup, dev):
    """Device time of ``steps`` calls (CUDA events on the current stream) after warm-up,
    plus each call's own duration for latency percentiles."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    ev[0].record(stream)
    for i in range(steps):
        fn()
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]
    return ev[0].elapsed_time(ev[-1]), per


def _line(args, workload_cfg, value, ms, extra, emit=True):
    """The workload's result: printed as its own JSON line (``--workload cN``), or
    returned as a summary for the headline line's ``configs``."""
    d = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
         "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
         "dtype": "c64", "data": "synthetic", "config": workload_cfg}
    d.update(extra)
    if emit:
        print(json.dumps(d), flush=True)
    return d


def run_c1(args, emit=True):
    """Small model: GeneralEncoder(rx, ry, rz, rx on 4 wires) + 2 x (U3 on every wire,
    CNOT ring) + Z on every wire, n=4, bsz=32, forward + backward per step."""
    import torch

    import torchquantum_gb300 as tq

    dev = torch.device("cuda")

    class Model(tq.QuantumModule):
        def __init__(self):
            super().__init__()
            self.enc = tq.GeneralEncoder([{"input_idx": [4 * g + w], "func": ["rx", "ry", "rz", "rx"][g],
                                           "wires": [w]} for g in range(4) for w in range(4)])
            self.u3 = tq.QuantumModuleList([tq.Op1QAllLayer(op=tq.U3, n_wires=4, has_params=True, trainable=True)
                                            for _ in range(2)])
            self.cx = tq.QuantumModuleList([tq.Op2QAllLayer(op=tq.CNOT, n_wires=4, circular=True) for _ in range(2)])
            self.meas = tq.MeasureAll(tq.PauliZ)

        def forward(self, x):
            q = tq.QuantumDevice(n_wires=4, bsz=x.shape[0], device=dev)
            self.enc(q, x)
            for a, b in zip(self.u3, self.cx):
                a(q)
                b(q)
            return self.meas(q)

    model = Model().to(dev)
    x = torch.rand(32, 16, device=dev, generator=torch.Generator(device=dev).manual_seed(0)) * np.pi

    def step():
        model.zero_grad(set_to_none=True)
        model(x).sum().backward()

    ms, per = _timed(step, args.steps, args.warmup, dev)
    return _line(args, {"workload": "n=4 bsz=32: encoder (16 rotations) + 2 x (U3 on each wire, CNOT ring), Z per "
                                    "wire, fwd + bwd", "n_wires": 4, "global_batch": 32},
                 32 * args.steps / (ms / 1e3), ms, {"p50_ms": float(np.percentile(per, 50)),
                                                    "p99_ms": float(np.percentile(per, 99))}, emit)


def run_c3(args, emit=True):
    """Fused forward at scale: the headline random circuit at (n=26, bsz=8) with fused
    widths k = 4, 5, 6 and (n=28, bsz=1) with k = 6; circuits/s of the forward pass."""
    import torch

    import torchquantum_gb300 as tq
    from torchquantum_gb300 import workloads as W

    dev = torch.device("cuda")
    res = {}
    widths = (4, 5, 6) if emit else (6,)
    for n, bsz, k in [(26, 8, k) for k in widths] + [(28, 1, 6)]:
        gates, ncols = W.random_circuit(n, args.depth, seed=0)
        th = torch.tensor(W.random_params(bsz, ncols, seed=1), device=dev)
        holder = {}

        def step():
            q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
            q.method = "fused"
            q.fuse_wires = k
            W.apply_circuit(q, gates, th)
            holder["out"] = q.get_states_1d()
            holder["q"] = q

        ms, _ = _timed(step, args.steps, args.warmup, dev)
        q = holder["q"]
        blocks = sum(len(sg.exec_ops) for sg in q._tape)
        tcb = sum(1 for sg in q._tape for op in sg.exec_ops if getattr(op, "tc", False))
        per_step = ms / args.steps
        S = bsz * (1 << n) * 8
        res[f"n{n}_bsz{bsz}_k{k}"] = {"circuits_per_s": bsz * 1e3 / per_step, "ms_per_step": per_step,
                                      "passes": blocks, "tensor_core_blocks": tcb,
                                      "hbm_GBps_2S_per_pass": 2 * S * blocks / (per_step / 1e3) / 1e9}
        del holder
    main = res["n26_bsz8_k6"]
    return _line(args, {"workload": f"random circuit depth {args.depth}, fused forward, n=26 bsz=8 (k="
                                    f"{','.join(str(k) for k in widths)}) and n=28 bsz=1 (k=6)", "n_wires": 26,
                        "global_batch": 8},
                 main["circuits_per_s"], main["ms_per_step"] * args.steps, {"cases": res}, emit)


def run_c5(args, emit=True):
    """Differentiation workload: n=20, bsz=64, 10 layers of (RY, RZ on every wire with
    shared parameters, CZ ladder) = 400 parameters, loss = sum_j w_j <P_j> over 50 random
    Pauli strings; fwd + adjoint bwd per step.  Literal variant (|0> input: all rows equal)
    and a variant with a per-sample RY(x_b) input layer."""
    import torch

    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf
    from torchquantum_gb300 import workloads as W

    dev = torch.device("cuda")
    n, bsz, layers, m = 20, 64, 10, 50
    gates, ncols = W.hea_circuit(n, layers)
    rng = np.random.default_rng(7)
    theta = torch.tensor(rng.uniform(-np.pi, np.pi, size=(1, ncols)).astype(np.float32), device=dev,
                         requires_grad=True)
    x = torch.tensor(rng.uniform(0, np.pi, size=(bsz, n)).astype(np.float32), device=dev)
    paulis = W.random_paulis(n, m, seed=8)
    w = torch.tensor(rng.normal(size=m).astype(np.float32), device=dev)
    out = {}
    # the default engine keeps every tensor-core block's input for the backward (when it
    # fits); "per_sample_input_in_place" runs the reverse sweep in place (O(1) states)
    for variant in ("literal", "per_sample_input", "per_sample_input_in_place"):
        def step():
            theta.grad = None
            q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
            q.method = "fused"
            q.fuse_wires = 6
            if variant.endswith("in_place"):
                q.checkpoint = False
            if variant.startswith("per_sample_input"):
                for wi in range(n):
                    tqf.ry(q, wires=wi, params=x[:, wi:wi + 1])
            W.apply_circuit(q, gates, theta)
            (tq.expval_joint_analytical_batch(q, paulis) * w).sum().backward()

        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        ms, _ = _timed(step, args.steps, args.warmup, dev)
        peak = torch.cuda.max_memory_allocated() - base
        S = bsz * (1 << n) * 8
        out[variant] = {"circuits_per_s": bsz * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                        "peak_bytes": int(peak), "peak_states": peak / S,
                        "autograd_estimate_bytes": int(len(gates) * S)}
    main = out["per_sample_input"]
    return _line(args, {"workload": "n=20 bsz=64, 10 x (RY, RZ per wire, shared params; CZ ladder), 400 params, "
                                    "sum of 50 weighted Pauli strings, fwd + adjoint bwd", "n_wires": n,
                        "global_batch": bsz},
                 main["circuits_per_s"], main["ms_per_step"] * args.steps, {"variants": out}, emit)


def c4_workload(rng):
    """256 circuits: (n, layers) with n ~ U{8..20}, L ~ U{2..40}, and their RY / RZ angles."""
    specs = [(int(rng.integers(8, 21)), int(rng.integers(2, 41))) for _ in range(256)]
    angles = [(rng.uniform(-np.pi, np.pi, (L, n)), rng.uniform(-np.pi, np.pi, (L, n))) for n, L in specs]
    return specs, angles


def run_c4(args, emit=True):
    """Uneven batching: 256 independent circuits, n ~ U{8..20}, L ~ U{2..40} layers of
    (RY, RZ on every wire, angles ~ U[-pi, pi); CZ ladder), output <Z_0> of each, run as
    one persistent kernel (tqk_batch_run) with the launch shape picked by the autotuner
    and captured in a CUDA graph.  value = circuits/s of graph replays (device time);
    e2e = new angles from the host every step (set_matrices: pinned host -> device),
    replay, and <Z> + latencies read back; latency = each circuit's completion time
    after the launch started."""
    import torch

    import torchquantum_gb300 as tq
    from torchquantum_gb300 import batch as B

    dev = torch.device("cuda")
    rng = np.random.default_rng(0)
    specs, angles = c4_workload(rng)
    cb = B.CircuitBatch()
    for (n, _), (ry, rz) in zip(specs, angles):
        cb.add_layered(n, ry, rz)
    t0 = time.perf_counter()
    pb = cb.prepare(dev, config="auto")
    t_tune = time.perf_counter() - t0
    pb.capture()
    for _ in range(args.warmup):
        pb.launch()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for i in range(args.steps):
        pb.graph.replay()
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[-1])
    pb.launch()
    res = pb.result()
    # end to end: new angles every step from the host, replay, read back
    new_mats = [np.concatenate([B.layered_matrices(n, rng.uniform(-np.pi, np.pi, (L, n)),
                                                   rng.uniform(-np.pi, np.pi, (L, n))) for n, L in specs])
                for _ in range(2)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        pb.set_matrices(new_mats[i % 2])
        pb.launch()
        pb.result()
    e2e_s = time.perf_counter() - t0
    h2d = int(new_mats[0].size * 8)  # complex64 matrices
    # default launch shape (no tuning, no graph) for comparison
    cb0 = B.CircuitBatch()
    for (n, _), (ry, rz) in zip(specs, angles):
        cb0.add_layered(n, ry, rz)
    pd = cb0.prepare(dev, config=B.DEFAULT_CONFIG)
    dms, _ = _timed(pd.launch, args.steps, args.warmup, dev)
    # the same circuits one at a time through the engine (fused method), on a sample; a
    # first untimed pass lets the autotuner measure each width once
    sample = list(range(0, 256, 16))

    def one_at_a_time():
        for i in sample:
            (n, L), (ry, rz) = specs[i], angles[i]
            q = tq.QuantumDevice(n_wires=n, bsz=1, device=dev)
            q.method = "fused"
            for l in range(L):
                for w in range(n):
                    tq.functional.ry(q, wires=w, params=float(ry[l, w]))
                    tq.functional.rz(q, wires=w, params=float(rz[l, w]))
                for w in range(n - 1):
                    tq.functional.cz(q, wires=[w, w + 1])
            tq.expval_joint_analytical(q, "Z" + "I" * (n - 1))

    one_at_a_time()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    one_at_a_time()
    torch.cuda.synchronize()
    per_circuit_engine = (time.perf_counter() - t0) / len(sample)
    cfg = pb.config
    # the batch kernel against its bounds: every planned op sweeps its circuit's tile in
    # shared memory (read + write each amplitude: 16 B per amplitude per op); circuits
    # wider than the tile stream their state through HBM once per pass (16 B per amplitude)
    per_launch_s = ms / args.steps / 1e3
    smem_bytes = sum(int(c["num_ops"]) * (1 << int(c["n"])) * 16 for c in pb.circ)
    hbm_bytes = sum(int(c["num_passes"]) * (1 << int(c["n"])) * 16 for c in pb.circ if int(c["state_off"]) >= 0)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    smem_peak = 128 * sms * 2.07e9 / 1e9  # 128 B per clock per SM at the 2070 MHz maximum SM clock
    hbm_peak, hbm_kind = _peaks()
    batch_kernel = {"smem_bytes_per_launch": smem_bytes, "smem_GB/s": smem_bytes / per_launch_s / 1e9,
                    "smem_peak_GB/s": smem_peak, "smem_frac": smem_bytes / per_launch_s / 1e9 / smem_peak,
                    "smem_peak_source": "nominal: 128 B/clock/SM x SMs x 2070 MHz",
                    "hbm_bytes_per_launch": hbm_bytes, "hbm_GB/s": hbm_bytes / per_launch_s / 1e9,
                    "hbm_frac": hbm_bytes / per_launch_s / 1e9 / hbm_peak, "hbm_peak_source": f"{hbm_kind} hbm_gbs"}
    return _line(args, {"workload": "256 circuits, n~U{8..20}, L~U{2..40} x (RY, RZ per wire; CZ ladder), <Z_0> each, one "
                             "persistent kernel in a CUDA graph", "circuits": 256, "n_range": [8, 20],
                 "layers_range": [2, 40],
                 "launch_shape": {"tile_bits": cfg.tile_bits, "threads": cfg.threads, "ctas_per_sm": cfg.ctas_per_sm,
                                  "chosen_by": "autotuner (measured candidates)", "tuning_s": t_tune}},
          256 * args.steps / (ms / 1e3), ms,
          {"e2e": {"value": 256 * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": 256 * 8 + 257 * 8,
                   "includes": "new angles host->device, graph replay, <Z> and latencies device->host"},
           "latency_ms": {"p50": float(np.percentile(res.latency_ms, 50)), "p99": float(np.percentile(res.latency_ms, 99)),
                          "max": float(res.latency_ms.max()),
                          "definition": "each circuit's completion time (%globaltimer) after its launch started"},
           "batch_kernel": batch_kernel,
           "default_launch_shape": {"circuits_per_s": 256 * args.steps / (dms / 1e3), "tile_bits": 14, "threads": 512,
                                    "ctas_per_sm": 1, "graph": False},
           "engine_one_circuit_at_a_time": {"circuits_per_s": 1.0 / per_circuit_engine,
                                            "sample": f"{len(sample)} of the 256 circuits, fused method, sequential"}},
                 emit)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.kernels:
        import torch

        dev = torch.device("cuda")
        roof, res = roofline(args, dev)
        print(json.dumps({"kernels": res, "n_wires": args.n, "bsz": args.bsz}), flush=True)
    elif args.workload == "c1":
        run_c1(args)
    elif args.workload == "c3":
        run_c3(args)
    elif args.workload == "c4":
        run_c4(args)
    elif args.workload == "c5":
        run_c5(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
