"""bench.py helpers that need no GPU: the plain method's gate-mix summary."""
import importlib.util
import os


def _bench():
    spec = importlib.util.spec_from_file_location(
        "bench_mod", os.path.join(os.path.dirname(os.path.dirname(__file__)), "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_plain_pass_summary_weights_the_gate_mix():
    b = _bench()
    S = 1 << 31
    kernels = {"dense1_fwd": {"bytes": 2 * S, "us": 600.0}, "cnot_fwd": {"bytes": S, "us": 300.0},
               "cz_fwd": {"bytes": S // 2, "us": 200.0}, "crx_fwd": {"bytes": S, "us": 300.0}}
    out = b.plain_pass_summary(kernels, S, 6800.0)
    t = (0.6 * 600 + 0.4 / 3 * (300 + 200 + 300)) * 1e-6
    nbytes = 0.6 * 2 * S + 0.4 / 3 * (S + S / 2 + S)
    assert abs(out["us_per_gate"] - t * 1e6) < 1e-9
    assert abs(out["GB/s"] - nbytes / t / 1e9) < 1e-6
    assert abs(out["uniform_2S_GB/s"] - 2 * S / t / 1e9) < 1e-6
    assert abs(out["frac"] - out["GB/s"] / 6800.0) < 1e-12
    assert abs(sum(b.PLAIN_GATE_MIX.values()) - 1.0) < 1e-12


def test_reference_arm_runs_upstream_on_the_host():
    """``bench.py --impl reference`` times upstream itself (baseline/_ref) when it is
    installed: one JSON line with kind "reference", the CPU model and positive rates."""
    import json
    import subprocess
    import sys

    import pytest

    from oracle import upstream as U

    if not U.available():
        pytest.skip("upstream torchquantum is not installed (baseline/_ref)")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--n", "8",
                        "--depth", "12", "--steps", "2", "--warmup", "1"], capture_output=True, text=True,
                       timeout=300, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "reference" and cb["cpu_model"] and cb["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0
