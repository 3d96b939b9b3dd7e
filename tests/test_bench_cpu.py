"""bench.py on the CPU: the reference arm's JSON line carries every key of the contract (impl,
metric, value, unit, n_gpus, steps, warmup, ms_per_step, higher_is_better, scaling, vs_baseline,
dtype, data, config.workload, cpu_baseline, e2e with zero transfer bytes), and the roofline
arithmetic: the algorithmic bytes of the 64^3 Hexa8 von Mises pass, recomputed here from its
parts, and achieved / peak."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_prints_the_contract_line():
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1", "--n", "8"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)  # fmt: skip
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):  # fmt: skip
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "elem/s"
    assert line["steps"] == 1 and line["warmup"] == 1 and line["vs_baseline"] is None
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_algorithmic_bytes_of_the_64cube_pass():
    import bench

    nEl, nQ, nNodes, nDof, nnz = 262144, 8, 65**3, 823875, 64701513
    parts = (nEl * nQ * 13 * 8 * 2  # history read + write
             + nEl * 8 * 4  # connectivity
             + nNodes * 3 * 8  # coordinates
             + nDof * 8  # dU
             + nnz * 4  # K values (FP32 tangent)
             + 2 * nDof * 8)  # R and F  # fmt: skip
    assert bench.algorithmic_bytes(nEl, nQ, 13, nNodes, nDof, nnz, 4) == parts == 729766276
    assert bench.bytes_per_pass(nEl, nQ, 13, nNodes, nDof, nnz, 4, 8, 3) == parts
    assert 2700 < parts / nEl < 2800  # ~2.78 kB per element


def test_roofline_fraction_is_achieved_over_peak():
    import bench

    r = bench.roofline_hbm(2.0e9, 1.0, traffic=3.0e9)
    peak, kind = bench.peaks()
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] == peak and r["peak_kind"] == kind
    assert r["achieved"] == pytest.approx(2000.0)
    assert r["frac"] == pytest.approx(2000.0 / peak)
    assert r["traffic"] == 3.0e9



def test_reference_arm_under_torchrun_prints_one_line():
    """Launched as the multi-GPU runs are (torch.distributed.run, two ranks, 127.0.0.1): rank 0
    alone runs the reference arm and prints its line; the other rank exits 0 without work."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--gpus", "2", "--impl", "reference", "--steps", "1",
           "--warmup", "1"]  # the driver's own arguments (torchrun would claim an abbreviated --n)  # fmt: skip
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
