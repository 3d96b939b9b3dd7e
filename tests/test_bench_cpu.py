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



def test_parity_selection_compares_like_with_like():
    """The at-size check of the headline pass compares the full mesh's P, F and CSR rows only on
    DOFs whose nodes lie in the oracle's block: with the oracle's own full-mesh pass standing in for
    the GPU's, every error is exactly zero and the column pattern agrees; a planted error in one
    state entry of a sample element and in one K entry of a checked row shows up."""
    import numpy as np

    import bench

    n = 6
    coords, conn, nodeDof, nDof, dU1, dU2 = bench.workload(n)
    sel = bench.parity_selection(conn, nodeDof, len(coords), block=72, sample=40)
    assert len(sel["rows"]) > 0 and len(sel["sample"]) == 40 and sel["sample"].min() >= 72
    full = bench._oracle_model(coords, conn, nodeDof, nDof, np.arange(len(conn)))
    st = full.accept_state(full.compute_elements(dU1, dU1, full.initial_state())["stateTemp"])
    r = full.compute_elements(dU1 + dU2, dU2, st)
    kpos, _ = bench.csr_row_positions(full.indptr, sel["rows"])
    sfull = r["stateTemp"][0]["state"]
    gpu = dict(P=r["P"][sel["rows"]], F=r["F"][sel["rows"]], K=r["Kdata"][kpos], Kcols=full.indices[kpos],
               st_block=sfull[sel["block"]], st_sample=sfull[sel["sample"]])  # fmt: skip
    blk = bench._oracle_model(coords, conn, nodeDof, nDof, sel["block"])
    sb = blk.accept_state(blk.compute_elements(dU1, dU1, blk.initial_state())["stateTemp"])
    rb = blk.compute_elements(dU1 + dU2, dU2, sb)
    orc_block = dict(P=rb["P"], F=rb["F"], Kdata=rb["Kdata"], indptr=blk.indptr, indices=blk.indices,
                     state=rb["stateTemp"][0]["state"])  # fmt: skip
    # P and F of the block model differ from the full mesh's outside the checked rows
    assert np.abs(rb["P"] - r["P"]).max() > 1e-6
    out = bench.oracle_parity(sel, gpu, orc_block, sfull[sel["sample"]])
    assert out["pattern_bit_exact"]
    assert out["R"] == 0.0 and out["F"] == 0.0 and out["K"] == 0.0 and out["state"] == 0.0
    assert set(out["state_per_field"]) == {"stress", "strain", "kappa"}
    bad = dict(gpu, st_sample=gpu["st_sample"].copy(), K=gpu["K"].copy())
    bad["st_sample"][3, 2, 12] *= 1 + 1e-9
    bad["K"][5] *= 1 + 1e-6
    out = bench.oracle_parity(sel, bad, orc_block, sfull[sel["sample"]])
    assert out["state_per_field"]["kappa"] > 1e-11 and out["K"] > 1e-10


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
