#!/usr/bin/env python3
"""Benchmark of the element-evaluation + CSR-assembly pass (one Newton iteration's element loop).

Workload (default, one GPU): boxGen C3D8 64x64x64 unit cube (262,144 elements, 8 quadrature
points, 823,875 DOFs, 64,701,513 CSR entries), interior nodes jittered +-5 % of the element size
(seed 1), von Mises J2 [E=210000, nu=0.3, fy0=250, H=1000].  The history is that of a plastic
uniaxial load path: increment 1 (uniaxial strain 0.25 %) is evaluated and accepted; every timed
step then evaluates increment 2 (a further 0.025 % plus seeded noise), so the radial return runs
at (nearly) every point.  A step = zero P, F, K + one pass over all elements: material update,
residual, tangent, scatter into CSR.  Inputs are larger than L2 (state 218 MB, CSR data
259/518 MB), so no explicit L2 flush is needed.

`value` is the mixed-precision mode (FP32 tangent, FP64 residual/state/return map) with inputs
resident in HBM; `fp64` holds the all-FP64 mode; `e2e` times the same pass through the public
API with host buffers (pinned U, dU in; P, F, K out).  `--impl reference` times the CPU oracle
port of the reference algorithm on all host cores.

Launch: python bench.py [--gpus N --steps K --warmup W] [--impl reference]; for N>1 under
torchrun, each rank runs an independent replica (the element pass does not shard across GPUs).
"""

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

METRIC = "assembled elem/s (K+R) mixed vs FP64 GPU, R rel err≤1e-12; adjoint grads/s"
VM = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]
N_CUBE = 64


def workload(n=N_CUBE):
    from edelweissfe_gb300 import meshes

    coords, conn, nodeDof, nDof = meshes.box(n, n, n, nNodes=8)
    coords = meshes.jitter(coords, 0.05, [1.0 / n] * 3, 1, [0, 0, 0], [1, 1, 1])
    rng = np.random.default_rng(2)
    y = coords[:, 1]
    dU1 = np.zeros(nDof)
    dU1[1::3] = 0.0025 * y
    dU2 = np.zeros(nDof)
    dU2[1::3] = 0.00025 * y
    dU2 += rng.uniform(-1, 1, nDof) * 1e-6
    return coords, conn, nodeDof, nDof, dU1, dU2


def algorithmic_bytes(nEl, nQ, nState, nNodes, nDof, nnz, kbytes, nn=8, dim=3):
    """Unique inputs read once, outputs written once: QP history read+write, connectivity, nodal
    coordinates, dU, K values, R and F.  Geometry tables, slot maps and CSR indices are
    implementation traffic and are not counted."""
    return (nEl * nQ * nState * 8 * 2 + nEl * nn * 4 + nNodes * dim * 8 + nDof * 8 + nnz * kbytes + 2 * nDof * 8)


class ClockSampler:
    FIELDS = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = os.path.join("/tmp", f"efe_clocks_{os.getpid()}.csv")
        self.gpu = gpu_index

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL,
            )  # fmt: skip
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        load = [s for s, w in zip(sm, pw)] if sm else []
        return {
            "sm_mhz": statistics.median(load) if load else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons,
            "samples": len(rows),
            "power_w_max": max(pw) if pw else None,
        }


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_value(name, key):
    """A figure recorded as `key: value` in the committed ncu summary profiles/<name>.txt, or None."""
    p = os.path.join(ROOT, "profiles", name + ".txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            return float(line.split(":")[1])
    return None


def ncu_traffic(name):
    """DRAM bytes per launch from the committed ncu summary (profiles/<name>.txt), or None."""
    return ncu_value(name, "traffic_bytes_per_launch_full_size")


# ------------------------------------------------------------------ shared measurement helpers
def bytes_per_pass(nEl, nQ, nState, nNodes, nDof, nnz, kbytes, nn, dim, state_read=True, n_props=0):
    """Algorithmic bytes of one element pass (unique inputs read once, outputs written once):
    QP history (read and written; written only for hyperelastic states), connectivity, nodal
    coordinates, the displacement vector, per-element properties, K values, R and F."""
    hist = nEl * nQ * nState * 8 * (2 if state_read else 1)
    return hist + nEl * nn * 4 + nNodes * dim * 8 + nDof * 8 + nEl * n_props * 8 + nnz * kbytes + 2 * nDof * 8


# Algorithmic FP64 FLOPs per quadrature point of the small-strain J2 pass (sparse-B forms, linear
# hardening, plastic branch): strain increment B.dU 72 FMA, von Mises update ~150 FLOP
# (vonmises.py:210-251), residual B^T sigma 72 FMA (element.py:322-344); J, J^-1 and dN/dX are
# formed once at set-up, as the reference's initializeElement does.  The FP64 mode adds the tangent
# K_e += B^T C B (C.B 6*3*24 = 432 FMA, B^T (C B) 3*24^2 = 1728 FMA per point, element.py:342); the
# mixed modes form it in FP32 (not counted here).  In mixed-ff the strain and residual run in
# float-float on the FP32 pipe, so only the material update stays FP64.
FP64_FLOP_PER_POINT = {"fp64": 2 * 72 + 150 + 2 * 72 + 2 * (432 + 1728), "mixed": 2 * 72 + 150 + 2 * 72,
                       "mixed-ff": 150}  # fmt: skip


def fma_peak_tflops(fp64, dev, reps=5):
    """Measured FMA throughput (TFLOP/s) of the FP64 (fp64=True) or FP32 pipe of this GPU:
    efe_fma_probe with 8 CTAs of 256 threads per SM, best of `reps` launches, each timed with CUDA
    events on the current stream (the stream of the launch)."""
    import ctypes

    import torch

    from edelweissfe_gb300 import _lib as L

    lib = L.load()
    blocks = 8 * torch.cuda.get_device_properties(dev).multi_processor_count
    iters = 4000 if fp64 else 200000
    sink = torch.zeros(1, dtype=torch.float64, device=dev)
    flops = ctypes.c_int64()
    stream = torch.cuda.current_stream(dev)
    best = None
    for _ in range(reps + 1):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        L.check(lib.efe_fma_probe(1 if fp64 else 0, blocks, iters, ctypes.c_void_p(sink.data_ptr()),
                                  ctypes.c_void_p(stream.cuda_stream), ctypes.byref(flops)), "efe_fma_probe")  # fmt: skip
        b.record(stream)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(b)
        best = ms if best is None else min(best, ms)  # the first launch is a warm-up
    return flops.value / (best * 1e-3) / 1e12


def roofline_fp64(nEl, nQ, precision, kernel_ms, peak_tflops):
    """FP64-pipe roofline of the small-strain J2 element pass: algorithmic FP64 FLOPs of the pass
    (FP64_FLOP_PER_POINT x points) / kernel time, against the probe-measured FP64 FMA peak."""
    flop = nEl * nQ * FP64_FLOP_PER_POINT[precision]
    achieved = flop / (kernel_ms * 1e-3) / 1e12
    return {"achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s", "frac": achieved / peak_tflops,
            "flop_per_element": nQ * FP64_FLOP_PER_POINT[precision], "algorithmic_flop_per_launch": flop,
            "peak_kind": "measured in this run (efe_fma_probe: FP64 FMA chains)"}  # fmt: skip


def roofline_hbm(abytes, kernel_ms, traffic=None):
    peak, kind = peaks()
    achieved = abytes / (kernel_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_kind": kind, "algorithmic_bytes_per_launch": abytes, "kernel_ms": kernel_ms}


def oracle_rate(elType, kind, props, n_side, disp, seed=0, reps=2):
    """Elements per second of the oracle port (the reference's element/material/assembly algorithm)
    on one core for a small n_side^3 (3D) or n_side^2 (2D) block of elType with nodal displacements
    `disp` x N(0, 1) (TL elements: total U; small strain: the increment); `disp` is chosen per call
    as about 1 % of the element size (1.2 % strain, plastic, for the von Mises sample)."""
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    from edelweissfe_gb300 import meshes
    from edelweissfe_gb300.library import element_type
    from oracle.assembly import Model

    et = element_type(elType)
    if et.dim == 3:
        coords, conn, nodeDof, nDof = meshes.box(n_side, n_side, n_side, nNodes=et.nNodes)
    else:
        coords, conn, nodeDof, nDof = meshes.rect(n_side, n_side, nNodes=et.nNodes)
    U = np.random.default_rng(seed).normal(0, disp, nDof)
    g = dict(elType=elType, kind=kind, props=np.tile(props, (len(conn), 1)), conn=conn.astype(np.int64),
             thickness=np.ones(len(conn)), order=np.arange(len(conn)))  # fmt: skip
    m = Model(coords, nodeDof, nDof, [g])
    st = m.initial_state()
    t = time.perf_counter()
    for _ in range(reps):
        m.compute_elements(U, U, st)
    secs = time.perf_counter() - t
    return len(conn) * reps / secs, len(conn) * reps, secs


# ------------------------------------------------------------------ parity at size against the oracle
def parity_selection(conn, nodeDof, nNodes, block=8192, sample=2048, seed=7, dim=3):
    """Elements and rows of the full mesh that the oracle can check at full size.

    block: the first `block` elements (the ones the CPU baseline evaluates); sample: `sample` further
    elements drawn over the whole mesh (seeded), for the state at element indices across every tile;
    rows: the DOFs of the nodes all of whose elements lie in the block -- there P, F and the CSR rows
    of the full mesh are sums over block elements only, the same sums an oracle model of the block
    forms (its DofManager numbering is the full mesh's)."""
    nEl = len(conn)
    blk = np.arange(min(block, nEl))
    rest = np.arange(len(blk), nEl)
    smp = np.sort(np.random.default_rng(seed).choice(rest, min(sample, len(rest)), replace=False))
    inside = np.zeros(nNodes, bool)
    inside[conn[blk].ravel()] = True
    inside[conn[rest].ravel()] = False
    nodes = np.nonzero(inside & (nodeDof >= 0))[0]
    rows = np.sort((nodeDof[nodes][:, None] + np.arange(dim)).ravel())
    return dict(block=blk, sample=smp, rows=rows)


def csr_row_positions(indptr, rows):
    """Positions in the CSR data of every entry of the given rows, row by row."""
    beg = indptr[rows].astype(np.int64)
    n = (indptr[rows + 1] - indptr[rows]).astype(np.int64)
    start = np.repeat(beg - np.concatenate([[0], np.cumsum(n)[:-1]]), n)
    return start + np.arange(int(n.sum())), n


def oracle_parity(sel, gpu, orc_block, orc_sample):
    """Errors of one GPU pass over the full mesh against the oracle on the parity selection.

    gpu: P, F (at sel['rows']), Kcols/K (every entry of those rows), st_block / st_sample ([E, nQ, S]
    state of the block / sample elements); orc_block: the oracle pass over the block elements
    (P, F, Kdata, indptr, indices, state); orc_sample: the oracle state of the sample elements.
    Relative errors are max-norm ratios (largest deviation / largest reference entry); state errors
    are also given per field (stress, strain, kappa each against its own largest entry)."""

    def rel(a, b):
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)) if b.size else 0.0

    rows = sel["rows"]
    pos, n = csr_row_positions(orc_block["indptr"], rows)
    pattern = bool(n.sum() == len(gpu["Kcols"]) and np.array_equal(orc_block["indices"][pos], gpu["Kcols"]))
    st_g = np.concatenate([gpu["st_block"], gpu["st_sample"]])
    st_o = np.concatenate([orc_block["state"], orc_sample])
    S = st_o.shape[-1]
    fields = {"stress": slice(0, 6), "strain": slice(6, 12)}
    if S > 12:
        fields["kappa"] = slice(12, S)
    per_field = {k: rel(st_g[..., s], st_o[..., s]) for k, s in fields.items()}
    return {
        "R": rel(gpu["P"], orc_block["P"][rows]),
        "F": rel(gpu["F"], orc_block["F"][rows]),
        "K": rel(gpu["K"], orc_block["Kdata"][pos]) if pattern else None,
        "state": rel(st_g, st_o),
        "state_per_field": per_field,
        "pattern_bit_exact": pattern,
    }


def max_over_ranks(values, device):
    """Element-wise maximum of per-rank timings over all ranks (every rank gets the result): the
    job's step time is its slowest replica's."""
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_throughput(units_per_rank, world, ms):
    """Whole-job units per second: every replica processes units_per_rank in the max-over-ranks ms."""
    return world * units_per_rank / (ms * 1e-3)


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, rank, world):
    import torch

    from edelweissfe_gb300 import ElementGroup, GPUAssembler

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    coords, conn, nodeDof, nDof, dU1, dU2 = workload(args.n)
    nEl = len(conn)
    sel = parity_selection(conn, nodeDof, len(coords))
    sampler = ClockSampler(dev.index)
    results = {}
    state = {}
    outs = {}
    sampler.start()
    for precision in (("fp64", "mixed", "mixed-ff") if args.precision == "both" else (args.precision,)):
        asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", VM, conn)], precision=precision,
                           device=dev)  # fmt: skip
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        d1 = torch.tensor(dU1, device=dev)
        asm.computeElements(None, d1, d1, P, K, F)  # increment 1
        asm.acceptLastState()
        U = torch.tensor(dU1 + dU2, device=dev)
        dU = torch.tensor(dU2, device=dev)
        stream = torch.cuda.current_stream(dev)
        if not args.no_autotune:
            # the tile shape per group, chosen by timing the variants on these inputs (untimed; the
            # pass reads stateRef and writes stateTemp only, so the state is unchanged)
            from edelweissfe_gb300.autotune import Autotuner

            tuner = Autotuner()
            tuner.tune_assembler(asm, U, dU, P, K, F)
            results.setdefault("tile_variants", {})[precision] = {
                "chosen": int(asm._groups_c[0].tileVariant), "ms": tuner.log[-1][1] if tuner.log else None}

        def step(ev=None):
            P.zero_()
            F.zero_()
            K.zero_()
            asm.status.zero_()
            if ev is not None:
                ev[0].record(stream)
            asm.launch(U, dU, P, K, F)
            if ev is not None:
                ev[1].record(stream)

        for _ in range(args.warmup):
            step()
        asm.check_status()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        t0.record(stream)
        for k in range(args.steps):
            step(evs[k])
        t1.record(stream)
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        ms = t0.elapsed_time(t1) / args.steps
        kms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
        if world > 1:
            ms, kms = max_over_ranks([ms, kms], dev)
        asm.check_status()
        state[precision] = dict(P=P.clone(), K=K.double().clone(), st=asm.group_state(0))
        # the outputs of the timed pass (same inputs every step) that the oracle checks at full size
        kpos, _ = csr_row_positions(asm.indptr_host, sel["rows"])
        rows_d = torch.as_tensor(sel["rows"], device=dev)
        outs[precision] = dict(P=P[rows_d].cpu().numpy(), F=F[rows_d].cpu().numpy(),
                               K=K[torch.as_tensor(kpos, device=dev)].double().cpu().numpy(),
                               Kcols=asm.indices_host[kpos], st_block=state[precision]["st"][sel["block"]],
                               st_sample=state[precision]["st"][sel["sample"]])  # fmt: skip
        results[precision] = dict(ms=ms, kernel_ms=kms, nnz=asm.nnz, asm=asm)
        if precision == "mixed":
            results["e2e"] = run_e2e(asm, dU1 + dU2, dU2, args, dev)
        del P, F, K
    # the arithmetic roofs of this GPU, measured in the same process and clock record as the pass
    results["fp64_peak_tflops"] = fma_peak_tflops(True, dev)
    results["fp32_peak_tflops"] = fma_peak_tflops(False, dev)
    clocks = sampler.stop()
    if len(state) < 2:
        return results, {}, clocks, nEl, nDof, len(coords), dict(sel=sel, outs=outs)
    errs = {
        "R_rel_mixed_ff_vs_fp64": float((state["mixed-ff"]["P"] - state["fp64"]["P"]).abs().max()
                                        / state["fp64"]["P"].abs().max()),
        "state_rel_mixed_ff_vs_fp64": float(np.abs(state["mixed-ff"]["st"] - state["fp64"]["st"]).max()
                                            / np.abs(state["fp64"]["st"]).max()),
        "R_rel_mixed_vs_fp64": float((state["mixed"]["P"] - state["fp64"]["P"]).abs().max()
                                     / state["fp64"]["P"].abs().max()),
        "K_rel_mixed_vs_fp64": float((state["mixed"]["K"] - state["fp64"]["K"]).abs().max()
                                     / state["fp64"]["K"].abs().max()),
        "state_rel_mixed_vs_fp64": float(np.abs(state["mixed"]["st"] - state["fp64"]["st"]).max()
                                         / np.abs(state["fp64"]["st"]).max()),
        "plastic_point_fraction": float((state["fp64"]["st"][..., 12] > 0).mean()),
    }  # fmt: skip
    return results, errs, clocks, nEl, nDof, len(coords), dict(sel=sel, outs=outs)


def run_e2e(asm, U_host, dU_host, args, dev):
    """The same pass through the public API with host buffers, every step moving its own data: pinned
    H2D of U and dU, zeroing, the element pass (GPUAssembler.launch), D2H of P, F, K and the status
    word, all inside the timed region (wall clock, synchronised at both ends).  Steps are pipelined
    over three streams with double-buffered device and host buffers: the read-back of step k
    overlaps the pass of step k+1; step k+2 reuses step k's buffers only after their copies are
    done.  Every step's status is checked after the loop (CutbackRequest as computeElements)."""
    import torch

    Uh = torch.tensor(U_host).pin_memory()
    dUh = torch.tensor(dU_host).pin_memory()
    nb = 2
    U = [asm.constructDofVector() for _ in range(nb)]
    dU = [asm.constructDofVector() for _ in range(nb)]
    P = [asm.constructDofVector() for _ in range(nb)]
    F = [asm.constructDofVector() for _ in range(nb)]
    K = [asm.constructSystemMatrix() for _ in range(nb)]
    st = [torch.zeros(4, dtype=torch.int32, device=dev) for _ in range(nb)]
    Ph = [torch.empty_like(P[0], device="cpu").pin_memory() for _ in range(nb)]
    Fh = [torch.empty_like(F[0], device="cpu").pin_memory() for _ in range(nb)]
    Kh = [torch.empty_like(K[0], device="cpu").pin_memory() for _ in range(nb)]
    nsteps = args.warmup + args.steps
    Sh = torch.zeros((nsteps, 4), dtype=torch.int32).pin_memory()
    s_in, s_run, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev = lambda: torch.cuda.Event()  # noqa: E731
    in_done = [ev() for _ in range(nb)]
    run_done = [ev() for _ in range(nb)]
    out_done = [ev() for _ in range(nb)]
    used = [False] * nb

    def step(k):
        b = k % nb
        with torch.cuda.stream(s_in):
            if used[b]:
                s_in.wait_event(run_done[b])  # the pass of step k-2 has read U[b], dU[b]
            U[b].copy_(Uh, non_blocking=True)
            dU[b].copy_(dUh, non_blocking=True)
            in_done[b].record(s_in)
        with torch.cuda.stream(s_run):
            s_run.wait_event(in_done[b])
            if used[b]:
                s_run.wait_event(out_done[b])  # step k-2's outputs have left the device
            P[b].zero_()
            F[b].zero_()
            K[b].zero_()
            st[b].zero_()
            asm.launch(U[b], dU[b], P[b], K[b], F[b], status=st[b])
            run_done[b].record(s_run)
        with torch.cuda.stream(s_out):
            s_out.wait_event(run_done[b])
            Ph[b].copy_(P[b], non_blocking=True)
            Fh[b].copy_(F[b], non_blocking=True)
            Kh[b].copy_(K[b], non_blocking=True)
            Sh[k].copy_(st[b], non_blocking=True)
            out_done[b].record(s_out)
        used[b] = True

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize(dev)
    t = time.perf_counter()
    for k in range(args.warmup, nsteps):
        step(k)
    torch.cuda.synchronize(dev)
    ms = (time.perf_counter() - t) * 1e3 / args.steps
    if (Sh[:, 0] & 1).any():
        from edelweissfe_gb300.exceptions import CutbackRequest

        raise CutbackRequest("material point failed in the end-to-end pass", 0.5)
    return dict(ms=ms, h2d=2 * U[0].numel() * 8, d2h=2 * P[0].numel() * 8 + K[0].numel() * K[0].element_size() + 16)


# ------------------------------------------------------------------ CPU baseline (oracle port)
_CPU = {}


def _oracle_model(coords, conn, nodeDof, nDof, elements):
    from oracle.assembly import Model

    sub = conn[elements].astype(np.int64)
    g = dict(elType="C3D8", kind="vonmises", props=np.tile(VM, (len(sub), 1)), conn=sub,
             thickness=np.ones(len(sub)), order=np.arange(len(sub)))  # fmt: skip
    return Model(coords, nodeDof, nDof, [g])


def _cpu_setup(n, block):
    """Oracle model of the first `block` elements of the workload, with the increment-1 history."""
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path.insert(0, ROOT)
    coords, conn, nodeDof, nDof, dU1, dU2 = workload(n)
    m = _oracle_model(coords, conn, nodeDof, nDof, np.arange(min(block, len(conn))))
    st = m.accept_state(m.compute_elements(dU1, dU1, m.initial_state())["stateTemp"])
    _CPU.update(model=m, state=st, U=dU1 + dU2, dU=dU2, block=len(m.dofs))


def _cpu_step(_=None):
    """One pass of the oracle over the block (element evaluation + CSR scatter); (elements, seconds)."""
    t = time.perf_counter()
    _CPU["last"] = _CPU["model"].compute_elements(_CPU["U"], _CPU["dU"], _CPU["state"])
    return _CPU["block"], time.perf_counter() - t


def cpu_baseline(n, block=4096, reps=3):
    """Single-core oracle port on `reps` passes over `block` contiguous elements."""
    _cpu_setup(n, block)
    done = 0
    secs = 0.0
    for _ in range(reps):
        d, s = _cpu_step()
        done += d
        secs += s
    return done / secs, done, secs


def oracle_reference_outputs(n, sel):
    """The oracle's outputs on the parity selection of the workload: the last CPU-baseline pass over
    the block (P, F, CSR data and pattern, state) and the state of the sample elements (increment 1
    evaluated and accepted, then increment 2, as on the GPU)."""
    last = _CPU["last"]
    m = _CPU["model"]
    block = dict(P=last["P"], F=last["F"], Kdata=last["Kdata"], indptr=m.indptr, indices=m.indices,
                 state=last["stateTemp"][0]["state"])  # fmt: skip
    coords, conn, nodeDof, nDof, dU1, dU2 = workload(n)
    ms = _oracle_model(coords, conn, nodeDof, nDof, sel["sample"])
    st = ms.accept_state(ms.compute_elements(dU1, dU1, ms.initial_state())["stateTemp"])
    sample = ms.compute_elements(dU1 + dU2, dU2, st)["stateTemp"][0]["state"]
    return block, sample


def run_reference(args):
    """The reference algorithm (oracle port) on all host cores: one process per core, each
    evaluating its own block of the workload per step; value = elements per wall second."""
    import multiprocessing as mp

    cores = os.cpu_count() or 1
    block = 512
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_cpu_setup, initargs=(args.n, block)) as pool:
        vals = []
        for k in range(args.warmup + args.steps):
            t = time.perf_counter()
            out = pool.map(_cpu_step, range(cores), chunksize=1)
            wall = time.perf_counter() - t
            if k >= args.warmup:
                vals.append(sum(o[0] for o in out) / wall)
    value = float(np.median(vals))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "elem/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": block * cores / value * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"C3D8 von Mises J2 {args.n}^3 unit cube (jitter 5%), plastic increment, one element pass",
                   "sample_per_step": f"{cores} processes x {block} elements"},
        "cpu_baseline": {"value": value, "unit": "elem/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} processes x {block} contiguous elements per step, oracle NumPy port "
                                   "of the reference element/material/assembly algorithm"},
        "e2e": {"value": value, "unit": "elem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }  # fmt: skip
    print(json.dumps(line))


# ------------------------------------------------------------------ batched uneven meshes
def batched_meshes(n_meshes=512, seed=3, scale=1.0):
    """512 meshes, element counts log-uniform in [1e3, 5e4] (times `scale`); even index: Quad8
    plane strain total-Lagrangian (CPE8RTL, 2x2 Gauss; the reference has no plane-stress Neo-Hooke),
    near-square nx ~ sqrt(n); odd index: C3D20TL, nx = ny ~ cbrt(n), nz = ceil(n / nx^2).  Neo-Hooke
    (a) with mu log-uniform in [1e2, 1e4], K = 10 mu per mesh.  Displacements: an affine field with a
    per-mesh F = I + 0.05 N(0,1), plus 0.2 % of the element size of seeded noise per node."""
    from edelweissfe_gb300 import meshes

    rng = np.random.default_rng(seed)
    m2, m3 = [], []
    for i in range(n_meshes):
        n = max(2, int(round(np.exp(rng.uniform(np.log(1e3), np.log(5e4))) * scale)))
        mu = float(np.exp(rng.uniform(np.log(1e2), np.log(1e4))))
        if i % 2 == 0:
            nx = max(1, int(round(np.sqrt(n))))
            ny = int(np.ceil(n / nx))
            coords, conn, nodeDof, nDof = meshes.rect(nx, ny, lX=1.0, lY=ny / nx, nNodes=8)
            h = 1.0 / nx
            d = 2
        else:
            nx = max(1, int(round(n ** (1 / 3))))
            nz = int(np.ceil(n / nx**2))
            coords, conn, nodeDof, nDof = meshes.box(nx, nx, nz, lX=1.0, lY=1.0, lZ=nz / nx, nNodes=20)
            h = 1.0 / nx
            d = 3
        Fbar = np.eye(d) + 0.05 * rng.normal(size=(d, d))
        disp = coords @ (Fbar - np.eye(d)).T + 0.002 * h * rng.normal(size=coords.shape)
        U = np.zeros(nDof)
        used = nodeDof >= 0
        for c in range(d):
            U[nodeDof[used] + c] = disp[used, c]
        rec = dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[mu, 10.0 * mu], thickness=1.0, U=U)
        (m2 if d == 2 else m3).append(rec)
    return m2, m3


def batched_e2e(bp, U_host, args):
    """The batched pass end to end through the public API with host buffers: per step, the pinned
    host U of every batch to the device, the captured pass (zeroing + launches), and P, F and the
    status word back to pinned host memory; wall clock, synchronised at both ends.  The tangent
    stays resident for the device linear solve (7.9e9 FP32 entries at full size would not cross the
    host link in a step); what a host Newton driver reads per iteration is the residual and flux."""
    import torch

    Uh = [torch.from_numpy(u).pin_memory() for u in U_host]
    Ph = [torch.empty(b.P.numel(), dtype=torch.float64).pin_memory() for b in bp.batches]
    Fh = [torch.empty(b.F.numel(), dtype=torch.float64).pin_memory() for b in bp.batches]
    Sh = torch.zeros(4, dtype=torch.int32).pin_memory()

    def step():
        for b, u in zip(bp.batches, Uh):
            b.U.copy_(u, non_blocking=True)
        bp.replay()
        for b, p, f in zip(bp.batches, Ph, Fh):
            p.copy_(b.P, non_blocking=True)
            f.copy_(b.F, non_blocking=True)
        Sh.copy_(bp.status, non_blocking=True)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t) * 1e3 / args.steps
    if int(Sh[0]) & 1:
        from edelweissfe_gb300.exceptions import CutbackRequest

        raise CutbackRequest("material point failed in the end-to-end batched pass", 0.5)
    h2d = sum(u.numel() * 8 for u in Uh)
    d2h = sum(p.numel() * 8 + f.numel() * 8 for p, f in zip(Ph, Fh)) + 16
    return ms, h2d, d2h


def run_batched(args):
    import torch

    from edelweissfe_gb300.autotune import Autotuner
    from edelweissfe_gb300.batch import BatchedPass, MeshBatch, chunk_meshes

    sampler = ClockSampler(torch.cuda.current_device())
    t0 = time.perf_counter()
    m2, m3 = batched_meshes(args.batch_meshes, 3, args.batch_scale)
    # batches whose CSR patterns fit int32 indexing (one batch per type unless the type is too large)
    batches = []
    U_host = []
    for ms, et in ((m3, "C3D20TL"), (m2, "CPE8RTL")):
        for chunk in chunk_meshes(ms, et):
            b = MeshBatch(chunk, et, "neohookewa", args.batch_precision, keep_host_pattern=False)
            U_host.append(np.concatenate([m["U"] for m in chunk]))
            b.U.copy_(torch.tensor(U_host[-1]))
            batches.append(b)
    nm2, nm3 = len(m2), len(m3)
    del m2[:], m3[:]  # the host meshes (the device holds the batches)
    setup_s = time.perf_counter() - t0
    bp = BatchedPass(batches, persistent=True)
    tuner = Autotuner()
    tuning = tuner.tune_batched(bp)  # tile variants per batch; persistent vs per-batch timed
    if args.batch_launch == "persistent" and bp.can_persist:
        bp.persistent = True
    bp.capture()
    sampler.start()
    for _ in range(args.warmup):
        bp.replay()
    torch.cuda.synchronize()
    bp.check_status()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.steps):
        bp.replay()
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / args.steps
    e2e_ms, h2d, d2h = batched_e2e(bp, U_host, args)
    clocks = sampler.stop()
    nEl = sum(b.nElements for b in batches)
    n2 = sum(b.nElements for b in batches if b.asm.dim == 2)
    abytes = sum(bytes_per_pass(b.nElements, b.asm.groups[0]._dev["type"].nInt, 13, b.asm.nNodes, b.asm.nDof,
                                b.asm.nnz, 4, b.asm.groups[0]._dev["type"].nNodes, b.asm.dim, state_read=False,
                                n_props=2) for b in batches)  # fmt: skip
    cpu = None
    if not args.no_cpu_baseline:
        r20, d20, s20 = oracle_rate("C3D20TL", "neohookewa", [1000.0, 10000.0], 3, 0.003, reps=10)
        r8, d8, s8 = oracle_rate("CPE8RTL", "neohookewa", [1000.0, 10000.0], 16, 0.0006, reps=40)
        rate = nEl / ((nEl - n2) / r20 + n2 / r8)
        cpu = {"value": rate, "unit": "elem/s", "cores": 1, "kind": "port",
               "sample": f"oracle port: {d20} C3D20TL evaluations ({s20:.1f} s) and {d8} CPE8RTL evaluations "
                         f"({s8:.1f} s), combined in the batch's element mix"}  # fmt: skip
    return {
        "metric": "assembled elem/s (K+R), batched uneven meshes, one CUDA graph (persistent or per-batch launches, "
                  "autotuned)",
        "value": nEl / (ms * 1e-3), "unit": "elem/s", "ms_per_step": ms, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True,
        "dtype": {"mixed": "f64 residual/state + f32 tangent (mixed)", "fp64": "f64",
                  "mixed-ff": "float-float F / residual, f64 Kirchhoff stress and state, f32 tangent (mixed-ff)"}[
            args.batch_precision], "data": "synthetic",
        "config": {"workload": f"{args.batch_meshes} meshes, sizes log-uniform [1e3, 5e4] x {args.batch_scale}: "
                               "CPE8RTL + C3D20TL Neo-Hooke (a)",
                   "elements_quad8": n2, "elements_hexa20": nEl - n2, "meshes_2d": nm2,
                   "meshes_3d": nm3, "batches": len(batches), "nnz": int(sum(b.asm.nnz for b in batches)),
                   "setup_s": setup_s, "l2": "inputs larger than L2 (CSR data 31.7 GB)"},
        "roofline": roofline_hbm(abytes, ms), "cpu_baseline": cpu,
        "e2e": {"value": nEl / (e2e_ms * 1e-3), "unit": "elem/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "result": "P, F and the status word; K stays on the device"},
        "clocks": clocks,
        "launch": "persistent" if bp.persistent else "per-batch",
        "tuning": {"persistent_ms": tuning.get(True), "per_batch_ms": tuning.get(False),
                   "tile_variants": [(k, v, best) for k, v, best in tuner.log if k != "persistent"]},
        "gpu_launches": args.steps * (1 if bp.persistent else len(batches)),
    }  # fmt: skip


# ------------------------------------------------------------------ the Hexa20 TL pass alone
def run_hexa20tl(args):
    """The C3D20TL Neo-Hooke (a) element pass on an n x n x n/2 box (default n = 32: 16,384 elements)
    under F = I + 0.05 N(0,1): CUDA-event time per pass for each precision with an FP32 tangent and
    tile variants 0 (SIMT tangent), 2 and 3 (tangent on the tensor cores), and the difference of each
    variant's K and P from variant 0's."""
    return _run_hexa20(args, "tl")


def run_hexa20ss(args):
    """The C3D20 (3x3x3 Gauss) von Mises element pass of a plastic increment on an n x n x n/2 box
    (default n = 32: 16,384 elements; E = 210 GPa, nu = 0.3, fy0 = 250 MPa, H = 1 GPa, saturation 50
    MPa at delta 10): a first increment of 0.3 % uniaxial strain plus noise is accepted, the timed
    pass runs the second (0.1 %).  Same report as the hexa20tl workload."""
    return _run_hexa20(args, "ss")


def _run_hexa20(args, kind):
    import torch

    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes

    n = args.n if args.n != N_CUBE else 32
    coords, conn, nodeDof, nDof = meshes.box(n, n, max(1, n // 2), nNodes=20)
    rng = np.random.default_rng(1)
    box = f"{n}x{n}x{max(1, n // 2)}"
    if kind == "tl":
        Fbar = np.eye(3) + 0.05 * rng.normal(size=(3, 3))
        disp = coords @ (Fbar - np.eye(3)).T
        U1 = np.zeros(nDof)
        for c in range(3):
            U1[nodeDof + c] = disp[:, c]
        dU2 = U1
        elType, material, props = "C3D20TL", "neohookewa", [300.0, 3000.0]
        metric, workload = "C3D20TL Neo-Hooke (a) element pass", f"C3D20TL {box} box, F = I + 0.05 N(0,1)"
    else:
        def uniaxial(strain, noise):
            U = np.zeros(nDof)
            U[nodeDof + 1] = strain * coords[:, 1]
            U[nodeDof + 0] = -0.3 * strain * coords[:, 0]
            U[nodeDof + 2] = -0.3 * strain * coords[:, 2]
            return U + rng.normal(0, noise / n, nDof)

        U1, dU2 = uniaxial(0.003, 1e-3), uniaxial(0.001, 5e-4)
        elType, material, props = "C3D20", "vonmises", [210e3, 0.3, 250.0, 1000.0, 50.0, 10.0]
        metric = "C3D20 von Mises element pass (plastic increment)"
        workload = f"C3D20 J2 {box} box, second increment of uniaxial strain"
    out = {"metric": f"assembled elem/s (K+R), {metric}", "unit": "elem/s",
           "config": {"workload": workload, "elements": len(conn)},
           "steps": args.steps, "warmup": args.warmup, "precisions": {}}  # fmt: skip
    for prec in ("mixed", "mixed-ff"):
        asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup(elType, material, props, conn)], precision=prec)
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        Ud = torch.tensor(U1, device=asm.device)
        if kind == "ss":
            asm.launch(Ud, Ud, P, K, F)  # the first increment, accepted: a plastic state
            asm.check_status()
            asm.acceptLastState()
            Ud = Ud + torch.tensor(dU2, device=asm.device)
        dUd = torch.tensor(dU2, device=asm.device)
        ref, res = None, {}
        for v in (0, 2, 3):
            asm._groups_c[0].tileVariant = v
            for _ in range(max(1, args.warmup)):
                P.zero_(), K.zero_(), F.zero_()
                asm.launch(Ud, dUd, P, K, F)
            torch.cuda.synchronize()
            asm.check_status()
            Kc, Pc = K.double().cpu().numpy(), P.cpu().numpy()
            ref = ref or (Kc, Pc)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(args.steps):
                asm.launch(Ud, dUd, P, K, F)
            b.record()
            torch.cuda.synchronize()
            ms = a.elapsed_time(b) / args.steps
            res[str(v)] = {"ms": ms, "elem_per_s": len(conn) / (ms * 1e-3),
                           "K_rel_vs_variant0": float(np.abs(Kc - ref[0]).max() / np.abs(ref[0]).max()),
                           "P_rel_vs_variant0": float(np.abs(Pc - ref[1]).max() / np.abs(ref[1]).max())}  # fmt: skip
        out["precisions"][prec] = res
        del asm, P, F, K
        torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------------ Newton iteration counts (64^3 J2)
def run_newton(args):
    """The 64^3 von Mises cube under uniaxial displacement: bottom u_y = 0, left u_x = 0, back u_z = 0,
    top u_y -> 0.005 in 20 increments (maxIncrement 0.05, no extrapolation), Newton to a flux
    residual of 1e-10 x the average flux (no absolute floor) with the device PCG, in FP64 and in
    mixed precision.  Reports the iterations per increment of both and the difference of the
    final displacement fields."""
    import torch

    from edelweissfe_gb300 import ElementGroup, GPUAssembler
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet, NISTGPU

    coords, conn, nodeDof, nDof, _, _ = workload(args.n)
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    dirichlets = [Dirichlet(nodeDof[y < 1e-9] + 1, 0.0), Dirichlet(nodeDof[x < 1e-9] + 0, 0.0),
                  Dirichlet(nodeDof[z < 1e-9] + 2, 0.0), Dirichlet(nodeDof[y > 1 - 1e-9] + 1, 0.005)]  # fmt: skip
    out = {}
    for precision in ("fp64", "mixed"):
        asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", VM, conn)], precision=precision)
        solver = NISTGPU(asm, linsolver="pcg", extrapolation="off", maxIter=15, fluxResidualTolerance=1e-10,
                         pcgPreconditioner=args.pcg_preconditioner,
                         fieldCorrectionTolerance=1e-10, fluxResidualFloor=0.0, pcgTolerance=1e-13)  # fmt: skip
        torch.cuda.synchronize()
        t = time.perf_counter()
        U = solver.solveStep(AdaptiveTimeStepper(maxIncrement=0.05, startIncrement=0.05), dirichlets)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t
        its = [h["iterations"] for h in solver.history]
        out[precision] = dict(U=U.cpu().numpy(), iterations=its, wall_s=wall, pcg_iterations=sum(solver.linearIterations),
                              final_flux=[h["residuals"][-1][0] / h["residuals"][-1][1] for h in solver.history
                                          if h["iterations"] is not None][-1],
                              plastic_fraction=float((asm.group_state(0, "ref")[..., 12] > 0).mean()))  # fmt: skip
        del asm, solver
        torch.cuda.empty_cache()
    f, m = out["fp64"], out["mixed"]
    extra = [b - a for a, b in zip(f["iterations"], m["iterations"]) if a is not None and b is not None]
    print(json.dumps({
        "metric": "Newton iterations per increment to 1e-10, FP64 vs mixed (FP32 tangent) element pass",
        "value": max(extra) if extra else None, "unit": "max extra iterations per increment (mixed - fp64)",
        "higher_is_better": False, "data": "synthetic",
        "config": {"workload": f"C3D8 von Mises J2 {args.n}^3 unit cube (jitter 5%), 20 uniaxial increments to "
                               f"0.5% strain, device PCG (rel. tol 1e-13, preconditioner {args.pcg_preconditioner})",
                   "dofs": nDof, "elements": len(conn)},
        "fp64": {k: v for k, v in f.items() if k != "U"},
        "mixed": {k: v for k, v in m.items() if k != "U"},
        "U_rel_diff_mixed_vs_fp64": float(np.abs(m["U"] - f["U"]).max() / np.abs(f["U"]).max()),
        "gpu_launches": None,
    }))


# ------------------------------------------------------------------ adjoint gradients (32^3 Neo-Hooke)
def adjoint_setup(n=32, seed=4):
    """boxGen C3D8TL n^3 unit cube, per-element E log-normal (median 1000, sigma 0.3, seed 4),
    nu = 0.3 (Neo-Hooke (a): mu = E/2.6, K = E/1.2); bottom fixed, top u_y = -0.01 in 5 increments;
    1000 sensor nodes off the bottom face (seed 5); targets = the solution for E x (1 + 0.1 N(0,1))
    (seed 6)."""
    from edelweissfe_gb300 import meshes

    coords, conn, nodeDof, nDof = meshes.box(n, n, n, nNodes=8)
    E = 1000.0 * np.exp(0.3 * np.random.default_rng(seed).normal(size=len(conn)))
    y = coords[:, 1]
    bottom = np.nonzero(y < 1e-9)[0]
    top = np.nonzero(y > 1 - 1e-9)[0]
    bdofs = (nodeDof[bottom][:, None] + np.arange(3)).ravel()
    tdofs = nodeDof[top] + 1
    cand = np.nonzero(y > 1e-9)[0]
    sensors = np.random.default_rng(seed + 1).choice(cand, min(1000, len(cand)), replace=False)
    sdofs = (nodeDof[sensors][:, None] + np.arange(3)).ravel()
    Epert = E * (1 + 0.1 * np.random.default_rng(seed + 2).normal(size=len(conn)))
    return coords, conn, nodeDof, nDof, E, Epert, bdofs, tdofs, sdofs


def run_adjoint(args):
    """dJ/dE (per element) and dJ/dX (nodal coordinates) of J = 1/2 sum_sensors |u - u*|^2 through
    TLEquilibrium (torch.autograd), timed as gradient evaluations per second at the converged
    solution.  `value` counts one gradient as the adjoint kernel (lambda^T dP/dp, all E_e and all
    X) with the linear solve excluded and timed separately, as the metric is defined for this
    workload; `with_adjoint_solve` counts the adjoint linear solve K^T lambda = dJ/dU (device PCG,
    tangent of the forward solve's last Newton pass, assembled at exactly the converged U) plus the
    kernel; also reported: with the tangent assembled again.  Checked against central differences
    (h = 1e-6) of J through full Newton solves on --fd-directions random directions in (E, X)."""
    import torch

    from edelweissfe_gb300 import ElementGroup, GPUAssembler
    from edelweissfe_gb300.adjoint import TLAdjoint, TLEquilibrium, TLProblem, young_to_lame
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet

    n = args.n if args.n != N_CUBE else 32
    coords, conn, nodeDof, nDof, E0, Epert, bdofs, tdofs, sdofs = adjoint_setup(n)
    dev = torch.device("cuda", 0)
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8TL", "neohookewa",
                       young_to_lame(torch.tensor(E0), 0.3).numpy(), conn)], precision="fp64")  # fmt: skip
    problem = TLProblem(asm, [Dirichlet(bdofs, 0.0), Dirichlet(tdofs, -0.01)],
                        lambda: AdaptiveTimeStepper(maxIncrement=0.2, startIncrement=0.2), linsolver="pcg",
                        extrapolation="linear", maxIter=25, fluxResidualTolerance=1e-12,
                        fieldCorrectionTolerance=1e-13, fluxResidualFloor=0.0, pcgTolerance=1e-14)  # fmt: skip
    X = torch.tensor(coords, device=dev)
    sd = torch.as_tensor(sdofs, device=dev)
    with torch.no_grad():
        target = TLEquilibrium.apply(young_to_lame(torch.tensor(Epert, device=dev), 0.3), X, problem)[sd].clone()

    def J(E, Xc):
        U = TLEquilibrium.apply(young_to_lame(E, 0.3), Xc, problem)
        return 0.5 * ((U[sd] - target) ** 2).sum()

    E = torch.tensor(E0, device=dev, requires_grad=True)
    Xg = X.clone().requires_grad_(True)
    torch.cuda.synchronize()
    t = time.perf_counter()
    J0 = J(E, Xg)
    torch.cuda.synchronize()
    forward_s = time.perf_counter() - t
    newton = [h["iterations"] for h in problem.solver.history]
    t = time.perf_counter()
    J0.backward()
    torch.cuda.synchronize()
    backward_s = time.perf_counter() - t
    gE, gX = E.grad.clone(), Xg.grad.clone()

    # timed gradient evaluations at the solution, solve timed apart: the adjoint kernel with the
    # forward solve's final tangent (assembled at exactly this U by the last Newton pass), and, for
    # reference, with the tangent assembled again
    with torch.no_grad():
        U = problem.solve(young_to_lame(E.detach(), 0.3), X)
        dJdU = torch.zeros(nDof, dtype=torch.float64, device=dev)
        dJdU[sd] = U[sd] - target
        adj = TLAdjoint(problem.solver)
        lam = adj.solve_adjoint(U, dJdU, problem.dirichletDofs)  # reuses solver.lastK
        pcg_its = adj.lastLinearIterations

        def gradient():
            lam = adj.solve_adjoint(U, dJdU, problem.dirichletDofs)
            return asm.adjointTL(U, lam)

        for _ in range(args.warmup):
            gradient()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(args.steps):
            gradient()
        torch.cuda.synchronize()
        gradient_ms = (time.perf_counter() - t) * 1e3 / args.steps  # host clock: the solve reads its residual

        def timed(fn):
            for _ in range(args.warmup):
                fn()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(args.steps):
                fn()
            b.record()
            torch.cuda.synchronize()
            return a.elapsed_time(b) / args.steps

        sampler = ClockSampler(dev.index)
        sampler.start()
        adjoint_ms = timed(lambda: asm.adjointTL(U, lam))
        tangent_ms = timed(lambda: problem.solver.tangentAt(U))
        ms = adjoint_ms
        solve_ms = gradient_ms - adjoint_ms
        # end to end through the public API with host buffers: pinned U and lambda to the device,
        # the adjoint kernel, dJ/dX and dJ/d(mu, K) back to pinned host memory (wall clock)
        Uh, lh = U.cpu().pin_memory(), lam.cpu().pin_memory()
        gXh = torch.empty((len(coords), 3), dtype=torch.float64).pin_memory()
        gPh = torch.empty((len(conn), 2), dtype=torch.float64).pin_memory()
        Ud, ld = torch.empty_like(U), torch.empty_like(lam)

        def e2e_step():
            Ud.copy_(Uh, non_blocking=True)
            ld.copy_(lh, non_blocking=True)
            gX, gP = asm.adjointTL(Ud, ld)
            gXh.copy_(gX, non_blocking=True)
            gPh.copy_(gP[0], non_blocking=True)

        for _ in range(args.warmup):
            e2e_step()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t) * 1e3 / args.steps
        clocks = sampler.stop()

    # central differences on random joint directions (E, X)
    rng = np.random.default_rng(7)
    errs = []
    with torch.no_grad():
        for _ in range(args.fd_directions):
            dE = torch.as_tensor(rng.normal(0, 1, len(conn)) * E0, device=dev)
            dX = torch.as_tensor(rng.normal(0, 1, coords.shape) / n, device=dev)
            h = 1e-6
            fd = (float(J(E.detach() + h * dE, X + h * dX)) - float(J(E.detach() - h * dE, X - h * dX))) / (2 * h)
            ad = float((gE * dE).sum() + (gX * dX).sum())
            errs.append(abs(ad - fd) / abs(fd))
    nEl = len(conn)
    # adjoint kernel algorithmic bytes: read U, lambda (DOF vectors), X, (mu, K); write dX, d(mu, K)
    adj_bytes = 2 * nDof * 8 + 2 * len(coords) * 3 * 8 + nEl * 2 * 8 * 2 + nEl * 8 * 4
    cpu = None
    if not args.no_cpu_baseline:
        r, d, secs = oracle_rate("C3D8TL", "neohookewa", [400.0, 800.0], 8, 0.001, reps=10)
        cpu = {"value": r, "unit": "elem/s", "cores": 1, "kind": "port",
               "sample": f"oracle port forward element pass (the reference has no derivatives): {d} C3D8TL "
                         f"Neo-Hooke evaluations in {secs:.1f} s"}  # fmt: skip
    return {
        "metric": "adjoint grads/s (dJ/dE per element + dJ/dX), excluding the adjoint linear solve, which is timed "
                  "separately (with_adjoint_solve)",
        "value": 1e3 / ms, "unit": "grad/s", "ms_per_step": ms, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"C3D8TL Neo-Hooke (a) {n}^3 unit cube, lognormal E (median 1000, sigma 0.3), "
                               "1000 sensor nodes, bottom fixed, top -0.01 in 5 increments",
                   "elements": nEl, "dofs": nDof, "nnz": int(asm.nnz)},
        "adjoint_kernel_ms": adjoint_ms, "tangent_ms": tangent_ms,
        "with_adjoint_solve": {"value": 1e3 / gradient_ms, "unit": "grad/s", "ms": gradient_ms},
        "with_tangent_reassembled": {"value": 1e3 / (gradient_ms + tangent_ms), "unit": "grad/s"},
        "adjoint_kernel_elem_per_s": nEl / (adjoint_ms * 1e-3),
        "adjoint_solve_ms": solve_ms, "adjoint_pcg_iterations": pcg_its,
        "forward_newton_s": forward_s, "forward_newton_iterations": newton, "autograd_backward_s": backward_s,
        "fd_check": {"directions": args.fd_directions, "h": 1e-6, "max_rel_err": max(errs) if errs else None,
                     "median_rel_err": float(np.median(errs)) if errs else None},
        "pcg_iteration_ms": solve_ms / max(sum(pcg_its), 1),
        "roofline": dict(roofline_hbm(adj_bytes, adjoint_ms),
                         fp64_pipe_active_pct=ncu_value("adjoint_tl_c3d8tl_16cube", "fp64_pipe_active_pct")),
        "cpu_baseline": cpu,
        "e2e": {"value": 1e3 / e2e_ms, "unit": "grad/s", "h2d_bytes_per_step": 2 * nDof * 8,
                "d2h_bytes_per_step": (len(coords) * 3 + nEl * 2) * 8, "ms_per_step": e2e_ms},
        "clocks": clocks,
        "gpu_launches": args.steps,
    }  # fmt: skip


# ------------------------------------------------------------------ plastic-path adjoint (Hexa20 J2)
def plastic_setup(n=96, seed=8):
    """boxGen C3D20 (3x3x3 Gauss) n x n x n/2 on [0,2]x[0,2]x[0,1]; von Mises with E = 210000,
    nu = 0.3 and per-element yield stress U[200, 300], hardening U[800, 1200] (seed 8); bottom
    u_y = 0, left u_x = 0, back u_z = 0, top u_y -> 0.01 (0.5 % strain) in 10 increments."""
    from edelweissfe_gb300 import meshes

    coords, conn, nodeDof, nDof = meshes.box(n, n, max(1, n // 2), lX=2.0, lY=2.0, lZ=1.0, nNodes=20)
    rng = np.random.default_rng(seed)
    E = len(conn)
    props = np.stack([np.full(E, 210e3), np.full(E, 0.3), rng.uniform(200, 300, E), rng.uniform(800, 1200, E),
                      np.zeros(E), np.zeros(E)], 1)  # fmt: skip
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    top = nodeDof[y > 2 - 1e-9] + 1
    bcs = [(nodeDof[y < 1e-9] + 1, 0.0), (nodeDof[x < 1e-9], 0.0), (nodeDof[z < 1e-9] + 2, 0.0), (top, 0.01)]
    return coords, conn, nodeDof, nDof, props, bcs, top


def run_plastic(args):
    """Gradient of the total top reaction after 10 plastic increments w.r.t. the per-element yield
    stress and hardening (config: C3D20 J2 96x96x48).  Forward: Newton (mixed: FP32 tangent, FP64
    residual and return map) with the device PCG, checkpointing the history per increment.
    Backward: PathAdjoint (tangent recomputed per increment from its checkpoint, two reverse
    passes, one adjoint PCG solve refined against the exact FP64 operator).  `value` = gradient
    evaluations per second of the element work of the backward sweep (recomputation + reverse
    passes over all increments), the adjoint solves excluded and timed separately, as for the
    32^3 adjoint; `with_adjoint_solves` = the whole backward sweep.  The forward simulation that
    it differentiates is reported apart.  Also reported: one element pass at the final increment
    in mixed and FP64 (elem/s)."""
    import torch

    from edelweissfe_gb300 import ElementGroup, GPUAssembler
    from edelweissfe_gb300.adjoint import PathAdjoint
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet, NISTGPU

    n = args.plastic_n or (args.n if args.n != N_CUBE else 96)
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    t0 = time.perf_counter()
    coords, conn, nodeDof, nDof, props, bcs, top = plastic_setup(n)
    dirichlets = [Dirichlet(d, v) for d, v in bcs]
    ddofs = np.unique(np.concatenate([d for d, _ in bcs]))

    def forward(pr, precision="mixed"):
        asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D20", "vonmises", pr, conn)], precision=precision)
        solver = NISTGPU(asm, linsolver="pcg", extrapolation="linear", maxIter=15, fluxResidualTolerance=1e-10,
                         fieldCorrectionTolerance=1e-10, fluxResidualFloor=0.0, pcgTolerance=args.pcg_tol,
                         pcgPreconditioner=args.pcg_preconditioner)  # fmt: skip
        adj = PathAdjoint(solver)
        torch.cuda.synchronize()
        t = time.perf_counter()
        solver.solveStep(AdaptiveTimeStepper(maxIncrement=0.1, startIncrement=0.1), dirichlets)
        torch.cuda.synchronize()
        J = -float(solver.lastP[torch.as_tensor(top, device=asm.device)].sum())
        return asm, solver, adj, J, time.perf_counter() - t

    asm, solver, adj, J, fwd_s = forward(props)
    setup_s = time.perf_counter() - t0 - fwd_s
    newton = [h["iterations"] for h in solver.history]
    pcg_fwd = sum(solver.linearIterations)
    cP = asm.constructDofVector()
    cP[torch.as_tensor(top, device=asm.device)] = -1.0
    solver.pcgTolerance = args.pcg_tol_adjoint
    timing = {}
    t = time.perf_counter()
    g = adj.gradient(ddofs, cP=cP, timing=timing)[0]
    torch.cuda.synchronize()
    bwd_s = time.perf_counter() - t
    pcg_adj = [sum(x) for x in adj.linearIterations]
    gH = g[:, 3].cpu().numpy()
    gy = g[:, 2].cpu().numpy()
    plastic = float((asm.groups[0]._dev["stateRef"][12] > 0).double().mean())

    # one element pass at the final increment, mixed and FP64, from the last checkpoint
    ck = adj.checkpoints[-1]
    passes = {}
    for precision in ("mixed", "fp64"):
        a2 = asm if precision == "mixed" else GPUAssembler(coords, nodeDof, nDof, [ElementGroup(
            "C3D20", "vonmises", props, conn)], precision="fp64")  # fmt: skip
        a2.groups[0]._dev["stateRef"].copy_(ck["states"][0])
        P, F, K = a2.constructDofVector(), a2.constructDofVector(), a2.constructSystemMatrix()
        evs = []
        for k in range(args.warmup + args.steps):
            P.zero_()
            F.zero_()
            K.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            a2.launch(ck["U"], ck["dU"], P, K, F)
            e1.record()
            if k >= args.warmup:
                evs.append((e0, e1))
        torch.cuda.synchronize()
        a2.check_status()
        ms = sum(a.elapsed_time(b) for a, b in evs) / len(evs)
        passes[precision] = {"ms": ms, "elem_per_s": len(conn) / (ms * 1e-3)}
        if precision == "fp64":
            del a2, P, F, K
            torch.cuda.empty_cache()

    fd = None
    if args.plastic_fd:
        rng = np.random.default_rng(11)
        errs = []
        for _ in range(args.plastic_fd):
            d = np.zeros_like(props)
            d[:, 2] = rng.normal(0, 1, len(conn)) * props[:, 2]
            d[:, 3] = rng.normal(0, 1, len(conn)) * props[:, 3]
            h = 1e-6
            Jp = forward(props + h * d)[3]
            Jm = forward(props - h * d)[3]
            f = (Jp - Jm) / (2 * h)
            ad = float(np.sum(gy * d[:, 2]) + np.sum(gH * d[:, 3]))
            errs.append(abs(ad - f) / abs(f))
        fd = {"directions": args.plastic_fd, "h": 1e-6, "max_rel_err": max(errs), "errors": errs}
    nInc = len(adj.checkpoints)
    # backward element work per increment: one element pass (the tangent) and two reverse passes,
    # each reading the checkpointed history, the reverse passes also the state adjoint (read + write)
    nQ = 27
    fwd = bytes_per_pass(len(conn), nQ, 13, len(coords), nDof, asm.nnz, 4, 20, 3, n_props=6)
    rev = len(conn) * nQ * 13 * 8 * 4 + len(conn) * 20 * 4 + 3 * nDof * 8 + len(conn) * 6 * 8 * 2
    cpu = None
    if not args.no_cpu_baseline:
        r, d, secs = oracle_rate("C3D20", "vonmises", VM, 3, 0.004, reps=15)
        cpu = {"value": r, "unit": "elem/s", "cores": 1, "kind": "port",
               "sample": f"oracle port forward element pass (the reference has no derivatives): {d} C3D20 von Mises "
                         f"evaluations in {secs:.1f} s"}  # fmt: skip
    clocks = sampler.stop()
    return {
        "metric": "adjoint grads/s (dJ/d(fy0, H) per element through the plastic path), excluding the adjoint solves, "
                  "which are timed separately (with_adjoint_solves)",
        "value": 1e3 / timing["kernel_ms"], "unit": "grad/s", "higher_is_better": True,
        "with_adjoint_solves": {"value": 1.0 / bwd_s, "unit": "grad/s", "backward_wall_s": bwd_s},
        "dtype": "f64 residual/state/return map + f32 tangent (mixed); reverse passes: f64 return map, "
                 "float-float B-products", "data": "synthetic",
        "config": {"workload": f"C3D20 von Mises J2 {n}x{n}x{max(1, n // 2)} on [0,2]x[0,2]x[0,1], per-element "
                               "fy0 ~ U[200,300], H ~ U[800,1200], 10 uniaxial increments to 0.5% strain; "
                               "J = total top reaction", "elements": len(conn), "dofs": nDof, "nnz": int(asm.nnz)},
        "backward_kernel_ms": timing["kernel_ms"], "backward_solve_ms": timing["solve_ms"], "backward_wall_s": bwd_s,
        "increments": nInc, "adjoint_pcg_iterations": pcg_adj,
        "forward_wall_s": fwd_s, "forward_newton_iterations": newton, "forward_pcg_iterations": pcg_fwd,
        "pcg_tolerance": {"forward": args.pcg_tol, "adjoint": args.pcg_tol_adjoint},
        "pcg_preconditioner": args.pcg_preconditioner,
        "J": J, "plastic_point_fraction": plastic,
        "grad_norm": {"fy0": float(np.linalg.norm(gy)), "H": float(np.linalg.norm(gH))},
        "element_pass": passes, "mixed_over_fp64": passes["fp64"]["ms"] / passes["mixed"]["ms"],
        "setup_s": setup_s, "fd_check": fd,
        "roofline": roofline_hbm(nInc * (fwd + 2 * rev), timing["kernel_ms"]), "cpu_baseline": cpu,
        # one gradient end to end through the public API: per-element properties from the host, the
        # forward Newton path with its checkpoints, the backward sweep with its adjoint solves, the
        # gradient back to the host
        "e2e": {"value": 1.0 / (fwd_s + bwd_s), "unit": "grad/s", "h2d_bytes_per_step": int(props.nbytes),
                "d2h_bytes_per_step": int(len(conn) * 2 * 8), "s_per_step": fwd_s + bwd_s},
        "clocks": clocks,
        "gpu_launches": 3 * nInc,  # tangent + two reverse passes per increment
    }  # fmt: skip


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_CUBE, help="elements per cube edge")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default tile variant (0)")
    ap.add_argument("--workload", default="all",
                    choices=["all", "cube", "batched", "newton", "adjoint", "plastic", "hexa20tl", "hexa20ss"],
                    help="all (default): the 64^3 von Mises headline line, with the batched, adjoint and plastic "
                         "workloads under its 'configs' key (one GPU); cube: the headline only; batched: the "
                         "uneven-mesh batch; newton: Newton iterations FP64 vs mixed on the 64^3 cube; adjoint: "
                         "32^3 Neo-Hooke gradients; plastic: Hexa20 J2 96x96x48 path adjoint; hexa20tl: the "
                         "C3D20TL Neo-Hooke pass alone (n x n x n/2) per precision and tile variant; hexa20ss: "
                         "the same for the C3D20 von Mises pass of a plastic increment")
    ap.add_argument("--plastic-fd", type=int, default=0, help="FD directions for the plastic workload")
    ap.add_argument("--plastic-n", type=int, default=0,
                    help="plastic workload mesh (n x n x n/2); 0: 96, or 48 inside the default 'all' run")
    ap.add_argument("--all-fd-directions", type=int, default=6,
                    help="central-difference directions of the adjoint workload inside the default 'all' run")
    ap.add_argument("--pcg-tol", type=float, default=1e-8, help="forward Newton PCG tolerance (plastic)")
    ap.add_argument("--pcg-preconditioner", default="jacobi", choices=["jacobi", "block", "amg"],
                    help="device CG preconditioner of the newton and plastic workloads (amg: aggregation multigrid)")
    ap.add_argument("--pcg-tol-adjoint", type=float, default=1e-10, help="adjoint PCG tolerance (plastic)")
    ap.add_argument("--fd-directions", type=int, default=50, help="central-difference directions (adjoint)")
    ap.add_argument("--batch-meshes", type=int, default=512)
    ap.add_argument("--batch-scale", type=float, default=1.0)
    ap.add_argument("--batch-precision", default="mixed", choices=["mixed", "mixed-ff", "fp64"],
                    help="batched workload: tangent/residual precision")
    ap.add_argument("--batch-launch", default="persistent", choices=["persistent", "auto"],
                    help="batched workload: one persistent launch over all batches, or the autotuner's choice")
    ap.add_argument("--precision", default="both", choices=["both", "mixed", "fp64", "mixed-ff"],
                    help="profiling aid: run one mode only (the JSON line needs both)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.workload in ("batched", "adjoint", "plastic", "hexa20tl", "hexa20ss"):
        if rank == 0:
            fn = {"batched": run_batched, "adjoint": run_adjoint, "plastic": run_plastic,
                  "hexa20tl": run_hexa20tl, "hexa20ss": run_hexa20ss}[args.workload]  # fmt: skip
            print(json.dumps(fn(args), default=str))
        return
    if args.workload == "newton":
        if rank == 0:
            run_newton(args)
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    results, errs, clocks, nEl, nDof, nNodes, checks = run_gpu(args, rank, world)
    if rank != 0:
        return
    if args.precision != "both":
        r = results[args.precision]
        print(json.dumps({"precision": args.precision, "ms_per_step": r["ms"], "kernel_ms": r["kernel_ms"],
                          "elem_per_s": nEl / (r["ms"] * 1e-3)}))
        return
    mixed, fp64, e2e = results["mixed"], results["fp64"], results["e2e"]
    value = job_throughput(nEl, world, mixed["ms"])
    peak, peak_kind = peaks()
    abytes = algorithmic_bytes(nEl, 8, 13, nNodes, nDof, mixed["nnz"], 4)
    achieved = abytes / (mixed["kernel_ms"] * 1e-3) / 1e9
    traffic = ncu_traffic("assemble_c3d8_vm_64cube")
    fp64_peak = results["fp64_peak_tflops"]
    rf64 = roofline_fp64(nEl, 8, "mixed", mixed["kernel_ms"], fp64_peak)
    cpu = None
    parity = None
    if not args.no_cpu_baseline and world == 1:
        v, done, secs = cpu_baseline(args.n, block=8192, reps=3)
        cpu = {"value": v, "unit": "elem/s", "cores": 1, "kind": "port",
               "sample": f"{done} element evaluations (3 passes over the first 8192 elements), oracle NumPy port "
                         f"of the reference algorithm, {secs:.1f} s"}  # fmt: skip
        sel = checks["sel"]
        orc_block, orc_sample = oracle_reference_outputs(args.n, sel)
        parity = {
            "against": "oracle (FP64 NumPy restatement of the reference, pinned to reference-recorded fixtures)",
            "selection": f"state: the first {len(sel['block'])} elements + {len(sel['sample'])} elements sampled "
                         f"over the whole mesh (seed 7); P, F and CSR rows (values and column pattern): the "
                         f"{len(sel['rows'])} DOFs whose nodes lie only in the first {len(sel['block'])} elements",
            "tolerance": {"R": 1e-12, "F": 1e-12, "state": 1e-12, "K_fp64": 1e-12, "K_fp32_tangent": 2e-6},
            "definition": "max |gpu - oracle| / max |oracle| over the selection (state also per field)",
            "tile_variants": {p: int(results[p]["asm"]._groups_c[0].tileVariant) for p in checks["outs"]},
        }  # fmt: skip
        for p, o in checks["outs"].items():
            parity[p] = oracle_parity(sel, o, orc_block, orc_sample)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "elem/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": mixed["ms"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 residual/state/return map + f32 tangent (mixed)",
        "data": "synthetic",
        "config": {
            "workload": f"C3D8 von Mises J2 {args.n}^3 unit cube (jitter 5%), plastic increment, one element pass",
            "elements": nEl,
            "dofs": nDof,
            "nnz": mixed["nnz"],
            "l2": "inputs larger than L2 (state 218 MB, CSR data 259 MB)",
            "parallelism": f"replicas x{world}",
        },
        "fp64": {"value": world * nEl / (fp64["ms"] * 1e-3), "ms_per_step": fp64["ms"], "kernel_ms": fp64["kernel_ms"],
                 "roofline": {"fp64": roofline_fp64(nEl, 8, "fp64", fp64["kernel_ms"], fp64_peak)}},
        "mixed_over_fp64": fp64["ms"] / mixed["ms"],
        "tile_variants": results.get("tile_variants"),
        "mixed_ff": {"value": world * nEl / (results["mixed-ff"]["ms"] * 1e-3), "ms_per_step": results["mixed-ff"]["ms"],
                     "kernel_ms": results["mixed-ff"]["kernel_ms"],
                     "roofline": {"fp64": roofline_fp64(nEl, 8, "mixed-ff", results["mixed-ff"]["kernel_ms"], fp64_peak),
                                  "hbm": roofline_hbm(abytes, results["mixed-ff"]["kernel_ms"])}},
        "errors": errs,
        "parity": parity,
        # the roof that binds the pass is the FP64 pipe (ncu: FP64 pipe ~80 % active, DRAM ~13 %);
        # the HBM fraction of the same launch is kept beside it
        "roofline": {
            "bound": "fp64",
            "achieved": rf64["achieved"],
            "peak": fp64_peak,
            "unit": "TFLOP/s",
            "frac": rf64["frac"],
            "traffic": traffic,
            "peak_kind": rf64["peak_kind"],
            "flop_per_element": rf64["flop_per_element"],
            "algorithmic_flop_per_launch": rf64["algorithmic_flop_per_launch"],
            "kernel_ms": mixed["kernel_ms"],
            "fp64_pipe_active_pct": ncu_value("assemble_c3d8_vm_64cube", "fp64_pipe_active_pct"),
            "fp32_peak_tflops": results["fp32_peak_tflops"],
            "hbm": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                    "algorithmic_bytes_per_launch": abytes, "traffic": traffic},
        },
        "cpu_baseline": cpu,
        "e2e": {
            "value": world * nEl / (e2e["ms"] * 1e-3),
            "unit": "elem/s",
            "h2d_bytes_per_step": e2e["h2d"],
            "d2h_bytes_per_step": e2e["d2h"],
            "ms_per_step": e2e["ms"],
        },
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if args.workload == "all" and world == 1:
        results.clear()
        checks.clear()
        line["configs"] = run_other_configs(args)
    print(json.dumps(line, default=str))


def run_other_configs(args):
    """The other workloads of the benchmark set, each timed on its own with its own roofline, CPU
    baseline, end-to-end figure and clock record: the 512-mesh batched pass (full size; FP64 residual
    and, without a second CPU baseline, float-float residual), the 32^3
    Neo-Hooke adjoint (with args.all_fd_directions finite-difference checks) and the plastic path
    adjoint at 48 x 48 x 24 (the full 96 x 96 x 48 run takes ~11 minutes: --workload plastic)."""
    import gc

    import torch

    out = {}
    jobs = (("batched_512_meshes", run_batched, {}),
            ("batched_512_meshes_mixed_ff", run_batched, {"batch_precision": "mixed-ff", "no_cpu_baseline": True}),
            ("adjoint_32cube", run_adjoint, {"fd_directions": args.all_fd_directions}),
            ("plastic_adjoint_48x48x24", run_plastic, {"plastic_n": args.plastic_n or 48}))  # fmt: skip
    for name, fn, over in jobs:
        gc.collect()
        torch.cuda.empty_cache()
        sub = argparse.Namespace(**dict(vars(args), **over))
        t = time.perf_counter()
        try:
            out[name] = fn(sub)
        except Exception as e:  # reported in the line, not hidden: the headline stays measured
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = time.perf_counter() - t
    return out


if __name__ == "__main__":
    main()
