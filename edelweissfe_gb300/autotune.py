"""Autotuner for the element pass: picks, per group, the CTA tile shape (EfeGroup.tileVariant) by
timing every variant on the caller's own inputs, and for batches whether the persistent launch or
per-batch launches are faster.  Results are cached in a JSON file keyed by GPU, element type,
material, precision and the element count (rounded to a power of two)."""

import json
import os

import torch

VARIANTS = (0, 1, 2)
TENSOR_VARIANT = 3  # the element tangent on the tensor cores (Hexa20 3x3x3 TL Neo-Hooke or small strain, FP32 tangent)


def variants_for(asm, gi):
    """Tile variants to time for group gi: the CTA shapes 0-2, and the tensor-core tangent where the
    library has it (Hexa20 3x3x3, total-Lagrangian with a hyperelastic material or small strain,
    with an FP32 tangent)."""
    from . import _lib as L
    from .library import element_type

    g = asm.groups[gi]
    et = element_type(g.elType)
    hyper = g.material.lower().startswith("neohooke")
    form_ok = (et.totalLagrangian and hyper) or (not et.totalLagrangian and not hyper)
    tc = (et.shape == L.EFE_HEXA20 and et.rule == L.EFE_RULE_3D_3X3X3 and form_ok
          and asm.kPrecision in (L.EFE_K_FP32, L.EFE_K_FP32_FF))  # fmt: skip
    return VARIANTS + ((TENSOR_VARIANT,) if tc else ())


def default_variant(asm, gi):
    """Tile variant of group gi before (or without) autotuning.  The tensor-core tangent for total-
    Lagrangian Hexa20 groups (faster than the SIMT tiles in both FP32-tangent modes) and for small-
    strain Hexa20 groups with an FP64 residual (mixed); 0 for small-strain Hexa20 groups with a
    float-float residual (mixed-ff), where the tensor-core tile, which runs the FP64 return map of an
    element's 27 points on one warp, is about even with the SIMT tile for linear hardening and slower
    for saturation hardening (C3D20 J2 plastic increment, 16,384 elements: 16.7 against 17.7 M
    elem/s)."""
    from . import _lib as L
    from .library import element_type

    if TENSOR_VARIANT not in variants_for(asm, gi):
        return 0
    et = element_type(asm.groups[gi].elType)
    if not et.totalLagrangian and asm.kPrecision == L.EFE_K_FP32_FF:
        return 0
    return TENSOR_VARIANT


def _key(asm, gi):
    g = asm.groups[gi]
    n = max(1, len(g.conn))
    return "|".join([torch.cuda.get_device_name(asm.device), g.elType.upper(), g.material.lower(), asm.precision,
                     str(1 << (n - 1).bit_length())])  # fmt: skip


def _time(fn, reps=5):
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


class Autotuner:
    def __init__(self, cache=None):
        self.cache_path = cache or os.environ.get(
            "EFE_AUTOTUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "efe_gb300_autotune.json")
        )
        self.cache = {}
        if os.path.exists(self.cache_path):
            try:
                self.cache = json.load(open(self.cache_path))
            except (OSError, ValueError):
                self.cache = {}
        self.log = []

    def save(self):
        try:
            os.makedirs(os.path.dirname(self.cache_path), exist_ok=True)
            json.dump(self.cache, open(self.cache_path, "w"), indent=1)
        except OSError:
            pass

    def tune_assembler(self, asm, U, dU, P, K, F, force=False):
        """Set the fastest tile variant of every group of `asm` (times asm.launch on these buffers).
        The state is not changed: the pass reads stateRef and writes stateTemp only."""
        for gi in range(len(asm.groups)):
            key = _key(asm, gi)
            if key in self.cache and not force:
                asm._groups_c[gi].tileVariant = int(self.cache[key]["variant"])
                continue
            times = {}
            for v in variants_for(asm, gi):
                asm._groups_c[gi].tileVariant = v

                def run():
                    P.zero_()
                    F.zero_()
                    K.zero_()
                    asm.launch(U, dU, P, K, F)

                times[v] = _time(run)
            best = min(times, key=times.get)
            asm._groups_c[gi].tileVariant = best
            self.cache[key] = {"variant": best, "ms": times}
            self.log.append((key, times, best))
        self.save()

    def tune_batched(self, bp):
        """Choose persistent vs per-batch launches for a BatchedPass (and the variants of its groups)."""
        for b in bp.batches:
            self.tune_assembler(b.asm, b.U, b.dU, b.P, b.K, b.F)
        if not bp.can_persist:
            bp.persistent = False
            return {}
        times = {}
        for mode in (True, False):
            bp.persistent = mode
            times[mode] = _time(bp.step)
        bp.persistent = min(times, key=times.get)
        self.log.append(("persistent", times, bp.persistent))
        return times
