"""Autotuner host logic on the CPU (timing replaced by a table): the fastest tile variant is chosen
per group, the choice is cached under (GPU, type, material, precision, element count rounded up to
a power of two), a second tuner takes it from the cache without timing, `force` re-times, and an
unreadable cache file starts an empty cache."""

from types import SimpleNamespace

import pytest

torch = pytest.importorskip("torch")


def _asm(n0, n1):
    groups = [SimpleNamespace(conn=[0] * n0, elType="C3D8", material="vonmises"),
              SimpleNamespace(conn=[0] * n1, elType="c3d20", material="NeoHookeWa")]  # fmt: skip
    gc = [SimpleNamespace(tileVariant=0), SimpleNamespace(tileVariant=0)]
    return SimpleNamespace(groups=groups, _groups_c=gc, device="cuda:0", precision="mixed", launch=lambda *a: None)


def test_tuner_picks_caches_and_reuses(tmp_path, monkeypatch):
    from edelweissfe_gb300 import autotune

    monkeypatch.setattr(autotune.torch.cuda, "get_device_name", lambda d: "FAKE GPU")
    table = {0: {0: 2.0, 1: 3.0, 2: 1.5}, 1: {0: 4.0, 1: 2.5, 2: 4.0}}  # group -> variant -> ms
    calls = []
    current = {}

    def fake_time(fn, reps=5):  # the tuner times the variants of one group after another, in order
        gi = (len(calls) // len(autotune.VARIANTS)) % 2
        v = current["asm"]._groups_c[gi].tileVariant
        calls.append((gi, v))
        return table[gi][v]

    monkeypatch.setattr(autotune, "_time", fake_time)
    path = tmp_path / "tune.json"
    t = autotune.Autotuner(cache=str(path))
    current["asm"] = asm = _asm(1000, 300)
    t.tune_assembler(asm, None, None, None, None, None)
    assert [c.tileVariant for c in asm._groups_c] == [2, 1]
    assert len(calls) == 6 and path.exists()
    keys = sorted(t.cache)
    assert keys == ["FAKE GPU|C3D20|neohookewa|mixed|512", "FAKE GPU|C3D8|vonmises|mixed|1024"]
    # a second tuner reads the cache: no timing
    calls.clear()
    current["asm"] = asm2 = _asm(1000, 300)
    autotune.Autotuner(cache=str(path)).tune_assembler(asm2, None, None, None, None, None)
    assert calls == [] and [c.tileVariant for c in asm2._groups_c] == [2, 1]
    # force re-times every group
    current["asm"] = asm3 = _asm(1000, 300)
    autotune.Autotuner(cache=str(path)).tune_assembler(asm3, None, None, None, None, None, force=True)
    assert len(calls) == 6 and [c.tileVariant for c in asm3._groups_c] == [2, 1]


def test_tensor_variant_only_where_the_library_has_it():
    """Tile variant 3 (the tensor-core tangent) is timed only for Hexa20 3x3x3 groups, total-Lagrangian
    hyperelastic or small strain, with an FP32 tangent."""
    from edelweissfe_gb300 import _lib as L
    from edelweissfe_gb300 import autotune

    def asm(elType, material, kp):
        return SimpleNamespace(groups=[SimpleNamespace(elType=elType, material=material)], kPrecision=kp)

    assert autotune.variants_for(asm("C3D20TL", "neohookewa", L.EFE_K_FP32), 0) == (0, 1, 2, 3)
    assert autotune.variants_for(asm("C3D20TL", "neohookewb", L.EFE_K_FP32_FF), 0) == (0, 1, 2, 3)
    assert autotune.variants_for(asm("C3D20TL", "neohookewa", L.EFE_K_FP64), 0) == (0, 1, 2)
    assert autotune.variants_for(asm("C3D20TL", "vonmises", L.EFE_K_FP32), 0) == (0, 1, 2)
    assert autotune.variants_for(asm("C3D20RTL", "neohookewa", L.EFE_K_FP32), 0) == (0, 1, 2)
    assert autotune.variants_for(asm("C3D20", "linearelastic", L.EFE_K_FP32), 0) == (0, 1, 2, 3)
    assert autotune.variants_for(asm("C3D20", "vonmises", L.EFE_K_FP32_FF), 0) == (0, 1, 2, 3)
    assert autotune.variants_for(asm("C3D20", "vonmises", L.EFE_K_FP64), 0) == (0, 1, 2)
    assert autotune.variants_for(asm("C3D20R", "vonmises", L.EFE_K_FP32), 0) == (0, 1, 2)
    assert autotune.variants_for(asm("C3D20TL", "vonmises", L.EFE_K_FP32), 0) == (0, 1, 2)
    assert autotune.variants_for(asm("C3D8TL", "neohookewa", L.EFE_K_FP32), 0) == (0, 1, 2)
    # the default before tuning: the tensor-core tile except for small strain with a float-float residual
    assert autotune.default_variant(asm("C3D20TL", "neohookewa", L.EFE_K_FP32), 0) == 3
    assert autotune.default_variant(asm("C3D20TL", "neohookewa", L.EFE_K_FP32_FF), 0) == 3
    assert autotune.default_variant(asm("C3D20", "vonmises", L.EFE_K_FP32), 0) == 3
    assert autotune.default_variant(asm("C3D20", "vonmises", L.EFE_K_FP32_FF), 0) == 0
    assert autotune.default_variant(asm("C3D20", "vonmises", L.EFE_K_FP64), 0) == 0
    assert autotune.default_variant(asm("C3D8", "vonmises", L.EFE_K_FP32), 0) == 0


def test_unreadable_cache_starts_empty(tmp_path, monkeypatch):
    from edelweissfe_gb300 import autotune

    path = tmp_path / "broken.json"
    path.write_text("{not json")
    assert autotune.Autotuner(cache=str(path)).cache == {}
