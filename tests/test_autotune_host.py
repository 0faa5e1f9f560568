"""Host logic of the tile autotuner: the candidate shapes per form and
lattice, and the per-GPU cache (a cached shape is used without a sweep)."""
import ewpt
from ewpt import _lib, autotune


def test_candidates_per_form_and_lattice():
    fp64 = autotune.candidates_for(ewpt.baseline_couplings(N=64))
    assert fp64 == autotune.CANDIDATES and all(t[3] == 0 for t in fp64)
    df64 = autotune.candidates_for(ewpt.baseline_couplings(N=64, precision=_lib.DF64))
    assert df64 == autotune.CANDIDATES
    fp32 = autotune.candidates_for(ewpt.baseline_couplings(N=64, precision=_lib.FP32))
    assert set(autotune.PAIR_CANDIDATES) <= set(fp32) and set(autotune.TMA_CANDIDATES) <= set(fp32)
    odd = autotune.candidates_for(ewpt.baseline_couplings(shape=(33, 32, 32), N=33, precision=_lib.FP32))
    assert not any(t[3] for t in odd)  # no paired or TMA shapes for odd nx
    ragged = autotune.candidates_for(ewpt.baseline_couplings(shape=(64, 30, 32), N=64, precision=_lib.FP32))
    assert (32, 2, 4, 2) in ragged and (32, 4, 4, 2) not in ragged  # ny % 4 != 0


def test_cached_tiling_is_used_without_a_sweep(tmp_path, monkeypatch):
    monkeypatch.setenv("EWPT_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_key", lambda p: "16x16x16:p1:b0:test-gpu")
    swept = []
    monkeypatch.setattr(autotune, "sweep", lambda p, steps=2, candidates=None: swept.append(p) or
                        [((32, 4, 0, 0), 2.0), ((64, 2, 2, 1), 1.0)])
    p = ewpt.baseline_couplings(N=16, precision=_lib.FP32)
    assert autotune.best_tiling(p) == (64, 2, 2, 1) and len(swept) == 1  # measured, then cached
    assert autotune.best_tiling(p) == (64, 2, 2, 1) and len(swept) == 1  # from the cache
    assert autotune._load_cache()["16x16x16:p1:b0:test-gpu"]["tile"] == [64, 2, 2, 1]
