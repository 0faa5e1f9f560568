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


def test_member_tilings_sweep_once_per_size(tmp_path, monkeypatch):
    """The ensemble's per-member shapes: one sweep per distinct member size
    (no TMA shapes offered; paired shapes only for even nx), cached, and the
    result mapped back onto every member."""
    monkeypatch.setenv("EWPT_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_key", lambda p: "x".join(map(str, p.dims)) + ":test-gpu")
    swept = []

    def fake_sweep(p, steps=2, candidates=None):
        swept.append((p.dims, list(candidates)))
        assert not any(t[3] == 2 for t in candidates)
        best = (8, 16, 2, 1) if p.dims[0] == 48 else (32, 4, 0, 0)
        return [(t, 1.0 if t == best else 2.0) for t in candidates]

    monkeypatch.setattr(autotune, "sweep", fake_sweep)
    ps = [ewpt.baseline_couplings(N=n, precision=_lib.FP32) for n in (48, 33, 48, 48, 33)]
    tiles = autotune.member_tilings(ps)
    assert tiles == [(8, 16, 2, 1), (32, 4, 0, 0), (8, 16, 2, 1), (8, 16, 2, 1), (32, 4, 0, 0)]
    assert [d for d, _ in swept] == [(48, 48, 48), (33, 33, 33)]
    odd = dict(swept)[(33, 33, 33)]
    assert not any(t[3] for t in odd)  # odd nx: one site per thread only
    assert (8, 16, 2, 1) in dict(swept)[(48, 48, 48)]
    assert autotune.member_tilings(ps) == tiles and len(swept) == 2  # from the cache
