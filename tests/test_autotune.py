"""Autotuner logic on the host (the GPU measurement is replaced by a model)."""
import pytest


def test_candidates_within_bounds(pkg):
    c = pkg.autotune.candidates(8, 1, 12)
    assert c == sorted(set(c)) and 8 in c and all(1 <= v <= 12 for v in c)
    assert pkg.autotune.candidates(1, 1, 6)[0] == 1
    assert max(pkg.autotune.candidates(6, 1, 6)) == 6


def test_tune_finds_the_optimum_of_a_separable_model(pkg):
    target = [12, 3, 24, 16, 8, 8]

    def model(k):
        return 100.0 + sum((a - b) ** 2 for a, b in zip(k, target))

    best, t, tried = pkg.autotune.tune(model, [6, 6, 12, 8, 8, 4], rounds=6, min_gain=0.0)
    assert model(best) == t <= model([6, 6, 12, 8, 8, 4])
    assert all(lo <= v <= hi for v, (lo, hi) in zip(best, pkg.LAUNCH_BOUNDS))
    assert sum((a - b) ** 2 for a, b in zip(best, target)) < sum((a - b) ** 2 for a, b in zip([6, 6, 12, 8, 8, 4], target))
    assert len(tried) > 1


def test_tune_keeps_start_when_nothing_is_better(pkg):
    best, _, _ = pkg.autotune.tune(lambda k: 1.0, [6, 6, 12, 8, 8, 4])
    assert best == [6, 6, 12, 8, 8, 4]


def test_cache_roundtrip(pkg, tmp_path):
    c = pkg.autotune.TuneCache(tmp_path / "tune.json")
    k = c.key("GB300", 16569, 16570.4, 25000)
    assert c.get(k) is None
    c.put(k, [8, 6, 16, 8, 8, 4])
    assert pkg.autotune.TuneCache(tmp_path / "tune.json").get(k) == [8, 6, 16, 8, 8, 4]


def test_set_launch_rejects_out_of_range_without_gpu(pkg):
    # argument checks happen on the host before any device work
    L = pkg.lib()
    import ctypes as C
    import numpy as np
    k = np.array([0, 6, 12, 8, 8, 4], np.int32)
    assert L.hg_ctx_set_launch(None, k.ctypes.data_as(C.c_void_p), 6) != 0
