"""The tuning table (ew_tune_set / ew_tune_set_staging, read by ew_create and
the batch runtime) and the autotuner's search space, on the CPU (no kernel
runs)."""
import pytest


def test_tuning_table_round_trip():
    from exwave_gb300 import _lib
    L = _lib.load()
    for prec in (0, 1, 2):
        old_cb, old_st = L.ew_tune_get(3, 5, prec), L.ew_tune_get_staging(3, 5, prec)
        assert L.ew_tune_set(3, 5, prec, 3) == 0
        assert L.ew_tune_set_staging(3, 5, prec, 1) == 0
        assert L.ew_tune_get(3, 5, prec) == 3 and L.ew_tune_get_staging(3, 5, prec) == 1
        L.ew_tune_set(3, 5, prec, old_cb)
        L.ew_tune_set_staging(3, 5, prec, old_st)
    assert L.ew_tune_set(3, 5, 3, 1) == -1          # no such precision
    assert L.ew_tune_set_staging(3, 5, 0, 3) == -1  # no such layout
    assert L.ew_tune_set(4, 5, 0, 1) == -1


def test_autotuner_search_space():
    from exwave_gb300 import autotune
    for dim, k in ((2, 4), (3, 5), (3, 7)):
        lines = dim * (k + 1) ** (dim - 1)
        assert all(c * lines <= max(512, lines) for c in autotune.candidates(dim, k))
    assert autotune.stagings(3, 5, "mixed_ff") == [1, 2]
    assert autotune.stagings(3, 3, "mixed") == [1, 2]
    assert autotune.stagings(3, 3, "mixed_ff") == [1]
    assert autotune.stagings(2, 7, "fp64") == [1]
