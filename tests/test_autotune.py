"""Host logic of the launch-shape autotuner (no GPU): candidate lists, the
choice with its tie rule, and the cache file."""
import json

import pytest

from pyquake3d_gb300 import autotune


def test_nsplit_candidates_bounded_by_column_blocks():
    assert autotune.nsplit_candidates(10000) == list(range(1, 17))
    assert autotune.nsplit_candidates(64) == [1, 2, 3, 4]        # 128 columns = 4 blocks of 32
    assert autotune.nsplit_candidates(8) == [1]


def test_pick_prefers_earlier_candidate_within_tie():
    order = [1, 2, 3, 4, 5]
    t = {1: 1.00, 2: 0.60, 3: 0.505, 4: 0.50, 5: 0.52}
    assert autotune.pick(t, order, tie=0.02) == 3      # 0.505 <= 0.50 * 1.02
    assert autotune.pick(t, order, tie=0.0) == 4
    assert autotune.pick(t, order, tie=1.0) == 1


def test_tune_times_every_candidate_once():
    seen = []

    def fake(c):
        seen.append(c)
        return {(1, 2): 3.0, (1, 1): 2.0, (2, 2): 1.0, (2, 1): 1.5}[c]

    order = [(1, 2), (1, 1), (2, 2), (2, 1)]
    choice, times = autotune.tune(order, fake)
    assert choice == (2, 2) and seen == order and times[(1, 1)] == 2.0


def test_cache_file_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv(autotune.ENV_CACHE, str(path))
    autotune.clear()
    k = autotune._key(None, "N=1000", "nsplit")
    assert autotune.lookup(k) is None
    autotune.store(k, 7)
    assert json.loads(path.read_text())[k] == 7
    autotune.clear()                      # a new process: read back from the file
    assert autotune.lookup(k) == 7
    monkeypatch.delenv(autotune.ENV_CACHE)
    autotune.clear()
    assert autotune.lookup(k) is None


def test_unreadable_cache_file_is_ignored(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    monkeypatch.setenv(autotune.ENV_CACHE, str(path))
    autotune.clear()
    assert autotune.lookup("anything") is None
    autotune.store("x", 3)                # rewritten as valid JSON
    assert json.loads(path.read_text()) == {"x": 3}
    autotune.clear()


@pytest.mark.parametrize("B,Bp", [(1, 16), (16, 16), (17, 32), (64, 64)])
def test_padded_runs(B, Bp):
    assert autotune.padded_runs(B) == Bp


def test_ensemble_rejects_unknown_attempt_arithmetic():
    import numpy as np
    import torch
    from pyquake3d_gb300.ensemble import Ensemble
    K = torch.zeros((3 * 4, 2 * 4), dtype=torch.float64)
    with pytest.raises(ValueError):
        Ensemble(K, np.zeros((1, 4, 10)), mu=3e10, Cs=3464.0, precision="fp64", attempt="fp16")
