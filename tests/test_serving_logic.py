"""Host logic of the serving loop (no GPU): Poisson arrivals, HBM-budget
admission, slot reuse, first-come-first-served order."""
import numpy as np
import pytest

from pyquake3d_gb300.serving import Request, Scheduler, percentile, poisson_arrivals


def _req(i, mesh, t=0.0):
    return Request(rid=i, mesh=mesh, arrival_s=t, table=np.zeros((1, 10)), span_s=1.0)


def test_poisson_arrivals_seeded_and_rate():
    a = poisson_arrivals(4000, 4.0, seed=3)
    b = poisson_arrivals(4000, 4.0, seed=3)
    assert np.array_equal(a, b) and np.all(np.diff(a) > 0)
    assert abs(len(a) / a[-1] - 4.0) < 0.25


def test_budget_admission_and_release():
    s = Scheduler({0: 100, 1: 50}, {0: 10, 1: 20}, {0: 3, 1: 2}, budget=195)
    slots = [s.try_admit(_req(i, 0)) for i in range(3)]
    assert slots == [0, 1, 2] and s.used == 180
    assert s.try_admit(_req(3, 0)) is None          # no free slot
    assert s.try_admit(_req(4, 1)) is None          # budget: 180 + 20 > 195
    s.release(0, 1)
    assert s.try_admit(_req(5, 1)) == 0              # 170 + 20 <= 195
    assert s.try_admit(_req(6, 0)) is None          # 190 + 10 > 195
    s.release(1, 0)
    assert s.try_admit(_req(7, 0)) == 1              # the freed slot is reused


def test_operators_over_budget_refused():
    with pytest.raises(MemoryError):
        Scheduler({0: 200}, {0: 1}, {0: 1}, budget=100)


def test_percentile_empty_is_nan():
    assert np.isnan(percentile([], 50))
    assert percentile([1.0, 2.0, 3.0], 50) == 2.0
