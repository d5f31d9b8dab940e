"""The barrier-profile analysis (vebisph_gb300/barrier_profile.py) on synthetic timestamps:
per barrier position of a period, the mean work before it and the wait in it."""
import numpy as np

from vebisph_gb300.barrier_profile import phases


def test_phases_recover_work_and_wait():
    period, iters = 3, 4
    work = np.array([10.0, 20.0, 30.0]) * 1e3  # ns
    wait = np.array([1.0, 2.0, 3.0]) * 1e3
    arrive, leave = [0.0], [500.0]  # the solve's first barrier
    t = 500.0
    for _ in range(iters):
        for q in range(period):
            t += work[q]
            arrive.append(t)
            t += wait[q]
            leave.append(t)
    out = phases(np.array(arrive), np.array(leave), period)
    assert out["iterations"] == iters
    assert np.allclose(out["work_us"], [10.0, 20.0, 30.0])
    assert np.allclose(out["wait_us"], [1.0, 2.0, 3.0])


def test_arrival_spread_names_the_late_block():
    from vebisph_gb300.barrier_profile import arrival_spread
    arr = np.zeros((64, 2048), np.uint64)
    arr[:, :4] = np.array([[1000, 1100, 3000, 1200]] * 64, np.uint64)
    sm = np.arange(2048, dtype=np.uint32) + 7
    out = arrival_spread(arr, sm)
    assert out["blocks"] == 4 and out["barriers"] == 64
    assert np.isclose(out["median_of_max_us"], 2.0)
    assert np.isclose(out["median_of_median_us"], 0.15)
    assert out["often_last"] == [(2, 9, 64)]


def test_infer_period():
    from vebisph_gb300.barrier_profile import infer_period
    assert infer_period(668, 22) == 31  # 4 grid-wide levels
    assert infer_period(2 + 20 * 35 - 10, 20) == 35
