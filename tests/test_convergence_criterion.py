"""The force-convergence criterion that judges the warm start and the aero map
(windtunnel/warmstart.py), against brute-force restatements on synthetic
coefficient series.

A run has converged at the first step after which the mean of Cd and of Cl
over the trailing window (all steps so far while fewer than the window) stays
within the tolerance of the reference values until the end of the series; the
reference is the mean over the last quarter of a long cold run.  The window
(5760 steps) is 12 s of the reference UI's averaging at 60 frames per second
and 8 steps per frame (src/main.ts:586-612)."""
import numpy as np
import pytest


def brute_trailing_mean(x, window):
    return np.array([np.mean(x[max(0, t + 1 - window):t + 1]) for t in range(len(x))])


def brute_convergence_step(cd, cl, ref_cd, ref_cl, window, tol):
    mcd, mcl = brute_trailing_mean(cd, window), brute_trailing_mean(cl, window)
    ok = [abs(a - ref_cd) <= tol * abs(ref_cd) and abs(b - ref_cl) <= tol * abs(ref_cl) for a, b in zip(mcd, mcl)]
    if not ok[-1]:
        return None
    t = len(ok)
    while t > 0 and ok[t - 1]:
        t -= 1
    return t + 1  # 1-based count of the first step of the final run of ok steps


@pytest.fixture(scope="module")
def ws():
    from windtunnel import warmstart
    return warmstart


def test_trailing_mean_matches_definition(ws):
    rng = np.random.default_rng(4)
    x = rng.standard_normal(300)
    for window in (1, 7, 64, 500):
        np.testing.assert_allclose(ws.trailing_mean(x, window), brute_trailing_mean(x, window), rtol=1e-12, atol=1e-12)


def test_window_is_twelve_seconds_of_frames(ws):
    assert ws.WINDOW == 12 * 60 * 8 and ws.TOLERANCE == 0.01


def test_settling_series(ws):
    t = np.arange(4000, dtype=np.float64)
    rng = np.random.default_rng(1)
    cd = 1.0 + 0.6 * np.exp(-t / 400.0) + 0.004 * rng.standard_normal(t.size)
    cl = -2.0 - 1.5 * np.exp(-t / 700.0) + 0.01 * rng.standard_normal(t.size)
    ref_cd, ref_cl = ws.reference_values(cd, cl)
    assert ref_cd == pytest.approx(np.mean(cd[3000:])) and ref_cl == pytest.approx(np.mean(cl[3000:]))
    for window in (50, 200):
        got = ws.convergence_step(cd, cl, ref_cd, ref_cl, window=window)
        want = brute_convergence_step(cd, cl, ref_cd, ref_cl, window, 0.01)
        assert got == want and got is not None and 1000 < got < 4000
        assert ws.convergence_step_cd(cd, ref_cd, window=window) <= got  # drag alone settles no later


def test_series_that_does_not_settle(ws):
    t = np.arange(3000, dtype=np.float64)
    cd = 1.0 + 0.05 * np.sin(t / 150.0)         # +-5 % swings, longer than the window
    cl = np.full(t.size, -2.0)
    assert ws.convergence_step(cd, cl, 1.0, -2.0, window=100) is None
    assert brute_convergence_step(cd, cl, 1.0, -2.0, 100, 0.01) is None


def test_series_that_leaves_and_returns(ws):
    """Within the band early, out of it in the middle, back at the end: the step
    counted is the start of the final stay."""
    cd = np.ones(3000)
    cd[1200:1500] = 1.2
    cl = np.full(3000, -2.0)
    got = ws.convergence_step(cd, cl, 1.0, -2.0, window=100)
    assert got == brute_convergence_step(cd, cl, 1.0, -2.0, 100, 0.01)
    assert 1500 < got < 1700  # the trailing mean clears the excursion ~100 steps after it ends
