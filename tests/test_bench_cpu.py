"""The bench's timed windows (host logic, no GPU).

The 3D plume adapts h every 50 steps (SML_UPDATE_INT, `main.cc`); the bench
times K steps centred on the second pass (step 100) and runs its e2e leg
over K steps centred on the next pass.  These tests pin the window
arithmetic: each window starts after the first pass, holds the same number
of passes, and for K a multiple of 50 holds one pass per 50 steps, the rate
of a run.
"""
import pytest

import bench

INTERVAL = bench.SML_INTERVAL


def _passes(first, last):
    return last // INTERVAL - (first - 1) // INTERVAL


@pytest.mark.parametrize("k", [2, 10, 20, 49, 50, 100, 150])
def test_timed_and_e2e_windows_hold_passes_at_the_same_rate(k):
    warmup = 5
    prep, first = bench.timed_window(warmup, k)
    last = first + k - 1
    assert prep + warmup + 1 == first
    assert first > INTERVAL  # after the first pass: h ~ 1.5 dx
    n = _passes(first, last)
    assert n >= 1
    if k % INTERVAL == 0:
        assert n == k // INTERVAL  # one pass per 50 steps
    e0 = bench.e2e_window(last, k)
    assert e0 > last
    assert _passes(e0, e0 + k - 1) == n


def test_default_window_is_steps_75_to_124():
    prep, first = bench.timed_window(5, 50)
    assert (first, first + 49) == (75, 124)
    assert bench.e2e_window(124, 50) == 125
