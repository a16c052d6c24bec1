"""Hydrostatic pressure column of the multicomponent solver (pressure_profile.hpp:
480-496, RK4) and its interpolation (26-41): the library's host routines against the
restatement in the oracle, bit for bit."""
import numpy as np
import pytest

from cases import gm, syn

import oracle


def _column(nc, n, h, top, seed):
    rng = np.random.default_rng(seed)
    y = top - h * np.arange(n + 1)
    T = 1300.0 + 50.0 * np.sin(y / 300.0)
    T1 = 1300.0 + 50.0 * np.sin((y - 0.5 * h) / 300.0)
    Y = np.clip(0.02 + 0.01 * rng.random((n + 1, nc - 1)), 0.0, 1.0)
    Y1 = np.clip(0.02 + 0.01 * rng.random((n + 1, nc - 1)), 0.0, 1.0)
    return y, T, T1, Y, Y1


@pytest.mark.parametrize("nc", [1, 2, 3, 4])
def test_rk4_column_matches_oracle(nc):
    mat = syn.material_for(nc, 0)
    y, T, T1, Y, Y1 = _column(nc, 400, 5.0, 2000.0, nc)
    got = gm.pressure_profile(mat, 1.0e5, 5.0, T, T1, Y, Y1)
    ref = oracle.pressure_profile(mat, 1.0e5, 5.0, T, T1, Y, Y1)
    assert np.array_equal(got, ref)
    assert np.all(np.diff(got) > 0)          # pressure grows downwards


def test_interpolation_matches_oracle_and_rejects_outside():
    mat = syn.material_for(2, 0)
    y, T, T1, Y, Y1 = _column(2, 200, 10.0, 1000.0, 1)
    p = gm.pressure_profile(mat, 2.0e5, 10.0, T, T1, Y, Y1)
    rng = np.random.default_rng(5)
    q = np.concatenate([rng.uniform(y[-1], y[0], 500), y[1:-1], [y[0]]])
    got = gm.pressure_interpolate(y, p, q)
    assert np.array_equal(got, oracle.pressure_interpolate(y, p, q))
    up = y[::-1].copy()                       # ascending columns take the other branch
    assert np.array_equal(gm.pressure_interpolate(up, p[::-1].copy(), q), oracle.pressure_interpolate(up, p[::-1], q))
    with pytest.raises(gm.GalesError):
        gm.pressure_interpolate(y, p, [y[-1] - 1.0])
