"""The closed-wake length behind a cylinder, on synthetic fields: a wake of
known length across two embedded levels, no reversed flow, and a wake that
is still open at the last cell."""
import numpy as np

from code_mge_gb300 import cases as K


def _level(n, h, u_of_x):
    """A w array (5, k, j, i) with two ghost layers whose span-averaged u on
    y = 0 is u_of_x, for a block of n x n x 2 cells centred on the origin."""
    sp = K.BlockSpec(n=(n, n, 2), h=(h, h, h), origin=(-0.5 * n * h, -0.5 * n * h, -h), bctype=(-20,) * 6)
    w = np.ones((5, 2 + 4, n + 4, n + 4))
    xc = sp.origin[0] + (np.arange(n) + 0.5) * h
    rho = 1.0 + 0.1 * np.arange(n + 4)[None, :, None]          # rho varies with j only
    w[0] = rho
    w[1] = rho * np.concatenate([[9.0, 9.0], u_of_x(xc), [9.0, 9.0]])[None, None, :]
    return w, sp


def test_length_crosses_levels_and_interpolates():
    u = lambda x: x - 2.7                                     # reattaches at x = 2.7
    fine = _level(64, 1.0 / 16.0, u)                          # covers |x| <= 2
    coarse = _level(64, 1.0 / 8.0, u)                         # covers |x| <= 4
    L = K.recirculation_length([fine, coarse], radius=0.5)
    assert abs(L - 2.2) < 1e-12


def test_no_reversed_flow_gives_zero():
    fine = _level(32, 1.0 / 8.0, lambda x: 0.3 + 0.0 * x)
    assert K.recirculation_length([fine], radius=0.5) == 0.0


def test_open_wake_gives_none():
    fine = _level(32, 1.0 / 8.0, lambda x: -0.1 + 0.0 * x)
    assert K.recirculation_length([fine], radius=0.5) is None
