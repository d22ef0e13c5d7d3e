"""Knot vectors for the B-spline basis.

explin_knots builds the exponential-then-linear grids the benchmark
configurations use; generate_grid restates the reference's own grid
(src/tools/grid_tools.f90:5-54).  Both return the full knot vector t(1:n+k)
with k-fold end knots, ready for Bs2e(knots, k, ...): the basis keeps
n_b = n - 2 splines (first and last dropped, bspline_tools.f90:33-34).
"""
import math

import numpy as np


def explin_knots(k, n_b, r_max, n_exp=15, r0=0.05, alpha=0.3):
    """First n_exp breakpoints r_i = r0 (exp(alpha i) - 1), i = 0..n_exp-1, then
    uniform spacing up to r_max chosen so that the basis has exactly n_b splines;
    end knots repeated k times."""
    n_knots = n_b + k + 2
    n_uniform = n_knots - (2 * k - 1) - (n_exp - 1)
    if n_uniform < 1:
        raise ValueError("n_b too small for this grid")
    r_exp = [r0 * (math.exp(alpha * i) - 1.0) for i in range(1, n_exp)]
    r_last = r_exp[-1]
    if r_last >= r_max:
        raise ValueError("r_max inside the exponential part")
    h = (r_max - r_last) / n_uniform
    uni = [r_last + h * u for u in range(1, n_uniform)] + [float(r_max)]
    t = [0.0] * k + r_exp + uni + [float(r_max)] * (k - 1)
    t = np.asarray(t, dtype=np.float64)
    assert t.size == n_knots
    return t


def generate_grid(k, m, Z, h_max, r_max):
    """generate_grid (src/tools/grid_tools.f90:5-54): k zeros, m steps of 2^-m,
    geometric growth until the step reaches Z*h_max, linear to Z*r_max, k-1
    repeated end knots, everything divided by Z."""
    h = 2.0 ** (-m)
    g = [0.0] * k
    for _ in range(m):
        g.append(g[-1] + h)
    while True:
        nxt = g[-1] * (1.0 + h)
        if nxt - g[-1] >= h_max * Z:
            break
        g.append(nxt)
    while g[-1] < Z * r_max:
        g.append(g[-1] + Z * h_max)
    g.extend([g[-1]] * (k - 1))
    return np.asarray(g, dtype=np.float64) / Z


def ragged_problems(n=64, seed=0):
    """The ragged batch of radial problems: per problem, in this draw order
    from numpy.random.default_rng(seed): order k from {6, 7, 8}, spline count
    N uniform in [100, 500], max_k uniform in [4, 16], and the largest channel
    l uniform in [0, 8] (it sizes the angular part only).  r_max = N a.u. on
    the exp-linear grid, k_GL = k + 4 Gauss-Legendre points per interval."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        k = int(rng.choice([6, 7, 8]))
        N = int(rng.integers(100, 501))
        max_k = int(rng.integers(4, 17))
        l_max = int(rng.integers(0, 9))
        out.append(dict(k=k, n_b=N, r_max=float(N), k_GL=k + 4, max_k=max_k, l_max=l_max))
    return out
