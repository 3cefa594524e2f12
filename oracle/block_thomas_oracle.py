"""CPU oracle for the batched block-Thomas solve.

TEST INFRASTRUCTURE ONLY (imported by ``tests/`` and ``bench.py``'s CPU
baseline leg).

:func:`block_thomas` restates ``pyrometheus/flamelets/linear_solver.py:6-103``
with numpy: a forward sweep that solves with the modified diagonal block twice
per row (``S = C'^-1 U``, ``t = C'^-1 b'``, ``:54-66``) and a backward sweep
that solves with it again (``:87-100``), each solve an LU with partial
pivoting (``np.linalg.solve``, LAPACK ``gesv``, like ``jnp.linalg.solve`` on
CPU).  :func:`make_systems` draws the benchmark's diagonally dominant random
blocks.
"""

from __future__ import annotations

import numpy as np


def block_thomas(lower, central, upper, rhs):
    """``lower``/``upper``: (N-1, nv, nv); ``central``: (N, nv, nv);
    ``rhs``: (N, nv).  Returns x: (N, nv)."""
    n = central.shape[0]
    c_tmp = [central[0]]
    b_tmp = [rhs[0]]
    for i in range(1, n):
        s = np.linalg.solve(c_tmp[-1], upper[i - 1])
        t = np.linalg.solve(c_tmp[-1], b_tmp[-1])
        c_tmp.append(central[i] - lower[i - 1] @ s)
        b_tmp.append(rhs[i] - lower[i - 1] @ t)
    x = [None] * n
    x[n - 1] = np.linalg.solve(c_tmp[n - 1], b_tmp[n - 1])
    for i in range(n - 2, -1, -1):
        x[i] = np.linalg.solve(c_tmp[i], b_tmp[i] - upper[i] @ x[i + 1])
    return np.stack(x)


def dense_matrix(lower, central, upper):
    """Assemble the full (N nv) x (N nv) matrix (for small checks)."""
    n, nv = central.shape[0], central.shape[1]
    a = np.zeros((n * nv, n * nv))
    for i in range(n):
        a[i * nv:(i + 1) * nv, i * nv:(i + 1) * nv] = central[i]
        if i < n - 1:
            a[i * nv:(i + 1) * nv, (i + 1) * nv:(i + 2) * nv] = upper[i]
            a[(i + 1) * nv:(i + 2) * nv, i * nv:(i + 1) * nv] = lower[i]
    return a


def make_systems(n_systems, nv, n_min=64, n_max=1024, seed=0,
                 diag_scale=10.0):
    """Seeded systems: lengths ~ U[n_min, n_max]; off-diagonal entries and
    right-hand sides ~ N(0, 1); diagonal blocks N(0, 1) + diag_scale * I.
    Returns (lengths, L, C, U, b) packed along rows (L, U padded with a
    zero block at each system's last row)."""
    rng = np.random.default_rng(seed)
    lengths = rng.integers(n_min, n_max + 1, size=n_systems)
    rows = int(lengths.sum())
    c = rng.standard_normal((rows, nv, nv)) + diag_scale * np.eye(nv)
    lo = rng.standard_normal((rows, nv, nv))
    up = rng.standard_normal((rows, nv, nv))
    b = rng.standard_normal((rows, nv))
    ends = np.cumsum(lengths) - 1
    lo[ends] = 0.0
    up[ends] = 0.0
    return lengths, lo, c, up, b


def solve_packed(lengths, lo, c, up, b):
    out = np.empty_like(b)
    r0 = 0
    for n in lengths:
        n = int(n)
        out[r0:r0 + n] = block_thomas(lo[r0:r0 + n - 1], c[r0:r0 + n],
                                      up[r0:r0 + n - 1], b[r0:r0 + n])
        r0 += n
    return out
