"""The cooperative kernel's blocked elimination (kern_coop.cu, factor_block) gives every LU
element the operations of the pivot-by-pivot order (kin_solver.h:97-113 applies them row by
row), in that order. Checked here on the algorithm itself: both orders emulated in Python with
exactly rounded FMAs (fractions), on random filled patterns, for blocks of 1, 2 and 4 pivots,
must agree bit for bit."""
import random
from fractions import Fraction

import pytest


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def filled_pattern(n, density, rnd):
    pat = [[i == j or rnd.random() < density for j in range(n)] for i in range(n)]
    for k in range(n):
        for i in range(k + 1, n):
            if pat[i][k]:
                for j in range(k + 1, n):
                    if pat[k][j]:
                        pat[i][j] = True
    return pat


def pivot_by_pivot(a, pat, n, ghinv):
    a = [r[:] for r in a]
    for k in range(n):
        inv = 1.0 / (a[k][k] + ghinv)
        a[k][k] = inv
        for i in range(k + 1, n):
            if not pat[i][k]:
                continue
            l = a[i][k] * inv
            for j in range(k + 1, n):
                if pat[k][j]:
                    a[i][j] = fma(-l, a[k][j], a[i][j])
            a[i][k] = l
    return a


def blocked(a, pat, n, ghinv, B):
    """factor_block<B>: panel rows by one warp, then each trailing row takes the block's pivots."""
    a = [r[:] for r in a]
    inv = [0.0] * B
    u = [[0.0] * n for _ in range(B)]
    for k in range(0, n, B):
        nb = min(B, n - k)
        for r in range(k, k + nb):   # the panel
            for q in range(k, r):
                if not pat[r][q]:
                    continue
                l = a[r][q] * inv[q - k]
                for j in range(q + 1, n):
                    if pat[q][j]:
                        a[r][j] = fma(-l, u[q - k][j], a[r][j])
                a[r][q] = l
            inv[r - k] = a[r][r] = 1.0 / (a[r][r] + ghinv)
            for j in range(r + 1, n):
                u[r - k][j] = a[r][j] if pat[r][j] else 0.0
        for i in range(k + nb, n):   # trailing rows
            bm = [p < nb and pat[i][k + p] for p in range(B)]
            if not any(bm):
                continue
            l = [0.0] * B
            for p in range(B):
                if bm[p]:
                    x = a[i][k + p]
                    for q in range(p):
                        if bm[q] and pat[k + q][k + p]:
                            x = fma(-l[q], u[q][k + p], x)
                    l[p] = x * inv[p]
            for j in range(k + nb, n):
                m = [bm[p] and pat[k + p][j] for p in range(B)]
                if any(m):
                    x = a[i][j]
                    for p in range(B):
                        if m[p]:
                            x = fma(-l[p], u[p][j], x)
                    a[i][j] = x
            for p in range(B):
                if bm[p]:
                    a[i][k + p] = l[p]
    return a


@pytest.mark.parametrize("B", [1, 2, 4])
def test_blocked_elimination_same_bits(B):
    rnd = random.Random(100 + B)
    for trial in range(30):
        n = rnd.choice([1, 2, 3, 4, 5, 7, 12, 17, 23])
        pat = filled_pattern(n, rnd.choice([0.05, 0.2, 0.5, 0.9]), rnd)
        a = [[rnd.uniform(-1, 1) * 10 ** rnd.uniform(-3, 3) if pat[i][j] else 0.0 for j in range(n)] for i in range(n)]
        ghinv = 10 ** rnd.uniform(0, 4)
        x, y = pivot_by_pivot(a, pat, n, ghinv), blocked(a, pat, n, ghinv, B)
        assert all(x[i][j].hex() == y[i][j].hex() for i in range(n) for j in range(n)), (trial, n)
