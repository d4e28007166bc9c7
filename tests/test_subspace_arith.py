"""The FP32 index arithmetic of the subspace-skipping kernels (sgpp_gb300/csrc/subspace.cu),
emulated exactly on the CPU: for every level 1..20 the cell index stays inside [0, 2^{l-1} - 1]
and the hat of the chosen cell equals the hat of the point's cell, for random points, the cube
faces, dyadic nodes, their float neighbours and points outside [0, 1]; for the float-float
(df64) kernel the hat pair is the exact hat of x_hi + x_lo."""
import math
from fractions import Fraction

import numpy as np

F = np.float32
MAGIC = 2.0 ** 23


def kernel_arith(x, S, L):
    """FP32 kernel: r = fma_rd(xc, S, 2^23), t = fma(x, L, fma(r, -2, 2^24 - 1))."""
    xc = np.minimum(np.maximum(x, F(0)), F(0.99999994))
    k = np.floor(np.float64(xc) * float(S))          # xc S is exact; rounding down gives floor
    r = MAGIC + k                                    # in [2^23, 2^24): spacing 1, exact
    n_i = r * -2.0 + (2.0 ** 24 - 1.0)               # -(2k + 1), exact
    t = (np.float64(x) * float(L) + n_i).astype(np.float32)  # exact in FP64, one FP32 rounding
    return k.astype(np.int64), np.clip(F(1) - np.abs(t), 0, 1)


def test_round_down_magic_gives_floor():
    # 2^23 + k for k in [0, 2^23) are consecutive floats: the round-down addend yields floor
    assert np.float32(MAGIC + 1) - np.float32(MAGIC) == 1.0
    assert float(np.float32(2.0 ** 24 - 1)) == 2.0 ** 24 - 1


def test_cell_index_in_range_and_hat_exact():
    rng = np.random.default_rng(0)
    worst = 0.0
    for level in range(1, 21):
        S, L = F(2.0 ** (level - 1)), F(2.0 ** level)
        nodes = (rng.integers(0, 2 ** level + 1, 4000) / 2.0 ** level).astype(np.float32)
        x = np.concatenate([rng.random(50000).astype(np.float32), nodes,
                            np.nextafter(nodes, F(0)), np.nextafter(nodes, F(1)),
                            np.array([0, 1, 0.99999994, 1e-30, -0.3, 1.7], np.float32)])
        k, h = kernel_arith(x, S, L)
        assert k.min() >= 0 and k.max() <= S - 1, level
        xd = np.float64(x)
        kt = np.clip(np.floor(xd * float(S)), 0, float(S) - 1)
        exact = np.maximum(1 - np.abs(xd * float(L) - (2 * kt + 1)), 0)
        worst = max(worst, float(np.abs(np.float64(h) - exact).max()))
    assert worst < 1e-7


def _f32_down(q: Fraction) -> np.float32:
    """Largest float32 <= q."""
    f = np.float32(float(q))
    while Fraction(float(f)) > q:
        f = np.nextafter(f, F(-np.inf))
    while Fraction(float(np.nextafter(f, F(np.inf)))) <= q:
        f = np.nextafter(f, F(np.inf))
    return f


def _f32_near(q: Fraction) -> np.float32:
    """float32 nearest to q (ties to even)."""
    f = _f32_down(q)
    up = np.nextafter(f, F(np.inf))
    d0, d1 = q - Fraction(float(f)), Fraction(float(up)) - q
    if d1 < d0 or (d1 == d0 and (int(up.view(np.uint32)) & 1) == 0):
        return up
    return f


def df_kernel_arith(xh, xl, L):
    """df64 kernel per dimension for a point inside (0, 1): returns (k, hat_hi, hat_lo)."""
    Lq = Fraction(float(L))
    sl = F(L) * xl                                   # exact (power of two)
    t2 = _f32_down(Fraction(float(xh)) * Lq + Fraction(float(sl)))
    rr = _f32_down(Fraction(float(t2)) / 2 + Fraction(MAGIC))
    m2k = _f32_near(Fraction(float(rr)) * -2 + Fraction(2 ** 24))
    a = _f32_near(Fraction(float(xh)) * Lq + Fraction(float(m2k)))
    b = _f32_near(-Fraction(float(xh)) * Lq + Fraction(float(F(2) - m2k)))
    c = F(F(2) * sl) + F(a - b)                      # fma(2, sl, a - b): 2 sl is exact
    rise = c <= 0
    k = int(float(rr) - MAGIC)
    return k, (a if rise else b), (sl if rise else -sl)


def test_float_float_cell_and_hat_exact():
    """df64 subspace kernel: the cell of x_hi + x_lo (not of x_hi alone) and an exact hat pair,
    for points within a float ulp of cell boundaries, random points and the (0, 1) filter."""
    rng = np.random.default_rng(1)
    for level in range(1, 21):
        S, L = 2.0 ** (level - 1), 2.0 ** level
        b = rng.integers(0, int(S) + 1, 150) / S
        x = np.concatenate([b + rng.normal(0, 1e-8, b.size) * rng.choice([0, 0.1, 1], b.size),
                            rng.random(100), np.array([0, 1, 1 - 1e-17, 1e-17, -1e-17, 1 - 2e-8])])
        xh = x.astype(np.float32)
        xl = (x - xh.astype(np.float64)).astype(np.float32)
        for h, lo in zip(xh, xl):
            xq = Fraction(float(h)) + Fraction(float(lo))
            inside = (h > 0 or (h == 0 and lo > 0)) and (h < 1 or (h == 1 and lo < 0))
            assert inside == (0 < xq < 1)
            if not inside:
                continue  # every Linear-grid hat is 0 outside (0, 1): the kernel writes 0
            k, hh, hl = df_kernel_arith(h, lo, L)
            kt = math.floor(xq * int(S))
            assert 0 <= k <= S - 1 and k == kt, (level, h, lo)
            exact = max(1 - abs(xq * int(L) - (2 * kt + 1)), 0)
            assert Fraction(float(hh)) + Fraction(float(hl)) == exact, (level, h, lo)
