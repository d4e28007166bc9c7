"""The FP32 index arithmetic of the subspace-skipping kernels (sgpp_gb300/csrc/subspace.cu),
emulated with numpy float32 operations: for every level 1..20 the cell index stays inside
[0, 2^{l-1} - 1] and the hat of the chosen cell equals the exact hat of x's cell, for random
points, the cube faces, dyadic nodes, their float neighbours and points outside [0, 1]."""
import numpy as np

F = np.float32
M = F(12582912.0)          # 1.5 * 2^23
M_BITS = np.uint32(0x4B400000)


def kernel_arith(x, S, L):
    xc = np.minimum(np.maximum(x, F(0)), F(0.99999994))
    y5 = (np.float64(xc) * np.float64(S) - 0.5).astype(np.float32)  # fma: one rounding
    r = (y5 + M).astype(np.float32)
    k = (r.view(np.uint32) - M_BITS).astype(np.int64)
    n_i = ((r - M).astype(np.float32) * F(-2) - F(1)).astype(np.float32)
    t = (np.float64(x) * np.float64(L) + np.float64(n_i)).astype(np.float32)
    return k, np.clip(F(1) - np.abs(t), 0, 1)


def test_magic_constant_with_half_is_not_fp32():
    # the reason the kernels subtract 0.5 in a separate step
    assert float(np.float32(12582911.5)) != 12582911.5


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
