"""The tensor exp's plan (wannier90_gb300/csrc/k_oz_exp.cu: halvings, exp_plan,
exp_plan_stable, abs_est) restated in NumPy.  The plan -- Taylor degree, block size and
squarings, the FP64 path's table (k_exp_u in k_fp64.cu) -- depends on ||X||_1 only through
which side of each theta 2^j the norm lies.  The kernel plans from an FP32 estimate of
the norm wherever the estimate is at least 2^-14 from every boundary, and forms the exact
FP64 norm otherwise.  Checked here: the integer halvings equal the halving loop, and on
anti-Hermitian matrices of every scale -- many placed within 1e-4 of a boundary -- every
estimate judged stable gives the exact norm's plan."""
import math
import struct

import numpy as np

THETA = [1.6e-3, 1.68e-2, 6.6e-2, 0.32, 0.78]
DEG, BLK, COST = [4, 6, 8, 12, 16], [4, 3, 4, 4, 4], [3, 3, 4, 5, 6]
MANT = (1 << 52) - 1


def _bits(x):
    return struct.unpack("<q", struct.pack("<d", float(x)))[0]


def halvings_loop(v, th):
    j = 0
    while v > th and j < 60:
        v *= 0.5
        j += 1
    return j


def halvings(v, th):
    vb, tb = _bits(v), _bits(th)
    if vb <= tb:
        return 0
    if (vb >> 52) == 0x7FF and (vb & MANT):
        return 0
    return min((vb >> 52) - (tb >> 52) + (1 if (vb & MANT) > (tb & MANT) else 0), 60)


def plan(nrm):
    best = (16, 4, 0, 1 << 30)
    for c in range(5):
        j = halvings(nrm, THETA[c])
        if COST[c] + j < best[3]:
            best = (DEG[c], BLK[c], j, COST[c] + j)
    return best[:3]


def stable(nrm):
    if not nrm < 1e300:
        return False
    nb = _bits(nrm)
    for th in THETA:
        j = halvings(nrm, th)
        lo, hi = _bits(th * (1 - 2.0 ** -14)), _bits(th * (1 + 2.0 ** -14))
        if j < 60 and not nb < lo + (j << 52):
            return False
        if j > 0 and not nb > hi + ((j - 1) << 52):
            return False
    return True


def _f32_trunc(x):
    """|x| truncated to FP32 through its bits (0 below 2^-60, inf above 2^60)."""
    b = np.abs(x).view(np.int64)
    e = (b >> 52) - 1023
    f = ((((e + 127) << 23) | ((b >> 29) & 0x7FFFFF)).astype(np.uint32)).view(np.float32)
    f = np.where(e < -60, np.float32(0), f)
    return np.where(e > 60, np.float32(np.inf), f)


def norm_estimate(X):
    a, b = _f32_trunc(X.real), _f32_trunc(X.imag)
    q = (a.astype(np.float64) ** 2 + b.astype(np.float64) ** 2).astype(np.float32)
    est = np.sqrt(q).astype(np.float32)
    col = np.zeros(X.shape[1], np.float32)
    for i in range(X.shape[0]):
        col = (col + est[i, :]).astype(np.float32)
    return float(col.max())


def norm_exact(X):
    return max(math.fsum(abs(complex(z)) for z in X[:, j]) for j in range(X.shape[1]))


def test_integer_halvings_equal_the_loop():
    rng = np.random.default_rng(1)
    for th in THETA:
        vs = [math.ldexp(rng.random() + 0.5, int(rng.integers(-80, 80))) for _ in range(20000)]
        vs += [th * f * 2.0 ** k for k in range(-5, 70) for f in (1.0, 1 + 2 ** -52, 1 - 2 ** -53)]
        vs += [0.0, 5e-324, float("inf")]
        assert all(halvings(v, th) == halvings_loop(v, th) for v in vs)


def test_stable_estimates_plan_as_the_exact_norm():
    rng = np.random.default_rng(2)
    n_stable = 0
    for t in range(6000):
        W = int(rng.choice([8, 20, 32]))
        X = rng.standard_normal((W, W)) + 1j * rng.standard_normal((W, W))
        X = X - X.conj().T
        if t % 2:
            # the exact norm within 1e-4 of a boundary theta 2^j
            th = THETA[int(rng.integers(0, 5))] * 2.0 ** int(rng.integers(0, 8))
            X *= th * (1 + rng.uniform(-1e-4, 1e-4)) / norm_exact(X)
        else:
            X *= 10.0 ** rng.uniform(-6, 2)
        est = norm_estimate(X)
        if stable(est):
            n_stable += 1
            assert plan(est) == plan(norm_exact(X)), (est, norm_exact(X))
    assert n_stable > 3000
