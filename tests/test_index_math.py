"""Host checks of the wavefront kernels' item index arithmetic
(fluid_gb300/csrc/k_pressure.cu: div_small, used by k_lexsor, k_lexsor_cl,
k_lexsor_grid and k_mg_coarse).

A step's item q (< 2^24) splits into (sweep, cell) = (q / n, q mod n) by a
float reciprocal and one correction:

    t = trunc(float(q) * float(1 / n));  r = q - t * n;  then one step of
    t -= 1 (r < 0) or t += 1 (r >= n).

With q < 2^24 exact in float and both roundings within 2^-24 relative, the
estimate is off by less than 2/n + 2^-23 q/n < 1 for n >= 3 (exact for n = 1,
2), so one correction suffices.  This restates the arithmetic in float32
(IEEE, round to nearest, like the device's default division and multiply) and
checks it against integer division at the worst places: the multiples of n
and their neighbours near the top of the range, for every n a step can have
(diagonal lengths up to 2^15, padded to 32 or not).
"""
import numpy as np


def div_small(q, n):
    q = np.asarray(q, np.int64)
    inv = np.float32(1.0) / np.float32(n)
    t = np.trunc(q.astype(np.float32) * inv).astype(np.int64)
    r = q - t * n
    lo, hi = r < 0, r >= n
    t = np.where(lo, t - 1, np.where(hi, t + 1, t))
    r = np.where(lo, r + n, np.where(hi, r - n, r))
    return t, r


def check(n):
    top = (1 << 24) - 1
    kmax = top // n
    ks = np.unique(np.concatenate([np.arange(0, min(kmax, 64) + 1),
                                   np.arange(max(0, kmax - 64), kmax + 1)]))
    q = (ks[:, None] * n + np.array([-1, 0, 1, n - 1])[None, :]).ravel()
    q = q[(q >= 0) & (q <= top)]
    t, r = div_small(q, n)
    ok = (t == q // n) & (r == q % n)
    assert ok.all(), (n, q[~ok][:5])


def test_div_small_every_divisor_up_to_2_pow_15():
    for n in range(1, (1 << 15) + 1):
        check(n)


def test_div_small_random_items():
    rng = np.random.default_rng(7)
    n = rng.integers(1, 1 << 15, 20000)
    q = rng.integers(0, 1 << 24, 20000)
    inv = np.float32(1.0) / n.astype(np.float32)
    t = np.trunc(q.astype(np.float32) * inv).astype(np.int64)
    r = q - t * n
    t = np.where(r < 0, t - 1, np.where(r >= n, t + 1, t))
    assert (t == q // n).all()
