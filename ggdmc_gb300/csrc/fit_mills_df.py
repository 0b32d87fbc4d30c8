"""Fit of the Mills ratio used, in double-float (hi + lo FP32) arithmetic, for
the per-proposal constants Phi(kappa) of the FP32 trial density.

M(x) = Q(x) / phi(x) = sqrt(pi/2) erfcx(x / sqrt(2)), x >= 0, approximated on
[0, 14] by a rational P8(t) / Q9(t) in t = x / 14 (q0 = 1), fitted for minimax
relative error by Lawson's iteratively reweighted least squares on the
linearised problem P(t) - M(x) Q(t) = 0, nodes denser near 0.  Beyond 14,
phi(x) is below 1e-42 and the tail it scales is irrelevant to the constants.

    python ggdmc_gb300/csrc/fit_mills_df.py

prints the coefficients as C double literals and the relative error on a fine
grid (about 1.4e-10).  Needs numpy and scipy.
"""

import numpy as np
from scipy.special import erfcx

XMAX = 14.0
M_DEG, N_DEG = 8, 9


def mills(x):
    return np.sqrt(np.pi / 2) * erfcx(x / np.sqrt(2))


def fit(m=M_DEG, n=N_DEG, iters=80):
    u = np.cos(np.linspace(0, np.pi, 6000)) * 0.5 + 0.5
    t = u ** 1.5
    x = XMAX * t
    f = mills(x)
    w = np.ones_like(x)
    best = None
    for _ in range(iters):
        A = np.hstack([t[:, None] ** np.arange(m + 1), -f[:, None] * t[:, None] ** np.arange(1, n + 1)])
        sw = np.sqrt(w) / f
        c, *_ = np.linalg.lstsq(A * sw[:, None], f * sw, rcond=None)
        p, q = c[:m + 1], np.concatenate([[1.0], c[m + 1:]])
        err = np.abs(np.polyval(p[::-1], t) / np.polyval(q[::-1], t) / f - 1)
        if best is None or err.max() < best[0]:
            best = (err.max(), p, q)
        w = w * err
        w /= w.sum()
    xt = np.linspace(0, XMAX, 200001)
    tt = xt / XMAX
    e = np.abs(np.polyval(best[1][::-1], tt) / np.polyval(best[2][::-1], tt) / mills(xt) - 1).max()
    return e, best[1], best[2]


if __name__ == "__main__":
    e, p, q = fit()
    print(f"relative error on [0, {XMAX:g}]: {e:.3e}")
    print("P (t^0..t^8):", ", ".join(repr(float(v)) for v in p))
    print("Q (t^0..t^9):", ", ".join(repr(float(v)) for v in q))
