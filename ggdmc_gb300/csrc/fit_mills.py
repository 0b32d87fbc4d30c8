"""Fit of the Mills-ratio approximation used by the FP32 trial densities.

M(x) = Q(x) / phi(x) = sqrt(pi/2) * erfcx(x / sqrt(2)) for x >= 0, where Q is
the upper normal tail.  The kernels evaluate Phi and Q from the phi(x) they
already hold as phi(x) * M(|x|), so one exp serves phi, Phi and Q.

M is approximated on [0, 14] by a rational function P4(x) / Q5(x) (q0 = 1),
fitted for minimax relative error by Lawson's iteratively reweighted least
squares on the linearised problem P(x) - M(x) Q(x) = 0.  Beyond x = 14,
phi(x) is below the FP32 range, so the product is zero whatever M returns.

    python ggdmc_gb300/csrc/fit_mills.py

prints the coefficients (as FP32 hex) and the errors in exact and in FP32
fused-multiply-add arithmetic.  Needs numpy and scipy.
"""

import numpy as np
from scipy.special import erfcx

XMAX = 14.0
M_DEG, N_DEG = 4, 5


def mills(x):
    return np.sqrt(np.pi / 2) * erfcx(x / np.sqrt(2))


def fit(m=M_DEG, n=N_DEG, iters=60):
    u = np.cos(np.linspace(0, np.pi, 4000)) * 0.5 + 0.5
    x = XMAX * u ** 2
    f = mills(x)
    w = np.ones_like(x)
    best = None
    for _ in range(iters):
        A = np.hstack([x[:, None] ** np.arange(m + 1),
                       -f[:, None] * x[:, None] ** np.arange(1, n + 1)])
        sw = np.sqrt(w) / f
        c, *_ = np.linalg.lstsq(A * sw[:, None], f * sw, rcond=None)
        p, q = c[:m + 1], np.concatenate([[1.0], c[m + 1:]])
        err = np.abs(np.polyval(p[::-1], x) / np.polyval(q[::-1], x) / f - 1)
        if best is None or err.max() < best[0]:
            best = (err.max(), p, q)
        w = w * err
        w /= w.sum()
    return best


def fp32_fma_error(p, q, n=400001):
    xs = np.linspace(0, XMAX, n).astype(np.float32)
    x64 = xs.astype(np.float64)

    def horner(c):
        acc = np.full_like(xs, np.float32(c[-1]))
        for k in range(len(c) - 2, -1, -1):   # one rounding per step, as fmaf
            acc = (acc.astype(np.float64) * x64 + np.float64(np.float32(c[k]))).astype(np.float32)
        return acc.astype(np.float64)

    return np.abs(horner(p) / horner(q) / mills(x64) - 1).max()


if __name__ == "__main__":
    e, p, q = fit()
    hexes = lambda c: [format(np.float32(v).view(np.uint32).item(), "08x") for v in c]
    print(f"exact-arithmetic max relative error {e:.3e}")
    print(f"FP32 FMA-Horner max relative error {fp32_fma_error(p, q):.3e}")
    print("P (x^0..x^4):", hexes(p))
    print("Q (x^0..x^5):", hexes(q))
