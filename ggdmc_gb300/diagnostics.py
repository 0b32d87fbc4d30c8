"""Posterior diagnostics of sampled chains: summaries and the Brooks-Gelman
potential scale reduction factor (host restatements; the device computes the
same quantities in ggdmc_handle_diagnostics).

The samples are in the C ABI's layout [nmc][nchain][npar], which is R's
posterior@theta [npar, nchain, nmc].

``gelman`` restates the reference's ``.gelman_diag`` (R/model-class.R:1559-1690).
It computes the within-chain covariance W (the mean of the chains'
covariances) and the between-chain covariance B = niter * var(chain means),
the univariate PSRF with its degrees-of-freedom adjustment and upper
confidence bound, and the multivariate PSRF from the largest eigenvalue of
W^-1 B.  As in the reference (form="reference"), the variance of W's rows
stands for the variance of the within-chain variances and the W-B covariance
term is left out; that changes only df_adj and the upper bound (with one
parameter the row variance is undefined and so is the PSRF, as in R).
form="coda" takes the variance of the chains' variances and includes the
covariance term (Brooks & Gelman 1998, as coda's gelman.diag).
"""

from __future__ import annotations

import numpy as np


def _theta(samples) -> np.ndarray:
    th = np.asarray(samples, np.float64)
    if th.ndim != 3:
        raise ValueError("samples must be [nmc][nchain][npar]")
    return th


def gelman(samples, start: int = 0, end: int | None = None, conf: float = 0.95,
           multivariate: bool = True, form: str = "reference") -> dict:
    """psrf [npar][2] (point estimate, upper C.I.) and mpsrf of iterations
    [start, end) of samples [nmc][nchain][npar]."""
    from scipy.stats import f as fdist
    th = _theta(samples)[start:end]
    niter, nchain, npar = th.shape
    if nchain < 3:
        raise ValueError("Minimum three chains needed")
    # within-chain covariances (denominator niter - 1), their mean W
    cov = np.stack([np.atleast_2d(np.cov(th[:, k, :], rowvar=False)) for k in range(nchain)])
    W = cov.mean(axis=0)
    xbar = th.mean(axis=0)                                  # [nchain][npar]
    B = niter * np.atleast_2d(np.cov(xbar, rowvar=False))
    w, b = np.diag(W), np.diag(B)
    var_b = 2.0 * b ** 2 / (nchain - 1)
    V = (niter - 1) / niter * w + (1 + 1 / nchain) / niter * b
    if form == "reference":
        with np.errstate(invalid="ignore", divide="ignore"):
            var_w = np.var(W, axis=1, ddof=1) / nchain if npar > 1 else np.full(1, np.nan)
        var_V = ((niter - 1) ** 2 * var_w + (1 + 1 / nchain) ** 2 * var_b) / niter ** 2
    elif form == "coda":
        s2 = np.stack([np.diag(c) for c in cov], axis=1)     # [npar][nchain] chain variances
        var_w = np.var(s2, axis=1, ddof=1) / nchain
        muhat = xbar.mean(axis=0)
        cross = lambda a, c: np.array([np.cov(a[p], c[p])[0, 1] for p in range(npar)])
        cov_wb = (niter / nchain) * (cross(s2, (xbar ** 2).T) - 2 * muhat * cross(s2, xbar.T))
        var_V = ((niter - 1) ** 2 * var_w + (1 + 1 / nchain) ** 2 * var_b
                 + 2 * (niter - 1) * (1 + 1 / nchain) * cov_wb) / niter ** 2
    else:
        raise ValueError("form must be 'reference' or 'coda'")
    df_V = 2 * V ** 2 / var_V
    df_adj = (df_V + 3) / (df_V + 1)
    r2_fixed = (niter - 1) / niter
    r2_random = (1 + 1 / nchain) * (1 / niter) * (b / w)
    r2_est = r2_fixed + r2_random
    with np.errstate(invalid="ignore", divide="ignore"):
        r2_up = r2_fixed + fdist.ppf(0.5 * (1 + conf), nchain - 1, 2 * w ** 2 / var_w) * r2_random
    psrf = np.stack([np.sqrt(df_adj * r2_est), np.sqrt(df_adj * r2_up)], axis=1)
    mpsrf = None
    if multivariate and npar >= 2:
        cw = np.linalg.cholesky(W).T                        # upper: W = cw' cw
        inv = np.linalg.inv(cw)
        emax = np.linalg.eigvalsh(inv.T @ B @ inv)[-1]
        mpsrf = float(np.sqrt((1 - 1 / niter) + (1 + 1 / npar) * emax / niter))
    return {"psrf": psrf, "mpsrf": mpsrf}


def spectrum0_ar(x) -> tuple[float, int]:
    """The spectral density at frequency zero of one chain from an AR fit,
    as R/model-class.R:257-275 (spectrum0_ar, which safespec0 wraps) computes
    it: 0 when the residual sd of lm(x ~ 1:n) is within all.equal's 1.5e-8 of
    zero; otherwise the Yule-Walker AR fit of stats::ar (order chosen by AIC
    up to min(n - 1, floor(10 log10 n)), autocovariances of the demeaned
    chain with denominator n, innovations variance scaled by n / (n - order -
    1)) and var.pred / (1 - sum(ar))^2.  Returns (spectrum, order)."""
    x = np.asarray(x, np.float64)
    n = x.size
    if n < 2:
        return float("nan"), 0
    xc = x - x.mean()
    zc = np.arange(n) - (n - 1) / 2.0
    sxz, szz = float(zc @ xc), float(zc @ zc)
    rss = max(float(xc @ xc) - sxz * sxz / szz, 0.0)
    if np.sqrt(rss / (n - 1)) <= 1.5e-8:
        return 0.0, 0
    kmax = min(n - 1, int(np.floor(10 * np.log10(n))))
    r = np.array([xc[: n - k] @ xc[k:] for k in range(kmax + 1)]) / n
    # Durbin-Levinson recursion for the Yule-Walker equations of orders 1..kmax
    var = np.empty(kmax + 1)
    var[0] = r[0]
    coef = [np.zeros(0)]
    phi = np.zeros(0)
    for k in range(1, kmax + 1):
        a = (r[k] - phi @ r[k - 1:0:-1]) / var[k - 1]
        phi = np.concatenate([phi - a * phi[::-1], [a]])
        var[k] = var[k - 1] * (1.0 - a * a)
        coef.append(phi)
    with np.errstate(divide="ignore", invalid="ignore"):
        aic = n * np.log(var) + 2.0 * np.arange(kmax + 1)
    order = int(np.nanargmin(aic))
    vp = var[order] * n / (n - (order + 1))
    return float(vp / (1.0 - coef[order].sum()) ** 2), order


def quantile7(x, probs) -> np.ndarray:
    """Quantiles of type 7 as R's quantile / matrixStats::rowQuantiles form
    them: h = 1 + (n - 1) p, (1 - (h - lo)) x[lo] + (h - lo) x[hi] of the
    sorted values (1-based lo = floor h, hi = ceiling h); x[lo] when the two
    order statistics are equal."""
    xs = np.sort(np.asarray(x, np.float64))
    n = xs.size
    out = np.empty(len(probs))
    for i, p in enumerate(probs):
        h = (n - 1) * p
        lo = int(np.floor(h))
        hi = min(lo + 1, n - 1)
        g = h - lo
        out[i] = xs[lo] if (g == 0.0 or xs[hi] == xs[lo]) else (1.0 - g) * xs[lo] + g * xs[hi]
    return out


def summary(samples, start: int = 0, end: int | None = None, probs=(0.05, 0.5, 0.975)) -> dict:
    """summary of a posterior (R/model-class.R:370-424) over iterations
    [start, end) of samples [nmc][nchain][npar] (R's start is 1-based and its
    end inclusive): per parameter over all chains and iterations the Mean,
    the SD, the Naive SE sqrt(var / niter * nchain) and the Time-series SE
    sqrt(mean_k spectrum0(chain k) / niter * nchain) -- the reference's
    formulas as written -- and the quantiles of type 7 at probs (the
    reference's default 0.05, 0.5, 0.975).  se_mean is the standard error of
    the mean from the chain means (chains as independent replicates)."""
    th = _theta(samples)[start:end]
    niter, nchain, npar = th.shape
    flat = th.reshape(-1, npar)
    var = flat.var(axis=0, ddof=1)
    ts = np.array([[spectrum0_ar(th[:, k, p])[0] for p in range(npar)] for k in range(nchain)])
    cm = th.mean(axis=0)
    return {"mean": flat.mean(axis=0), "sd": np.sqrt(var),
            "naive_se": np.sqrt(var / niter * nchain),
            "ts_se": np.sqrt(ts.mean(axis=0) / niter * nchain),
            "quantiles": np.stack([quantile7(flat[:, p], probs) for p in range(npar)], axis=1),
            "probs": np.asarray(probs),
            "se_mean": cm.std(axis=0, ddof=1) / np.sqrt(nchain)}
