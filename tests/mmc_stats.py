"""Statistical comparison of MiniMC tally histograms (weighted histograms:
content = sum w, errorsq = sum w^2 per bin)."""
import numpy as np

GROUPS = ["NOSCAT", "SINGLESCAT_ELAS", "SINGLESCAT_INELAS", "MULTISCAT_PUREELAS", "MULTISCAT_OTHER"]


def hist_from_result(res, tally, part):
    t = res["output"]["tally"][tally]
    h = t["total"] if part == "total" else t["breakdown"][part]
    b = h["bindata"]
    c = np.array([b["underflow"]] + list(b["content"]) + [b["overflow"]], dtype=float)
    e = np.array([b["underflow_errorsq"]] + list(b["errorsq"]) + [b["overflow_errorsq"]], dtype=float)
    return c, e, (b["xmin"], b["xmax"], b["nbins"])


def chi2_compare(c1, e1, n1, c2, e2, n2, min_neff=50.0):
    """Two-sample chi-square of per-neutron normalised weighted histograms over
    the bins where both sides have at least min_neff effective entries.
    Returns (chi2, ndf, p, worst) where worst lists bins one side fills
    heavily and the other leaves empty."""
    from scipy.stats import chi2 as _chi2
    a, b = c1 / n1, c2 / n2
    va, vb = e1 / n1 ** 2, e2 / n2 ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        na = np.where(e1 > 0, c1 * c1 / e1, 0.0)
        nb = np.where(e2 > 0, c2 * c2 / e2, 0.0)
    m = (na >= min_neff) & (nb >= min_neff)
    worst = np.nonzero(((na >= 1000) & (c2 == 0)) | ((nb >= 1000) & (c1 == 0)))[0]
    if not m.any():
        return 0.0, 0, 1.0, worst
    x = float(np.sum((a[m] - b[m]) ** 2 / (va[m] + vb[m])))
    ndf = int(m.sum())
    return x, ndf, float(_chi2.sf(x, ndf)), worst
