"""Chi-square homogeneity tests for win/draw/loss counts."""
from __future__ import annotations

import numpy as np
from scipy import stats


def chi2_2xk(a, b):
    """Chi-square statistic and dof of a 2 x k table (empty columns dropped)."""
    t = np.array([a, b], dtype=np.float64)
    t = t[:, t.sum(0) > 0]
    if t.shape[1] < 2:
        return 0.0, 0
    exp = t.sum(1, keepdims=True) * t.sum(0, keepdims=True) / t.sum()
    return float(((t - exp) ** 2 / exp).sum()), t.shape[1] - 1


def wdl_agreement(counts_a, counts_b, alpha=0.01):
    """Per-position 2x3 tests with Bonferroni over positions, plus the pooled sum.

    Returns (ok, details).  With a family-wise alpha the chance that two
    samplers of the same distribution fail this check is at most about 2*alpha.
    """
    counts_a = np.asarray(counts_a)
    counts_b = np.asarray(counts_b)
    n = counts_a.shape[0]
    per_alpha = alpha / n
    worst = (0.0, None)
    total_stat, total_dof = 0.0, 0
    fails = []
    for i in range(n):
        s, dof = chi2_2xk(counts_a[i], counts_b[i])
        total_stat += s
        total_dof += dof
        if dof == 0:
            continue
        p = stats.chi2.sf(s, dof)
        if p < per_alpha:
            fails.append((i, s, dof, p))
        if worst[1] is None or p < worst[1]:
            worst = (s, p)
    pooled_p = stats.chi2.sf(total_stat, total_dof) if total_dof else 1.0
    ok = not fails and pooled_p >= alpha
    return ok, {"fails": fails, "pooled_stat": total_stat, "pooled_dof": total_dof,
                "pooled_p": pooled_p, "min_p": worst[1]}
