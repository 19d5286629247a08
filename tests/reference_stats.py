"""Statistical agreement of an implementation with the reference's own estimator (the committed
reference fixtures), shared by the CPU test (oracle) and the GPU test (engine).

Both sides run the same estimator on the same scene and points with different random streams
(the reference: std::mt19937 per point; here: Philox per path), so agreement is distributional:

1. per-point z-scores z = (m_ref - m) / sqrt(v_ref/N + v/N) over every (point, component):
   max |z| below the Bonferroni bound for a family-wise error of 1e-3, and the mean of z within
   4 / sqrt(M) of zero;
2. the distribution of those z-scores against a null sample of z-scores formed the same way
   from two further independent runs of the implementation (two-sample Kolmogorov-Smirnov,
   p > 1e-3). The null is empirical because these estimators' path values are heavy-tailed: at a
   few hundred paths the z-statistic is measurably lighter-tailed than N(0, 1) (kurtosis -0.4 to
   -1.1 on the star and sphere workloads), so a test against N(0, 1) would reject two runs of
   one and the same estimator;
3. every path value at a few points against the reference's path values at those points
   (two-sample Kolmogorov-Smirnov, p > 1e-3 / number of points): the whole distribution of a
   path's contribution, not only its mean.
"""
from __future__ import annotations

import numpy as np
from scipy import stats

FWER = 1e-3


def zscores(s_a, q_a, s_b, q_b, n):
    m_a, m_b = s_a / n, s_b / n
    v_a = np.maximum(q_a / n - m_a ** 2, 0.0)
    v_b = np.maximum(q_b / n - m_b ** 2, 0.0)
    se = np.sqrt(v_a / n + v_b / n)
    ok = se > 0
    z = np.zeros_like(m_a)
    z[ok] = (m_a[ok] - m_b[ok]) / se[ok]
    # a component that is exactly equal on both sides with zero variance (e.g. a gradient of a
    # constant) carries no information; one that differs with zero variance is a failure
    assert np.all(ok | (m_a == m_b)), "a zero-variance component differs"
    return z[ok]


def check_against_reference(fix, run_sums, run_per_path, label):
    """fix: the loaded fixture. run_sums(seed) -> (sum, sumsq) over fix's n_paths at fix's points;
    run_per_path(seed) -> [n_pp, pp_paths] path values of u at the first n_pp points."""
    n = int(fix["n_paths"])
    s0, q0 = run_sums(101)
    z = zscores(fix["sum"], fix["sumsq"], s0, q0, n)
    s1, q1 = run_sums(202)
    s2, q2 = run_sums(303)
    z_null = zscores(s1, q1, s2, q2, n)
    M = z.size
    bound = stats.norm.isf(FWER / (2 * M))
    report = {"points": len(fix["points"]), "paths": n, "M": M, "max_abs_z": float(np.abs(z).max()),
              "bonferroni_bound": float(bound), "mean_z_sqrtM": float(z.mean() * np.sqrt(M))}
    assert np.abs(z).max() < bound, (label, report)
    assert abs(z.mean()) * np.sqrt(M) < 4.0, (label, report)
    ks = stats.ks_2samp(z, z_null)
    report["ks_vs_null_p"] = float(ks.pvalue)
    assert ks.pvalue > FWER, (label, report)
    pp_ref = fix["per_path"]
    pp = run_per_path(404)
    ps = [float(stats.ks_2samp(pp_ref[i], pp[i]).pvalue) for i in range(len(pp_ref))]
    report["per_path_ks_min_p"] = min(ps)
    assert min(ps) > FWER / len(ps), (label, report)
    return report
