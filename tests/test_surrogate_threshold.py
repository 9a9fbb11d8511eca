"""The surrogate's acceptance threshold (surrogate.accept_threshold) on
synthetic calibration splits: the largest estimate whose accepted prefix
keeps the share of true errors above the bound within the risk, with the
minimum prefix size, ties and the all/none cases."""
import numpy as np


def test_threshold_controls_risk_on_the_accepted_prefix(pkg):
    S = pkg.surrogate
    rng = np.random.default_rng(3)
    est = rng.uniform(0.1, 3.0, 4000)
    err = est * rng.lognormal(0.0, 0.3, est.size)  # errors grow with the estimate
    for b in (0.5, 1.0, 2.0):
        t = S.accept_threshold(est, err, b, risk=0.05, min_count=20)
        acc = est <= t
        assert acc.sum() >= 20
        assert np.mean(err[acc] > b) <= 0.05
        # the brute-force maximum over all candidate thresholds
        best = -np.inf
        for c in np.sort(est):
            a = est <= c
            if a.sum() >= 20 and np.mean(err[a] > b) <= 0.05:
                best = c
        assert t == (np.inf if best == est.max() else best)


def test_threshold_edge_cases(pkg):
    S = pkg.surrogate
    est = np.linspace(0.1, 1.0, 100)
    # every calibration query within the bound: accept everything
    assert S.accept_threshold(est, np.zeros(100), 1.0) == np.inf
    # every one above: accept nothing
    assert S.accept_threshold(est, np.full(100, 5.0), 1.0) == -np.inf
    # too few queries under any admissible prefix
    err = np.where(np.arange(100) < 10, 0.0, 5.0)
    assert S.accept_threshold(est, err, 1.0, risk=0.05, min_count=20) == -np.inf
    assert S.accept_threshold(est, err, 1.0, risk=0.05, min_count=5) == est[9]
    # ties stay together: a tied group that breaks the risk is not split
    est_t = np.array([0.1] * 30 + [0.2] * 30)
    err_t = np.array([0.0] * 30 + [0.0] * 25 + [5.0] * 5)
    assert S.accept_threshold(est_t, err_t, 1.0, risk=0.05, min_count=20) == 0.1
    # an empty calibration split accepts nothing
    assert S.accept_threshold([], [], 1.0) == -np.inf
