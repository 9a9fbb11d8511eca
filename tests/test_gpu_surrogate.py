"""The learned spectral surrogate against the method without it (DG for every
query), on a small configuration (10 x 10 grid meshes, 400 RK4 steps, 600
training runs) so that DG data generation and training take seconds.

What the network gains: it answers queries at >= 100x the rate of the DG
runs it replaces (timed at the shipped DG configuration), it predicts
held-out spectra better than the best constant guess (the mean training
spectrum), its error network's estimate follows the true error, and its
fallback hands every query whose estimate is above the bound's acceptance
threshold back to DG, whose answers it returns unchanged."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRID, STEPS = 10, 400


@pytest.fixture(scope="module")
def trained(pkg):
    S = pkg.surrogate
    P_train = S.draw_params(600, 15)
    P_test = S.draw_params(48, 16)
    Y_train, _ = S.dg_spectra(P_train, steps=STEPS, grid=GRID)
    Y_test, dg_s = S.dg_spectra(P_test, steps=STEPS, grid=GRID)
    sur = S.Surrogate.fit(P_train[:500], Y_train[:500], steps=1500, batch=100, lr=2e-3, lr_final=2e-5,
                          grid=GRID, dg_steps=STEPS)
    sur.calibrate(P_train[500:], Y_train[500:])
    yield S, sur, P_train, Y_train, P_test, Y_test, dg_s
    sur.close()


def test_targets_are_finite_spectra(trained):
    S, _, _, Y_train, _, Y_test, _ = trained
    assert Y_train.shape == (600, S.N_OBS, S.N_BINS)
    assert np.all(np.isfinite(Y_train)) and np.all(np.isfinite(Y_test))
    # floored at most the dynamic range below each observer's peak
    span = Y_train.max(axis=2) - Y_train.min(axis=2)
    assert np.all(span <= S.DYN_RANGE_DB + 1e-6)


def test_surrogate_beats_constant_guess(trained):
    S, sur, _, Y_train, P_test, Y_test, _ = trained
    mean, est = sur.predict(P_test)
    err = S.rms_db(mean, Y_test)
    base = S.rms_db(np.broadcast_to(Y_train[:500].mean(axis=0), Y_test.shape), Y_test)
    assert np.median(err) < 0.7 * np.median(base), (np.median(err), np.median(base))
    assert np.all(est > 0)


def test_error_estimate_follows_true_error(trained):
    """The error network ranks held-out queries by their true error better
    than chance (rank correlation), and the out-of-fold errors it learned
    from are of the size of the held-out errors."""
    S, sur, _, _, P_test, Y_test, _ = trained
    mean, est = sur.predict(P_test)
    err = S.rms_db(mean, Y_test)
    r = np.corrcoef(np.argsort(np.argsort(est)), np.argsort(np.argsort(err)))[0, 1]
    assert r > 0.2, r
    assert 0.5 < np.median(sur.oof_rms_db) / np.median(err) < 2.0


def test_surrogate_throughput_over_dg(trained):
    """Queries per second of each method: the batched DG runs that a query
    of the shipped configuration costs (3000 RK4 steps on the 25 x 25 meshes,
    48 queries in one batch) against the network (4096 queries, host arrays
    in and out). The network's cost does not depend on the DG configuration
    it was trained on."""
    S, sur, _, _, _, _, _ = trained
    P = S.draw_params(4096, 17)
    _, dg_s = S.dg_spectra(P[:48], steps=S.STEPS, grid=S.GRID)
    sur.predict(P)
    t0 = time.perf_counter()
    for _ in range(10):
        sur.predict(P)
    sur_rate = 10 * len(P) / (time.perf_counter() - t0)
    dg_rate = 48 / dg_s
    assert sur_rate >= 100 * dg_rate, (sur_rate, dg_rate)


def test_fallback_returns_dg_answers(trained):
    S, sur, _, _, P_test, Y_test, _ = trained
    q = P_test[:12]
    # a bound no estimate meets: every query goes to DG and comes back as DG
    # answers it (a re-run is another batch, whose FP32 kernel variant the
    # autotuner may pick differently: round-off level differences)
    spec, from_dg, _ = sur.query(q, bound_db=-1.0)
    assert from_dg.all()
    np.testing.assert_allclose(spec, Y_test[:12], rtol=0, atol=1e-3)
    # an unbounded tolerance: every query is answered by the network
    spec2, from_dg2, _ = sur.query(q, bound_db=np.inf)
    assert not from_dg2.any()
    mean, _ = sur.predict(q)
    np.testing.assert_array_equal(spec2, mean)
    # a mixed bound: accepted rows come from the network, the others from DG
    _, est = sur.predict(q)
    t = float(np.median(est))
    # the loosest bound whose acceptance threshold is below t
    b = max((x for x in np.sort(sur.calib_err) if sur.threshold(x) < t), default=-1.0)
    spec3, from_dg3, _ = sur.query(q, bound_db=b)
    assert np.array_equal(from_dg3, est > sur.threshold(b))
    np.testing.assert_allclose(spec3[from_dg3], Y_test[:12][from_dg3], rtol=0, atol=1e-3)
    np.testing.assert_array_equal(spec3[~from_dg3], mean[~from_dg3])


def test_save_load_round_trip(trained, tmp_path):
    S, sur, _, _, P_test, _, _ = trained
    path = str(tmp_path / "s.npz")
    sur.save(path)
    s2 = S.Surrogate.load(path)
    a, ea = sur.predict(P_test)
    b, eb = s2.predict(P_test)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(ea, eb)
    assert (s2.grid, s2.steps) == (GRID, STEPS)
    s2.close()
