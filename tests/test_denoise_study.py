"""Host-side pieces of the denoised-vs-plain study (no GPU): the relMSE with
the reference's own noise removed, and the time at which a measured
(time, error) curve reaches a target."""
import numpy as np

from rendertoy_gb300 import denoise as D


def _noisy(mu, rel, rng):
    return mu * (1.0 + rng.normal(0.0, rel, mu.shape))


def test_corrected_relmse_removes_reference_noise():
    rng = np.random.RandomState(0)
    mu = rng.exponential(1.0, (300, 300, 3)) + 0.02
    x = _noisy(mu, 0.03, rng)
    true = ((x - mu) ** 2 / (mu ** 2 + D.EPS)).mean()
    # two half references, each noisier than x: the raw error is dominated
    # by the reference, the corrected one is not
    a, b = _noisy(mu, 0.1, rng), _noisy(mu, 0.1, rng)
    raw, corr, noise, bad = D.relmse_corrected(x, a, b)
    assert bad == 0
    assert raw > 3 * true
    assert abs(corr - true) < 0.25 * true, (corr, true)
    assert abs(noise - (raw - true)) < 0.25 * noise


def test_corrected_relmse_masks_non_finite_pixels():
    rng = np.random.RandomState(1)
    mu = rng.exponential(1.0, (20, 30, 3)) + 0.1
    x = mu.copy()
    a, b = mu.copy(), mu.copy()
    x[0, 0, 1] = np.nan
    a[3, 4, 0] = np.inf
    raw, corr, noise, bad = D.relmse_corrected(x, a, b)
    assert bad == 2
    assert raw == 0.0 and corr == 0.0 and noise == 0.0


def test_time_to_target_interpolates_in_log_log():
    pts = [(10.0, 1.0), (40.0, 0.1), (160.0, 0.01)]
    # exactly on a measured point
    assert abs(D._time_to(pts, 0.1) - 40.0) < 1e-9
    # halfway in log error between 40 ms and 160 ms -> halfway in log time
    t = D._time_to(pts, 10 ** -1.5)
    assert abs(np.log(t) - 0.5 * (np.log(40.0) + np.log(160.0))) < 1e-9
    # already below the target at the first point; never reaching it
    assert D._time_to([(5.0, 0.01)], 0.1) == 5.0
    assert D._time_to(pts, 1e-4) is None
