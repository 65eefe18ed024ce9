"""The Cv-error helpers of the bench's plain-against-delayed-acceptance comparison
(sad-monte-carlo_gb300/cv.py), on synthetic curves with known answers."""
import numpy as np
import pytest

import cv as CV


def test_cv_error_of_exact_and_scaled_curves():
    ref = np.array([90.0, 100.0, 115.0, 120.0])
    walkers = np.array([ref, 1.1 * ref, 0.8 * ref])
    e = CV.cv_error(walkers, ref)
    # per walker max relative errors 0, 0.1, 0.2: median 0.1; median curve = ref
    assert e["median_max_rel"] == pytest.approx(0.1)
    assert e["max_rel_of_median"] == pytest.approx(0.0)
    assert e["median_rel"] == pytest.approx([0.1] * 4)
    # a walker with a non-finite Cv counts as infinitely wrong, not as exact
    walkers = np.array([ref, [np.nan, 100.0, 115.0, 120.0], 1.3 * ref])
    assert CV.cv_error(walkers, ref)["median_max_rel"] == pytest.approx(0.3)


def test_time_to_error_interpolates_the_running_minimum():
    t = [1.0, 2.0, 3.0, 4.0]
    err = [0.4, 0.2, 0.3, 0.1]
    assert CV.time_to_error(t, err, 0.5) == 1.0
    assert CV.time_to_error(t, err, 0.2) == pytest.approx(2.0)
    # between 0.4 at t=1 and 0.2 at t=2, linear in log error
    got = CV.time_to_error(t, err, np.sqrt(0.4 * 0.2))
    assert got == pytest.approx(1.5)
    # 0.25 is first reached at t=2 (the running minimum holds it through t=3)
    assert 1.0 < CV.time_to_error(t, err, 0.25) <= 2.0
    assert CV.time_to_error(t, err, 0.05) is None


def test_reference_interpolation_is_the_mean_of_the_curves():
    a = (np.array([0.1, 0.3]), np.array([10.0, 30.0]))
    b = (np.array([0.1, 0.3]), np.array([20.0, 40.0]))
    got = CV.interp_reference(np.array([0.1, 0.2, 0.3]), [a, b])
    np.testing.assert_allclose(got, [15.0, 25.0, 35.0])
