"""se(3) helpers used by the pose tests and the bench (meshhashing_gb300/pose.py):
the closed-form exponential against the matrix exponential of the twist,
log as its inverse (both branches), and the left-increment convention
wTc <- exp(xi) wTc with xi = (translation, rotation), Sophus's tangent order."""
import numpy as np
import pytest

from meshhashing_gb300.pose import hat, left_update, pose_error, se3_exp, se3_log


def _twist(xi):
    M = np.zeros((4, 4))
    M[:3, :3] = hat(xi[3:])
    M[:3, 3] = xi[:3]
    return M


@pytest.mark.parametrize("scale", [1e-7, 1e-3, 0.3, 2.5])
def test_exp_matches_matrix_exponential_and_log_inverts_it(scale):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(5)
    for _ in range(20):
        xi = rng.standard_normal(6)
        xi[3:] *= scale / max(np.linalg.norm(xi[3:]), 1e-12)
        T = se3_exp(xi)
        np.testing.assert_allclose(T, scipy_linalg.expm(_twist(xi)), rtol=0, atol=1e-12)
        np.testing.assert_allclose(T[:3, :3] @ T[:3, :3].T, np.eye(3), atol=1e-12)
        np.testing.assert_allclose(se3_log(T), xi, rtol=0, atol=1e-9 * max(1.0, np.abs(xi).max()))


def test_left_update_convention():
    rng = np.random.default_rng(6)
    T = se3_exp(rng.standard_normal(6) * 0.5)
    a, b = rng.standard_normal(6) * 0.1, rng.standard_normal(6) * 0.1
    np.testing.assert_allclose(left_update(T, a), se3_exp(a) @ T, atol=1e-14)
    np.testing.assert_allclose(left_update(left_update(T, a), b), se3_exp(b) @ se3_exp(a) @ T, atol=1e-13)
    # to first order a point moves by v + w x p
    p = np.array([0.3, -0.2, 1.5, 1.0])
    h = 1e-7
    e = np.array([0.2, -0.1, 0.4, 0.3, 0.5, -0.2])
    dp = (left_update(T, h * e) @ p - left_update(T, -h * e) @ p)[:3] / (2 * h)
    pw = (T @ p)[:3]
    np.testing.assert_allclose(dp, e[:3] + np.cross(e[3:], pw), atol=1e-6)


def test_pose_error():
    T = se3_exp(np.array([0.1, 0.2, -0.3, 0.2, -0.1, 0.05]))
    t0, r0 = pose_error(T, T)
    assert t0 == 0.0 and r0 < 1e-5
    D = se3_exp(np.array([0.01, 0.0, 0.0, 0.0, 0.0, np.radians(2.0)]))
    t_err, r_err = pose_error(D @ T, T)
    assert abs(r_err - 2.0) < 1e-9 and t_err > 0.0
