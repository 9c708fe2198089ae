"""The reference's point-to-PSDF tracker on the GPU
(mh_point_to_psdf_normal_equations, mh_track_point_to_psdf) against the FP32
oracle on the same map, and the behaviour of its Gauss-Newton loop.

Per pixel both sides run the same single-precision arithmetic; the sums are
doubles of float partials on the GPU and of single terms in the oracle, so A,
b and err agree to 1e-5 of their largest entry and the count exactly.
"""
import numpy as np
import pytest

from meshhashing_gb300 import Volume, config, scene
from meshhashing_gb300.pose import left_update, pose_error
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _map():
    wl = scene.small_circle(60)
    f = 262.5 * 160 / 320
    wl.camera = scene.Camera(160, 120, f, f, 79.5, 59.5)
    p = config.params_for(wl, value_capacity=1 << 17, bucket_count=1 << 16)
    v = Volume(p)
    for i in range(0, 36, 2):
        v.integrate_frame(wl.frame(i), wl.pose(i))
    return wl, p, v


@pytest.mark.parametrize("reference_jacobian", [True, False])
def test_tracker_equations_match_oracle(built, reference_jacobian):
    wl, p, v = _map()
    pos, f = v.dump_blocks()
    o = Oracle(p, fp64=False)
    o.set_blocks(pos, f["sdf"], f["w"], f["a"], f["b"])
    rng = np.random.default_rng(11)
    for fi in (38, 44):
        T = left_update(wl.pose(fi).astype(np.float64),
                        np.concatenate([rng.standard_normal(3) * 0.01, rng.standard_normal(3) * 0.01]))
        T = T.astype(np.float32)
        v.set_frame(wl.frame(fi), T)
        o.frame_set(wl.frame(fi), T)
        A, b, e, n = v.point_to_psdf(T, reference_jacobian=reference_jacobian)
        A2, b2, e2, n2 = o.point_to_psdf(T, fix_jacobian=not reference_jacobian)
        assert n == n2 and n > 1000
        assert np.abs(A - A2).max() <= 1e-5 * np.abs(A2).max()
        assert np.abs(b - b2).max() <= 1e-5 * np.abs(b2).max()
        assert abs(e - e2) <= 1e-5 * e2
        assert np.array_equal(A[:, 2], A[:, 0]) == reference_jacobian


def test_tracker_loop(built):
    """The Gauss-Newton loop lowers its objective (mean squared sdf of the
    frame's points); with the reference's damping (lambda = 1e5) it moves
    the pose by well under a millimetre per call; with no valid pixel it
    stops and returns the pose unchanged."""
    wl, p, v = _map()
    rng = np.random.default_rng(6)
    fi = 42
    T_true = wl.pose(fi).astype(np.float64)
    T0 = left_update(T_true, np.concatenate([rng.standard_normal(3) * 0.005,
                                             rng.standard_normal(3) * np.radians(0.25)]))
    v.set_frame(wl.frame(fi), T0)
    _, _, e0, n0 = v.point_to_psdf(T0.astype(np.float32), reference_jacobian=False)
    T1, e1, n1 = v.track_point_to_psdf(T0, iterations=10, lam=1.0, reference_jacobian=False)
    _, _, e2, n2 = v.point_to_psdf(T1.astype(np.float32), reference_jacobian=False)
    assert n1 > 1000 and e2 / n2 < 0.9 * (e0 / n0), (e0 / n0, e2 / n2)
    v.set_frame(wl.frame(fi), T0)
    T3, _, _ = v.track_point_to_psdf(T0, iterations=3, lam=1e5, reference_jacobian=True)
    assert pose_error(T3, T0)[0] < 1e-3
    v.set_frame(np.zeros_like(wl.frame(fi)), T0)
    T4, e4, n4 = v.track_point_to_psdf(T0, iterations=5)
    assert n4 == 0 and np.array_equal(T4.astype(np.float32), T0.astype(np.float32))
    assert v.stats()["error"] == 0
