"""The GPU library against golden outputs of the reference's own code.

Same fixtures and bars as tests/test_golden.py, through the C ABI with
compat_arithmetic = 1: block sets, voxel values, cube indices, mesh topology
and raycast depth bit-identical to the reference's kernels.  Huber-TV: the
data weight is CUDA's expf against the host's (a few ulp apart), so the
smoothed sdf agrees within 2e-6 of the field's range and mostly bit for bit.
"""
import pytest

from tests import _golden

pytestmark = pytest.mark.gpu


def test_gpu_matches_reference_simple_chain(built):
    ntri, other_end = _golden.check_simple(_golden.GpuRunner)
    assert ntri > 500


def test_gpu_matches_reference_compress_mesh(built):
    nt, close = _golden.check_compress(_golden.GpuRunner)
    assert nt > 10000


def test_gpu_matches_reference_psdf_chain(built):
    _golden.check_psdf(_golden.GpuRunner)


def test_gpu_matches_reference_tracker_equations(built):
    _golden.check_track(_golden.GpuRunner)


class _GpuHuber:
    def __init__(self, params, pos, sdf, w, cand):
        import numpy as np
        from meshhashing_gb300 import Volume
        self.v = Volume(params)
        z = np.zeros_like(sdf)
        self.v.load_blocks(pos, sdf, w, z, z)
        self.v.set_candidates(cand)
        self.v.huber_tv_init()

    def iterate(self, lam, sigma, tau):
        return self.v.huber_tv_iterate(lam, sigma, tau, 1)

    def sdf(self, cand):
        pos, f = self.v.dump_blocks(("sdf",))
        return _golden.rows(pos, f["sdf"], cand)


def test_gpu_matches_reference_huber_tv(built):
    import numpy as np
    got, want, before = _golden.check_huber(_GpuHuber)
    np.testing.assert_allclose(got, want, rtol=0, atol=2e-6 * np.abs(before).max())
    assert np.mean(got == want) > 0.95
