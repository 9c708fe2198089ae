"""The GPU library against golden outputs of the reference's own code.

Same fixtures and bars as tests/test_golden.py, through the C ABI with
compat_arithmetic = 1: block sets, voxel values, cube indices, mesh topology
and raycast depth bit-identical to the reference's kernels.
"""
import pytest

from tests import _golden

pytestmark = pytest.mark.gpu


def test_gpu_matches_reference_simple_chain(built):
    ntri, other_end = _golden.check_simple(_golden.GpuRunner)
    assert ntri > 500


def test_gpu_matches_reference_psdf_chain(built):
    _golden.check_psdf(_golden.GpuRunner)
