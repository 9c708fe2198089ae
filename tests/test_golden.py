"""The oracle against golden outputs of the reference's own code.

tests/golden/*.npz hold seeded inputs and the outputs of the reference's
kernels built for the CPU (see tests/golden/make_golden.py).  With
compat_arithmetic = 1 the oracle must reproduce them bit for bit (voxel
values, block sets, mesh topology, raycast depth); PSDF values within a few
ulp (expf).  The GPU counterpart is tests/test_gpu_golden.py.
"""
import os

import pytest

from tests import _golden


def test_oracle_matches_reference_simple_chain(built):
    ntri, other_end = _golden.check_simple(_golden.OracleRunner)
    assert ntri > 500


def test_oracle_matches_reference_psdf_chain(built):
    _golden.check_psdf(_golden.OracleRunner)


@pytest.mark.skipif(not os.path.isdir("/root/reference"), reason="reference sources not present")
def test_fixtures_regenerate_from_reference(built, tmp_path):
    """The committed fixtures are what the reference's code produces now."""
    import numpy as np
    from oracle import refcpu
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(_golden.GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    refcpu.build()
    p, depth, poses = mg.simple_case()
    fx = _golden.load("simple_room96.npz")
    np.testing.assert_array_equal(depth, fx["depth"])
    out = mg.run_simple(refcpu, p, depth, poses)
    for k in ("counts", "blocks", "sample_sdf", "sample_w", "tris", "ray_depth"):
        np.testing.assert_array_equal(out[k], fx[k])
