"""The oracle against golden outputs of the reference's own code.

tests/golden/*.npz hold seeded inputs and the outputs of the reference's
kernels built for the CPU (see tests/golden/make_golden.py).  With
compat_arithmetic = 1 the oracle must reproduce them bit for bit (voxel
values, block sets, mesh topology, raycast depth); PSDF values within a few
ulp (expf); the volumetric Huber-TV (optimize/primal_dual.cu) bit for bit.
The GPU counterpart is tests/test_gpu_golden.py.
"""
import os

import pytest

from tests import _golden


def _have_reference():
    from oracle.refcpu import have_reference
    return have_reference()


def test_oracle_matches_reference_simple_chain(built):
    ntri, other_end = _golden.check_simple(_golden.OracleRunner)
    assert ntri > 500


def test_oracle_matches_reference_compress_mesh(built):
    nt, close = _golden.check_compress(_golden.OracleRunner)
    assert nt > 10000


def test_oracle_matches_reference_psdf_chain(built):
    _golden.check_psdf(_golden.OracleRunner)


class _OracleHuber:
    def __init__(self, params, pos, sdf, w, cand):
        import numpy as np
        from oracle.oracle import Oracle
        self.o = Oracle(params, fp64=False)
        z = np.zeros_like(sdf)
        self.o.set_blocks(pos, sdf, w, z, z)
        self.o.set_candidates(cand)
        self.o.huber_tv_init()

    def iterate(self, lam, sigma, tau):
        return self.o.huber_tv_iterate(lam, sigma, tau, 1)

    def sdf(self, cand):
        pos, s = self.o.blocks()[:2]
        return _golden.rows(pos, s, cand)


def test_oracle_matches_reference_tracker_equations(built):
    _golden.check_track(_golden.OracleRunner)


def test_oracle_matches_reference_huber_tv(built):
    import numpy as np
    got, want, _ = _golden.check_huber(_OracleHuber)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.skipif(not _have_reference(), reason="reference sources not present")
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
    out = mg.run_huber(refcpu, p, depth, poses)
    fx = _golden.load("huber_room96.npz")
    for k in ("pre_pos", "pre_sdf", "pre_w", "cand", "post_sdf", "errs"):
        np.testing.assert_array_equal(out[k], fx[k])
    out = mg.run_track(refcpu, p, depth, poses)
    fx = _golden.load("track_room96.npz")
    for k in ("depth", "poses", "A", "b", "err", "count"):
        np.testing.assert_array_equal(out[k], fx[k])
