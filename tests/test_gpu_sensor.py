"""Raw 16-bit depth input (mh_frame_set_u16) against the reference's
ConvertDepthFormatKernel (sensor/preprocess.cu:25-42), restated in numpy by
oracle.convert_depth_u16: depth = range_factor * (short)raw in single
precision, valid inside [min_depth_range, max_depth_range], else -inf; the
inlier-ratio image is reset to 0.1 (preprocess.cu:10-23)."""
import numpy as np
import pytest

from meshhashing_gb300 import Volume, config, scene
from oracle.oracle import convert_depth_u16

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("range_factor", [0.0002, 0.001])
def test_u16_depth_matches_reference_conversion(built, range_factor):
    wl = scene.full_spline(2, width=160, height=120)
    p = config.params_for(wl, value_capacity=1 << 14, bucket_count=1 << 14, max_vertex_count=1 << 16,
                          max_triangle_count=1 << 16)
    p.range_factor = range_factor
    v = Volume(p)
    rng = np.random.default_rng(7)
    raw = rng.integers(0, 65536, size=(p.height, p.width), dtype=np.int64).astype(np.uint16)
    # the edges of the valid range, zero, and raw values that are negative as a short
    lo, hi = int(round(p.min_depth_range / range_factor)), int(round(p.max_depth_range / range_factor))
    edge = np.array([0, 1, lo - 1, lo, lo + 1, hi - 1, hi, hi + 1, 32767, 32768, 40000, 65535], np.uint16)
    raw.reshape(-1)[:edge.size] = edge
    v.set_frame_u16(raw, wl.pose(0))
    got = v.depth()
    want = convert_depth_u16(raw, range_factor, p.min_depth_range, p.max_depth_range)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.all(v.inlier() == np.float32(0.1))
    assert np.isfinite(got).sum() > 0 and (~np.isfinite(got)).sum() > 0


def test_u16_frame_fuses_like_its_float_depth(built):
    """A frame given as raw 16-bit depth allocates and fuses exactly what the
    same depths given as float32 metres do."""
    wl = scene.full_spline(2, width=160, height=120)
    kw = dict(value_capacity=1 << 15, bucket_count=1 << 15, max_vertex_count=1 << 16, max_triangle_count=1 << 16)
    p = config.params_for(wl, **kw)
    d = wl.frame(0)
    raw = np.clip(np.round(np.nan_to_num(d, nan=0.0, posinf=0.0, neginf=0.0) / p.range_factor), 0, 65535).astype(np.uint16)
    a, b = Volume(p), Volume(p)
    a.set_frame_u16(raw, wl.pose(0))
    b.set_frame(convert_depth_u16(raw, p.range_factor, p.min_depth_range, p.max_depth_range), wl.pose(0))
    for v in (a, b):
        v.alloc_block_array()
        v.collect_blocks_in_frustum()
        v.predict_outlier_ratio()
        v.update_blocks_bayesian()
    pa, fa = a.dump_blocks()
    pb, fb = b.dump_blocks()
    oa, ob = np.lexsort(pa.T[::-1]), np.lexsort(pb.T[::-1])
    assert len(pa) > 0 and np.array_equal(pa[oa], pb[ob])
    np.testing.assert_array_equal(fa["sdf"][oa].view(np.uint32), fb["sdf"][ob].view(np.uint32))
