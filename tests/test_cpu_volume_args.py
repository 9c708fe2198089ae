"""Argument checks of the Python host layer (meshhashing_gb300.Volume and
Batch), on the CPU: the C library trusts the pointers it is given, so frame, raycast and
gradient buffers passed as arrays or tensors must be refused with ValueError
when their size, type, layout or device is wrong, before any call reaches the
library.  The library is replaced by a recorder, so no GPU is needed."""
import ctypes as C
from types import SimpleNamespace

import numpy as np
import pytest

from meshhashing_gb300.volume import Volume

W, H = 8, 6


class Recorder:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def call(*args):
            self.calls.append(name)
            return 0
        return call


class FakeTensor:
    """The attributes of a torch tensor the checks read."""

    def __init__(self, n, dtype="torch.float32", contiguous=True, cuda=True):
        self.n, self.dtype, self.contiguous, self.is_cuda = n, dtype, contiguous, cuda

    def numel(self):
        return self.n

    def is_contiguous(self):
        return self.contiguous

    def data_ptr(self):
        return 0x10000


def volume():
    v = object.__new__(Volume)
    v.L = Recorder()
    v.h = C.c_void_p()
    v.stream = C.c_void_p(0)
    v.params = SimpleNamespace(value_capacity=16)
    v.W, v.H, v.RW, v.RH = W, H, W, H
    return v


T = np.eye(4)


def test_frame_inputs():
    v = volume()
    v.set_frame(np.zeros((H, W), np.float64), T)          # converted to float32
    with pytest.raises(ValueError):
        v.set_frame(np.zeros((H, W + 1), np.float32), T)
    with pytest.raises(ValueError):
        v.set_frame_u16(np.zeros((H - 1, W), np.uint16), T)
    v.set_frame(FakeTensor(W * H), T, on_device=True)
    with pytest.raises(ValueError):
        v.set_frame(FakeTensor(W * H - 1), T, on_device=True)
    with pytest.raises(ValueError):
        v.set_frame(FakeTensor(W * H, cuda=False), T, on_device=True)
    v.set_frame(0x20000, T, on_device=True)                # a raw device pointer is taken as given
    assert v.L.calls == ["mh_frame_set", "mh_frame_set", "mh_frame_set"]


def test_integrate_frame_buffers():
    v = volume()
    d = np.zeros((H, W), np.float32)
    out = np.empty((H, W), np.float32)
    v.integrate_frame(d, T, ray_depth=out, ray_normal=np.empty((H, W, 4), np.float32))
    for bad in (np.empty((H, W), np.float64), np.empty((H, W + 1), np.float32), np.empty((W, H), np.float32).T,
                FakeTensor(W * H, cuda=True)):
        with pytest.raises(ValueError):
            v.integrate_frame(d, T, ray_depth=bad)
    with pytest.raises(ValueError):
        v.integrate_frame(np.zeros(W * H + 1, np.float32), T)
    with pytest.raises(ValueError):
        v.integrate_frame(FakeTensor(W * H, dtype="torch.float64", cuda=False), T)
    v.integrate_frame(FakeTensor(W * H, cuda=False), T, ray_depth=FakeTensor(W * H, cuda=False))
    # device inputs and outputs
    v.integrate_frame(FakeTensor(W * H), T, on_device=True, ray_depth=FakeTensor(W * H),
                      ray_vertex=FakeTensor(4 * W * H), ray_normal=FakeTensor(4 * W * H), outputs_on_device=True)
    with pytest.raises(ValueError):
        v.integrate_frame(FakeTensor(W * H), T, on_device=True, ray_normal=FakeTensor(W * H), outputs_on_device=True)
    with pytest.raises(ValueError):
        v.integrate_frame(FakeTensor(W * H, contiguous=False), T, on_device=True)
    assert v.L.calls == ["mh_integrate_frame"] * 3


def test_raycast_and_backward_buffers():
    v = volume()
    cTw = np.eye(4, dtype=np.float32)
    v.raycast(cTw, depth_out=FakeTensor(W * H), normal_out=FakeTensor(4 * W * H))
    with pytest.raises(ValueError):
        v.raycast(cTw, depth_out=FakeTensor(W * H + 1))
    with pytest.raises(ValueError):
        v.raycast(cTw, depth_out=FakeTensor(W * H, cuda=False))
    v.raycast_backward(cTw, FakeTensor(W * H), FakeTensor(4 * W * H), FakeTensor(16 * 512))
    with pytest.raises(ValueError):
        v.raycast_backward(cTw, FakeTensor(W * H), None, FakeTensor(15 * 512))
    with pytest.raises(ValueError):
        v.raycast_backward(cTw, FakeTensor(W * H, dtype="torch.float16"), None, None)
    assert v.L.calls == ["mh_raycast", "mh_raycast_backward"]


def test_batch_step_inputs():
    from meshhashing_gb300.batch import Batch
    b = object.__new__(Batch)
    b.L = Recorder()
    b.h = C.c_void_p()
    b.volumes = [SimpleNamespace(W=W, H=H), SimpleNamespace(W=2 * W, H=2 * H)]
    d0, d1 = np.zeros((H, W), np.float32), np.zeros((2 * H, 2 * W), np.float32)
    b.step([d0, d1], [T, T])
    b.step([d0, None], [T, None], active=[1, 0])
    with pytest.raises(ValueError):
        b.step([d1, d0], [T, T])                            # sizes swapped
    with pytest.raises(ValueError):
        b.step([d0], [T])                                   # one entry per scene
    with pytest.raises(ValueError):
        b.step([d0, d1], [T, T], active=[1])
    b.step([FakeTensor(W * H), FakeTensor(4 * W * H)], [T, T], on_device=True)
    with pytest.raises(ValueError):
        b.step([FakeTensor(W * H), FakeTensor(W * H)], [T, T], on_device=True)
    with pytest.raises(ValueError):
        b.step([FakeTensor(W * H, cuda=False), None], [T, None], on_device=True)
    assert b.L.calls == ["mh_batch_step"] * 3


def test_pose_and_field_buffers():
    v = volume()
    v.normal_equations(np.eye(4), FakeTensor(W * H))
    v.refine_pose(np.eye(4), obs_depth=None)
    with pytest.raises(ValueError):
        v.refine_pose(np.eye(4), obs_depth=FakeTensor(W * H - 1))
    v.dump_block_field(FakeTensor(16 * 512))
    with pytest.raises(ValueError):
        v.dump_block_field(FakeTensor(16 * 511))
    assert v.L.calls == ["mh_raycast_normal_equations", "mh_refine_pose", "mh_dump_block_field",
                         "mh_dump_block_field"]
