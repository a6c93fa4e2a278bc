"""xr_read_output_async / xr_wait_output: frames in flight with double-buffered RGBA8 images.

Two contexts render the same frames.  One reads every image synchronously
(xr_read_output).  The other reads asynchronously while the next frames render,
and its images must be identical:
* one frame in flight;
* a read still pending when two more frames are submitted, the second of which
  writes the buffer being read: that frame waits for the read on the device;
* two frames in flight (the host loop bench.py's e2e leg runs): reads are waited
  for oldest first, a third read in flight is refused;
* the same through replayed frame graphs;
* frames of one parity back to back: they share the UBO staging slot and the
  RGBA8 buffer, so each waits for the previous frame's upload and image read.
Misuse is refused before anything is enqueued.
"""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from tests.helpers import camera_sequence

pytestmark = pytest.mark.gpu
L = xr._lib
W, H = 320, 180


def _scene():
    return xr.Scene.procedural(seed=4, n_objects=256, n_lights=4, extent=10.0)


def _renderer(scene, graphs):
    r = xr.Renderer(W, H)
    r.set_params(xr.params_default(W, H))
    r.upload_scene(scene)
    r.build_bvh()
    if graphs:
        r.set_graphs(True)
    return r


def _sync_images(scene, ubos):
    with _renderer(scene, False) as r:
        out = []
        for u in ubos:
            r.render(u)
            out.append(r.read_output(L.XR_OUT_LDR8).copy())
    return out


@pytest.mark.parametrize("graphs", [False, True])
def test_async_reads_match_sync_reads(graphs):
    scene = _scene()
    ubos = camera_sequence(scene, W, H, 10, 4)
    ref = _sync_images(scene, ubos)
    assert len({img.tobytes() for img in ref}) == len(ref)   # the frames differ
    pinned = [xr.PinnedBuffer(W * H * 4) for _ in range(2)]
    try:
        with _renderer(scene, graphs) as r:
            # one frame in flight
            got = []
            for f, u in enumerate(ubos[:6]):
                r.render(u)
                if f:
                    r.wait_output()
                    got.append(pinned[(f - 1) % 2].array.copy())
                r.read_output_async(pinned[f % 2].array)
            r.wait_output()
            got.append(pinned[5 % 2].array.copy())
            for f in range(6):
                assert np.array_equal(got[f].view(np.uint32), ref[f].reshape(-1).view(np.uint32)), f"frame {f}"
            # frame 6's read is pending while frames 7 and 8 are submitted; frame 8 writes
            # the buffer being read and waits for the read on the device
            r.render(ubos[6])
            r.read_output_async(pinned[0].array)
            r.render(ubos[7])
            r.render(ubos[8])
            r.wait_output()
            assert np.array_equal(pinned[0].array.view(np.uint32), ref[6].reshape(-1).view(np.uint32))
            r.sync()
            assert np.array_equal(r.read_output(L.XR_OUT_LDR8), ref[8])
    finally:
        for p in pinned:
            p.free()


def test_two_frames_in_flight():
    scene = _scene()
    ubos = camera_sequence(scene, W, H, 9, 4)
    ref = _sync_images(scene, ubos)
    pinned = [xr.PinnedBuffer(W * H * 4) for _ in range(3)]
    try:
        with _renderer(scene, True) as r:
            got = {}
            for f, u in enumerate(ubos):
                r.render(u)
                if f >= 2:
                    r.wait_output()                       # frame f-2's image
                    got[f - 2] = pinned[(f - 2) % 3].array.copy()
                r.read_output_async(pinned[f % 3].array)
                if f == 4:                                # a third read in flight is refused
                    with pytest.raises(xr.XrError, match="two reads"):
                        r.read_output_async(pinned[(f + 1) % 3].array)
            for f in (len(ubos) - 2, len(ubos) - 1):
                r.wait_output()
                got[f] = pinned[f % 3].array.copy()
            for f in range(len(ubos)):
                assert np.array_equal(got[f].view(np.uint32), ref[f].reshape(-1).view(np.uint32)), f"frame {f}"
    finally:
        for p in pinned:
            p.free()


@pytest.mark.parametrize("graphs", [False, True])
def test_frames_of_one_parity_back_to_back(graphs):
    scene = _scene()
    ubos = []
    for f, u in enumerate(camera_sequence(scene, W, H, 7, 4)):
        v = L.XrUniformBufferObject.from_buffer_copy(u)
        v.current_frame = 2 * f                           # every frame even
        ubos.append(v)
    ref = _sync_images(scene, ubos)
    pinned = [xr.PinnedBuffer(W * H * 4) for _ in range(3)]
    try:
        with _renderer(scene, graphs) as r:
            got = {}
            for f, u in enumerate(ubos):
                r.render(u)
                if f >= 2:
                    r.wait_output()
                    got[f - 2] = pinned[(f - 2) % 3].array.copy()
                r.read_output_async(pinned[f % 3].array)
            for f in (len(ubos) - 2, len(ubos) - 1):
                r.wait_output()
                got[f] = pinned[f % 3].array.copy()
            for f in range(len(ubos)):
                assert np.array_equal(got[f].view(np.uint32), ref[f].reshape(-1).view(np.uint32)), f"frame {f}"
    finally:
        for p in pinned:
            p.free()


def test_async_read_refuses_misuse():
    scene = _scene()
    with _renderer(scene, False) as r:
        buf = np.zeros(W * H * 4, np.uint8)
        with pytest.raises(RuntimeError, match="no frame rendered"):
            r.read_output_async(buf)
        r.wait_output()                                   # nothing pending: returns at once
        r.render(camera_sequence(scene, W, H, 1, 4)[0])
        lib = L.load()
        assert lib.xr_read_output_async(r.ctx, buf.ctypes.data, buf.nbytes - 4) == L.XR_ERR_INVALID_ARGUMENT
        with pytest.raises(ValueError):
            r.read_output_async(buf[:-4])
