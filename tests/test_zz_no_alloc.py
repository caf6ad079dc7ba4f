"""tr_render_frame_noalloc: rendering into caller-owned device buffers with no
device allocation, for callers that cannot allocate where they render (a
render loop that must not stall the device on cudaMalloc/cudaFree, a host that
owns all device memory). Checked against tr_render_frame, which renders the
same frame from the context's own buffers, on two calls in a row.

Named to run last: it loads the library's device scratch array on the GPU."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

import trayracer_gb300 as tr
from trayracer_gb300 import _abi

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

RTOL = 1e-4  # the per-path / per-pixel tolerance of the parity tests


def _close(a, b):
    return np.abs(a - b) <= RTOL * np.maximum(1.0, np.abs(b)) + 1e-6


def test_noalloc_matches_render_frame_on_two_calls():
    scene = tr.cornell_box(width=64, height=48)
    st = tr.settings_for(scene, multi_sample=2)
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((64, 48))
    r.SetSettings(st)
    # the same two frames through the context's own buffers
    r.RenderFrame()
    want1 = r.ColorBuffer().copy()
    r.RenderFrame()
    want2 = r.ColorBuffer().copy()

    lib = _abi.load_library()
    acc = torch.full((48, 64, 4), 7.0, dtype=torch.float32, device="cuda")  # stale contents on purpose
    col = torch.zeros((48, 64, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert lib.tr_render_frame_noalloc(r.handle, None, acc.data_ptr(), col.data_ptr(), 0) == 0
    torch.cuda.synchronize()
    got1 = col.cpu().numpy()
    assert lib.tr_render_frame_noalloc(r.handle, None, acc.data_ptr(), col.data_ptr(), 2) == 0
    torch.cuda.synchronize()
    got2 = col.cpu().numpy()
    assert _close(got1, want1).all()
    assert _close(got2, want2).all()
    assert np.array_equal(acc.cpu().numpy()[..., 3], np.full((48, 64), 4.0, np.float32))
    # the statistics of a no-allocation frame come from the shared array
    s = r.Statistics()
    assert s["device_error"] == 0 and s["extend_rays"][0] == 64 * 48 * 2 and s["sample_count"] == 4

    # a traversal that runs out of its bound is reported through tr_get_statistics; the next
    # call starts clean
    r.SetSettings(dataclasses.replace(st, traversalStepLimit=2))
    assert lib.tr_render_frame_noalloc(r.handle, None, acc.data_ptr(), col.data_ptr(), 0) == 0
    assert r.Statistics()["device_error"] != 0
    r.SetSettings(st)
    assert lib.tr_render_frame_noalloc(r.handle, None, acc.data_ptr(), col.data_ptr(), 0) == 0
    assert r.Statistics()["device_error"] == 0
    torch.cuda.synchronize()
    assert _close(col.cpu().numpy(), want1).all()

    # other render modes are refused, not path-traced
    assert lib.tr_set_render_mode(r.handle, 0, 0, C.c_float(1.0), C.c_float(1.0)) == 0  # ambient occlusion
    assert lib.tr_render_frame_noalloc(r.handle, None, acc.data_ptr(), col.data_ptr(), 0) == 1
    assert b"path-tracing" in lib.tr_last_error(r.handle)
    assert lib.tr_set_render_mode(r.handle, 7, 0, C.c_float(1.0), C.c_float(1.0)) == 0

    # beyond the scratch array: rejected with a status, nothing launched
    r.Resize((512, 512))
    assert lib.tr_render_frame_noalloc(r.handle, None, acc.data_ptr(), col.data_ptr(), 0) == 6  # TR_ERR_LIMIT
    assert b"131072" in lib.tr_last_error(r.handle)
    assert lib.tr_render_frame_noalloc(r.handle, None, None, col.data_ptr(), 0) == 1
    r.close()
