"""The allocation-free deblocking entry point (rc_h264_deblock_noalloc).

It serves callers that cannot allocate device memory while running (their
allocator owns the device memory, or allocation would stall a real-time or
captured stream).  The test checks, through the C ABI, that it filters a
picture exactly as rc_h264_submit does, on two calls in a row (an intra then
an inter picture, the second predicted from the first one's filtered
output), at a small size and at its documented limit (68 x 128 MBs: 8704
MBs in 128 rows), and that it rejects what it cannot take.  One case runs
in a fresh child process, so that the first call's set-up (looking up the
static array's device address in a new context) is exercised on its own.
Collected last so that a run stopping at its first failure has already run
every other test."""
from __future__ import annotations

import ctypes
import pathlib
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MB_W, MB_H = 20, 12
HERE = pathlib.Path(__file__).resolve().parent


def _unfiltered(engine, pic):
    """The picture's records with the loop filter off in every slice."""
    bufs = pic.buffers()
    sl = (engine.H264Slice * pic.pic.num_slices).from_buffer_copy(bufs["slices"])
    for s in sl:
        s.disable_deblocking_filter_idc = 1
    bufs["slices"] = bytes(sl)
    return engine.PictureBuffers(bufs, pic.pic.num_slices, pic.pic.num_weights)


def _device_picture(engine, pic, keep):
    """An RC_MEM_DEVICE copy of the picture's records (torch owns the memory)."""
    import torch
    d = engine.H264Picture()
    d.mem = engine.RC_MEM_DEVICE
    d.num_slices, d.num_weights, d.num_levels = pic.pic.num_slices, pic.pic.num_weights, pic.pic.num_levels
    for key, raw in pic.buffers().items():
        if key in ("scaling4", "scaling8") or not raw:
            continue
        t = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
        keep.append(t)
        setattr(d, key, t.data_ptr())
    return d


def compare_twice(engine, mb_w, mb_h, seed):
    """Two pictures in a row (intra, then inter from the first): the
    allocation-free filter on unfiltered planes equals rc_h264_submit."""
    import torch
    L = engine.lib()
    filt = engine.ReconStream(engine.RC_CODEC_H264, mb_w * 16, mb_h * 16, 8, 2)
    raw = engine.ReconStream(engine.RC_CODEC_H264, mb_w * 16, mb_h * 16, 8, 2)
    keep = []
    try:
        for n in range(2):
            refs = [(0, 0, 0)] if n else None
            p = engine.SynthH264(seed=seed + n, mb_w=mb_w, mb_h=mb_h, intra_only=int(n == 0), refs=refs, frame_id=n)
            filt.submit_h264(p, n)
            raw.submit_h264(_unfiltered(engine, p), n)
            assert filt.sync() == 0 and raw.sync() == 0
            dpic = _device_picture(engine, p, keep)
            y, u, v = raw.device_planes(n)
            status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            rc = L.rc_h264_deblock_noalloc(ctypes.addressof(dpic), mb_w, mb_h, y, u, v, raw.pitch, raw.cpitch,
                                           status.data_ptr(), raw.cuda_stream())
            assert rc == engine.RC_OK
            assert raw.sync() == 0
            torch.cuda.synchronize()
            assert int(status.item()) == 0
            for a, b in zip(raw.download(n), filt.download(n)):
                assert np.array_equal(a, b), f"picture {n}: allocation-free filter differs from rc_h264_submit"
    finally:
        filt.close()
        raw.close()


def test_noalloc_deblock_matches_submit_twice(engine):
    pytest.importorskip("torch")
    compare_twice(engine, MB_W, MB_H, 909)


def test_noalloc_deblock_at_its_limit(engine):
    """68 x 128 MBs: exactly RC_NOALLOC_MAX_MBS macroblocks in
    RC_NOALLOC_MAX_ROWS rows."""
    pytest.importorskip("torch")
    assert 68 * 128 == 8704
    compare_twice(engine, 68, 128, 919)


def test_noalloc_first_call_in_a_fresh_process():
    """A child process in which nothing called this entry point before, so
    that its first call sets up the static array's address there."""
    pytest.importorskip("torch")
    code = ("import sys; sys.path.insert(0, {tests!r}); import conftest, test_zz_no_alloc as t; "
            "t.compare_twice(conftest.load_engine(), 20, 12, 929); print('child ok')").format(tests=str(HERE))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "child ok" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]


def test_noalloc_rejects_what_it_cannot_take(engine):
    torch = pytest.importorskip("torch")
    L = engine.lib()
    keep = []
    p = engine.SynthH264(seed=5, mb_w=4, mb_h=3, intra_only=1)
    dpic = _device_picture(engine, p, keep)
    planes = torch.zeros(16 * 3 * 64 + 2 * 8 * 3 * 32 + 64, dtype=torch.uint8, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    y = planes.data_ptr()
    u = y + 64 * 48
    v = u + 32 * 24
    args = (y, u, v, 64, 32, status.data_ptr(), None)
    # more macroblocks than the static scratch holds
    assert L.rc_h264_deblock_noalloc(ctypes.addressof(dpic), 120, 80, *args) == engine.RC_EINVAL
    assert L.rc_h264_deblock_noalloc(ctypes.addressof(dpic), 1, 129, *args) == engine.RC_EINVAL
    # host-memory records would need a staging copy
    assert L.rc_h264_deblock_noalloc(p.ptr, 4, 3, *args) == engine.RC_EINVAL
    # misaligned luma pitch
    assert L.rc_h264_deblock_noalloc(ctypes.addressof(dpic), 4, 3, y, u, v, 72, 32, status.data_ptr(),
                                     None) == engine.RC_EINVAL
