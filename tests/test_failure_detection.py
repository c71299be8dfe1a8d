"""Failure detection on the GPU, in forms that leave the device usable.

- A device-side wait that runs out: every wait in the wavefront kernels
  polls at most `wait_limit` times, then records RC_ETIMEOUT in the stream's
  sticky error word, and its launch unwinds.  rc_stream_set_wait_limit(1)
  makes the first wait that finds its neighbour not yet done give up.
- A record the device finds out of range (RC_MEM_DEVICE records skip the
  host-side validation): the kernel records RC_EDEVICE and skips it.

In both cases the test then reads the sticky error (rc_stream_error clears
it), restores the defaults and checks that the next pictures on the same
stream are bit-exact with the oracle.  Nothing here faults, traps or hangs
the GPU: a wait that gives up returns, a bad record is not accessed.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RC_HEVC_TU_CBF = 2


def _same(got, want, what):
    for name, g, w in zip("YUV", got, want):
        assert np.array_equal(g.astype(np.uint16), w.astype(np.uint16)), f"{what}: plane {name} differs"


def test_h264_wait_runs_out_then_stream_recovers(engine, oracle):
    mb_w, mb_h = 40, 23
    st = engine.ReconStream(engine.RC_CODEC_H264, mb_w * 16, mb_h * 16, 8, 4)
    dpb = oracle.H264Dpb(mb_w, mb_h, 4)
    try:
        bad = engine.SynthH264(seed=3101, mb_w=mb_w, mb_h=mb_h, intra_only=1, frame_id=0)
        st.set_wait_limit(1)
        st.submit_h264(bad, 0)
        assert st.sync() == engine.RC_ETIMEOUT
        assert st.sync() == engine.RC_ETIMEOUT  # sticky until read
        assert st.error() == engine.RC_ETIMEOUT
        assert st.sync() == 0
        st.set_wait_limit(0)
        for n in (1, 2):
            refs = [(0, 1, 1)] if n == 2 else None
            p = engine.SynthH264(seed=3100 + n, mb_w=mb_w, mb_h=mb_h, intra_only=int(n == 1), refs=refs,
                                 frame_id=n)
            st.submit_h264(p, n)
            assert dpb.recon(p.ptr, n) == 0
            assert st.sync() == 0
            _same(st.download(n), dpb.planes(n), f"H.264 picture {n} after the timeout")
    finally:
        st.close()


def test_hevc_wait_runs_out_then_stream_recovers(engine, oracle):
    W, H = 512, 256
    st = engine.ReconStream(engine.RC_CODEC_HEVC, W, H, 8, 4)
    dpb = oracle.HevcDpb(W, H, 8, 4)
    try:
        bad = engine.SynthHevc(seed=3201, width=W, height=H, log2_ctb=5, intra_only=1, frame_id=0)
        st.set_wait_limit(1)
        st.submit_hevc(bad, 0)
        assert st.sync() == engine.RC_ETIMEOUT
        assert st.error() == engine.RC_ETIMEOUT
        assert st.sync() == 0
        st.set_wait_limit(0)
        for n in (1, 2):
            refs = [(0, 1, 1)] if n == 2 else None
            p = engine.SynthHevc(seed=3200 + n, width=W, height=H, log2_ctb=5, intra_only=int(n == 1), refs=refs,
                                 frame_id=n)
            st.submit_hevc(p, n)
            assert dpb.recon(p.ptr, n, 3) == 0
            assert st.sync() == 0
            _same(st.download(n), dpb.planes(n), f"HEVC picture {n} after the timeout")
    finally:
        st.close()


def _device_hevc(engine, bufs, src, keep):
    """An RC_MEM_DEVICE rc_hevc_picture over device copies of `bufs`."""
    import torch
    d = engine.HevcPicture()
    d.mem = engine.RC_MEM_DEVICE
    for k in engine.HevcPictureBuffers.HEADER:
        setattr(d, k, getattr(src, k))
    d.num_levels = len(bufs["levels"]) // 2
    d.num_tus = len(bufs["tus"]) // ctypes.sizeof(engine.HevcTu)
    for key in ("ctbs", "blk", "mvf", "tus", "slices", "levels"):
        t = torch.frombuffer(bytearray(bufs[key]), dtype=torch.uint8).cuda()
        keep.append(t)
        setattr(d, key, t.data_ptr())
    return d


def test_hevc_out_of_range_record_reported_then_stream_recovers(engine, oracle):
    torch = pytest.importorskip("torch")
    W, H, ctb = 128, 64, 32
    st = engine.ReconStream(engine.RC_CODEC_HEVC, W, H, 8, 4)
    dpb = oracle.HevcDpb(W, H, 8, 4)
    keep = []
    try:
        i0 = engine.SynthHevc(seed=3301, width=W, height=H, log2_ctb=5, intra_only=1, frame_id=0)
        st.submit_hevc(i0, 0)
        assert dpb.recon(i0.ptr, 0, 3) == 0
        assert st.sync() == 0
        _same(st.download(0), dpb.planes(0), "HEVC intra picture")
        # an all-inter picture whose transform-block list ends with one block
        # that reaches past the picture's right edge, inside the last CTB in
        # decode order (so that every CTB's block range stays as it was)
        p = engine.SynthHevc(seed=3302, width=W, height=H, log2_ctb=5, intra_permille=0, refs=[(0, 0, 0)],
                             frame_id=1)
        bufs = p.buffers()
        t = engine.HevcTu()
        t.x0, t.y0, t.log2, t.c = W - 4, H - 4, 5, 0
        t.flags, t.qp, t.max_x, t.max_y, t.coef_off = RC_HEVC_TU_CBF, 30, 0, 0, 0
        assert (W - 4) // ctb == W // ctb - 1 and (H - 4) // ctb == H // ctb - 1
        bufs["tus"] = bufs["tus"] + bytes(t)
        d = _device_hevc(engine, bufs, p.pic, keep)
        torch.cuda.synchronize()
        st.submit_hevc(ctypes.addressof(d), 1)
        assert st.sync() == engine.RC_EDEVICE
        assert st.error() == engine.RC_EDEVICE
        assert st.sync() == 0
        # the same picture from host records is rejected before any launch
        with pytest.raises(engine.ReconError) as e:
            st.submit_hevc(engine.HevcPictureBuffers(bufs, {**{k: getattr(p.pic, k) for k in
                                                              engine.HevcPictureBuffers.HEADER},
                                                           "num_tus": p.pic.num_tus + 1}), 1)
        assert e.value.code == engine.RC_EINVAL
        # and the stream goes on: a valid inter picture from the intra one
        q = engine.SynthHevc(seed=3303, width=W, height=H, log2_ctb=5, refs=[(0, 0, 0)], frame_id=2)
        st.submit_hevc(q, 2)
        assert dpb.recon(q.ptr, 2, 3) == 0
        assert st.sync() == 0
        _same(st.download(2), dpb.planes(2), "HEVC picture after the bad record")
    finally:
        st.close()

