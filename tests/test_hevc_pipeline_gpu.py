"""HEVC pictures submitted back to back: parity of the overlapped inter passes.

A picture's inter prediction runs in two passes: the units whose references
are final run on the side stream beside the previous picture's intra and
loop-filter kernels, and the units that read the previous picture run on
the main stream after it.  These tests submit whole sequences without a
sync between pictures, fetch every picture with an asynchronous download
issued right after its submit, and compare each plane bit-exactly with the
oracle.  They also check which passes ran (per-kernel launch counts): none
for a picture that does not reference its predecessor (host records show
it), always for device-memory records, whose reference lists the host does
not read.  One case writes a reference slot through the caller's own stream
between two submits."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INTER, INTER_LATE = 4, 7


def _pinned(torch, W, H, bd):
    dt = torch.uint16 if bd > 8 else torch.uint8
    return tuple(torch.zeros(n, dtype=dt).pin_memory() for n in (W * H, W * H // 4, W * H // 4))


def _same(got, want, W, H, what):
    for name, g, w, (h, ww) in zip("YUV", got, want, ((H, W), (H // 2, W // 2), (H // 2, W // 2))):
        g = g.numpy().astype(np.uint16).reshape(h, ww)
        d = np.argwhere(g != w)
        assert len(d) == 0, f"{what} plane {name}: first mismatch at {tuple(d[0][::-1])}, {len(d)} samples"


class _DevicePlane:
    """A slot plane as a CUDA array (torch.as_tensor takes it without a copy)."""

    def __init__(self, ptr, h, w, pitch):
        self.__cuda_array_interface__ = {"shape": (h, w), "strides": (pitch, 1), "typestr": "|u1",
                                         "data": (ptr, False), "version": 2}


def _device(engine, p, keep):
    """An RC_MEM_DEVICE copy of synthetic picture p's records."""
    import torch
    bufs = p.buffers()
    d = engine.HevcPicture()
    d.mem = engine.RC_MEM_DEVICE
    for k in engine.HevcPictureBuffers.HEADER:
        setattr(d, k, getattr(p.pic, k))
    d.num_levels = len(bufs["levels"]) // 2
    d.num_tus = len(bufs["tus"]) // ctypes.sizeof(engine.HevcTu)
    for key in ("ctbs", "blk", "mvf", "tus", "slices", "levels"):
        t = torch.frombuffer(bytearray(bufs[key]), dtype=torch.uint8).cuda()
        keep.append(t)
        setattr(d, key, t.data_ptr())
    return d


def run_pipelined(engine, oracle, W, H, frames, seed, bd=8, slots=5, refs_of=None, device=False, **opts):
    torch = pytest.importorskip("torch")
    refs_of = refs_of or (lambda n: [(0, (n - k) % slots, n - k) for k in (1, 2, 3, 4) if n - k >= 0])
    pics = [engine.SynthHevc(seed=seed * 1000 + n, width=W, height=H, bit_depth=bd, intra_only=int(n == 0),
                             refs=refs_of(n), frame_id=n, **opts) for n in range(frames)]
    dpb = oracle.HevcDpb(W, H, bd, slots)
    want = []
    for n, p in enumerate(pics):
        assert dpb.recon(p.ptr, n % slots, 3) == 0
        want.append([np.array(x, copy=True) for x in dpb.planes(n % slots)])
    outs = [_pinned(torch, W, H, bd) for _ in range(frames)]
    keep = []
    st = engine.ReconStream(engine.RC_CODEC_HEVC, W, H, bd, slots)
    try:
        recs = [_device(engine, p, keep) for p in pics] if device else None
        torch.cuda.synchronize()
        st.profile(True)
        for n, p in enumerate(pics):
            st.submit_hevc(ctypes.addressof(recs[n]) if device else p, n % slots)
            y, u, v = outs[n]
            st.download_async(n % slots, (0, 0, W, H), y.data_ptr(), u.data_ptr(), v.data_ptr())
        assert st.sync() == 0
        counts = {k: c for k, (ms, c) in st.profile_read().items()}
    finally:
        st.close()
    for n in range(frames):
        _same(outs[n], want[n], W, H, f"picture {n}")
    return counts


def test_back_to_back_8bit(engine, oracle):
    counts = run_pipelined(engine, oracle, 416, 240, 12, seed=71, log2_ctb=5)
    # every picture after the first reads its predecessor: two passes each
    assert counts[INTER] == 12 and counts[INTER_LATE] == 11


def test_back_to_back_10bit_two_lists(engine, oracle):
    slots = 6
    refs = lambda n: ([(0, (n - k) % slots, n - k) for k in (1, 2) if n - k >= 0] +
                      [(1, (n - k) % slots, n - k) for k in (3, 1) if n - k >= 0])
    counts = run_pipelined(engine, oracle, 352, 208, 10, seed=72, bd=10, slots=slots, refs_of=refs, log2_ctb=4)
    assert counts[INTER] == 10 and counts[INTER_LATE] == 9


def test_pictures_that_skip_their_predecessor_need_one_pass(engine, oracle):
    slots = 5
    # odd pictures reference only pictures two and three back
    refs = lambda n: [(0, (n - k) % slots, n - k) for k in ((2, 3) if n % 2 else (1, 2)) if n - k >= 0]
    counts = run_pipelined(engine, oracle, 320, 192, 11, seed=73, slots=slots, refs_of=refs, log2_ctb=5)
    # pictures 2, 4, .., 10 read their predecessor; 1, 3, .., 9 do not
    assert counts[INTER] == 11 and counts[INTER_LATE] == 5


def test_device_records_always_take_both_passes(engine, oracle):
    counts = run_pipelined(engine, oracle, 256, 160, 8, seed=74, device=True, log2_ctb=6)
    assert counts[INTER] == 8 and counts[INTER_LATE] == 7


def test_1080p_back_to_back(engine, oracle):
    counts = run_pipelined(engine, oracle, 1920, 1080, 5, seed=75)
    assert counts[INTER] == 5 and counts[INTER_LATE] == 4


def test_slot_written_on_the_callers_stream_between_submits(engine, oracle):
    """A reference written into a slot through rc_picture_device_planes on
    the stream's own CUDA stream, between two submits with no sync, then
    rc_stream_cuda_stream called again (the ordering rule for such writes):
    the next picture's first inter pass, on the side stream, runs after the
    write."""
    torch = pytest.importorskip("torch")
    W, H, slots = 320, 192, 5
    rng = np.random.default_rng(76)
    ref = [rng.integers(0, 256, (H, W), dtype=np.uint8), rng.integers(0, 256, (H // 2, W // 2), dtype=np.uint8),
           rng.integers(0, 256, (H // 2, W // 2), dtype=np.uint8)]
    p0 = engine.SynthHevc(seed=7600, width=W, height=H, intra_only=1, frame_id=0, log2_ctb=5)
    # picture 1 reads slot 3 (written by the caller) and picture 0
    p1 = engine.SynthHevc(seed=7601, width=W, height=H, refs=[(0, 3, 7), (0, 0, 0)], frame_id=1, log2_ctb=5)
    dpb = oracle.HevcDpb(W, H, 8, slots)
    assert dpb.recon(p0.ptr, 0, 3) == 0
    for pl, r in zip(dpb.planes(3), ref):
        pl[:] = r
    assert dpb.recon(p1.ptr, 1, 3) == 0
    want = [np.array(x, copy=True) for x in dpb.planes(1)]
    out = _pinned(torch, W, H, 8)
    st = engine.ReconStream(engine.RC_CODEC_HEVC, W, H, 8, slots)
    try:
        planes = st.device_planes(3)
        dst = [torch.as_tensor(_DevicePlane(ptr, h, w, pitch), device="cuda")
               for ptr, (h, w), pitch in zip(planes, ((H, W), (H // 2, W // 2), (H // 2, W // 2)),
                                             (st.pitch, st.cpitch, st.cpitch))]
        cs = torch.cuda.ExternalStream(st.cuda_stream())
        src = [torch.from_numpy(r).cuda() for r in ref]
        torch.cuda.synchronize()
        st.submit_hevc(p0, 0)
        with torch.cuda.stream(cs):
            # a long kernel first, so that the copies land well after the
            # submit above returned
            torch.cuda._sleep(2_000_000)
            for d, s in zip(dst, src):
                d.copy_(s)
        assert st.cuda_stream() == cs.cuda_stream
        st.submit_hevc(p1, 1)
        y, u, v = out
        st.download_async(1, (0, 0, W, H), y.data_ptr(), u.data_ptr(), v.data_ptr())
        assert st.sync() == 0
    finally:
        st.close()
    _same(out, want, W, H, "picture 1")
