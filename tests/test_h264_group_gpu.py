"""GPU parity of H.264 picture groups (rc_stream_set_h264_group) against the
oracle.

A group launch reconstructs several consecutive pictures at once: the intra
+ loop-filter wavefront of each beside the MB phase of all of them, an inter
MB of a later picture waiting only for the rows of the earlier ones that its
motion vectors reach.  Every test here submits pictures without waiting, so
that they form groups, and compares every picture bit-exactly with the
oracle, which reconstructs them one at a time.  A picture's planes are read
back before any later picture overwrites its DPB slot: pictures are
submitted in runs whose output slots are distinct, and the first download of
a run launches what is still queued."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def first_diff(a: np.ndarray, b: np.ndarray, blk: int):
    d = np.argwhere(a != b)
    if len(d) == 0:
        return None
    y, x = d[0]
    return f"first mismatch at ({x},{y}) block ({x // blk},{y // blk}): gpu {a[y, x]} oracle {b[y, x]}; {len(d)} samples"


def runs(slots_of):
    """Split pictures into runs of distinct output slots."""
    out, cur = [], []
    for i, s in enumerate(slots_of):
        if s in [slots_of[j] for j in cur]:
            out.append(cur)
            cur = []
        cur.append(i)
    if cur:
        out.append(cur)
    return out


def run_grouped(engine, oracle, pics, slots_of, mb_w, mb_h, dpb_slots, group, submit=None):
    """Reconstruct `pics` (SynthH264 or PictureBuffers) into slots_of[i] on
    the GPU with groups of `group` pictures and on the oracle; compares every
    picture and returns the stream's per-kernel launch counts.  submit(st, i,
    slot), if given, submits picture i instead of st.submit_h264."""
    st = engine.ReconStream(engine.RC_CODEC_H264, mb_w * 16, mb_h * 16, 8, dpb_slots)
    dpb = oracle.H264Dpb(mb_w, mb_h, dpb_slots)
    want = []
    for p, s in zip(pics, slots_of):
        assert dpb.recon(p.ptr, s) == 0
        want.append([np.array(x, copy=True) for x in dpb.planes(s)])
    try:
        assert st.set_h264_group(group) == group
        st.profile(True)
        for r in runs(slots_of):
            for i in r:
                if submit:
                    submit(st, i, slots_of[i])
                else:
                    st.submit_h264(pics[i], slots_of[i])
            for i in r:
                for name, g, w, blk in zip("YUV", st.download(slots_of[i]), want[i], (16, 8, 8)):
                    msg = first_diff(g, w, blk)
                    assert msg is None, f"picture {i} plane {name}: {msg}"
        assert st.sync() == 0
        return {k: n for k, (ms, n) in st.profile_read().items()}
    finally:
        st.close()


def ipp_sequence(engine, mb_w, mb_h, frames, seed, slots, lists=1, **opts):
    pics = []
    for n in range(frames):
        refs = [(0, (n - k) % slots, n - k) for k in (1, 2) if n - k >= 0]
        if lists == 2:
            refs += [(1, (n - k) % slots, n - k) for k in (2, 1) if n - k >= 0]
        pics.append(engine.SynthH264(seed=seed * 1000 + n, mb_w=mb_w, mb_h=mb_h, intra_only=int(n == 0), refs=refs,
                                     frame_id=n, **opts))
    return pics, [n % slots for n in range(frames)]


@pytest.mark.parametrize("group", [2, 3, 4])
def test_group_sizes_small_pictures(engine, oracle, group):
    pics, slots = ipp_sequence(engine, 8, 6, 12, seed=31, slots=8)
    counts = run_grouped(engine, oracle, pics, slots, 8, 6, 8, group)
    # every picture went through the pre-pass (ids 2, 0) and the group
    # kernel (id 8), none through the one-picture band kernel (id 1)
    assert counts.get(8, 0) >= 12 // group and 1 not in counts
    assert counts.get(0, 0) == 12 and counts.get(2, 0) == 12


def test_group_far_motion_dense_residual_two_lists(engine, oracle):
    # motion vectors reaching far down and right make inter MBs wait for
    # late rows of the picture before them in the group
    pics, slots = ipp_sequence(engine, 13, 9, 10, seed=32, slots=8, lists=2, mv_range=256, zero_permille=0,
                               bipred_permille=600, wp_permille=400)
    run_grouped(engine, oracle, pics, slots, 13, 9, 8, 4)


def test_group_intra_mix_constrained_and_filter_offsets(engine, oracle):
    pics, slots = ipp_sequence(engine, 11, 10, 9, seed=33, slots=8, intra_permille=500, constrained_intra_pred=1,
                               alpha_offset=6, beta_offset=-4, num_slices=3, pcm_permille=30)
    run_grouped(engine, oracle, pics, slots, 11, 10, 8, 3)


def test_group_with_slot_reuse_flushes(engine, oracle):
    # four slots and references two back: from the second run of slots on,
    # the third picture of a group would overwrite a slot that the first one
    # reads, so those groups end after two pictures: runs [0..3] (one group),
    # [4..7] (two), [8, 9] (one)
    pics, slots = ipp_sequence(engine, 10, 7, 10, seed=34, slots=4)
    counts = run_grouped(engine, oracle, pics, slots, 10, 7, 4, 4)
    assert counts.get(8, 0) == 4


def test_group_1080p_bench_sequence(engine, oracle):
    pics, slots = ipp_sequence(engine, 120, 68, 10, seed=35, slots=8)
    run_grouped(engine, oracle, pics, slots, 120, 68, 8, 4)


def test_group_scaling_list_change_and_device_records(engine, oracle):
    """A change of scaling lists launches what is queued first; a picture
    whose records are in device memory joins the group like the others (its
    reference slots are read back from its slices); the output is
    unchanged."""
    torch = pytest.importorskip("torch")
    mb_w, mb_h, slots = 9, 8, 8
    pics = []
    for n in range(10):
        refs = [(0, (n - k) % slots, n - k) for k in (1, 2) if n - k >= 0]
        pics.append(engine.SynthH264(seed=36000 + n, mb_w=mb_w, mb_h=mb_h, intra_only=int(n == 0), refs=refs,
                                     frame_id=n, custom_scaling=int(n in (4, 5))))
    keep = []

    def device_copy(p):
        d = engine.H264Picture()
        d.mem = engine.RC_MEM_DEVICE
        d.num_slices, d.num_weights, d.num_levels = p.pic.num_slices, p.pic.num_weights, p.pic.num_levels
        d.constrained_intra_pred = p.pic.constrained_intra_pred
        d.scaling4, d.scaling8 = p.pic.scaling4, p.pic.scaling8
        for key, raw in p.buffers().items():
            if key in ("scaling4", "scaling8") or not raw:
                continue
            t = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
            keep.append(t)
            setattr(d, key, t.data_ptr())
        return d

    dev = {i: device_copy(pics[i]) for i in (2, 3, 7)}
    torch.cuda.synchronize()

    def submit(st, i, slot):
        st.submit_h264(ctypes.addressof(dev[i]) if i in dev else pics[i], slot)

    counts = run_grouped(engine, oracle, pics, [n % slots for n in range(10)], mb_w, mb_h, slots, 4, submit=submit)
    assert counts.get(8, 0) >= 3 and 1 not in counts


def test_group_timeout_is_reported_and_stream_recovers(engine, oracle):
    """A wait cap of one poll makes the group's waits give up (RC_ETIMEOUT in
    the sticky word, the launch unwinds); with the cap restored the same
    pictures reconstruct exactly."""
    mb_w, mb_h, slots = 30, 17, 8
    pics, slot_of = ipp_sequence(engine, mb_w, mb_h, 4, seed=37, slots=slots)
    st = engine.ReconStream(engine.RC_CODEC_H264, mb_w * 16, mb_h * 16, 8, slots)
    try:
        assert st.set_h264_group(4) == 4
        st.set_wait_limit(1)
        for p, s in zip(pics, slot_of):
            st.submit_h264(p, s)
        assert st.sync() == engine.RC_ETIMEOUT
        assert st.error() == engine.RC_ETIMEOUT  # read and cleared
        assert st.error() == 0
        st.set_wait_limit(0)
        dpb = oracle.H264Dpb(mb_w, mb_h, slots)
        for p, s in zip(pics, slot_of):
            st.submit_h264(p, s)
            assert dpb.recon(p.ptr, s) == 0
        for s in slot_of:
            for g, w in zip(st.download(s), dpb.planes(s)):
                assert np.array_equal(g, w)
        assert st.sync() == 0
    finally:
        st.close()


def test_group_async_downloads_wait_for_their_group(engine, oracle):
    """rc_picture_download_async right after each submit (the e2e pattern):
    a download of a queued picture's slot is issued when its group launches,
    so groups still form, and every copy holds its picture."""
    torch = pytest.importorskip("torch")
    mb_w, mb_h, slots, frames = 12, 9, 8, 14
    pics, slot_of = ipp_sequence(engine, mb_w, mb_h, frames, seed=38, slots=slots)
    dpb = oracle.H264Dpb(mb_w, mb_h, slots)
    want = []
    for p, sl in zip(pics, slot_of):
        assert dpb.recon(p.ptr, sl) == 0
        want.append([np.array(x, copy=True) for x in dpb.planes(sl)])
    W, H = mb_w * 16, mb_h * 16
    outs = [tuple(torch.zeros(n, dtype=torch.uint8).pin_memory() for n in (W * H, W * H // 4, W * H // 4))
            for _ in range(frames)]
    st = engine.ReconStream(engine.RC_CODEC_H264, W, H, 8, slots)
    try:
        assert st.set_h264_group(4) == 4
        st.profile(True)
        for n, (p, sl) in enumerate(zip(pics, slot_of)):
            st.submit_h264(p, sl)
            y, u, v = outs[n]
            st.download_async(sl, (0, 0, W, H), y.data_ptr(), u.data_ptr(), v.data_ptr())
        assert st.sync() == 0
        counts = {k: c for k, (ms, c) in st.profile_read().items()}
    finally:
        st.close()
    assert counts.get(8, 0) < frames and 1 not in counts
    for n in range(frames):
        y, u, v = (t.numpy() for t in outs[n])
        assert np.array_equal(y.reshape(H, W), want[n][0]), f"picture {n} Y"
        assert np.array_equal(u.reshape(H // 2, W // 2), want[n][1]), f"picture {n} U"
        assert np.array_equal(v.reshape(H // 2, W // 2), want[n][2]), f"picture {n} V"
