"""Motion derived on the GPU from motion syntax (rc_h264_picture.motion),
against the oracle's derivation, on generated pictures.

The golden streams pin the derivation to the reference (tests/
test_golden_h264.py); these cases add what those streams hold little of:
every partition shape with 8x4 / 4x8 / 4x4 sub-partitions, up to four
references per list, two lists in one picture, weight entries per
reference pair, P_Skip, and 1080p.  Every picture is compared bit-exactly
with the oracle, which derives the same vectors on the CPU."""
from __future__ import annotations

import numpy as np
import pytest


def sequence(engine, mb_w, mb_h, frames, seed, slots, lists=1, **opts):
    pics = []
    for n in range(frames):
        refs = [(0, (n - k) % slots, n - k) for k in (1, 2, 3) if n - k >= 0]
        if lists == 2:
            refs += [(1, (n - k) % slots, n - k) for k in (2, 1) if n - k >= 0]
        pics.append(engine.SynthH264(seed=seed * 1000 + n, mb_w=mb_w, mb_h=mb_h, intra_only=int(n == 0), refs=refs,
                                     frame_id=n, motion_syntax=1, **opts))
    return pics


def test_generated_motion_syntax_validates(engine, oracle):
    L = engine.lib()
    for lists in (1, 2):
        pics = sequence(engine, 9, 7, 5, seed=51 + lists, slots=6, lists=lists, bipred_permille=500)
        dpb = oracle.H264Dpb(9, 7, 6)
        for n, p in enumerate(pics):
            assert p.pic.motion and p.pic.slice_motion
            assert L.rc_h264_validate(9, 7, 6, p.ptr) == 0
            assert dpb.recon(p.ptr, n % 6) == 0


def run(engine, oracle, mb_w, mb_h, frames, seed, slots=6, lists=1, group=1, **opts):
    pics = sequence(engine, mb_w, mb_h, frames, seed, slots, lists, **opts)
    st = engine.ReconStream(engine.RC_CODEC_H264, mb_w * 16, mb_h * 16, 8, slots)
    dpb = oracle.H264Dpb(mb_w, mb_h, slots)
    try:
        assert st.set_h264_group(group) == group
        st.profile(True)
        for n, p in enumerate(pics):
            st.submit_h264(p, n % slots)
            assert dpb.recon(p.ptr, n % slots) == 0
            for g, w in zip(st.download(n % slots), dpb.planes(n % slots)):
                assert np.array_equal(g, w), f"picture {n}"
        assert st.sync() == 0
        counts = {k: c for k, (ms, c) in st.profile_read().items()}
        assert counts.get(9, 0) == frames  # h264_mv_kernel once per picture
    finally:
        st.close()


@pytest.mark.gpu
def test_motion_one_list_all_shapes(engine, oracle):
    run(engine, oracle, 13, 9, 6, seed=61)


@pytest.mark.gpu
def test_motion_two_lists_weights_slices(engine, oracle):
    run(engine, oracle, 12, 10, 6, seed=62, lists=2, bipred_permille=500, wp_permille=400, num_slices=3)


@pytest.mark.gpu
def test_motion_in_picture_groups(engine, oracle):
    run(engine, oracle, 11, 8, 6, seed=63, slots=8, group=3)


@pytest.mark.gpu
def test_motion_1080p(engine, oracle):
    run(engine, oracle, 120, 68, 3, seed=64)
