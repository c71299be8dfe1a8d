"""GPU parity of the H.264 reconstruction kernels against the oracle.

Every test runs pictures through the C ABI (rc_h264_submit on a device DPB)
and through the oracle on the same seeded syntax records, and compares every
plane bit-exactly (integer path: no tolerance)."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def first_diff(a: np.ndarray, b: np.ndarray, blk: int):
    d = np.argwhere(a != b)
    if len(d) == 0:
        return None
    y, x = d[0]
    return f"first mismatch at ({x},{y}) block ({x // blk},{y // blk}): gpu {a[y, x]} oracle {b[y, x]}; {len(d)} samples"


def run_sequence(engine, oracle, mb_w, mb_h, frames, seed, slots=4, lists=1, filter_check=True, **opts):
    """Reconstruct `frames` pictures (the first intra) on the GPU and the
    oracle; returns the per-frame MD5 of the three planes."""
    st = engine.ReconStream(engine.RC_CODEC_H264, mb_w * 16, mb_h * 16, 8, slots)
    dpb = oracle.H264Dpb(mb_w, mb_h, slots)
    md5s = []
    try:
        for n in range(frames):
            slot = n % slots
            refs = [(0, (n - k) % slots, n - k) for k in (1, 2) if n - k >= 0]
            if lists == 2:
                refs += [(1, (n - k) % slots, n - k) for k in (2, 1) if n - k >= 0]
            p = engine.SynthH264(seed=seed * 1000 + n, mb_w=mb_w, mb_h=mb_h, intra_only=int(n == 0),
                                 refs=refs, frame_id=n, **opts)
            st.submit_h264(p, slot)
            assert dpb.recon(p.ptr, slot) == 0
            assert st.sync() == 0
            got = st.download(slot)
            want = dpb.planes(slot)
            for name, g, w, blk in zip("YUV", got, want, (16, 8, 8)):
                assert g.shape == w.shape
                msg = first_diff(g, w, blk)
                assert msg is None, f"frame {n} plane {name}: {msg}"
            md5s.append(tuple(hashlib.md5(g.tobytes()).hexdigest() for g in got))
    finally:
        st.close()
    return md5s


def test_small_sequence_default_mix(engine, oracle):
    run_sequence(engine, oracle, 8, 6, 6, seed=1)


def test_no_loop_filter_isolates_reconstruction(engine, oracle):
    run_sequence(engine, oracle, 9, 7, 4, seed=2, deblock_idc=1)


def test_odd_size_slices_pcm_offsets(engine, oracle):
    run_sequence(engine, oracle, 11, 7, 5, seed=3, num_slices=3, deblock_idc=2, alpha_offset=6,
                 beta_offset=-4, pcm_permille=80)


def test_constrained_intra_and_filter_offsets(engine, oracle):
    run_sequence(engine, oracle, 10, 6, 4, seed=4, constrained_intra_pred=1, alpha_offset=-12, beta_offset=12,
                 intra_permille=600)


def test_bipred_weighted_two_lists(engine, oracle):
    run_sequence(engine, oracle, 8, 8, 5, seed=5, lists=2, bipred_permille=600, wp_permille=400)


def test_custom_scaling_matrices_and_qp_extremes(engine, oracle):
    run_sequence(engine, oracle, 7, 5, 4, seed=6, custom_scaling=1, qp_min=0, qp_max=51, chroma_qp_offset=-4)


def test_far_motion_and_dense_residual(engine, oracle):
    run_sequence(engine, oracle, 6, 6, 4, seed=7, mv_range=400, outside_permille=300, zero_permille=200)


def test_intra_only_pictures(engine, oracle):
    run_sequence(engine, oracle, 12, 9, 1, seed=8)
    run_sequence(engine, oracle, 1, 1, 1, seed=9)


def test_1080p_frames(engine, oracle):
    md5 = run_sequence(engine, oracle, 120, 68, 3, seed=10)
    assert len(md5) == 3


def test_small_config_geometry_qp26_60_frames(engine, oracle):
    """The small plain configuration's shape: 640x360 (40 x 23 MBs, coded
    640x368), 60 frames, QP 26, one intra picture then P pictures; seeded
    syntax records stand in for the reference encoder's stream."""
    run_sequence(engine, oracle, 40, 23, 60, seed=30, qp_min=26, qp_max=26)


def test_largest_picture(engine, oracle):
    """The largest coded size a stream accepts, 8192 x 8192 (512 x 512 MBs,
    128 bands): an intra picture, then a P picture with far and off-picture
    motion."""
    run_sequence(engine, oracle, 512, 512, 2, seed=31, mv_range=512)


@pytest.mark.parametrize("mb_h", [200, 204, 308])
def test_band_launch_forms(engine, oracle, mb_h):
    """Heights that give the band launch each of its forms on a 152-SM GB300
    (one band CTA per SM, 4 MB rows per band): 50 bands take three CTAs per
    band (intra, luma filter, chroma filter), 51 bands two (intra with the
    luma filter, the chroma filter apart), 77 bands one.  Narrow pictures
    with intra MBs and far motion keep the oracle quick."""
    run_sequence(engine, oracle, 6, mb_h, 3, seed=40 + mb_h, mv_range=256)


def test_deterministic(engine, oracle):
    a = run_sequence(engine, oracle, 8, 6, 3, seed=11)
    b = run_sequence(engine, oracle, 8, 6, 3, seed=11)
    assert a == b


def test_invalid_picture_rejected_before_launch(engine):
    import ctypes
    with engine.ReconStream(engine.RC_CODEC_H264, 64, 48, 8, 2) as st:
        p = engine.SynthH264(seed=1, mb_w=4, mb_h=3, refs=[(0, 5, 1)])  # slot 5 outside a 2-slot DPB
        before = st.launches()
        with pytest.raises(engine.ReconError) as e:
            st.submit_h264(p, 0)
        assert e.value.code == engine.RC_EINVAL
        assert st.launches() == before
        with pytest.raises(engine.ReconError):
            st.submit_h264(engine.SynthH264(seed=1, mb_w=4, mb_h=3, intra_only=1), 7)
        with pytest.raises(engine.ReconError):
            st.download(0, crop=(0, 0, 65, 48))
        assert st.sync() == 0


def test_hbm_budget_enforced(engine):
    with pytest.raises(engine.ReconError) as e:
        engine.ReconStream(engine.RC_CODEC_H264, 1920, 1080, 8, 8, hbm_budget=1 << 20)
    assert e.value.code == engine.RC_ENOMEM


def test_cropped_download_matches_planes(engine, oracle):
    with engine.ReconStream(engine.RC_CODEC_H264, 100, 60, 8, 2) as st:
        p = engine.SynthH264(seed=12, mb_w=7, mb_h=4, intra_only=1)
        st.submit_h264(p, 0)
        assert st.sync() == 0
        Y, U, V = st.download(0)
        y, u, v = st.download(0, crop=(2, 4, 99, 55))
        assert np.array_equal(y, Y[4:59, 2:101])
        assert np.array_equal(u, U[2:30, 1:51])
        assert np.array_equal(v, V[2:30, 1:51])


def test_launch_count_and_profile(engine):
    with engine.ReconStream(engine.RC_CODEC_H264, 64, 64, 8, 2) as st:
        st.profile(True)
        p = engine.SynthH264(seed=3, mb_w=4, mb_h=4, intra_only=1)
        n0 = st.launches()
        st.submit_h264(p, 0)
        assert st.launches() - n0 == 3  # edge words, MB kernel, band kernel
        prof = st.profile_read()
        assert all(prof[k][1] == 1 for k in (0, 1, 2)) and prof[1][0] > 0


def test_streams_of_different_widths_coexist(engine, oracle):
    """A narrower stream created after a wider one must not break the wider
    one's launches (the band kernel's shared-memory limit is per process)."""
    wide = engine.ReconStream(engine.RC_CODEC_H264, 1920, 1088, 8, 2)
    narrow = engine.ReconStream(engine.RC_CODEC_H264, 320, 192, 8, 2)
    try:
        for st, (mw, mh) in ((wide, (120, 68)), (narrow, (20, 12)), (wide, (120, 68))):
            p = engine.SynthH264(seed=77 + mw, mb_w=mw, mb_h=mh, intra_only=1)
            st.submit_h264(p, 0)
            assert st.sync() == 0
            dpb = oracle.H264Dpb(mw, mh, 2)
            assert dpb.recon(p.ptr, 0) == 0
            for g, w in zip(st.download(0), dpb.planes(0)):
                assert np.array_equal(g, w)
    finally:
        wide.close()
        narrow.close()


def _bench():
    import importlib.util
    import pathlib
    import sys
    if "bench" in sys.modules:
        return sys.modules["bench"]
    path = pathlib.Path(__file__).resolve().parent.parent / "bench.py"
    spec = importlib.util.spec_from_file_location("bench", path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules["bench"] = mod
    spec.loader.exec_module(mod)
    return mod


def test_benched_1080p_sequence_first_30_frames(engine, oracle):
    """The bench's own workload (same generator, seed, references and DPB
    slots), its first 30 frames at 1920x1088, every plane against the oracle."""
    B = _bench()
    wl = B.H264Workload(engine)
    pics = wl.sequence(B.SEED, 30)
    st = engine.ReconStream(engine.RC_CODEC_H264, wl.W, wl.H, 8, wl.slots)
    dpb = wl.oracle_dpb(oracle)
    try:
        for n, p in enumerate(pics):
            slot = n % wl.slots
            st.submit_h264(p, slot)
            assert dpb.recon(p.ptr, slot) == 0
            assert st.sync() == 0
            for name, g, w, blk in zip("YUV", st.download(slot), dpb.planes(slot), (16, 8, 8)):
                msg = first_diff(g, w, blk)
                assert msg is None, f"frame {n} plane {name}: {msg}"
    finally:
        st.close()
