"""GPU parity of the HEVC reconstruction kernels against the oracle.

Pictures go through the C ABI (rc_hevc_submit on a device DPB) and through
the oracle on the same seeded syntax records; every plane is compared
bit-exactly (integer path: no tolerance), 8-bit and 10-bit."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def first_diff(a, b):
    d = np.argwhere(a != b)
    if len(d) == 0:
        return None
    y, x = d[0]
    return f"first mismatch at ({x},{y}): gpu {a[y, x]} oracle {b[y, x]}; {len(d)} samples"


def run_sequence(engine, oracle, width, height, frames, seed, bit_depth=8, slots=5, lists=1, stages=3, lf_rows=None,
                 log2_ctbs=None, **opts):
    st = engine.ReconStream(engine.RC_CODEC_HEVC, width, height, bit_depth, slots)
    if lf_rows:
        st.set_lf_tile(lf_rows)
        assert st.lf_tile() == lf_rows
    dpb = oracle.HevcDpb(width, height, bit_depth, slots)
    md5s = []
    try:
        for n in range(frames):
            slot = n % slots
            refs = [(0, (n - k) % slots, n - k) for k in (1, 2, 3, 4) if n - k >= 0]
            if lists == 2:
                refs = [(0, (n - k) % slots, n - k) for k in (1, 2) if n - k >= 0]
                refs += [(1, (n - k) % slots, n - k) for k in (2, 1) if n - k >= 0]
            if log2_ctbs:  # a CTB size per picture
                opts["log2_ctb"] = log2_ctbs[n % len(log2_ctbs)]
            p = engine.SynthHevc(seed=seed * 1000 + n, width=width, height=height, bit_depth=bit_depth,
                                 intra_only=int(n == 0), refs=refs, frame_id=n, **opts)
            st.submit_hevc(p, slot)
            assert dpb.recon(p.ptr, slot, stages) == 0
            assert st.sync() == 0
            got = st.download(slot)
            want = dpb.planes(slot)
            for name, g, w in zip("YUV", got, want):
                g = g.astype(np.uint16)
                assert g.shape == w.shape
                msg = first_diff(g, w)
                assert msg is None, f"frame {n} plane {name}: {msg}"
            md5s.append(tuple(hashlib.md5(g.tobytes()).hexdigest() for g in got))
    finally:
        st.close()
    return md5s


def test_ctb_size_changes_between_pictures(engine, oracle):
    """One stream whose pictures change CTB size (64, 16, 16, 32, 64): the
    intra task order follows the CTB grid, built again only when it changes."""
    run_sequence(engine, oracle, 200, 120, 5, seed=8, log2_ctbs=[6, 4, 4, 5, 6])


def test_small_8bit_default_mix(engine, oracle):
    run_sequence(engine, oracle, 128, 72, 4, seed=1, log2_ctb=5)


def test_small_10bit_default_mix(engine, oracle):
    run_sequence(engine, oracle, 136, 88, 4, seed=2, bit_depth=10, log2_ctb=4)


def test_no_loop_filters(engine, oracle):
    run_sequence(engine, oracle, 96, 64, 3, seed=3, log2_ctb=5, deblock_disabled=1, sao=0)


def test_tiles_slices_offsets(engine, oracle):
    run_sequence(engine, oracle, 192, 128, 3, seed=4, log2_ctb=5, tile_cols=2, tile_rows=2, num_slices=3,
                 lf_across_slices=0, loop_filter_across_tiles=0, beta_offset=4, tc_offset=-2,
                 cb_qp_offset=3, cr_qp_offset=-5)


@pytest.mark.parametrize("rows", [16, 32, 64])
def test_loop_filter_tile_heights(engine, oracle, rows):
    """The loop filter's tile height is a schedule knob: every height gives
    the oracle's bytes, across tiles, slices, deblocking offsets, PCM and
    bypass blocks, SAO at 8 and 10 bits, and a picture height that is not a
    multiple of the tile."""
    run_sequence(engine, oracle, 192, 136, 3, seed=40 + rows, log2_ctb=5, tile_cols=2, tile_rows=2, num_slices=3,
                 lf_across_slices=0, loop_filter_across_tiles=0, beta_offset=4, tc_offset=-2, lf_rows=rows)
    run_sequence(engine, oracle, 128, 72, 3, seed=50 + rows, bit_depth=10, log2_ctb=4, pcm_permille=150,
                 pcm_loop_filter_disabled=1, bypass_permille=100, lf_rows=rows)


def test_loop_filter_tile_knob_rejects_bad_heights(engine):
    with engine.ReconStream(engine.RC_CODEC_HEVC, 64, 64, 8, 2) as st:
        assert st.lf_tile() == 64
        for bad in (0, 8, 48, 128):
            with pytest.raises(engine.ReconError):
                st.set_lf_tile(bad)
        assert st.lf_tile() == 64
    with engine.ReconStream(engine.RC_CODEC_H264, 64, 64, 8, 2) as st:
        assert st.lf_tile() == 0
        with pytest.raises(engine.ReconError):
            st.set_lf_tile(32)


def test_pcm_bypass_transform_skip(engine, oracle):
    run_sequence(engine, oracle, 128, 64, 3, seed=5, log2_ctb=5, pcm_permille=150, pcm_loop_filter_disabled=1,
                 bypass_permille=100, transform_skip_permille=400, intra_permille=500)


def test_scaling_lists_constrained_intra_no_strong(engine, oracle):
    run_sequence(engine, oracle, 128, 96, 3, seed=6, log2_ctb=6, scaling_lists=1, constrained_intra_pred=1,
                 strong_intra_smoothing=0, intra_permille=600)


def test_weighted_bipred(engine, oracle):
    run_sequence(engine, oracle, 96, 96, 4, seed=7, log2_ctb=5, lists=2, bipred_permille=600, weighted=1)
    run_sequence(engine, oracle, 96, 64, 3, seed=8, bit_depth=10, log2_ctb=4, lists=2, bipred_permille=500,
                 weighted=1)


def test_dense_residual_and_far_motion(engine, oracle):
    run_sequence(engine, oracle, 64, 64, 3, seed=9, log2_ctb=6, zero_tu_permille=100, mv_range=300)


def test_tiny_pictures_partial_groups(engine, oracle):
    """Pictures smaller than one 16x16 inter area in a dimension, and chroma
    rows of 20 and 12 samples: every thread group at a picture edge is partial."""
    run_sequence(engine, oracle, 40, 24, 3, seed=14, log2_ctb=4)
    run_sequence(engine, oracle, 24, 40, 3, seed=15, bit_depth=10, log2_ctb=4, mv_range=40)


def test_1080p_8bit_and_10bit(engine, oracle):
    run_sequence(engine, oracle, 1920, 1080, 3, seed=10)
    run_sequence(engine, oracle, 1920, 1080, 2, seed=11, bit_depth=10)


def test_2160p_one_picture_each_depth(engine, oracle):
    run_sequence(engine, oracle, 3840, 2160, 2, seed=12)
    run_sequence(engine, oracle, 3840, 2160, 1, seed=13, bit_depth=10)


def test_largest_picture_10bit(engine, oracle):
    """The largest coded size a stream accepts, 8192 x 8192, at 10 bits: an
    intra picture, then a P picture whose inter passes list units from every
    part of the picture."""
    run_sequence(engine, oracle, 8192, 8192, 2, seed=32, bit_depth=10)


def test_deterministic(engine, oracle):
    a = run_sequence(engine, oracle, 128, 64, 3, seed=14, log2_ctb=5)
    b = run_sequence(engine, oracle, 128, 64, 3, seed=14, log2_ctb=5)
    assert a == b


def test_invalid_hevc_rejected(engine):
    with engine.ReconStream(engine.RC_CODEC_HEVC, 64, 64, 8, 2) as st:
        p = engine.SynthHevc(seed=1, width=64, height=64, log2_ctb=5, refs=[(0, 3, 1)])
        n0 = st.launches()
        with pytest.raises(engine.ReconError) as e:
            st.submit_hevc(p, 0)
        assert e.value.code == engine.RC_EINVAL
        assert st.launches() == n0
        assert st.sync() == 0
    with pytest.raises(engine.ReconError):
        engine.ReconStream(engine.RC_CODEC_HEVC, 100, 64, 8, 2)  # width not a multiple of 8


def test_benched_1080p_sequences_first_frames(engine, oracle):
    """The bench's own HEVC workloads (same generator, seed, references and
    DPB slots), the first 8 frames at 8 and 10 bit, against the oracle."""
    import importlib.util
    import pathlib
    import sys
    if "bench" not in sys.modules:
        spec = importlib.util.spec_from_file_location("bench", pathlib.Path(__file__).resolve().parent.parent / "bench.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules["bench"] = mod
        spec.loader.exec_module(mod)
    B = sys.modules["bench"]
    for name in ("hevc_1080p_8", "hevc_1080p_10"):
        wl = B.workload(engine, name)
        pics = wl.sequence(B.SEED, 8)
        st = engine.ReconStream(engine.RC_CODEC_HEVC, wl.W, wl.H, wl.bd, wl.slots)
        dpb = wl.oracle_dpb(oracle)
        try:
            for n, p in enumerate(pics):
                slot = n % wl.slots
                st.submit_hevc(p, slot)
                assert dpb.recon(p.ptr, slot, 3) == 0
                assert st.sync() == 0
                for pn, g, w in zip("YUV", st.download(slot), dpb.planes(slot)):
                    msg = first_diff(g.astype(np.uint16), w)
                    assert msg is None, f"{name} frame {n} plane {pn}: {msg}"
        finally:
            st.close()
