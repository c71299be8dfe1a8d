"""Known-answer tests of the oracle's H.264 arithmetic.

Expected values are worked out by hand from the published H.264 algorithms
the reference implements (src/h264/dec/transform.rs, inter.rs, intra.rs,
deblock.rs), so they check the restatement independently of its code."""
from __future__ import annotations

import ctypes

import numpy as np


def i32(a):
    return np.ascontiguousarray(np.array(a, dtype=np.int32))


def test_idct4_dc_and_first_ac(oracle):
    L = oracle.lib()
    dst = np.full((4, 4), 100, np.uint8)
    d = i32([64] + [0] * 15)
    L.oracle_h264_idct4_add(d.ctypes.data, dst.ctypes.data, 4)
    assert np.all(dst == 101)  # (64 + 32) >> 6 = 1 everywhere
    dst[:] = 100
    d = i32([0, 64] + [0] * 14)
    L.oracle_h264_idct4_add(d.ctypes.data, dst.ctypes.data, 4)
    # row pass [64, 32, -32, -64]; (v + 32) >> 6 -> [1, 1, 0, -1]
    assert np.all(dst == np.array([101, 101, 100, 99], np.uint8)[None, :])


def test_idct4_clips(oracle):
    L = oracle.lib()
    dst = np.full((4, 4), 250, np.uint8)
    d = i32([64 * 40] + [0] * 15)
    L.oracle_h264_idct4_add(d.ctypes.data, dst.ctypes.data, 4)
    assert np.all(dst == 255)


def test_idct8_dc(oracle):
    L = oracle.lib()
    dst = np.full((8, 8), 50, np.uint8)
    d = i32([64] + [0] * 63)
    L.oracle_h264_idct8_add(d.ctypes.data, dst.ctypes.data, 8)
    assert np.all(dst == 51)


def test_luma_dc_dequant_impulse(oracle):
    L = oracle.lib()
    c = i32([16] + [0] * 15)
    # Hadamard of an impulse is flat 16; qp 28: (16 * 256 + 2) >> 2 = 1024
    L.oracle_h264_luma_dc_dequant(c.ctypes.data, 28, 256)
    assert np.all(c == 1024)
    c = i32([16] + [0] * 15)
    # qp 42 >= 36: (16 * 256) << (42 / 6 - 6) = 8192
    L.oracle_h264_luma_dc_dequant(c.ctypes.data, 42, 256)
    assert np.all(c == 8192)


def test_chroma_dc_dequant(oracle):
    L = oracle.lib()
    c = i32([4, 0, 0, 0])
    # ((4 * 160) << 5) >> 5 = 640
    L.oracle_h264_chroma_dc_dequant(c.ctypes.data, 30, 160)
    assert np.all(c == 640)
    c = i32([1, 1, 0, 0])
    # f = [2, 0, 2, 0]; qp 12: ((2 * 100) << 2) >> 5 = 25
    L.oracle_h264_chroma_dc_dequant(c.ctypes.data, 12, 100)
    assert list(c) == [25, 0, 25, 0]


def test_level_scale_flat(oracle):
    L = oracle.lib()
    ls4 = np.zeros((6, 6, 16), np.int32)
    ls8 = np.zeros((6, 6, 64), np.int32)
    L.oracle_h264_level_scale(None, None, ls4.ctypes.data, ls8.ctypes.data)
    assert ls4[0, 0, 0] == 160 and ls4[0, 0, 5] == 256 and ls4[0, 0, 1] == 208
    assert ls8[1, 5, 0] == 16 * 36 and ls8[1, 5, 9] == 16 * 32


def test_mc_luma_constant_and_ramp(oracle):
    L = oracle.lib()
    W, H = 32, 32
    plane = np.full((H, W), 77, np.uint8)
    out = np.zeros((4, 4), np.uint8)
    for mvx in range(4):
        for mvy in range(4):
            L.oracle_h264_mc_luma(plane.ctypes.data, W, H, 8, 8, mvx, mvy, 4, 4, out.ctypes.data, 4)
            assert np.all(out == 77)
    ramp = np.tile(np.arange(W, dtype=np.uint8) * 4, (H, 1))
    # half-pel of a ramp 4x: tap6 = 32 * 4x + 64 -> (128x + 64 + 16) >> 5 = 4x + 2
    L.oracle_h264_mc_luma(ramp.ctypes.data, W, H, 8, 8, 2, 0, 4, 4, out.ctypes.data, 4)
    assert np.all(out == (np.arange(8, 12) * 4 + 2)[None, :])
    # quarter-pel: avg(4x, 4x + 2) = 4x + 1
    L.oracle_h264_mc_luma(ramp.ctypes.data, W, H, 8, 8, 1, 0, 4, 4, out.ctypes.data, 4)
    assert np.all(out == (np.arange(8, 12) * 4 + 1)[None, :])


def test_mc_edge_extension(oracle):
    L = oracle.lib()
    W, H = 16, 16
    plane = np.zeros((H, W), np.uint8)
    plane[0, 0] = 200
    out = np.zeros((4, 4), np.uint8)
    # a full-pel vector far above-left of the picture reads the clamped corner
    L.oracle_h264_mc_luma(plane.ctypes.data, W, H, 0, 0, -4 * 40, -4 * 40, 4, 4, out.ctypes.data, 4)
    assert np.all(out == 200)
    cplane = np.zeros((8, 8), np.uint8)
    cplane[7, 7] = 90
    L.oracle_h264_mc_chroma(cplane.ctypes.data, 8, 8, 6, 6, 8 * 30, 8 * 30, 2, 2, out.ctypes.data, 4)
    assert np.all(out[:2, :2] == 90)


def test_mc_chroma_bilinear(oracle):
    L = oracle.lib()
    W = 16
    ramp = np.tile(np.arange(W, dtype=np.uint8) * 8, (8, 1))
    out = np.zeros((2, 2), np.uint8)
    # fx = 4: (32 * 8x + 32 * 8(x + 1) + 32) >> 6 = 8x + 4
    L.oracle_h264_mc_chroma(ramp.ctypes.data, W, 8, 4, 2, 4, 0, 2, 2, out.ctypes.data, 2)
    assert np.all(out == (np.arange(4, 6) * 8 + 4)[None, :])


def _i16_picture(engine, levels_per_mb):
    """A 2x1-MB intra picture of Intra16x16 DC macroblocks whose luma DC
    levels are all in the first (DC) coefficient."""
    n = len(levels_per_mb)
    mbs = (engine.H264Mb * n)()
    lv = []
    for i, L in enumerate(levels_per_mb):
        m = mbs[i]
        m.kind = engine.RC_H264_I16x16
        m.qp = 28
        m.qpc[0] = m.qpc[1] = 28
        m.i16_mode = 2
        m.chroma_mode = 0
        m.dc_coded = 1
        m.coef_off = len(lv)
        for b in range(4):
            m.ref_idx[0][b] = m.ref_idx[1][b] = -1
            m.wp[b] = 0xFF
        lv += [L] + [0] * 15
    sl = engine.H264Slice()
    bufs = {"mbs": bytes(mbs), "slices": bytes(sl), "weights": b"",
            "levels": np.array(lv, np.int16).tobytes(), "scaling4": b"", "scaling8": b""}
    return engine.PictureBuffers(bufs, 1, 0)


def test_intra16_dc_residual_and_strong_edge(engine, oracle):
    # MB0: DC pred 128, DC level -28 -> every 4x4 DC = 64 * -28 -> residual -28 -> 100.
    # MB1: DC pred from its left neighbour = 100, level 10 -> 110.
    # Loop filter at the MB edge (bS 4, qp 28: alpha 20, beta 6; |p0 - q0| = 10
    # is not < (20 >> 2) + 2, so the weak bS-4 form): p0 = (2*100+100+110+2)>>2
    # = 103, q0 = (2*110+110+100+2)>>2 = 108.  Flat areas stay flat.
    pb = _i16_picture(engine, [-28, 10])
    dpb = oracle.H264Dpb(2, 1, 1)
    assert dpb.recon(pb.ptr, 0, filter=False) == 0
    y, u, v = dpb.planes(0)
    assert np.all(y[:, :16] == 100) and np.all(y[:, 16:] == 110)
    assert np.all(u == 128) and np.all(v == 128)
    dpb = oracle.H264Dpb(2, 1, 1)
    assert dpb.recon(pb.ptr, 0, filter=True) == 0
    y, _, _ = dpb.planes(0)
    expect = np.array([100] * 15 + [103, 108] + [110] * 15, np.uint8)
    assert np.all(y == expect[None, :])


def test_filter_is_recon_then_deblock(engine, oracle):
    d1 = oracle.H264Dpb(8, 6, 4)
    d2 = oracle.H264Dpb(8, 6, 4)
    for n, seed in enumerate((11, 12, 13)):
        refs = [(0, n - k, n - k) for k in (1, 2) if n - k >= 0]
        p = engine.SynthH264(seed=seed, mb_w=8, mb_h=6, intra_only=int(n == 0), refs=refs, pcm_permille=50)
        slot = n
        assert d1.recon(p.ptr, slot) == 0
        assert d2.recon(p.ptr, slot, filter=False) == 0
        y, u, v = d2.planes(slot)
        oracle.lib().oracle_h264_deblock(8, 6, p.ptr, y.ctypes.data, u.ctypes.data, v.ctypes.data)
        for a, b in zip(d1.planes(slot), d2.planes(slot)):
            assert np.array_equal(a, b)
