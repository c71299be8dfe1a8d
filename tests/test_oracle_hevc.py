"""Known-answer tests of the oracle's HEVC arithmetic.

Expected values are worked out by hand from the published HEVC algorithms
the reference implements (src/hevc/transform.rs, intra.rs); picture-level
tests check properties of the restatement (stage consistency, determinism,
validation)."""
from __future__ import annotations

import ctypes

import numpy as np


def i16(a):
    return np.ascontiguousarray(np.array(a, dtype=np.int16))


def test_inverse_dc_hand_values(oracle):
    L = oracle.lib()
    # dc 64, 8-bit (bd_shift 12): e = (64*64+64)>>7 = 32; (64*32 + 2048) >> 12 = 1
    assert L.oracle_hevc_inverse_dc(64, 12) == 1
    # 10-bit (bd_shift 10): (2048 + 512) >> 10 = 2
    assert L.oracle_hevc_inverse_dc(64, 10) == 2
    assert L.oracle_hevc_inverse_dc(-64, 12) == 0  # (64*-32 + 2048) >> 12 = 0


def test_dc_only_equals_full_transform(oracle):
    L = oracle.lib()
    for log2 in (3, 4, 5):
        n = 1 << log2
        for dc in (-300, -64, 1, 64, 1000):
            co = np.zeros(n * n, np.int16)
            co[0] = dc
            L.oracle_hevc_inverse(co.ctypes.data, log2, 0, 0, 0, 12)
            assert np.all(co == L.oracle_hevc_inverse_dc(dc, 12))


def test_dst_4x4_impulse(oracle):
    L = oracle.lib()
    co = np.zeros(16, np.int16)
    co[0] = 64
    L.oracle_hevc_inverse(co.ctypes.data, 2, 1, 0, 0, 12)
    r = co.reshape(4, 4)
    # column pass [15, 28, 37, 42]; row y=3: (2048 + 42*[29,55,74,84]) >> 12 = [0,1,1,1]
    assert list(r[3]) == [0, 1, 1, 1]
    assert list(r[0]) == [0, 0, 0, 0]


def test_inverse_linear_in_dc_sign(oracle):
    L = oracle.lib()
    a = np.zeros(64, np.int16)
    a[1] = 200
    b = a.copy()
    b[1] = -200
    L.oracle_hevc_inverse(a.ctypes.data, 3, 0, 1, 0, 12)
    L.oracle_hevc_inverse(b.ctypes.data, 3, 0, 1, 0, 12)
    # first horizontal basis function is odd-symmetric across the block
    assert np.array_equal(a.reshape(8, 8)[:, ::-1], b.reshape(8, 8))


def _refs(left, top):
    l = np.zeros(129, np.uint16)
    t = np.zeros(129, np.uint16)
    l[:len(left)] = left
    t[:len(top)] = top
    return l, t


def test_intra_dc_and_planar_flat(oracle):
    L = oracle.lib()
    for mode in (0, 1):
        l, t = _refs([100] * 17, [100] * 17)
        out = np.zeros(64, np.int32)
        L.oracle_hevc_intra_predict_refs(l.ctypes.data, t.ctypes.data, mode, 3, 1, 1, 8, out.ctypes.data)
        assert np.all(out == 100)


def test_intra_vertical_edge_filter(oracle):
    L = oracle.lib()
    # mode 26 (vertical) copies the top row; luma n<32 adjusts column 0 by
    # (left[1+y] - corner) >> 1
    left = [50] + [60] * 16
    top = [50] + list(range(100, 116))
    l, t = _refs(left, top)
    out = np.zeros(64, np.int32)
    L.oracle_hevc_intra_predict_refs(l.ctypes.data, t.ctypes.data, 26, 3, 1, 1, 8, out.ctypes.data)
    o = out.reshape(8, 8)
    assert np.all(o[:, 1:] == np.arange(101, 108)[None, :])
    assert np.all(o[:, 0] == 100 + (60 - 50) // 2)


def test_intra_pure_diagonal(oracle):
    L = oracle.lib()
    # mode 34 (angle 32): sample (x, y) = top[x + y + 2]
    top = [0] + list(range(10, 26))
    l, t = _refs([0] * 17, top)
    out = np.zeros(16, np.int32)
    L.oracle_hevc_intra_predict_refs(l.ctypes.data, t.ctypes.data, 34, 2, 0, 0, 8, out.ctypes.data)
    o = out.reshape(4, 4)
    for y in range(4):
        for x in range(4):
            assert o[y, x] == top[x + y + 2]


def _run(engine, oracle, stages, **kw):
    p = engine.SynthHevc(**kw)
    d = oracle.HevcDpb(kw["width"], kw["height"], kw.get("bit_depth", 8), 2)
    assert d.recon(p.ptr, 0, stages) == 0
    return p, d.planes(0)


def test_hevc_oracle_deterministic_and_staged(engine, oracle):
    kw = dict(seed=3, width=128, height=72, log2_ctb=5, intra_only=1)
    _, a = _run(engine, oracle, 3, **kw)
    _, b = _run(engine, oracle, 3, **kw)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # SAO and deblocking change something on a dense picture; recon alone is stable
    _, r0 = _run(engine, oracle, 0, **kw)
    _, r1 = _run(engine, oracle, 1, **kw)
    assert not all(np.array_equal(x, y) for x, y in zip(r0, r1))
    assert not all(np.array_equal(x, y) for x, y in zip(r1, a))


def test_hevc_validate(engine):
    L = engine.lib()
    p = engine.SynthHevc(seed=5, width=64, height=64, log2_ctb=5, refs=[(0, 1, 1)])
    assert L.rc_hevc_validate(64, 64, 8, 2, p.ptr) == 0
    assert L.rc_hevc_validate(64, 64, 8, 1, p.ptr) == engine.RC_EINVAL  # ref slot 1 outside
    assert L.rc_hevc_validate(64, 60, 8, 2, p.ptr) == engine.RC_EINVAL  # height not a multiple of 8
    bufs = p.buffers()
    tus = np.frombuffer(bufs["tus"], np.uint8).copy().reshape(-1, 16)
    tus[0, engine.HevcTu.log2.offset] = 6
    keep = ctypes.create_string_buffer(tus.tobytes(), len(tus.tobytes()))
    pic = engine.HevcPicture.from_buffer_copy(bytes(engine.HevcPicture.from_address(p.ptr)))
    pic.tus = ctypes.addressof(keep)
    assert L.rc_hevc_validate(64, 64, 8, 2, ctypes.addressof(pic)) == engine.RC_EINVAL


# record flags of include/pito_recon.h
TU_CBF, TU_BYPASS, TU_PCM = 2, 8, 16
F_INTRA, F_CODED = 1, 16


def test_hevc_validate_each_check(engine):
    """Every host-side check of rc_hevc_validate rejects its bad field, and
    the limits themselves (QP 51, a block ending on the picture edge, levels
    ending on the last one) are accepted."""
    L = engine.lib()
    W = H = 64
    p = engine.SynthHevc(seed=21, width=W, height=H, log2_ctb=5, refs=[(0, 1, 1)], intra_permille=300)
    base = engine.HevcPicture.from_buffer_copy(bytes(engine.HevcPicture.from_address(p.ptr)))
    bufs = p.buffers()
    keep = []

    def arr(key, cls):
        return np.frombuffer(bufs[key], dtype=np.dtype(cls)).copy()

    def check(**recs):
        pic = engine.HevcPicture.from_buffer_copy(bytes(base))
        for key, a in recs.items():
            b = ctypes.create_string_buffer(a.tobytes(), a.nbytes)
            keep.append(b)
            setattr(pic, key, ctypes.addressof(b))
        return L.rc_hevc_validate(W, H, 8, 2, ctypes.addressof(pic))

    tus, blk, mvf, ctbs = arr("tus", engine.HevcTu), arr("blk", engine.HevcBlk), arr("mvf", engine.HevcMvf), arr(
        "ctbs", engine.HevcCtb)
    assert check() == 0
    nlev = base.num_levels
    luma = int(np.flatnonzero((tus["c"] == 0) & ((tus["flags"] & (TU_CBF | TU_BYPASS | TU_PCM)) == TU_CBF))[0])
    n = 1 << int(tus[luma]["log2"])

    def tu(field, value, i=luma, flags=None):
        t = tus.copy()
        t[i][field] = value
        if flags is not None:
            t[i]["flags"] = flags
        return check(tus=t)

    for field, value in (("log2", 1), ("log2", 6), ("c", 3), ("mode", 35), ("x0", W - n + 4), ("y0", H - n + 4),
                         ("max_x", n), ("max_y", n), ("qp", -1), ("qp", 52), ("coef_off", nlev)):
        assert tu(field, value) == engine.RC_EINVAL, (field, value)
    for field, value in (("x0", W - n), ("y0", H - n), ("qp", 51), ("qp", 0)):
        assert tu(field, value) == 0, (field, value)
    # transquant bypass: the QP is not used
    assert tu("qp", 60, flags=TU_CBF | TU_BYPASS) == 0
    # PCM: n x n levels from coef_off, the last one included
    assert tu("coef_off", nlev - n * n, flags=TU_PCM) == 0
    assert tu("coef_off", nlev - n * n + 1, flags=TU_PCM) == engine.RC_EINVAL
    # no coefficients: the level range is not read
    assert tu("coef_off", nlev + 1000, flags=0) == 0

    inter = int(np.flatnonzero((blk["flags"] & (F_CODED | F_INTRA)) == F_CODED)[0])
    intra = int(np.flatnonzero((blk["flags"] & (F_CODED | F_INTRA)) == (F_CODED | F_INTRA))[0])

    def blk_qp(i, qp):
        b = blk.copy()
        b[i]["qp"] = qp
        return check(blk=b)

    assert blk_qp(inter, 52) == engine.RC_EINVAL and blk_qp(intra, -1) == engine.RC_EINVAL
    assert blk_qp(inter, 51) == 0 and blk_qp(intra, 0) == 0

    def refs(i, r0, r1):
        m = mvf.copy()
        m[i]["ref_idx"][0], m[i]["ref_idx"][1] = r0, r1
        return check(mvf=m)

    for r0, r1 in ((1, -1), (-1, -1), (-2, 0), (0, -2), (0, 0)):  # one reference in list 0, none in list 1
        assert refs(inter, r0, r1) == engine.RC_EINVAL, (r0, r1)
    assert refs(inter, 0, -1) == 0
    assert refs(intra, 5, 5) == 0  # an intra block's motion field is not read
    c = ctbs.copy()
    c[len(c) - 1]["slice"] = base.num_slices
    assert check(ctbs=c) == engine.RC_EINVAL


def test_hevc_validate_large_picture_in_pieces(engine):
    """A 2160p picture is validated in pieces on host threads: a bad record in
    the last piece of block rows or of transform blocks is still found, also
    while other threads validate at the same time."""
    import threading
    L = engine.lib()
    W, H = 3840, 2160
    p = engine.SynthHevc(seed=22, width=W, height=H, bit_depth=10, refs=[(0, 1, 1)], frame_id=1)
    base = engine.HevcPicture.from_buffer_copy(bytes(engine.HevcPicture.from_address(p.ptr)))
    bufs = p.buffers()
    blk = np.frombuffer(bufs["blk"], dtype=np.dtype(engine.HevcBlk)).copy()
    tus = np.frombuffer(bufs["tus"], dtype=np.dtype(engine.HevcTu)).copy()
    blk[-1]["qp"] = 70
    tus[-1]["mode"] = 40
    keep = []

    def pic_with(key, a):
        pic = engine.HevcPicture.from_buffer_copy(bytes(base))
        b = ctypes.create_string_buffer(a.tobytes(), a.nbytes)
        keep.append((pic, b))
        setattr(pic, key, ctypes.addressof(b))
        return ctypes.addressof(pic)

    cases = [(p.ptr, 0), (pic_with("blk", blk), engine.RC_EINVAL), (pic_with("tus", tus), engine.RC_EINVAL)]
    for ptr, want in cases:
        assert L.rc_hevc_validate(W, H, 10, 2, ptr) == want
    errors = []

    def worker(k):
        for j in range(6):
            ptr, want = cases[(k + j) % 3]
            got = L.rc_hevc_validate(W, H, 10, 2, ptr)
            if got != want:
                errors.append((k, j, got, want))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
