"""End-to-end parity against the reference's golden H.264 streams.

tests/golden/h264_<name>.npz holds the syntax records of the reference's x264
stream tests/refs/h264/<name>.h264 (made by tests/golden/make_h264_golden.py:
h264_cavlc.py parses the Baseline stream, h264_cabac.py the Main and High
ones), with each picture's DPB slot, picture order count and crop.  EXPECTED
below is the sha256 the reference's manifest records for the stream's
reconstruction (tests/refs/h264/manifest.toml, the "<name>.yuv" entry, kind
bit-exact: the reconstruction x264 dumped while encoding).  The digest
covers the pictures in output order, each cropped, Y then Cb then Cr row by
row (src/testref.rs:570-578).  The oracle (CPU) and the engine (GPU, through
the C ABI) must both reproduce it.

  baseline          Baseline, CAVLC, 2 slices, I and P with 3 references
  main_cabac_b      Main, CABAC, B pictures (spatial direct, implicit
                    weights), explicit P weights with duplicated references
  high_bpyramid     High, 8x8 transform and I8x8, B pyramid, temporal
                    direct, explicit weights, 4 references
  high_crop_slices  High, JVT scaling matrices (PPS, fall-back rule A), 4
                    slices, B pictures, 238x158 cropped from 240x160

Every fixture also holds each picture's motion syntax (partitions, parsed
ref_idx and mvd, direct modes, per-slice direct and weight tables); the
"derived" cases reconstruct from it, the vectors derived by the oracle (CPU)
or by the engine's h264_mv_kernel (GPU).
"""
from __future__ import annotations

import hashlib
import json
import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
EXPECTED = {
    "baseline": "5a978004cf205415f059349e9fa14714e1d7578b1c5165c48520fca71a11ef00",
    "main_cabac_b": "9f7179ab822f155adc7cbe0586f3d7447cf78f3863cb720335cbf927cc5b33a7",
    "high_bpyramid": "25379e94ff635e93d66808405de5fbbad27595ab1b32e3ea6e7b0259ea92b21e",
    "high_crop_slices": "6da5d2d112e7128e7a88af29d226fc4c300a95c4b795f0d0162ee9053fb901fc",
}
KEYS = ("mbs", "slices", "weights", "levels", "scaling4", "scaling8")
MOTION_KEYS = ("motion", "slice_motion")
DPB_SLOTS = 16


def load_fixture(engine, name, motion=False):
    """The fixture's pictures; motion=True attaches the motion syntax, so
    that the oracle and the engine derive every vector themselves."""
    z = np.load(GOLDEN / f"h264_{name}.npz")
    meta = json.loads(bytes(z["meta"]).decode())
    pics = []
    for i, m in enumerate(meta["pictures"]):
        bufs = {k: z[f"{k}_{i}"].tobytes() for k in KEYS + (MOTION_KEYS if motion else ())}
        pics.append((m, engine.PictureBuffers(bufs, m["num_slices"], m["num_weights"], m["constrained_intra"],
                                              m["frame_id"])))
    return meta, pics


def cropped(planes, crop):
    y, u, v = planes
    l, r, t, b = crop
    H, W = y.shape
    out = [y[2 * t:H - 2 * b, 2 * l:W - 2 * r]]
    out += [c[t:H // 2 - b, l:W // 2 - r] for c in (u, v)]
    return [np.ascontiguousarray(p) for p in out]


def output_digest(metas, planes_after) -> str:
    outs = {}
    for i, m in enumerate(metas):
        outs[(m["period"], m["poc"])] = [np.array(p, copy=True) for p in planes_after(i)]
    h = hashlib.sha256()
    for k in sorted(outs):
        for pl in outs[k]:
            h.update(pl.tobytes())
    return h.hexdigest()


def test_every_fixture_is_a_reference_stream():
    assert sorted(p.stem[5:] for p in GOLDEN.glob("h264_*.npz")) == sorted(EXPECTED)
    for name, want in EXPECTED.items():
        z = np.load(GOLDEN / f"h264_{name}.npz")
        meta = json.loads(bytes(z["meta"]).decode())
        assert meta["expected_sha256"] == want and meta["stream"] == f"tests/refs/h264/{name}.h264"


@pytest.mark.parametrize("motion", [False, True], ids=["resolved", "derived"])
@pytest.mark.parametrize("name", sorted(EXPECTED))
def test_oracle_reproduces_reference_digest(engine, oracle, name, motion):
    """Resolved: the records' own vectors.  Derived: the vectors the oracle
    derives from the motion syntax (MV prediction, P_Skip, B direct spatial
    and temporal from the co-located picture, weight entries)."""
    meta, pics = load_fixture(engine, name, motion)
    m0 = meta["pictures"][0]
    dpb = oracle.H264Dpb(m0["mb_w"], m0["mb_h"], DPB_SLOTS)

    def planes_after(i):
        m, p = pics[i]
        assert dpb.recon(p.ptr, m["slot"]) == 0
        return cropped(dpb.planes(m["slot"]), m["crop"])

    assert output_digest([m for m, _ in pics], planes_after) == EXPECTED[name]


@pytest.mark.gpu
@pytest.mark.parametrize("motion", [False, True], ids=["resolved", "derived"])
@pytest.mark.parametrize("name", sorted(EXPECTED))
def test_engine_reproduces_reference_digest(engine, name, motion):
    """Derived: the engine derives every vector on the GPU (h264_mv_kernel)
    from the motion syntax."""
    meta, pics = load_fixture(engine, name, motion)
    m0 = meta["pictures"][0]
    W, H = m0["mb_w"] * 16, m0["mb_h"] * 16
    with engine.ReconStream(engine.RC_CODEC_H264, W, H, 8, DPB_SLOTS) as st:
        def planes_after(i):
            m, p = pics[i]
            st.submit_h264(p, m["slot"])
            assert st.sync() == 0
            return cropped(st.download(m["slot"]), m["crop"])

        assert output_digest([m for m, _ in pics], planes_after) == EXPECTED[name]


@pytest.mark.gpu
@pytest.mark.parametrize("motion", [False, True], ids=["resolved", "derived"])
@pytest.mark.parametrize("group", [2, 4])
@pytest.mark.parametrize("name", sorted(EXPECTED))
def test_engine_grouped_reproduces_reference_digest(engine, name, group, motion):
    """The same streams with several pictures per launch
    (rc_stream_set_h264_group): pictures are submitted in runs of distinct
    DPB slots without waiting, and read back after each run."""
    meta, pics = load_fixture(engine, name, motion)
    metas = [m for m, _ in pics]
    m0 = metas[0]
    W, H = m0["mb_w"] * 16, m0["mb_h"] * 16
    planes = {}
    with engine.ReconStream(engine.RC_CODEC_H264, W, H, 8, DPB_SLOTS) as st:
        assert st.set_h264_group(group) == group
        i = 0
        while i < len(pics):
            run = []
            while i < len(pics) and metas[i]["slot"] not in [metas[j]["slot"] for j in run]:
                st.submit_h264(pics[i][1], metas[i]["slot"])
                run.append(i)
                i += 1
            for j in run:
                planes[j] = cropped(st.download(metas[j]["slot"]), metas[j]["crop"])
        assert st.sync() == 0
    assert output_digest(metas, lambda j: planes[j]) == EXPECTED[name]


def _motion_picture(engine, name, i):
    """Picture i of a fixture with its motion syntax, and its buffers."""
    z = np.load(GOLDEN / f"h264_{name}.npz")
    meta = json.loads(bytes(z["meta"]).decode())
    m = meta["pictures"][i]
    bufs = {k: bytearray(z[f"{k}_{i}"].tobytes()) for k in KEYS + MOTION_KEYS}
    return m, bufs


def test_validate_rejects_bad_motion_syntax(engine):
    """rc_h264_validate checks motion syntax like the kernel would: shapes,
    sub-partitions, prediction lists, ref_idx within the lists, direct modes
    only in B slices, weight entries that exist."""
    import ctypes
    L = engine.lib()
    # a P picture of the Baseline stream (list 0 only)
    m, bufs = _motion_picture(engine, "baseline", 1)
    mb_w, mb_h, n = m["mb_w"], m["mb_h"], m["mb_w"] * m["mb_h"]

    def check(mutate):
        b = {k: bytearray(v) for k, v in bufs.items()}
        mos = (engine.H264Motion * n).from_buffer(b["motion"])
        recs = (engine.H264Mb * n).from_buffer(b["mbs"])
        sms = (engine.H264SliceMotion * m["num_slices"]).from_buffer(b["slice_motion"])
        mutate(mos, recs, sms)
        pb = engine.PictureBuffers({k: bytes(v) for k, v in b.items()}, m["num_slices"], m["num_weights"],
                                   m["constrained_intra"], m["frame_id"])
        return L.rc_h264_validate(mb_w, mb_h, DPB_SLOTS, pb.ptr)

    inter = [a for a in range(n) if (engine.H264Mb * n).from_buffer(bufs["mbs"])[a].kind == engine.RC_H264_INTER]
    part = [a for a in inter if (engine.H264Motion * n).from_buffer(bufs["motion"])[a].shape
            == engine.RC_H264_MOTION_16x16]
    assert check(lambda mo, r, sm: None) == 0
    a, q = inter[0], part[0]

    def shape_mismatch(mo, r, sm):
        mo[a].shape = engine.RC_H264_MOTION_NONE

    def bad_shape(mo, r, sm):
        mo[a].shape = 9

    def ref_past_list(mo, r, sm):
        mo[q].ref_idx[0][0] = 31

    def list1_in_p(mo, r, sm):
        mo[q].pred[0] = 2

    def direct_in_p(mo, r, sm):
        mo[q].shape = engine.RC_H264_MOTION_8x8
        for i in range(4):
            mo[q].sub[i], mo[q].pred[i], mo[q].ref_idx[0][i] = engine.RC_H264_SUB_DIRECT, 0, 0

    def bad_weight(mo, r, sm):
        sm[0].wp_map[1 * 33 + 0] = 7  # (ref0 0, list 1 unused) -> an entry that does not exist

    for fn in (shape_mismatch, bad_shape, ref_past_list, list1_in_p, direct_in_p, bad_weight):
        assert check(fn) == engine.RC_EINVAL, fn.__name__


@pytest.mark.gpu
def test_engine_rejects_b_picture_without_stored_colocated_motion(engine):
    """A B slice's co-located picture must have been submitted with motion
    syntax (its stored motion is what direct prediction reads)."""
    meta, pics = load_fixture(engine, "main_cabac_b", motion=True)
    _, plain = load_fixture(engine, "main_cabac_b", motion=False)
    metas = [m for m, _ in pics]
    m0 = metas[0]
    b = next(i for i, (m, p) in enumerate(pics)
             if any((engine.H264SliceMotion * m["num_slices"]).from_address(p.pic.slice_motion)[j].b_slice
                    for j in range(m["num_slices"])))
    with engine.ReconStream(engine.RC_CODEC_H264, m0["mb_w"] * 16, m0["mb_h"] * 16, 8, DPB_SLOTS) as st:
        # every earlier picture with resolved motion only: no stored motion
        for i in range(b):
            st.submit_h264(plain[i][1], metas[i]["slot"])
        with pytest.raises(engine.ReconError):
            st.submit_h264(pics[b][1], metas[b]["slot"])
        # with motion syntax, the same pictures are accepted
        for i in range(b + 1):
            st.submit_h264(pics[i][1], metas[i]["slot"])
        assert st.sync() == 0
