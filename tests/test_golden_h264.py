"""End-to-end parity against the reference's golden H.264 stream.

tests/golden/h264_baseline.npz holds the syntax records of the reference's
tests/refs/h264/baseline.h264 (x264 Baseline, 10 frames, 2 slices per
picture, I and P with 3 reference frames, deblocking on), parsed by
tests/golden/h264_cavlc.py, and the sha256 the reference's manifest records
for the stream's reconstruction (tests/refs/h264/manifest.toml, kind
bit-exact; digest of every frame's cropped Y, Cb, Cr rows as in
src/testref.rs:570-578).  The oracle and the engine must both reproduce it.
"""
from __future__ import annotations

import hashlib
import json
import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "h264_baseline.npz"


def load_fixture(engine):
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    pics = []
    for i, m in enumerate(meta["pictures"]):
        bufs = {k: z[f"{k}_{i}"].tobytes() for k in ("mbs", "slices", "levels")}
        bufs["weights"] = b""
        pics.append((m, engine.PictureBuffers(bufs, m["num_slices"], 0, m["constrained_intra"], m["frame_id"])))
    return meta, pics


def cropped(planes, crop):
    y, u, v = planes
    l, r, t, b = crop
    H, W = y.shape
    out = [y[2 * t:H - 2 * b, 2 * l:W - 2 * r]]
    out += [c[t:H // 2 - b, l:W // 2 - r] for c in (u, v)]
    return [np.ascontiguousarray(p) for p in out]


def test_fixture_is_the_reference_stream(engine):
    meta, pics = load_fixture(engine)
    assert len(pics) == 10
    assert meta["expected_sha256"] == "5a978004cf205415f059349e9fa14714e1d7578b1c5165c48520fca71a11ef00"


def test_oracle_reproduces_reference_digest(engine, oracle):
    meta, pics = load_fixture(engine)
    m0 = meta["pictures"][0]
    dpb = oracle.H264Dpb(m0["mb_w"], m0["mb_h"], 8)
    h = hashlib.sha256()
    for m, p in pics:
        assert dpb.recon(p.ptr, m["slot"]) == 0
        for plane in cropped(dpb.planes(m["slot"]), m["crop"]):
            h.update(plane.tobytes())
    assert h.hexdigest() == meta["expected_sha256"]


@pytest.mark.gpu
def test_engine_reproduces_reference_digest(engine):
    meta, pics = load_fixture(engine)
    m0 = meta["pictures"][0]
    W, H = m0["mb_w"] * 16, m0["mb_h"] * 16
    h = hashlib.sha256()
    with engine.ReconStream(engine.RC_CODEC_H264, W, H, 8, 8) as st:
        for m, p in pics:
            st.submit_h264(p, m["slot"])
            assert st.sync() == 0
            for plane in cropped(st.download(m["slot"]), m["crop"]):
                h.update(plane.tobytes())
    assert h.hexdigest() == meta["expected_sha256"]
