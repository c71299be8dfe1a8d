"""Output order of decoded pictures: the DPB bumping process (rc_output_*).

Host-only (no GPU).  Unit cases for each bumping condition -- the reorder
limit, the latency limit, the DPB capacity with references still held, a
new coded video sequence with and without no_output_of_prior_pics -- and,
for every golden HEVC stream of the reference, the output order the process
gives with the stream's own SPS limits (max_dec_pic_buffering,
max_num_reorder_pics, max latency) and reference marking, which must be the
order of the reference's digest: picture order count within each coded
video sequence (src/syntax/hevc/dpb.rs:76-160)."""
from __future__ import annotations

import ctypes
import json
import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


def test_reorder_zero_outputs_each_picture_at_once(engine):
    d = engine.OutputOrder(capacity=4, max_num_reorder=0)
    assert d.begin(new_sequence=True) == []
    for i, poc in enumerate([0, 1, 2, 3]):
        assert d.begin() == []
        assert d.insert(i, poc) == [i]
    assert d.flush() == []


def test_reorder_limit_bumps_smallest_poc(engine):
    # a three-level B pyramid in decoding order (POC 0, 8, 4, 2, 1, 3, 6, 5,
    # 7): up to three pictures wait ahead of the one being output
    d = engine.OutputOrder(capacity=8, max_num_reorder=3)
    order = [0, 8, 4, 2, 1, 3, 6, 5, 7]
    out = []
    for i, poc in enumerate(order):
        out += d.begin(new_sequence=i == 0)
        out += d.insert(poc, poc, reference=False)  # only the reorder limit bumps
    out += d.flush()
    assert out == sorted(order)
    # with two pictures allowed to wait, POC 0 leaves when the third arrives
    d = engine.OutputOrder(capacity=8, max_num_reorder=2)
    d.begin(new_sequence=True)
    assert d.insert(0, 0) == [] and d.insert(8, 8) == [] and d.insert(4, 4) == [0]


def test_latency_limit(engine):
    d = engine.OutputOrder(capacity=8, max_num_reorder=8, max_latency_pictures=2)
    d.begin(new_sequence=True)
    assert d.insert(10, 10) == []
    assert d.insert(20, 20) == []
    # POC 10 has now waited through two later pictures
    assert d.insert(30, 30) == [10]


def test_capacity_with_references_held(engine):
    d = engine.OutputOrder(capacity=2, max_num_reorder=8)
    d.begin(new_sequence=True)
    assert d.insert(1, 0, reference=True) == []
    assert d.begin() == []
    assert d.insert(2, 1, reference=True) == []
    # full: the next picture's start bumps while the DPB stays full; both
    # pictures are still references, so both are output and both stay
    assert d.begin() == [1, 2]
    assert d.count() == 2
    d.unref(1)
    assert d.count() == 1
    assert d.insert(3, 2, reference=False) == []
    # full again (the reference and the waiting picture): POC 2 is bumped
    assert d.begin() == [3]
    assert d.flush() == [] and d.count() == 0


def test_new_sequence_outputs_or_drops_prior_pictures(engine):
    d = engine.OutputOrder(capacity=8, max_num_reorder=8)
    d.begin(new_sequence=True)
    d.insert(1, 4)
    d.insert(2, 2)
    assert d.begin(new_sequence=True) == [2, 1]
    d.insert(3, 0)
    d.insert(4, 8)
    assert d.begin(new_sequence=True, no_output_of_prior_pics=True) == []
    assert d.count() == 0


def test_output_flag_off_and_room_checked(engine):
    d = engine.OutputOrder(capacity=4, max_num_reorder=0)
    d.begin(new_sequence=True)
    assert d.insert(7, 0, output=False) == []
    L = engine.lib()
    n = ctypes.c_int()
    assert L.rc_output_insert(d._h, 8, 1, 1, 1, None, 0, ctypes.byref(n)) == engine.RC_EINVAL
    assert d.count() == 1  # nothing changed
    assert d.insert(8, 1) == [8]
    with pytest.raises(engine.ReconError):
        engine.OutputOrder(capacity=0, max_num_reorder=0)


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("hevc_*.npz")), ids=lambda p: p.stem)
def test_golden_hevc_output_order(engine, path):
    meta = json.loads(bytes(np.load(path)["meta"]).decode())
    pics = meta["pictures"]
    cap, reorder, latency = pics[0]["dpb"]
    d = engine.OutputOrder(capacity=cap, max_num_reorder=reorder, max_latency_pictures=latency)
    out = []
    for m in pics:
        for u in m["unref"]:
            d.unref(u)
        out += d.begin(new_sequence=m["new_sequence"], no_output_of_prior_pics=m["no_output_of_prior_pics"])
        out += d.insert(m["frame_id"], m["poc"], output=m["output"], reference=True)
        assert d.count() <= cap
    out += d.flush()
    want = [m["frame_id"] for m in sorted((m for m in pics if m["output"]), key=lambda m: (m["cvs"], m["poc"]))]
    assert out == want
