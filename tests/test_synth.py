"""The synthetic syntax generator: seeded determinism and the workload's
statistics (intra share, weighted-prediction share, zero blocks, QP range)."""
from __future__ import annotations

import hashlib

import numpy as np


def digest(pic) -> str:
    h = hashlib.sha256()
    for k, v in sorted(pic.buffers().items()):
        h.update(k.encode())
        h.update(v)
    return h.hexdigest()


def test_same_seed_same_records(engine):
    a = engine.SynthH264(seed=42, mb_w=20, mb_h=12, refs=[(0, 1, 1), (0, 2, 2)])
    b = engine.SynthH264(seed=42, mb_w=20, mb_h=12, refs=[(0, 1, 1), (0, 2, 2)])
    c = engine.SynthH264(seed=43, mb_w=20, mb_h=12, refs=[(0, 1, 1), (0, 2, 2)])
    assert digest(a) == digest(b)
    assert digest(a) != digest(c)


def test_workload_statistics(engine):
    p = engine.SynthH264(seed=5, mb_w=120, mb_h=68, refs=[(0, 1, 1), (0, 2, 2)])
    recs = p.mbs().reshape(-1, 176)
    kind = recs[:, engine.H264Mb.kind.offset]
    intra = np.isin(kind, [1, 2, 3, 4]).mean()
    assert 0.27 < intra < 0.33
    inter = kind == engine.RC_H264_INTER
    wp = recs[inter, engine.H264Mb.wp.offset] != 0xff
    assert 0.17 < wp.mean() < 0.23
    qp = recs[:, engine.H264Mb.qp.offset]
    assert qp.min() >= 20 and qp.max() <= 40
    lc = recs[:, engine.H264Mb.luma_coded.offset:engine.H264Mb.luma_coded.offset + 2].copy().view(np.uint16)[:, 0]
    t8 = recs[:, engine.H264Mb.transform_8x8.offset] == 1
    coded4 = np.array([bin(int(v)).count("1") for v in lc[~t8 & inter]]).sum() / (16 * (~t8 & inter).sum())
    assert 0.17 < coded4 < 0.23  # 80% all-zero blocks
    ref = recs[inter, engine.H264Mb.ref_idx.offset:engine.H264Mb.ref_idx.offset + 4].view(np.int8)
    assert set(np.unique(ref)) <= {0, 1}
    assert 0.4 < (ref == 1).mean() < 0.6


def test_intra_picture_has_no_inter(engine):
    p = engine.SynthH264(seed=1, mb_w=10, mb_h=6, intra_only=1)
    kind = p.mbs().reshape(-1, 176)[:, engine.H264Mb.kind.offset]
    assert np.all(np.isin(kind, [1, 2, 3, 4]))
