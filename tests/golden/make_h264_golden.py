#!/usr/bin/env python3
"""Make tests/golden/h264_<name>.npz from the reference's golden H.264 streams.

Parses each x264 stream of the reference (tests/refs/h264/<name>.h264) into
per-picture syntax records -- with tests/golden/h264_cavlc.py (Baseline,
CAVLC) or tests/golden/h264_cabac.py (Main / High, CABAC) -- reconstructs
them with the oracle, and checks the sha256 of the output pictures against
the reference's manifest (tests/refs/h264/manifest.toml, the "<name>.yuv"
entry of kind bit-exact: the reconstruction x264 dumped while encoding).
The digest covers every picture in output order (picture order count within
each IDR period), each cropped, Y then Cb then Cr row by row (the
Digest::frame of src/testref.rs:570-578).  The oracle must reproduce it
twice: from the records with their resolved motion vectors, and from the
motion syntax alone (rc_h264_motion / rc_h264_slice_motion: partitions,
parsed ref_idx and mvd, direct modes), deriving every vector itself.
Writes the records, the motion syntax, each picture's DPB slot, POC and
crop, and the expected digest; the tests replay them through the oracle and
the engine.  Run where a checkout of the
reference exists, naming its root with --reference or the PITO_REFERENCE
environment variable:

    python tests/golden/make_h264_golden.py --reference <checkout> [name ...]
                                                      (default: every stream)
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import pathlib
import re
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "tests"))
sys.path.insert(0, str(HERE))

STREAMS = {"baseline": "cavlc", "main_cabac_b": "cabac", "high_bpyramid": "cabac", "high_crop_slices": "cabac"}
KEYS = ("mbs", "slices", "weights", "levels", "scaling4", "scaling8")
# motion syntax (rc_h264_picture.motion / slice_motion): with it the oracle
# and the engine derive every vector themselves
MOTION_KEYS = ("motion", "slice_motion")
DPB_SLOTS = 16
REFS = None  # <reference checkout>/tests/refs/h264, set by main()


def manifest_digest(name: str) -> str:
    text = (REFS / "manifest.toml").read_text()
    for block in text.split("[[ref]]"):
        if re.search(rf'name = "{re.escape(name)}.yuv"', block):
            return re.search(r'sha256 = "([0-9a-f]+)"', block).group(1)
    raise KeyError(name)


def parse(E, name, data):
    if STREAMS[name] == "cavlc":
        import h264_cavlc
        pics = h264_cavlc.Decoder(E).decode(data)
        for i, p in enumerate(pics):  # Baseline: P pictures only, output order is decode order
            p.update(poc=i, period=0, num_weights=0, scaling4=b"", scaling8=b"")
        return pics
    import h264_cabac
    return h264_cabac.Decoder(E, DPB_SLOTS).decode(data)


def cropped(planes, crop):
    l, r, t, b = crop
    y, u, v = planes
    H, W = y.shape
    out = [y[2 * t:H - 2 * b, 2 * l:W - 2 * r]]
    out += [c[t:H // 2 - b, l:W // 2 - r] for c in (u, v)]
    return [np.ascontiguousarray(p) for p in out]


def output_digest(pictures, planes_after) -> str:
    outs = {}
    for i, p in enumerate(pictures):
        outs[(p["period"], p["poc"])] = [np.array(x, copy=True) for x in planes_after(i)]
    h = hashlib.sha256()
    for k in sorted(outs):
        for pl in outs[k]:
            h.update(pl.tobytes())
    return h.hexdigest()


def main(names):
    from conftest import load_engine, load_oracle
    E, O = load_engine(), load_oracle()
    for name in names:
        data = (REFS / f"{name}.h264").read_bytes()
        pics = parse(E, name, data)
        want = manifest_digest(name)
        for keys, how in ((KEYS, "resolved motion"), (KEYS + MOTION_KEYS, "motion derived from syntax")):
            dpb = O.H264Dpb(pics[0]["mb_w"], pics[0]["mb_h"], DPB_SLOTS)

            def planes_after(i):
                p = pics[i]
                buf = E.PictureBuffers({k: p[k] for k in keys}, p["num_slices"], p["num_weights"],
                                       p["constrained_intra"], p["frame_id"])
                if dpb.recon(buf.ptr, p["slot"]) != 0:
                    raise RuntimeError("oracle rejected a parsed picture")
                return cropped(dpb.planes(p["slot"]), p["crop"])

            got = output_digest(pics, planes_after)
            print(f"{name} ({how}): {len(pics)} pictures, oracle {got}, reference {want}: "
                  f"{'MATCH' if got == want else 'DIFFER'}")
            if got != want:
                raise SystemExit(1)
        arrays = {}
        meta = {"stream": f"tests/refs/h264/{name}.h264", "stream_sha256": hashlib.sha256(data).hexdigest(),
                "expected_sha256": want,
                "expected_source": f"tests/refs/h264/manifest.toml [[ref]] {name}.yuv (kind bit-exact)",
                "pictures": []}
        for i, p in enumerate(pics):
            for k in KEYS + MOTION_KEYS:
                arrays[f"{k}_{i}"] = np.frombuffer(p[k], np.uint8)
            meta["pictures"].append({k: p[k] for k in ("num_slices", "num_weights", "slot", "frame_id",
                                                        "constrained_intra", "mb_w", "mb_h", "crop", "poc",
                                                        "period")})
        arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
        np.savez_compressed(HERE / f"h264_{name}.npz", **arrays)
        print(f"wrote tests/golden/h264_{name}.npz")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PITO_REFERENCE"),
                    help="root of the reference checkout (default: $PITO_REFERENCE)")
    ap.add_argument("names", nargs="*", default=list(STREAMS))
    a = ap.parse_args()
    if not a.reference:
        raise SystemExit("name the reference checkout with --reference or PITO_REFERENCE")
    REFS = pathlib.Path(a.reference) / "tests" / "refs" / "h264"
    main(a.names)
