#!/usr/bin/env python3
"""Make tests/golden/h264_<name>.npz from the reference's golden H.264 streams.

Parses the stream with tests/golden/h264_cavlc.py into per-picture syntax
records, reconstructs them with the oracle, and checks the sha256 of the
cropped planes (all frames, Y then Cb then Cr row by row, the Digest::frame
of src/testref.rs:570-578) against the reference's manifest
(tests/refs/h264/manifest.toml, kind "bit-exact").  Writes the records and
the expected digest; the tests replay them through the oracle and the
engine.  Run here, where the reference checkout exists:

    python tests/golden/make_h264_golden.py [name ...]   (default: baseline)
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
REFS = None  # <reference checkout>/tests/refs/h264, set by main()
sys.path.insert(0, str(REPO / "tests"))
sys.path.insert(0, str(HERE))


def manifest_digest(name: str) -> str:
    text = (REFS / "manifest.toml").read_text()
    for block in text.split("[[ref]]"):
        if re.search(rf'name = "{re.escape(name)}.yuv"', block):
            return re.search(r'sha256 = "([0-9a-f]+)"', block).group(1)
    raise KeyError(name)


def oracle_digest(E, O, pics) -> str:
    mb_w, mb_h = pics[0]["mb_w"], pics[0]["mb_h"]
    dpb = O.H264Dpb(mb_w, mb_h, 8)
    h = hashlib.sha256()
    for p in pics:
        buf = E.PictureBuffers({k: p[k] for k in ("mbs", "slices", "weights", "levels")}, p["num_slices"], 0,
                               p["constrained_intra"], p["frame_id"])
        if dpb.recon(buf.ptr, p["slot"]) != 0:
            raise RuntimeError("oracle rejected a parsed picture")
        l, r, t, bm = p["crop"]
        y, u, v = dpb.planes(p["slot"])
        H, W = y.shape
        h.update(np.ascontiguousarray(y[2 * t:H - 2 * bm, 2 * l:W - 2 * r]).tobytes())
        for c in (u, v):
            h.update(np.ascontiguousarray(c[t:H // 2 - bm, l:W // 2 - r]).tobytes())
    return h.hexdigest()


def main(names):
    from conftest import load_engine, load_oracle
    import h264_cavlc
    E, O = load_engine(), load_oracle()
    for name in names:
        data = (REFS / f"{name}.h264").read_bytes()
        pics = h264_cavlc.Decoder(E).decode(data)
        want = manifest_digest(name)
        got = oracle_digest(E, O, pics)
        print(f"{name}: {len(pics)} pictures, oracle {got}, reference {want}: {'MATCH' if got == want else 'DIFFER'}")
        if got != want:
            raise SystemExit(1)
        arrays = {}
        meta = {"stream": f"tests/refs/h264/{name}.h264", "stream_sha256": hashlib.sha256(data).hexdigest(),
                "expected_sha256": want,
                "expected_source": f"tests/refs/h264/manifest.toml [[ref]] {name}.yuv (kind bit-exact)",
                "pictures": []}
        for i, p in enumerate(pics):
            for k in ("mbs", "slices", "levels"):
                arrays[f"{k}_{i}"] = np.frombuffer(p[k], np.uint8)
            meta["pictures"].append({k: p[k] for k in ("num_slices", "slot", "frame_id", "constrained_intra",
                                                        "mb_w", "mb_h", "crop")})
        arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
        np.savez_compressed(HERE / f"h264_{name}.npz", **arrays)
        print(f"wrote tests/golden/h264_{name}.npz")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PITO_REFERENCE"),
                    help="root of the reference checkout (default: $PITO_REFERENCE)")
    ap.add_argument("names", nargs="*", default=["baseline"])
    a = ap.parse_args()
    if not a.reference:
        raise SystemExit("name the reference checkout with --reference or PITO_REFERENCE")
    REFS = pathlib.Path(a.reference) / "tests" / "refs" / "h264"
    main(a.names)
