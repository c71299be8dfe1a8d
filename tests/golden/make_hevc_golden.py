#!/usr/bin/env python3
"""Make tests/golden/hevc_<name>.npz from the reference's golden HEVC streams.

Parses each x265 stream of the reference (tests/refs/hevc/<name>.hevc) with
tests/golden/hevc_cabac.py into per-picture syntax records, reconstructs
them with the oracle, and checks the sha256 of the output pictures against
the reference's manifest (tests/refs/hevc/manifest.toml, the "<name>.yuv"
entry of kind bit-exact: the reconstruction x265 wrote while encoding).
The digest covers every output picture in output order (picture order
count within each coded video sequence), each cropped to the conformance
window, Y then Cb then Cr row by row, 8-bit samples as bytes and 10-bit
samples as little-endian 16-bit words (the Digest::frame of
src/testref.rs:570-578).  Writes the records, the DPB slot, POC and crop of
every picture and the expected digest; the tests replay them through the
oracle and the engine.  Run where a checkout of the reference exists,
naming its root with --reference or the PITO_REFERENCE environment variable:

    python tests/golden/make_hevc_golden.py --reference <checkout> [name ...]
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

STREAMS = ["intra_main10", "medium", "slow_main10", "bframes", "weightp_main10", "open_gop", "tools", "lossless",
           "odd_350x238", "wpp_crop_66x70", "wpp_slices_main10", "long_b_runs", "pyramid_weightb_main10",
           "weightp_8bit", "scaling_tskip_main10", "cu_qp_chroma_offsets", "intra_tools", "cu_lossless",
           "one_ctb_no_deblock", "scaling_list_file", "open_gop_cut"]
KEYS = ("ctbs", "blk", "mvf", "tus", "slices", "levels", "scaling")


def manifest_digest(refs: pathlib.Path, name: str) -> str:
    text = (refs / "manifest.toml").read_text()
    for block in text.split("[[ref]]"):
        if re.search(rf'name = "{re.escape(name)}.yuv"', block):
            return re.search(r'sha256 = "([0-9a-f]+)"', block).group(1)
    raise KeyError(name)


def output_digest(pictures, planes_of) -> str:
    """sha256 of the output pictures: planes_of(i) gives picture i's cropped
    (Y, Cb, Cr) right after it is reconstructed."""
    outs = {}
    for i, p in enumerate(pictures):
        planes = planes_of(i)
        if p["output"]:
            outs[(p["cvs"], p["poc"])] = [np.array(pl, copy=True) for pl in planes]
    h = hashlib.sha256()
    dt = np.dtype("<u2") if pictures[0]["bit_depth"] > 8 else np.dtype(np.uint8)
    for k in sorted(outs):
        for pl in outs[k]:
            h.update(np.ascontiguousarray(pl.astype(dt)).tobytes())
    return h.hexdigest()


def cropped(planes, crop):
    x, y, w, h = crop
    Y, U, V = planes
    return [Y[y:y + h, x:x + w], U[y // 2:(y + h) // 2, x // 2:(x + w) // 2], V[y // 2:(y + h) // 2, x // 2:(x + w) // 2]]


def main(refs: pathlib.Path, names):
    from conftest import load_engine, load_oracle
    import hevc_cabac
    E, O = load_engine(), load_oracle()
    for name in names:
        data = (refs / f"{name}.hevc").read_bytes()
        pics = hevc_cabac.Decoder().decode(data)
        want = manifest_digest(refs, name)
        p0 = pics[0]
        dpb = O.HevcDpb(p0["W"], p0["H"], p0["bit_depth"], 16)

        def planes_of(i):
            p = pics[i]
            buf = E.HevcPictureBuffers(p["bufs"], p["header"])
            if dpb.recon(buf.ptr, p["slot"], 3) != 0:
                raise RuntimeError("oracle rejected a parsed picture")
            return cropped(dpb.planes(p["slot"]), p["crop"])

        got = output_digest(pics, planes_of)
        print(f"{name}: {len(pics)} pictures, oracle {got}, reference {want}: {'MATCH' if got == want else 'DIFFER'}")
        if got != want:
            raise SystemExit(1)
        arrays = {}
        meta = {"stream": f"tests/refs/hevc/{name}.hevc", "stream_sha256": hashlib.sha256(data).hexdigest(),
                "expected_sha256": want,
                "expected_source": f"tests/refs/hevc/manifest.toml [[ref]] {name}.yuv (kind bit-exact)",
                "pictures": []}
        for i, p in enumerate(pics):
            for k in KEYS:
                arrays[f"{k}_{i}"] = np.frombuffer(p["bufs"][k], np.uint8)
            meta["pictures"].append({k: p[k] for k in ("W", "H", "bit_depth", "slot", "poc", "cvs", "output", "crop",
                                                        "header", "frame_id", "new_sequence",
                                                        "no_output_of_prior_pics", "unref", "dpb")})
        arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
        np.savez_compressed(HERE / f"hevc_{name}.npz", **arrays)
        print(f"wrote tests/golden/hevc_{name}.npz")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PITO_REFERENCE"),
                    help="root of the reference checkout (default: $PITO_REFERENCE)")
    ap.add_argument("names", nargs="*", default=STREAMS)
    a = ap.parse_args()
    if not a.reference:
        raise SystemExit("name the reference checkout with --reference or PITO_REFERENCE")
    main(pathlib.Path(a.reference) / "tests" / "refs" / "hevc", a.names)
