"""End-to-end parity against the reference's golden HEVC streams.

tests/golden/hevc_<name>.npz holds the syntax records of the reference's
x265 stream tests/refs/hevc/<name>.hevc, parsed by tests/golden/hevc_cabac.py
(made by tests/golden/make_hevc_golden.py), with each picture's DPB slot,
picture order count and crop.  EXPECTED below is the sha256 the reference's
manifest records for the stream's reconstruction (tests/refs/hevc/
manifest.toml, the "<name>.yuv" entry, kind bit-exact: the reconstruction
x265 wrote while encoding).  The digest covers the output pictures in output
order, each cropped, Y then Cb then Cr row by row, 10-bit samples as
little-endian 16-bit words (src/testref.rs:570-578).  The oracle (CPU) and
the engine (GPU, through the C ABI) must both reproduce it.

The streams cover Main and Main10; all-intra, P and B pictures with up to 6
references and pyramids; explicit weighted uni- and bi-prediction; scaling
lists (default and from a file), transform skip, lossless and CU-level
transquant bypass; slices, WPP, CTBs of 16 and 64; chroma QP offsets; AMP
and rectangular partitions; odd picture sizes with conformance cropping;
deblocking offsets and off; SAO; open GOPs.
"""
from __future__ import annotations

import hashlib
import json
import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"

EXPECTED = {
    "bframes": "bbafb7ec04216cc5be52591ea23ff7acaf0063517ab0eff17df7f5337c367e71",
    "cu_lossless": "b37f770a55a17f4b5cfea921f2a01659b14875f368b6cc36624f926191ce6778",
    "cu_qp_chroma_offsets": "e0a9085e49d104da89f914d8a2183090c7103b143bc97f4798e18b4f41ff15ca",
    "intra_main10": "b1f10d3fda9502dc01e5f5c5e68c829d6ab7a62a2b277fd37b6fa904724a7629",
    "intra_tools": "51c96c1616b5466fe22b86fccd643318580427eb8b52a0daf9c16bda537d4c4e",
    "long_b_runs": "ad850749969561ddf6dfa99cbc8c70b5c4448200000aab7735c7478cfa9b2288",
    "lossless": "f7723c040d9452cb0ea6253eb134c07f42467a0c0f5b2e2f8a575fbd7acffdf3",
    "medium": "a104a551b4fb1c1c9caa35057ce05979e2e86627fa29bd5a24249b6ec1ec3c78",
    "odd_350x238": "38800fae9af00f7bbb144f6fbc3733ace4aa4b28a5efa2c4fc762194e69e849e",
    "one_ctb_no_deblock": "e3507f48c707bc8503080188aa4d597edf1cafdfe965982bc76a720f01318420",
    "open_gop": "c1eec277f39f9fd1d9a0a9093bca2d7091d1cab076d407af6abd4f7331177d7f",
    "open_gop_cut": "98ca6574cb354724d993ae3510acc6c7aec6c75b7772fa9c9fb278a1bc59d8d2",
    "pyramid_weightb_main10": "d27e802adfc7dbeb4f0bbba857dd45861a6b1ff569dcb1020d3b2dcfc6e7d934",
    "scaling_list_file": "69b3bf09651389c53b06cb15a59390909d5995484cc0f491bf1bd8047bec6cd4",
    "scaling_tskip_main10": "b14aa6b3f8aafa4425b6cb85c0efd257fa39e04d082d7d7fb2c6e10a78ae3248",
    "slow_main10": "881f0e049f029b325743a69efb4e815f608b181bf5f40960f8e816e2001140e6",
    "tools": "7bb369c4adbefb98af1545c973ab0101a2e9878893975797ebb9a62372010d2f",
    "weightp_8bit": "b42bc08a7d4b2b64ed90588636a7408390a60daf7098fca52c562ea3ba520e6d",
    "weightp_main10": "afd77e99b268360038bfce1ed6a96f145bdfa2fbe80b302261b52f074a38c2d2",
    "wpp_crop_66x70": "be6bd3c45921e3b86ec17b184f8145146f8e12ae8fe0e31cca56c3c5549779d4",
    "wpp_slices_main10": "78ac94f5059a0f68e481a471bc57611d5573dae34d9856e02e84f1bc72cf6246",
}
KEYS = ("ctbs", "blk", "mvf", "tus", "slices", "levels", "scaling")
DPB_SLOTS = 16


def load_fixture(engine, name):
    z = np.load(GOLDEN / f"hevc_{name}.npz")
    meta = json.loads(bytes(z["meta"]).decode())
    pics = []
    for i, m in enumerate(meta["pictures"]):
        bufs = {k: z[f"{k}_{i}"].tobytes() for k in KEYS}
        pics.append((m, engine.HevcPictureBuffers(bufs, m["header"])))
    return meta, pics


def cropped(planes, crop):
    x, y, w, h = crop
    Y, U, V = planes
    return [Y[y:y + h, x:x + w], U[y // 2:(y + h) // 2, x // 2:(x + w) // 2], V[y // 2:(y + h) // 2, x // 2:(x + w) // 2]]


def output_digest(metas, planes_after) -> str:
    """Reconstruct picture by picture (planes_after(i) -> its cropped planes,
    taken before its DPB slot can be reused) and hash the output pictures in
    output order."""
    outs = {}
    for i, m in enumerate(metas):
        planes = [np.array(p, copy=True) for p in planes_after(i)]
        if m["output"]:
            outs[(m["cvs"], m["poc"])] = planes
    dt = np.dtype("<u2") if metas[0]["bit_depth"] > 8 else np.dtype(np.uint8)
    h = hashlib.sha256()
    for k in sorted(outs):
        for pl in outs[k]:
            h.update(np.ascontiguousarray(pl.astype(dt)).tobytes())
    return h.hexdigest()


def test_every_fixture_is_a_reference_stream():
    assert sorted(p.stem[5:] for p in GOLDEN.glob("hevc_*.npz")) == sorted(EXPECTED)
    for name, want in EXPECTED.items():
        z = np.load(GOLDEN / f"hevc_{name}.npz")
        meta = json.loads(bytes(z["meta"]).decode())
        assert meta["expected_sha256"] == want
        assert meta["stream"] == f"tests/refs/hevc/{name}.hevc"


@pytest.mark.parametrize("name", sorted(EXPECTED))
def test_oracle_reproduces_reference_digest(engine, oracle, name):
    meta, pics = load_fixture(engine, name)
    m0 = meta["pictures"][0]
    dpb = oracle.HevcDpb(m0["W"], m0["H"], m0["bit_depth"], DPB_SLOTS)

    def planes_after(i):
        m, p = pics[i]
        assert dpb.recon(p.ptr, m["slot"], 3) == 0
        return cropped(dpb.planes(m["slot"]), m["crop"])

    assert output_digest([m for m, _ in pics], planes_after) == EXPECTED[name]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(EXPECTED))
def test_engine_reproduces_reference_digest(engine, name):
    meta, pics = load_fixture(engine, name)
    m0 = meta["pictures"][0]
    with engine.ReconStream(engine.RC_CODEC_HEVC, m0["W"], m0["H"], m0["bit_depth"], DPB_SLOTS) as st:
        def planes_after(i):
            m, p = pics[i]
            st.submit_hevc(p, m["slot"])
            assert st.sync() == 0
            return st.download(m["slot"], m["crop"])

        assert output_digest([m for m, _ in pics], planes_after) == EXPECTED[name]
