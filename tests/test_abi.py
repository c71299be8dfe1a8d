"""The C ABI library loads, exports every entry point include/*.h declares,
and validates syntax records on the host (no GPU needed)."""
from __future__ import annotations

import ctypes
import pathlib
import re

import pytest

REPO = pathlib.Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (REPO / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^[A-Za-z_][\w \t\*]*?\b(rc_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("rc_stream_create", "rc_stream_destroy", "rc_h264_submit", "rc_stream_sync", "rc_stream_error",
              "rc_picture_download", "rc_picture_upload", "rc_h264_validate"):
        assert n in names


def test_library_exports_every_declared_symbol(engine):
    L = engine.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"not exported: {missing}"


def test_struct_sizes_match_header(engine):
    assert ctypes.sizeof(engine.H264Mb) == 176
    assert ctypes.sizeof(engine.H264Slice) == 4 * (5 + 64 + 64)
    assert ctypes.sizeof(engine.H264Weight) == 64
    assert ctypes.sizeof(engine.H264Picture) == 96


def _mutate(engine, pic, fn):
    """Copy a generated picture's buffers, apply fn to the MB record array,
    and return a PictureBuffers view."""
    import numpy as np
    bufs = pic.buffers()
    mbs = np.frombuffer(bufs["mbs"], dtype=np.uint8).copy().reshape(-1, 176)
    fn(mbs)
    bufs["mbs"] = mbs.tobytes()
    return engine.PictureBuffers(bufs, pic.pic.num_slices, pic.pic.num_weights)


@pytest.fixture(scope="module")
def ppic(engine):
    return engine.SynthH264(seed=7, mb_w=6, mb_h=4, refs=[(0, 1, 1), (0, 2, 2)], frame_id=3)


def test_validate_accepts_generated_picture(engine, ppic):
    assert engine.lib().rc_h264_validate(6, 4, 4, ppic.ptr) == 0


def test_validate_rejects_bad_records(engine, ppic):
    L = engine.lib()
    mb = engine.H264Mb
    off_kind, off_slice = mb.kind.offset, mb.slice.offset
    off_ref, off_coef = mb.ref_idx.offset, mb.coef_off.offset
    recs = ppic.mbs().reshape(-1, 176)
    inter = int(next(i for i in range(len(recs)) if recs[i][off_kind] == engine.RC_H264_INTER))

    def bad_kind(m):
        m[0, off_kind] = 9

    def bad_slice(m):
        m[0, off_slice] = 5

    def bad_ref(m):
        m[inter, off_ref] = 7  # ref_idx[0][0] beyond num_ref

    def no_list(m):
        m[inter, off_ref:off_ref + 8] = 0xff  # -1 in both lists

    def bad_payload(m):
        m[inter, off_coef:off_coef + 4] = [0xff, 0xff, 0xff, 0x7f]
        m[inter, mb.luma_coded.offset] = 1

    for fn in (bad_kind, bad_slice, bad_ref, no_list, bad_payload):
        pb = _mutate(engine, ppic, fn)
        assert L.rc_h264_validate(6, 4, 4, pb.ptr) == engine.RC_EINVAL, fn.__name__
    # a reference slot outside the DPB
    assert L.rc_h264_validate(6, 4, 2, ppic.ptr) == engine.RC_EINVAL


def test_stream_create_without_gpu_reports_nodev(engine, gpu_available):
    if gpu_available:
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = engine.lib().rc_stream_create(engine.RC_CODEC_H264, 64, 64, 8, 2, 0, ctypes.byref(h))
    assert rc == engine.RC_ENODEV


def test_stream_create_rejects_bad_arguments(engine):
    L = engine.lib()
    h = ctypes.c_void_p()
    assert L.rc_stream_create(engine.RC_CODEC_H264, 0, 64, 8, 2, 0, ctypes.byref(h)) == engine.RC_EINVAL
    assert L.rc_stream_create(99, 64, 64, 8, 2, 0, ctypes.byref(h)) == engine.RC_EINVAL
    assert L.rc_stream_create(engine.RC_CODEC_H264, 64, 64, 8, 0, 0, ctypes.byref(h)) == engine.RC_EINVAL
    # the shared-GPU flag is the only bit a codec may carry
    assert L.rc_stream_create(engine.RC_CODEC_HEVC | 0x200, 64, 64, 8, 2, 0, ctypes.byref(h)) == engine.RC_EINVAL
    assert L.rc_stream_create(engine.RC_STREAM_SHARED_GPU, 64, 64, 8, 2, 0, ctypes.byref(h)) == engine.RC_EINVAL


def test_shared_gpu_flag_matches_header(engine):
    import re
    text = (pathlib.Path(__file__).resolve().parents[1] / "include" / "pito_recon.h").read_text()
    assert int(re.search(r"#define RC_STREAM_SHARED_GPU (0x[0-9a-f]+)", text).group(1), 16) == engine.RC_STREAM_SHARED_GPU


def test_stream_calls_reject_null_streams(engine):
    """Every stream call checks its handle before touching the GPU."""
    L = engine.lib()
    assert L.rc_stream_set_h264_group(None, 2) == engine.RC_EINVAL
    assert L.rc_stream_set_wait_limit(None, 0) == engine.RC_EINVAL
    assert L.rc_stream_sync(None) == engine.RC_EINVAL
    assert L.rc_stream_cuda_stream(None) is None
