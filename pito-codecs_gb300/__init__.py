"""GB300 block-reconstruction engine for H.264 / HEVC decode (host mirror).

The product is the C ABI of include/pito_recon.h, implemented by
libpito_recon.so (CUDA kernels for sm_103a + the C layer).  This module is a
thin ctypes mirror of that ABI so Python callers and tests drive the same
entry points a C caller (or the reference's Rust FFI) would:

    ReconStream(codec, width, height, bit_depth, dpb_slots)
        .submit_h264(picture, out_slot)   # rc_h264_submit
        .sync() / .error()                # rc_stream_sync / rc_stream_error
        .download(slot, crop)             # rc_picture_download
        .upload(slot, y, u, v)            # rc_picture_upload

There is no CPU path: if the CUDA library cannot be loaded, or no GPU is
present, construction fails with ReconError.
"""
from __future__ import annotations

import ctypes
import os
import pathlib

import numpy as np

PKG = pathlib.Path(__file__).resolve().parent
REPO = PKG.parent

RC_OK, RC_EINVAL, RC_ENOMEM, RC_ECUDA, RC_ETIMEOUT, RC_EDEVICE, RC_ENODEV = 0, -1, -2, -3, -4, -5, -6
RC_CODEC_H264, RC_CODEC_HEVC = 1, 2
RC_STREAM_SHARED_GPU = 0x100  # or-ed into the codec: one of many streams on the GPU
RC_MEM_HOST, RC_MEM_DEVICE = 0, 1
ERROR_NAMES = {RC_EINVAL: "RC_EINVAL", RC_ENOMEM: "RC_ENOMEM", RC_ECUDA: "RC_ECUDA",
               RC_ETIMEOUT: "RC_ETIMEOUT", RC_EDEVICE: "RC_EDEVICE", RC_ENODEV: "RC_ENODEV"}

RC_H264_NONE, RC_H264_I4x4, RC_H264_I8x8, RC_H264_I16x16, RC_H264_IPCM, RC_H264_INTER = range(6)
RC_KERNEL_NAMES = {0: "h264_mb_kernel", 1: "h264_band_kernel", 2: "h264_edge_kernel", 3: "hevc_residual_kernel",
                   4: "hevc_inter_kernel", 5: "hevc_intra_kernel", 6: "hevc_loopfilter_kernel", 7: "hevc_inter_kernel_late",
                   8: "h264_group_kernel", 9: "h264_mv_kernel"}
RC_KERNEL_COUNT = 10


class ReconError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what}: {ERROR_NAMES.get(code, code)}")
        self.code = code


# ---- C struct mirrors (layouts fixed by include/pito_recon.h) -------------
class H264Mb(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint8), ("transform_8x8", ctypes.c_uint8), ("qp", ctypes.c_uint8),
                ("qpc", ctypes.c_uint8 * 2), ("i16_mode", ctypes.c_uint8), ("chroma_mode", ctypes.c_uint8),
                ("dc_coded", ctypes.c_uint8), ("slice", ctypes.c_uint16), ("nz_mask", ctypes.c_uint16),
                ("luma_coded", ctypes.c_uint16), ("chroma_coded", ctypes.c_uint8), ("reserved0", ctypes.c_uint8),
                ("coef_off", ctypes.c_uint32), ("intra_modes", ctypes.c_uint8 * 16),
                ("ref_idx", (ctypes.c_int8 * 4) * 2), ("wp", ctypes.c_uint8 * 4),
                ("mv", ((ctypes.c_int16 * 2) * 16) * 2)]


class H264Slice(ctypes.Structure):
    _fields_ = [("disable_deblocking_filter_idc", ctypes.c_int32), ("alpha_offset", ctypes.c_int32),
                ("beta_offset", ctypes.c_int32), ("num_ref", ctypes.c_int32 * 2),
                ("ref_slot", (ctypes.c_int32 * 32) * 2), ("ref_id", (ctypes.c_uint32 * 32) * 2)]


class H264Weight(ctypes.Structure):
    _fields_ = [("explicit_mask", ctypes.c_uint8), ("reserved", ctypes.c_uint8 * 3), ("log_wd", ctypes.c_int32 * 3),
                ("w0", ctypes.c_int32 * 3), ("w1", ctypes.c_int32 * 3), ("o0", ctypes.c_int32 * 3),
                ("o1", ctypes.c_int32 * 3)]


class H264Picture(ctypes.Structure):
    _fields_ = [("mem", ctypes.c_int32), ("constrained_intra_pred", ctypes.c_int32), ("frame_id", ctypes.c_uint32),
                ("num_slices", ctypes.c_int32), ("num_weights", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("num_levels", ctypes.c_size_t), ("mbs", ctypes.c_void_p), ("slices", ctypes.c_void_p),
                ("weights", ctypes.c_void_p), ("levels", ctypes.c_void_p), ("scaling4", ctypes.c_void_p),
                ("scaling8", ctypes.c_void_p), ("motion", ctypes.c_void_p), ("slice_motion", ctypes.c_void_p)]


class H264Motion(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_uint8), ("pred", ctypes.c_uint8 * 4), ("sub", ctypes.c_uint8 * 4),
                ("reserved", ctypes.c_uint8 * 3), ("ref_idx", (ctypes.c_int8 * 4) * 2),
                ("mvd", ((ctypes.c_int16 * 2) * 16) * 2)]


class H264SliceMotion(ctypes.Structure):
    _fields_ = [("b_slice", ctypes.c_int32), ("direct_spatial", ctypes.c_int32),
                ("direct_8x8_inference", ctypes.c_int32), ("col_slot", ctypes.c_int32),
                ("col_short_term", ctypes.c_int32), ("dist_scale", ctypes.c_int16 * 32),
                ("direct_copy", ctypes.c_uint8 * 32), ("wp_map", ctypes.c_uint8 * (33 * 33)),
                ("reserved", ctypes.c_uint8 * 3)]


RC_H264_MOTION_NONE, RC_H264_MOTION_SKIP, RC_H264_MOTION_16x16, RC_H264_MOTION_16x8, RC_H264_MOTION_8x16, \
    RC_H264_MOTION_8x8 = range(6)
RC_H264_SUB_8x8, RC_H264_SUB_8x4, RC_H264_SUB_4x8, RC_H264_SUB_4x4, RC_H264_SUB_DIRECT = range(5)
assert ctypes.sizeof(H264Motion) == 148 and ctypes.sizeof(H264SliceMotion) == 1208
assert ctypes.sizeof(H264Mb) == 176 and ctypes.sizeof(H264Weight) == 64 and ctypes.sizeof(H264Picture) == 96


class SynthH264Opts(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("mb_w", ctypes.c_int32), ("mb_h", ctypes.c_int32),
                ("intra_only", ctypes.c_int32), ("intra_permille", ctypes.c_int32), ("pcm_permille", ctypes.c_int32),
                ("wp_permille", ctypes.c_int32), ("zero_permille", ctypes.c_int32),
                ("outside_permille", ctypes.c_int32), ("mv_range", ctypes.c_int32), ("t8_permille", ctypes.c_int32),
                ("bipred_permille", ctypes.c_int32), ("qp_min", ctypes.c_int32), ("qp_max", ctypes.c_int32),
                ("num_slices", ctypes.c_int32), ("constrained_intra_pred", ctypes.c_int32),
                ("deblock_idc", ctypes.c_int32), ("alpha_offset", ctypes.c_int32), ("beta_offset", ctypes.c_int32),
                ("custom_scaling", ctypes.c_int32), ("chroma_qp_offset", ctypes.c_int32),
                ("num_ref", ctypes.c_int32 * 2), ("ref_slot", (ctypes.c_int32 * 4) * 2),
                ("ref_id", (ctypes.c_uint32 * 4) * 2), ("frame_id", ctypes.c_uint32),
                ("motion_syntax", ctypes.c_int32)]


class HevcBlk(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_uint8), ("edges", ctypes.c_uint8), ("qp", ctypes.c_int8), ("ipm", ctypes.c_uint8)]


class HevcMvf(ctypes.Structure):
    _fields_ = [("mv", (ctypes.c_int16 * 2) * 2), ("ref_idx", ctypes.c_int8 * 2), ("reserved", ctypes.c_uint16)]


class HevcSao(ctypes.Structure):
    _fields_ = [("type_idx", ctypes.c_uint8 * 3), ("band_pos", ctypes.c_uint8 * 3), ("eo_class", ctypes.c_uint8 * 3),
                ("reserved", ctypes.c_uint8), ("offsets", (ctypes.c_int16 * 4) * 3)]


class HevcCtb(ctypes.Structure):
    _fields_ = [("slice", ctypes.c_uint16), ("tile", ctypes.c_uint16), ("ts", ctypes.c_uint32), ("sao", HevcSao),
                ("reserved", ctypes.c_uint16)]


class HevcTu(ctypes.Structure):
    _fields_ = [("x0", ctypes.c_uint16), ("y0", ctypes.c_uint16), ("log2", ctypes.c_uint8), ("c", ctypes.c_uint8),
                ("flags", ctypes.c_uint8), ("mode", ctypes.c_uint8), ("qp", ctypes.c_int8), ("max_x", ctypes.c_uint8),
                ("max_y", ctypes.c_uint8), ("reserved", ctypes.c_uint8), ("coef_off", ctypes.c_uint32)]


class HevcSlice(ctypes.Structure):
    _fields_ = [("slice_addr", ctypes.c_uint32), ("deblock_disabled", ctypes.c_int32), ("beta_offset", ctypes.c_int32),
                ("tc_offset", ctypes.c_int32), ("lf_across", ctypes.c_int32), ("sao_luma", ctypes.c_int32),
                ("sao_chroma", ctypes.c_int32), ("weighted", ctypes.c_int32), ("luma_log2_denom", ctypes.c_int32),
                ("chroma_log2_denom", ctypes.c_int32), ("num_ref", ctypes.c_int32 * 2),
                ("ref_slot", (ctypes.c_int32 * 16) * 2), ("ref_id", (ctypes.c_uint32 * 16) * 2),
                ("luma_w", (ctypes.c_int16 * 16) * 2), ("luma_o", (ctypes.c_int16 * 16) * 2),
                ("chroma_w", ((ctypes.c_int16 * 2) * 16) * 2), ("chroma_o", ((ctypes.c_int16 * 2) * 16) * 2)]


class HevcPicture(ctypes.Structure):
    _fields_ = [("mem", ctypes.c_int32), ("log2_ctb", ctypes.c_int32), ("constrained_intra_pred", ctypes.c_int32),
                ("strong_intra_smoothing", ctypes.c_int32), ("loop_filter_across_tiles", ctypes.c_int32),
                ("cb_qp_offset", ctypes.c_int32), ("cr_qp_offset", ctypes.c_int32), ("num_slices", ctypes.c_int32),
                ("num_tus", ctypes.c_int32), ("frame_id", ctypes.c_uint32), ("num_levels", ctypes.c_size_t),
                ("ctbs", ctypes.c_void_p), ("blk", ctypes.c_void_p), ("mvf", ctypes.c_void_p), ("tus", ctypes.c_void_p),
                ("slices", ctypes.c_void_p), ("levels", ctypes.c_void_p), ("scaling", ctypes.c_void_p)]


assert (ctypes.sizeof(HevcBlk), ctypes.sizeof(HevcMvf), ctypes.sizeof(HevcCtb), ctypes.sizeof(HevcTu),
        ctypes.sizeof(HevcSlice), ctypes.sizeof(HevcPicture)) == (4, 12, 44, 16, 688, 104)


class SynthHevcOpts(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("bit_depth", ctypes.c_int32), ("log2_ctb", ctypes.c_int32), ("intra_only", ctypes.c_int32),
                ("intra_permille", ctypes.c_int32), ("zero_tu_permille", ctypes.c_int32),
                ("split_permille", ctypes.c_int32), ("mv_range", ctypes.c_int32), ("bipred_permille", ctypes.c_int32),
                ("qp_min", ctypes.c_int32), ("qp_max", ctypes.c_int32), ("cb_qp_offset", ctypes.c_int32),
                ("cr_qp_offset", ctypes.c_int32), ("transform_skip_permille", ctypes.c_int32),
                ("pcm_permille", ctypes.c_int32), ("pcm_loop_filter_disabled", ctypes.c_int32),
                ("bypass_permille", ctypes.c_int32), ("scaling_lists", ctypes.c_int32),
                ("constrained_intra_pred", ctypes.c_int32), ("strong_intra_smoothing", ctypes.c_int32),
                ("weighted", ctypes.c_int32), ("num_slices", ctypes.c_int32), ("tile_cols", ctypes.c_int32),
                ("tile_rows", ctypes.c_int32), ("loop_filter_across_tiles", ctypes.c_int32),
                ("lf_across_slices", ctypes.c_int32), ("deblock_disabled", ctypes.c_int32),
                ("beta_offset", ctypes.c_int32), ("tc_offset", ctypes.c_int32), ("sao", ctypes.c_int32),
                ("num_ref", ctypes.c_int32 * 2), ("ref_slot", (ctypes.c_int32 * 4) * 2),
                ("ref_id", (ctypes.c_uint32 * 4) * 2), ("frame_id", ctypes.c_uint32)]


# ---- library loading ------------------------------------------------------
_LIBS: dict = {}


def _load(name: str, path: pathlib.Path, build_fn):
    if name in _LIBS:
        return _LIBS[name]
    if not path.exists():
        build_fn()
    if not path.exists():
        raise ReconError(RC_ENODEV, f"{path.name} missing and could not be built")
    lib = ctypes.CDLL(str(path))
    _LIBS[name] = lib
    return lib


def _build():
    from importlib import util

    spec = util.spec_from_file_location("_pito_build", PKG / "build.py")
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


def lib() -> ctypes.CDLL:
    """The CUDA engine (libpito_recon.so) with argument types declared."""
    if "recon" in _LIBS:
        return _LIBS["recon"]
    L = _load("recon", PKG / "libpito_recon.so", _build)
    vp, i32, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    L.rc_stream_create.argtypes = [i32, i32, i32, i32, i32, sz, ctypes.POINTER(vp)]
    L.rc_stream_create.restype = i32
    L.rc_device_select.argtypes = [i32]
    L.rc_device_select.restype = i32
    L.rc_stream_destroy.argtypes = [vp]
    L.rc_stream_destroy.restype = None
    L.rc_h264_submit.argtypes = [vp, vp, i32]
    L.rc_h264_submit.restype = i32
    L.rc_h264_validate.argtypes = [i32, i32, i32, vp]
    L.rc_h264_validate.restype = i32
    L.rc_hevc_submit.argtypes = [vp, vp, i32]
    L.rc_hevc_submit.restype = i32
    L.rc_hevc_validate.argtypes = [i32, i32, i32, i32, vp]
    L.rc_hevc_validate.restype = i32
    L.rc_stream_sync.argtypes = [vp]
    L.rc_stream_set_intra_ctas.argtypes = [vp, i32]
    L.rc_stream_set_intra_ctas.restype = i32
    L.rc_stream_intra_ctas.argtypes = [vp]
    L.rc_stream_intra_ctas.restype = i32
    L.rc_stream_set_lf_tile.argtypes = [vp, i32]
    L.rc_stream_set_lf_tile.restype = i32
    L.rc_stream_lf_tile.argtypes = [vp]
    L.rc_stream_lf_tile.restype = i32
    L.rc_stream_set_wait_limit.argtypes = [vp, ctypes.c_uint]
    L.rc_stream_set_wait_limit.restype = i32
    L.rc_stream_set_h264_group.argtypes = [vp, i32]
    L.rc_stream_set_h264_group.restype = i32
    L.rc_stream_sync.restype = i32
    L.rc_stream_error.argtypes = [vp]
    L.rc_stream_error.restype = i32
    L.rc_picture_download.argtypes = [vp, i32, i32, i32, i32, i32, vp, vp, vp]
    L.rc_picture_download.restype = i32
    L.rc_picture_download_async.argtypes = [vp, i32, i32, i32, i32, i32, vp, vp, vp]
    L.rc_picture_download_async.restype = i32
    L.rc_stream_profile.argtypes = [vp, i32]
    L.rc_stream_profile.restype = i32
    L.rc_stream_profile_read.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong), i32]
    L.rc_stream_profile_read.restype = i32
    L.rc_picture_upload.argtypes = [vp, i32, vp, vp, vp]
    L.rc_picture_upload.restype = i32
    L.rc_stream_geometry.argtypes = [vp] + [ctypes.POINTER(i32)] * 4
    L.rc_stream_geometry.restype = i32
    L.rc_picture_device_planes.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.rc_picture_device_planes.restype = i32
    L.rc_stream_launches.argtypes = [vp]
    L.rc_stream_launches.restype = ctypes.c_longlong
    L.rc_stream_cuda_stream.argtypes = [vp]
    L.rc_stream_cuda_stream.restype = vp
    L.rc_stream_mark.argtypes = [vp, ctypes.POINTER(ctypes.c_ulonglong)]
    L.rc_stream_mark.restype = i32
    L.rc_stream_mark_done.argtypes = [vp, ctypes.c_ulonglong]
    L.rc_stream_mark_done.restype = i32
    L.rc_stream_device_bytes.argtypes = [vp]
    L.rc_stream_device_bytes.restype = sz
    L.rc_h264_deblock_noalloc.argtypes = [vp, i32, i32, vp, vp, vp, i32, i32, vp, vp]
    L.rc_h264_deblock_noalloc.restype = i32
    u64p = ctypes.POINTER(ctypes.c_uint64)
    L.rc_output_create.argtypes = [i32, i32, i32, ctypes.POINTER(vp)]
    L.rc_output_create.restype = i32
    L.rc_output_destroy.argtypes = [vp]
    L.rc_output_destroy.restype = None
    L.rc_output_begin.argtypes = [vp, i32, i32, u64p, i32, ctypes.POINTER(i32)]
    L.rc_output_begin.restype = i32
    L.rc_output_unref.argtypes = [vp, ctypes.c_uint64]
    L.rc_output_unref.restype = i32
    L.rc_output_insert.argtypes = [vp, ctypes.c_uint64, ctypes.c_int32, i32, i32, u64p, i32, ctypes.POINTER(i32)]
    L.rc_output_insert.restype = i32
    L.rc_output_flush.argtypes = [vp, u64p, i32, ctypes.POINTER(i32)]
    L.rc_output_flush.restype = i32
    L.rc_output_count.argtypes = [vp]
    L.rc_output_count.restype = i32
    return L


def synth_lib() -> ctypes.CDLL:
    """The synthetic syntax generators (libpito_synth.so)."""
    if "synth" in _LIBS:
        return _LIBS["synth"]
    L = _load("synth", PKG / "libpito_synth.so", _build)
    L.rc_synth_h264_defaults.argtypes = [ctypes.POINTER(SynthH264Opts)]
    L.rc_synth_h264_defaults.restype = None
    L.rc_synth_h264_new.argtypes = [ctypes.POINTER(SynthH264Opts)]
    L.rc_synth_h264_new.restype = ctypes.c_void_p
    L.rc_synth_h264_picture.argtypes = [ctypes.c_void_p]
    L.rc_synth_h264_picture.restype = ctypes.c_void_p
    L.rc_synth_h264_bytes.argtypes = [ctypes.c_void_p]
    L.rc_synth_h264_bytes.restype = ctypes.c_size_t
    L.rc_synth_h264_free.argtypes = [ctypes.c_void_p]
    L.rc_synth_h264_free.restype = None
    L.rc_synth_hevc_defaults.argtypes = [ctypes.POINTER(SynthHevcOpts)]
    L.rc_synth_hevc_defaults.restype = None
    L.rc_synth_hevc_new.argtypes = [ctypes.POINTER(SynthHevcOpts)]
    L.rc_synth_hevc_new.restype = ctypes.c_void_p
    L.rc_synth_hevc_picture.argtypes = [ctypes.c_void_p]
    L.rc_synth_hevc_picture.restype = ctypes.c_void_p
    L.rc_synth_hevc_bytes.argtypes = [ctypes.c_void_p]
    L.rc_synth_hevc_bytes.restype = ctypes.c_size_t
    L.rc_synth_hevc_free.argtypes = [ctypes.c_void_p]
    L.rc_synth_hevc_free.restype = None
    return L


# ---- synthetic H.264 pictures ---------------------------------------------
class SynthH264:
    """One generated picture (owns the C buffers)."""

    def __init__(self, **kw):
        L = synth_lib()
        o = SynthH264Opts()
        L.rc_synth_h264_defaults(ctypes.byref(o))
        refs = kw.pop("refs", None)  # [(list, slot, id), ...]
        for k, v in kw.items():
            if not hasattr(o, k):
                raise TypeError(f"unknown generator option {k}")
            setattr(o, k, v)
        if refs is not None:
            o.num_ref[0] = o.num_ref[1] = 0
            for (l, slot, rid) in refs:
                i = o.num_ref[l]
                o.ref_slot[l][i] = slot
                o.ref_id[l][i] = rid
                o.num_ref[l] = i + 1
        self.opts = o
        self._h = L.rc_synth_h264_new(ctypes.byref(o))
        if not self._h:
            raise ValueError("generator rejected its options")
        self.ptr = L.rc_synth_h264_picture(self._h)
        self.pic = H264Picture.from_address(self.ptr)
        self.nbytes = L.rc_synth_h264_bytes(self._h)

    @property
    def mb_count(self) -> int:
        return self.opts.mb_w * self.opts.mb_h

    def mbs(self) -> np.ndarray:
        """The MB records as a structured view (bytes)."""
        return np.ctypeslib.as_array((ctypes.c_uint8 * (176 * self.mb_count)).from_address(self.pic.mbs))

    def buffers(self) -> dict:
        """Raw bytes of every syntax buffer (for fixtures / device copies)."""
        p = self.pic
        def raw(addr, n):
            return bytes((ctypes.c_uint8 * n).from_address(addr)) if n else b""
        return {"mbs": raw(p.mbs, 176 * self.mb_count),
                "slices": raw(p.slices, ctypes.sizeof(H264Slice) * p.num_slices),
                "weights": raw(p.weights, 64 * p.num_weights) if p.weights else b"",
                "levels": raw(p.levels, 2 * p.num_levels) if p.levels else b"",
                "scaling4": raw(p.scaling4, 96) if p.scaling4 else b"",
                "scaling8": raw(p.scaling8, 384) if p.scaling8 else b""}

    def close(self):
        if self._h:
            synth_lib().rc_synth_h264_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SynthHevc:
    """One generated HEVC picture (owns the C buffers)."""

    def __init__(self, **kw):
        L = synth_lib()
        o = SynthHevcOpts()
        L.rc_synth_hevc_defaults(ctypes.byref(o))
        refs = kw.pop("refs", None)  # [(list, slot, id), ...]
        for k, v in kw.items():
            if not hasattr(o, k):
                raise TypeError(f"unknown generator option {k}")
            setattr(o, k, v)
        if refs is not None:
            o.num_ref[0] = o.num_ref[1] = 0
            for (l, slot, rid) in refs:
                i = o.num_ref[l]
                o.ref_slot[l][i] = slot
                o.ref_id[l][i] = rid
                o.num_ref[l] = i + 1
        self.opts = o
        self._h = L.rc_synth_hevc_new(ctypes.byref(o))
        if not self._h:
            raise ValueError("generator rejected its options")
        self.ptr = L.rc_synth_hevc_picture(self._h)
        self.pic = HevcPicture.from_address(self.ptr)
        self.nbytes = L.rc_synth_hevc_bytes(self._h)

    def buffers(self) -> dict:
        p, o = self.pic, self.opts
        w4, h4 = o.width // 4, o.height // 4
        ctb = 1 << o.log2_ctb
        nctb = ((o.width + ctb - 1) // ctb) * ((o.height + ctb - 1) // ctb)
        def raw(addr, n):
            return bytes((ctypes.c_uint8 * n).from_address(addr)) if (n and addr) else b""
        return {"ctbs": raw(p.ctbs, 44 * nctb), "blk": raw(p.blk, 4 * w4 * h4), "mvf": raw(p.mvf, 12 * w4 * h4),
                "tus": raw(p.tus, 16 * p.num_tus), "slices": raw(p.slices, 688 * p.num_slices),
                "levels": raw(p.levels, 2 * p.num_levels),
                "scaling": raw(p.scaling, 6 * (16 + 64 + 256 + 1024))}

    def close(self):
        if self._h:
            synth_lib().rc_synth_hevc_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PictureBuffers:
    """An rc_h264_picture rebuilt from raw buffers (e.g. fixture files),
    keeping the buffers alive."""

    def __init__(self, bufs: dict, num_slices: int, num_weights: int, constrained_intra_pred: int = 0,
                 frame_id: int = 0):
        self._keep = {k: ctypes.create_string_buffer(v, len(v)) if v else None for k, v in bufs.items()}
        p = H264Picture()
        p.mem = RC_MEM_HOST
        p.constrained_intra_pred = constrained_intra_pred
        p.frame_id = frame_id
        p.num_slices = num_slices
        p.num_weights = num_weights
        p.num_levels = len(bufs["levels"]) // 2
        addr = lambda k: ctypes.addressof(self._keep[k]) if self._keep.get(k) is not None else None
        p.mbs, p.slices, p.weights, p.levels = addr("mbs"), addr("slices"), addr("weights"), addr("levels")
        p.scaling4, p.scaling8 = addr("scaling4"), addr("scaling8")
        p.motion, p.slice_motion = addr("motion"), addr("slice_motion")
        self.pic = p
        self.ptr = ctypes.addressof(p)


class HevcPictureBuffers:
    """An rc_hevc_picture rebuilt from raw buffers (fixture files, parsed
    streams, edited records), keeping the buffers alive.  `header` holds the
    scalar fields of rc_hevc_picture (log2_ctb, num_slices, num_tus, ...)."""

    HEADER = ("log2_ctb", "constrained_intra_pred", "strong_intra_smoothing", "loop_filter_across_tiles",
              "cb_qp_offset", "cr_qp_offset", "num_slices", "num_tus", "frame_id")

    def __init__(self, bufs: dict, header: dict):
        self._keep = {k: ctypes.create_string_buffer(v, len(v)) if v else None for k, v in bufs.items()}
        p = HevcPicture()
        p.mem = RC_MEM_HOST
        for k in self.HEADER:
            setattr(p, k, int(header.get(k, 0)))
        p.num_levels = len(bufs.get("levels", b"")) // 2
        addr = lambda k: ctypes.addressof(self._keep[k]) if self._keep.get(k) is not None else None
        for k in ("ctbs", "blk", "mvf", "tus", "slices", "levels", "scaling"):
            setattr(p, k, addr(k))
        self.pic = p
        self.ptr = ctypes.addressof(p)


class OutputOrder:
    """Output order of decoded pictures (rc_output_*: DPB bumping).  Each
    call returns the ids it outputs, in order."""

    def __init__(self, capacity: int, max_num_reorder: int, max_latency_pictures: int = 0):
        h = ctypes.c_void_p()
        _check(lib().rc_output_create(capacity, max_num_reorder, max_latency_pictures, ctypes.byref(h)),
               "rc_output_create")
        self._h = h

    def _call(self, fn, *args):
        cap = lib().rc_output_count(self._h) + 1
        ids = (ctypes.c_uint64 * cap)()
        n = ctypes.c_int()
        _check(fn(self._h, *args, ids, cap, ctypes.byref(n)), fn.__name__)
        return [ids[i] for i in range(n.value)]

    def begin(self, new_sequence: bool = False, no_output_of_prior_pics: bool = False):
        return self._call(lib().rc_output_begin, int(new_sequence), int(no_output_of_prior_pics))

    def unref(self, pic_id: int):
        _check(lib().rc_output_unref(self._h, pic_id), "rc_output_unref")

    def insert(self, pic_id: int, poc: int, output: bool = True, reference: bool = True):
        return self._call(lib().rc_output_insert, pic_id, poc, int(output), int(reference))

    def flush(self):
        return self._call(lib().rc_output_flush)

    def count(self) -> int:
        return lib().rc_output_count(self._h)

    def close(self):
        if self._h:
            lib().rc_output_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- the stream -------------------------------------------------------------
def _check(rc: int, what: str):
    if rc != RC_OK:
        raise ReconError(rc, what)


class ReconStream:
    """One decode stream: a device-resident DPB plus the CUDA stream its
    pictures are reconstructed on (rc_stream)."""

    def __init__(self, codec: int, width: int, height: int, bit_depth: int = 8, dpb_slots: int = 4,
                 hbm_budget: int = 0, shared_gpu: bool = False):
        L = lib()
        h = ctypes.c_void_p()
        flags = RC_STREAM_SHARED_GPU if shared_gpu else 0
        _check(L.rc_stream_create(codec | flags, width, height, bit_depth, dpb_slots, hbm_budget, ctypes.byref(h)),
               "rc_stream_create")
        self._h = h
        self.codec, self.bit_depth, self.slots = codec, bit_depth, dpb_slots
        self.h264_group = 1
        w, hh, p, cp = (ctypes.c_int() for _ in range(4))
        _check(L.rc_stream_geometry(h, ctypes.byref(w), ctypes.byref(hh), ctypes.byref(p), ctypes.byref(cp)),
               "rc_stream_geometry")
        self.coded_w, self.coded_h, self.pitch, self.cpitch = w.value, hh.value, p.value, cp.value

    @property
    def handle(self):
        return self._h

    def submit_h264(self, picture, out_slot: int):
        ptr = picture.ptr if hasattr(picture, "ptr") else picture
        _check(lib().rc_h264_submit(self._h, ptr, out_slot), "rc_h264_submit")

    def submit_hevc(self, picture, out_slot: int):
        ptr = picture.ptr if hasattr(picture, "ptr") else picture
        _check(lib().rc_hevc_submit(self._h, ptr, out_slot), "rc_hevc_submit")

    def sync(self) -> int:
        return lib().rc_stream_sync(self._h)

    def error(self) -> int:
        return lib().rc_stream_error(self._h)

    def launches(self) -> int:
        return lib().rc_stream_launches(self._h)

    def cuda_stream(self) -> int:
        return lib().rc_stream_cuda_stream(self._h)

    def mark(self) -> int:
        """A completion mark after all work submitted so far."""
        m = ctypes.c_ulonglong()
        _check(lib().rc_stream_mark(self._h, ctypes.byref(m)), "rc_stream_mark")
        return m.value

    def device_bytes(self) -> int:
        return lib().rc_stream_device_bytes(self._h)

    def mark_done(self, mark: int) -> bool:
        r = lib().rc_stream_mark_done(self._h, mark)
        if r < 0:
            raise ReconError(r, "rc_stream_mark_done")
        return r == 1

    def profile(self, enable: bool):
        _check(lib().rc_stream_profile(self._h, int(enable)), "rc_stream_profile")

    def set_intra_ctas(self, ctas: int):
        """HEVC intra kernel CTAs per launch (0: the default); a schedule knob."""
        _check(lib().rc_stream_set_intra_ctas(self._h, int(ctas)), "rc_stream_set_intra_ctas")

    def intra_ctas(self) -> int:
        return lib().rc_stream_intra_ctas(self._h)

    def set_lf_tile(self, rows: int):
        """HEVC loop-filter tile height in luma rows (64, 32 or 16)."""
        _check(lib().rc_stream_set_lf_tile(self._h, int(rows)), "rc_stream_set_lf_tile")

    def lf_tile(self) -> int:
        return lib().rc_stream_lf_tile(self._h)

    def set_wait_limit(self, limit: int):
        """Iteration cap of the device-side waits (0: the default)."""
        _check(lib().rc_stream_set_wait_limit(self._h, int(limit)), "rc_stream_set_wait_limit")

    def set_h264_group(self, pictures: int) -> int:
        """H.264: pictures reconstructed per launch (1: one launch per
        picture; 0: the library's default); returns the value in effect."""
        r = lib().rc_stream_set_h264_group(self._h, int(pictures))
        if r < 0:
            raise ReconError(r, "rc_stream_set_h264_group")
        self.h264_group = r
        return r

    def profile_read(self) -> dict:
        ms = (ctypes.c_double * RC_KERNEL_COUNT)()
        n = (ctypes.c_longlong * RC_KERNEL_COUNT)()
        k = lib().rc_stream_profile_read(self._h, ms, n, RC_KERNEL_COUNT)
        if k < 0:
            raise ReconError(k, "rc_stream_profile_read")
        return {i: (ms[i], n[i]) for i in range(k) if n[i]}

    def download_async(self, slot: int, crop, Y, U, V):
        """Queue a cropped copy of a slot into caller buffers (pinned host
        or device addresses); valid after sync()."""
        x, y, w, h = crop
        _check(lib().rc_picture_download_async(self._h, slot, x, y, w, h, Y, U, V), "rc_picture_download_async")

    def device_planes(self, slot: int):
        y, u, v = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib().rc_picture_device_planes(self._h, slot, ctypes.byref(y), ctypes.byref(u), ctypes.byref(v)),
               "rc_picture_device_planes")
        return y.value, u.value, v.value

    def download(self, slot: int, crop=None):
        """Planes of a DPB slot (coded size unless crop=(x, y, w, h))."""
        x, y, w, h = crop if crop else (0, 0, self.coded_w, self.coded_h)
        dt = np.uint16 if self.bit_depth > 8 else np.uint8
        cw, ch = (w + 1) // 2, (h + 1) // 2
        Y = np.empty((h, w), dt)
        U = np.empty((ch, cw), dt)
        V = np.empty((ch, cw), dt)
        _check(lib().rc_picture_download(self._h, slot, x, y, w, h, Y.ctypes.data, U.ctypes.data, V.ctypes.data),
               "rc_picture_download")
        return Y, U, V

    def upload(self, slot: int, Y: np.ndarray, U: np.ndarray, V: np.ndarray):
        Y, U, V = (np.ascontiguousarray(a) for a in (Y, U, V))
        _check(lib().rc_picture_upload(self._h, slot, Y.ctypes.data, U.ctypes.data, V.ctypes.data),
               "rc_picture_upload")

    def close(self):
        if self._h:
            lib().rc_stream_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
