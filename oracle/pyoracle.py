"""ctypes binding of the oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The engine never loads it.
"""
from __future__ import annotations

import ctypes
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
_lib = None


def build() -> None:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB))
        vp, i32 = ctypes.c_void_p, ctypes.c_int
        for name in ("oracle_h264_recon", "oracle_h264_recon_nofilter"):
            f = getattr(_lib, name)
            f.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp, vp]
            f.restype = i32
        _lib.oracle_h264_recon_motion.argtypes = [i32, i32, vp, vp, i32, vp, vp, vp, vp, vp, vp, vp, i32]
        _lib.oracle_h264_recon_motion.restype = i32
        _lib.oracle_h264_deblock.argtypes = [i32, i32, vp, vp, vp, vp]
        _lib.oracle_h264_deblock.restype = None
        _lib.oracle_h264_idct4_add.argtypes = [vp, vp, i32]
        _lib.oracle_h264_idct8_add.argtypes = [vp, vp, i32]
        _lib.oracle_h264_luma_dc_dequant.argtypes = [vp, i32, ctypes.c_int32]
        _lib.oracle_h264_chroma_dc_dequant.argtypes = [vp, i32, ctypes.c_int32]
        _lib.oracle_h264_level_scale.argtypes = [vp, vp, vp, vp]
        _lib.oracle_h264_mc_luma.argtypes = [vp, i32, i32, i32, i32, i32, i32, i32, i32, vp, i32]
        _lib.oracle_h264_mc_chroma.argtypes = [vp, i32, i32, i32, i32, i32, i32, i32, i32, vp, i32]
        _lib.oracle_hevc_recon.argtypes = [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, i32]
        _lib.oracle_hevc_recon.restype = i32
        _lib.oracle_hevc_inverse.argtypes = [vp, i32, i32, i32, i32, i32]
        _lib.oracle_hevc_inverse_dc.argtypes = [i32, i32]
        _lib.oracle_hevc_inverse_dc.restype = i32
        _lib.oracle_hevc_intra_predict_refs.argtypes = [vp, vp, i32, i32, i32, i32, i32, vp]
    return _lib


COLMB_BYTES = 172  # sizeof(oracle_h264_colmb)


class H264Dpb:
    """CPU decoded-picture buffer: planes per slot at the coded size, and
    each slot's co-located motion (for pictures whose motion is derived
    from motion syntax, rc_h264_picture.motion)."""

    def __init__(self, mb_w: int, mb_h: int, slots: int):
        self.mb_w, self.mb_h, self.slots = mb_w, mb_h, slots
        W, H = mb_w * 16, mb_h * 16
        self.y = [np.zeros((H, W), np.uint8) for _ in range(slots)]
        self.u = [np.zeros((H // 2, W // 2), np.uint8) for _ in range(slots)]
        self.v = [np.zeros((H // 2, W // 2), np.uint8) for _ in range(slots)]
        self.col = [None] * slots

    def _ptrs(self, planes):
        arr = (ctypes.c_void_p * self.slots)(*[p.ctypes.data for p in planes])
        return arr

    def recon(self, picture_ptr: int, out_slot: int, filter: bool = True) -> int:
        L = lib()
        ry, ru, rv = self._ptrs(self.y), self._ptrs(self.u), self._ptrs(self.v)
        # the output slot is never its own reference: reconstruct into fresh planes
        y = self.y[out_slot].copy()
        u = self.u[out_slot].copy()
        v = self.v[out_slot].copy()
        col = (ctypes.c_void_p * self.slots)(*[c.ctypes.data if c is not None else None for c in self.col])
        out_col = np.zeros(self.mb_w * self.mb_h * COLMB_BYTES, np.uint8)
        rc = L.oracle_h264_recon_motion(self.mb_w, self.mb_h, picture_ptr, col, self.slots, out_col.ctypes.data,
                                        ry, ru, rv, y.ctypes.data, u.ctypes.data, v.ctypes.data, int(filter))
        if rc == 0:
            self.y[out_slot], self.u[out_slot], self.v[out_slot] = y, u, v
            self.col[out_slot] = out_col
        return rc

    def planes(self, slot: int):
        return self.y[slot], self.u[slot], self.v[slot]


class HevcDpb:
    """CPU decoded-picture buffer for HEVC: uint16 planes per slot."""

    def __init__(self, width: int, height: int, bit_depth: int, slots: int):
        self.W, self.H, self.bd, self.slots = width, height, bit_depth, slots
        self.y = [np.zeros((height, width), np.uint16) for _ in range(slots)]
        self.u = [np.zeros((height // 2, width // 2), np.uint16) for _ in range(slots)]
        self.v = [np.zeros((height // 2, width // 2), np.uint16) for _ in range(slots)]

    def recon(self, picture_ptr: int, out_slot: int, stages: int = 3) -> int:
        L = lib()
        arr = lambda planes: (ctypes.c_void_p * self.slots)(*[p.ctypes.data for p in planes])
        y = self.y[out_slot].copy()
        u = self.u[out_slot].copy()
        v = self.v[out_slot].copy()
        rc = L.oracle_hevc_recon(self.W, self.H, self.bd, picture_ptr, arr(self.y), arr(self.u), arr(self.v),
                                 y.ctypes.data, u.ctypes.data, v.ctypes.data, stages)
        if rc == 0:
            self.y[out_slot], self.u[out_slot], self.v[out_slot] = y, u, v
        return rc

    def planes(self, slot: int):
        return self.y[slot], self.u[slot], self.v[slot]
