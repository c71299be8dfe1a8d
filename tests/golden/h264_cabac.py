"""H.264 Main / High (CABAC) parse into reconstruction records.

TEST INFRASTRUCTURE: this module turns an H.264 Main- or High-profile
elementary stream (progressive, 4:2:0, 8-bit, CABAC) into the per-picture
syntax records of include/pito_recon.h (rc_h264_mb, rc_h264_slice,
rc_h264_weight, levels, scaling matrices), so that the reference's golden
x264 streams (tests/refs/h264/{main_cabac_b,high_bpyramid,high_crop_slices}
.h264) can drive the oracle and the GPU engine end to end.  It restates, in
this project's own code, the parse half of the reference decoder:

  parameter sets, slice headers, scaling lists   src/syntax/h264/{params,slice}.rs
  POC, reference marking and lists               src/syntax/h264/dpb.rs, src/h264/dec/decoder.rs
  CABAC engine and macroblock layer              src/h264/dec/{cabac,cabac_mb}.rs
  MV prediction, direct modes, implicit weights  src/h264/dec/slicedec.rs:411-471,473-937

following ITU-T H.264 clauses 7.3-7.4, 8.2, 8.4.1-8.4.2 and 9.3: I, P and
B slices; I4x4 / I8x8 / I16x16 / I_PCM; P and B partitions down to 4x4 with
MV prediction; spatial and temporal direct (direct_8x8_inference); explicit
and implicit weighted prediction; the 8x8 transform; sequence and picture
scaling matrices with the fall-back rules; several slices per picture;
short-term references with sliding-window and memory-management marking.
Field coding, MBAFF, long-term references and data partitioning raise
NotImplementedError.  Nothing in the engine imports it.
"""
from __future__ import annotations

import array

from h264_cavlc import _BLK_RASTER, _QPC, Bits, nal_units
from hevc_cabac import _LPS_BY_STATE, _NEXT_LPS, _NEXT_MPS

# ---------------------------------------------------------------------------
# Tables
# ---------------------------------------------------------------------------
# (m, n) of ctxIdx 0..459, flattened m0, n0, m1, n1, ... per table (H.264 Tables
# 9-12..9-33, frame-coded contexts; entries a slice type never uses hold 0, 0).
_MN = [
    # cabac_init_idc 0 (P, B)
    [20, -15, 2, 54, 3, 74, 20, -15, 2, 54, 3, 74, -28, 127, -23, 104, -6, 53, -1, 54, 7, 51, 23, 33, 23, 2, 21,
     0, 1, 9, 0, 49, -37, 118, 5, 57, -13, 78, -11, 65, 1, 62, 12, 49, -4, 73, 17, 50, 18, 64, 9, 43, 29, 0, 26,
     67, 16, 90, 9, 104, -46, 127, -20, 104, 1, 67, -13, 78, -11, 65, 1, 62, -6, 86, -17, 95, -6, 61, 9, 45, -3,
     69, -6, 81, -11, 96, 6, 55, 7, 67, -5, 86, 2, 88, 0, 58, -3, 76, -10, 94, 5, 54, 4, 69, -3, 81, 0, 88, -7,
     67, -5, 74, -4, 74, -5, 80, -7, 72, 1, 58, 0, 41, 0, 63, 0, 63, 0, 63, -9, 83, 4, 86, 0, 97, -7, 72, 13, 41,
     3, 62, 0, 45, -4, 78, -3, 96, -27, 126, -28, 98, -25, 101, -23, 67, -28, 82, -20, 94, -16, 83, -22, 110, -21,
     91, -18, 102, -13, 93, -29, 127, -7, 92, -5, 89, -7, 96, -13, 108, -3, 46, -1, 65, -1, 57, -9, 93, -3, 74,
     -9, 92, -8, 87, -23, 126, 5, 54, 6, 60, 6, 59, 6, 69, -1, 48, 0, 68, -4, 69, -8, 88, -2, 85, -6, 78, -1, 75,
     -7, 77, 2, 54, 5, 50, -3, 68, 1, 50, 6, 42, -4, 81, 1, 63, -4, 70, 0, 67, 2, 57, -2, 76, 11, 35, 4, 64, 1,
     61, 11, 35, 18, 25, 12, 24, 13, 29, 13, 36, -10, 93, -7, 73, -2, 73, 13, 46, 9, 49, -7, 100, 9, 53, 2, 53, 5,
     53, -2, 61, 0, 56, 0, 56, -13, 63, -5, 60, -1, 62, 4, 57, -6, 69, 4, 57, 14, 39, 4, 51, 13, 68, 3, 64, 1, 61,
     9, 63, 7, 50, 16, 39, 5, 44, 4, 52, 11, 48, -5, 60, -1, 59, 0, 59, 22, 33, 5, 44, 14, 43, -1, 78, 0, 60, 9,
     69, 11, 28, 2, 40, 3, 44, 0, 49, 0, 46, 2, 44, 2, 51, 0, 47, 4, 39, 2, 62, 6, 46, 0, 54, 3, 54, 2, 58, 4, 63,
     6, 51, 6, 57, 7, 53, 6, 52, 6, 55, 11, 45, 14, 36, 8, 53, -1, 82, 7, 55, -3, 78, 15, 46, 22, 31, -1, 84, 25,
     7, 30, -7, 28, 3, 28, 4, 32, 0, 34, -1, 30, 6, 30, 6, 32, 9, 31, 19, 26, 27, 26, 30, 37, 20, 28, 34, 17, 70,
     1, 67, 5, 59, 9, 67, 16, 30, 18, 32, 18, 35, 22, 29, 24, 31, 23, 38, 18, 43, 20, 41, 11, 63, 9, 59, 9, 64,
     -1, 94, -2, 89, -9, 108, -6, 76, -2, 44, 0, 45, 0, 52, -3, 64, -2, 59, -4, 70, -4, 75, -8, 82, -17, 102, -9,
     77, 3, 24, 0, 42, 0, 48, 0, 55, -6, 59, -7, 71, -12, 83, -11, 87, -30, 119, 1, 58, -3, 29, -1, 36, 1, 38, 2,
     43, -6, 55, 0, 58, 0, 64, -3, 74, -10, 90, 0, 70, -4, 29, 5, 31, 7, 42, 1, 59, -2, 58, -3, 72, -3, 81, -11,
     97, 0, 58, 8, 5, 10, 14, 14, 18, 13, 27, 2, 40, 0, 58, -3, 70, -6, 79, -8, 85, 0, 0, -13, 106, -16, 106, -10,
     87, -21, 114, -18, 110, -14, 98, -22, 110, -21, 106, -18, 103, -21, 107, -23, 108, -26, 112, -10, 96, -12,
     95, -5, 91, -9, 93, -22, 94, -5, 86, 9, 67, -4, 80, -10, 85, -1, 70, 7, 60, 9, 58, 5, 61, 12, 50, 15, 50, 18,
     49, 17, 54, 10, 41, 7, 46, -1, 51, 7, 49, 8, 52, 9, 41, 6, 47, 2, 55, 13, 41, 10, 44, 6, 50, 5, 53, 13, 49,
     4, 63, 6, 64, -2, 69, -2, 59, 6, 70, 10, 44, 9, 31, 12, 43, 3, 53, 14, 34, 10, 38, -3, 52, 13, 40, 17, 32, 7,
     44, 7, 38, 13, 50, 10, 57, 26, 43, 14, 11, 11, 14, 9, 11, 18, 11, 21, 9, 23, -2, 32, -15, 32, -15, 34, -21,
     39, -23, 42, -33, 41, -31, 46, -28, 38, -12, 21, 29, 45, -24, 53, -45, 48, -26, 65, -43, 43, -19, 39, -10,
     30, 9, 18, 26, 20, 27, 0, 57, -14, 82, -5, 75, -19, 97, -35, 125, 27, 0, 28, 0, 31, -4, 27, 6, 34, 8, 30, 10,
     24, 22, 33, 19, 22, 32, 26, 31, 21, 41, 26, 44, 23, 47, 16, 65, 14, 71, 8, 60, 6, 63, 17, 65, 21, 24, 23, 20,
     26, 23, 27, 32, 28, 23, 28, 24, 23, 40, 24, 32, 28, 29, 23, 42, 19, 57, 22, 53, 22, 61, 11, 86, 12, 40, 11,
     51, 14, 59, -4, 79, -7, 71, -5, 69, -9, 70, -8, 66, -10, 68, -19, 73, -12, 69, -16, 70, -15, 67, -20, 62,
     -19, 70, -16, 66, -22, 65, -20, 63, 9, -2, 26, -9, 33, -9, 39, -7, 41, -2, 45, 3, 49, 9, 45, 27, 36, 59, -6,
     66, -7, 35, -7, 42, -8, 45, -5, 48, -12, 56, -6, 60, -5, 62, -8, 66, -8, 76, -5, 85, -6, 81, -10, 77, -7, 81,
     -17, 80, -18, 73, -4, 74, -10, 83, -9, 71, -9, 67, -1, 61, -8, 66, -14, 66, 0, 59, 2, 59, 21, -13, 33, -14,
     39, -7, 46, -2, 51, 2, 60, 6, 61, 17, 55, 34, 42, 62],
    # cabac_init_idc 1 (P, B)
    [20, -15, 2, 54, 3, 74, 20, -15, 2, 54, 3, 74, -28, 127, -23, 104, -6, 53, -1, 54, 7, 51, 22, 25, 34, 0, 16,
     0, -2, 9, 4, 41, -29, 118, 2, 65, -6, 71, -13, 79, 5, 52, 9, 50, -3, 70, 10, 54, 26, 34, 19, 22, 40, 0, 57,
     2, 41, 36, 26, 69, -45, 127, -15, 101, -4, 76, -6, 71, -13, 79, 5, 52, 6, 69, -13, 90, 0, 52, 8, 43, -2, 69,
     -5, 82, -10, 96, 2, 59, 2, 75, -3, 87, -3, 100, 1, 56, -3, 74, -6, 85, 0, 59, -3, 81, -7, 86, -5, 95, -1, 66,
     -1, 77, 1, 70, -2, 86, -5, 72, 0, 61, 0, 41, 0, 63, 0, 63, 0, 63, -9, 83, 4, 86, 0, 97, -7, 72, 13, 41, 3,
     62, 13, 15, 7, 51, 2, 80, -39, 127, -18, 91, -17, 96, -26, 81, -35, 98, -24, 102, -23, 97, -27, 119, -24, 99,
     -21, 110, -18, 102, -36, 127, 0, 80, -5, 89, -7, 94, -4, 92, 0, 39, 0, 65, -15, 84, -35, 127, -2, 73, -12,
     104, -9, 91, -31, 127, 3, 55, 7, 56, 7, 55, 8, 61, -3, 53, 0, 68, -7, 74, -9, 88, -13, 103, -13, 91, -9, 89,
     -14, 92, -8, 76, -12, 87, -23, 110, -24, 105, -10, 78, -20, 112, -17, 99, -78, 127, -70, 127, -50, 127, -46,
     127, -4, 66, -5, 78, -4, 71, -8, 72, 2, 59, -1, 55, -7, 70, -6, 75, -8, 89, -34, 119, -3, 75, 32, 20, 30, 22,
     -44, 127, 0, 54, -5, 61, 0, 58, -1, 60, -3, 61, -8, 67, -25, 84, -14, 74, -5, 65, 5, 52, 2, 57, 0, 61, -9,
     69, -11, 70, 18, 55, -4, 71, 0, 58, 7, 61, 9, 41, 18, 25, 9, 32, 5, 43, 9, 47, 0, 44, 0, 51, 2, 46, 19, 38,
     -4, 66, 15, 38, 12, 42, 9, 34, 0, 89, 4, 45, 10, 28, 10, 31, 33, -11, 52, -43, 18, 15, 28, 0, 35, -22, 38,
     -25, 34, 0, 39, -18, 32, -12, 102, -94, 0, 0, 56, -15, 33, -4, 29, 10, 37, -5, 51, -29, 39, -9, 52, -34, 69,
     -58, 67, -63, 44, -5, 32, 7, 55, -29, 32, 1, 0, 0, 27, 36, 33, -25, 34, -30, 36, -28, 38, -28, 38, -27, 34,
     -18, 35, -16, 34, -14, 32, -8, 37, -6, 35, 0, 30, 10, 28, 18, 26, 25, 29, 41, 0, 75, 2, 72, 8, 77, 14, 35,
     18, 31, 17, 35, 21, 30, 17, 45, 20, 42, 18, 45, 27, 26, 16, 54, 7, 66, 16, 56, 11, 73, 10, 67, -10, 116, -23,
     112, -15, 71, -7, 61, 0, 53, -5, 66, -11, 77, -9, 80, -9, 84, -10, 87, -34, 127, -21, 101, -3, 39, -5, 53,
     -7, 61, -11, 75, -15, 77, -17, 91, -25, 107, -25, 111, -28, 122, -11, 76, -10, 44, -10, 52, -10, 57, -9, 58,
     -16, 72, -7, 69, -4, 69, -5, 74, -9, 86, 2, 66, -9, 34, 1, 32, 11, 31, 5, 52, -2, 55, -2, 67, 0, 73, -8, 89,
     3, 52, 7, 4, 10, 8, 17, 8, 16, 19, 3, 37, -1, 61, -5, 73, -1, 70, -4, 78, 0, 0, -21, 126, -23, 124, -20, 110,
     -26, 126, -25, 124, -17, 105, -27, 121, -27, 117, -17, 102, -26, 117, -27, 116, -33, 122, -10, 95, -14, 100,
     -8, 95, -17, 111, -28, 114, -6, 89, -2, 80, -4, 82, -9, 85, -8, 81, -1, 72, 5, 64, 1, 67, 9, 56, 0, 69, 1,
     69, 7, 69, -7, 69, -6, 67, -16, 77, -2, 64, 2, 61, -6, 67, -3, 64, 2, 57, -3, 65, -3, 66, 0, 62, 9, 51, -1,
     66, -2, 71, -2, 75, -1, 70, -9, 72, 14, 60, 16, 37, 0, 47, 18, 35, 11, 37, 12, 41, 10, 41, 2, 48, 12, 41, 13,
     41, 0, 59, 3, 50, 19, 40, 3, 66, 18, 50, 19, -6, 18, -6, 14, 0, 26, -12, 31, -16, 33, -25, 33, -22, 37, -28,
     39, -30, 42, -30, 47, -42, 45, -36, 49, -34, 41, -17, 32, 9, 69, -71, 63, -63, 66, -64, 77, -74, 54, -39, 52,
     -35, 41, -10, 36, 0, 40, -1, 30, 14, 28, 26, 23, 37, 12, 55, 11, 65, 37, -33, 39, -36, 40, -37, 38, -30, 46,
     -33, 42, -30, 40, -24, 49, -29, 38, -12, 40, -10, 38, -3, 46, -5, 31, 20, 29, 30, 25, 44, 12, 48, 11, 49, 26,
     45, 22, 22, 23, 22, 27, 21, 33, 20, 26, 28, 30, 24, 27, 34, 18, 42, 25, 39, 18, 50, 12, 70, 21, 54, 14, 71,
     11, 83, 25, 32, 21, 49, 21, 54, -5, 85, -6, 81, -10, 77, -7, 81, -17, 80, -18, 73, -4, 74, -10, 83, -9, 71,
     -9, 67, -1, 61, -8, 66, -14, 66, 0, 59, 2, 59, 17, -10, 32, -13, 42, -9, 49, -5, 53, 0, 64, 3, 68, 10, 66,
     27, 47, 57, -5, 71, 0, 24, -1, 36, -2, 42, -2, 52, -9, 57, -6, 63, -4, 65, -4, 67, -7, 82, -3, 81, -3, 76,
     -7, 72, -6, 78, -12, 72, -14, 68, -3, 70, -6, 76, -5, 66, -5, 62, 0, 57, -4, 61, -9, 60, 1, 54, 2, 58, 17,
     -10, 32, -13, 42, -9, 49, -5, 53, 0, 64, 3, 68, 10, 66, 27, 47, 57],
    # cabac_init_idc 2 (P, B)
    [20, -15, 2, 54, 3, 74, 20, -15, 2, 54, 3, 74, -28, 127, -23, 104, -6, 53, -1, 54, 7, 51, 29, 16, 25, 0, 14,
     0, -10, 51, -3, 62, -27, 99, 26, 16, -4, 85, -24, 102, 5, 57, 6, 57, -17, 73, 14, 57, 20, 40, 20, 10, 29, 0,
     54, 0, 37, 42, 12, 97, -32, 127, -22, 117, -2, 74, -4, 85, -24, 102, 5, 57, -6, 93, -14, 88, -6, 44, 4, 55,
     -11, 89, -15, 103, -21, 116, 19, 57, 20, 58, 4, 84, 6, 96, 1, 63, -5, 85, -13, 106, 5, 63, 6, 75, -3, 90, -1,
     101, 3, 55, -4, 79, -2, 75, -12, 97, -7, 50, 1, 60, 0, 41, 0, 63, 0, 63, 0, 63, -9, 83, 4, 86, 0, 97, -7, 72,
     13, 41, 3, 62, 7, 34, -9, 88, -20, 127, -36, 127, -17, 91, -14, 95, -25, 84, -25, 86, -12, 89, -17, 91, -31,
     127, -14, 76, -18, 103, -13, 90, -37, 127, 11, 80, 5, 76, 2, 84, 5, 78, -6, 55, 4, 61, -14, 83, -37, 127, -5,
     79, -11, 104, -11, 91, -30, 127, 0, 65, -2, 79, 0, 72, -4, 92, -6, 56, 3, 68, -8, 71, -13, 98, -4, 86, -12,
     88, -5, 82, -3, 72, -4, 67, -8, 72, -16, 89, -9, 69, -1, 59, 5, 66, 4, 57, -4, 71, -2, 71, 2, 58, -1, 74, -4,
     44, -1, 69, 0, 62, -7, 51, -4, 47, -6, 42, -3, 41, -6, 53, 8, 76, -9, 78, -11, 83, 9, 52, 0, 67, -5, 90, 1,
     67, -15, 72, -5, 75, -8, 80, -21, 83, -21, 64, -13, 31, -25, 64, -29, 94, 9, 75, 17, 63, -8, 74, -5, 35, -2,
     27, 13, 91, 3, 65, -7, 69, 8, 77, -10, 66, 3, 62, -3, 68, -20, 81, 0, 30, 1, 7, -3, 23, -21, 74, 16, 66, -23,
     124, 17, 37, 44, -18, 50, -34, -22, 127, 4, 39, 0, 42, 7, 34, 11, 29, 8, 31, 6, 37, 7, 42, 3, 40, 8, 33, 13,
     43, 13, 36, 4, 47, 3, 55, 2, 58, 6, 60, 8, 44, 11, 44, 14, 42, 7, 48, 4, 56, 4, 52, 13, 37, 9, 49, 19, 58,
     10, 48, 12, 45, 0, 69, 20, 33, 8, 63, 35, -18, 33, -25, 28, -3, 24, 10, 27, 0, 34, -14, 52, -44, 39, -24, 19,
     17, 31, 25, 36, 29, 24, 33, 34, 15, 30, 20, 22, 73, 20, 34, 19, 31, 27, 44, 19, 16, 15, 36, 15, 36, 21, 28,
     25, 21, 30, 20, 31, 12, 27, 16, 24, 42, 0, 93, 14, 56, 15, 57, 26, 38, -24, 127, -24, 115, -22, 82, -9, 62,
     0, 53, 0, 59, -14, 85, -13, 89, -13, 94, -11, 92, -29, 127, -21, 100, -14, 57, -12, 67, -11, 71, -10, 77,
     -21, 85, -16, 88, -23, 104, -15, 98, -37, 127, -10, 82, -8, 48, -8, 61, -8, 66, -7, 70, -14, 75, -10, 79, -9,
     83, -12, 92, -18, 108, -4, 79, -22, 69, -16, 75, -2, 58, 1, 58, -13, 78, -9, 83, -4, 81, -13, 99, -13, 81,
     -6, 38, -13, 62, -6, 58, -2, 59, -16, 73, -10, 76, -13, 86, -9, 83, -10, 87, 0, 0, -22, 127, -25, 127, -25,
     120, -27, 127, -19, 114, -23, 117, -25, 118, -26, 117, -24, 113, -28, 118, -31, 120, -37, 124, -10, 94, -15,
     102, -10, 99, -13, 106, -50, 127, -5, 92, 17, 57, -5, 86, -13, 94, -12, 91, -2, 77, 0, 71, -1, 73, 4, 64, -7,
     81, 5, 64, 15, 57, 1, 67, 0, 68, -10, 67, 1, 68, 0, 77, 2, 64, 0, 68, -5, 78, 7, 55, 5, 59, 2, 65, 14, 54,
     15, 44, 5, 60, 2, 70, -2, 76, -18, 86, 12, 70, 5, 64, -12, 70, 11, 55, 5, 56, 0, 69, 2, 65, -6, 74, 5, 54, 7,
     54, -6, 76, -11, 82, -2, 77, -2, 77, 25, 42, 17, -13, 16, -9, 17, -12, 27, -21, 37, -30, 41, -40, 42, -41,
     48, -47, 39, -32, 46, -40, 52, -51, 46, -41, 52, -39, 43, -19, 32, 11, 61, -55, 56, -46, 62, -50, 81, -67,
     45, -20, 35, -2, 28, 15, 34, 1, 39, 1, 30, 17, 20, 38, 18, 45, 15, 54, 0, 79, 36, -16, 37, -14, 37, -17, 32,
     1, 34, 15, 29, 15, 24, 25, 34, 22, 31, 16, 35, 18, 31, 28, 33, 41, 36, 28, 27, 47, 21, 62, 18, 31, 19, 26,
     36, 24, 24, 23, 27, 16, 24, 30, 31, 29, 22, 41, 22, 42, 16, 60, 15, 52, 14, 60, 3, 78, -16, 123, 21, 53, 22,
     56, 25, 61, 21, 33, 19, 50, 17, 61, -3, 78, -8, 74, -9, 72, -10, 72, -18, 75, -12, 71, -11, 63, -5, 70, -17,
     75, -14, 72, -16, 67, -8, 53, -14, 59, -9, 52, -11, 68, 9, -2, 30, -10, 31, -4, 33, -1, 33, 7, 31, 12, 37,
     23, 31, 38, 20, 64, -9, 71, -7, 37, -8, 44, -11, 49, -10, 56, -12, 59, -8, 63, -9, 67, -6, 68, -10, 79, -3,
     78, -8, 74, -9, 72, -10, 72, -18, 75, -12, 71, -11, 63, -5, 70, -17, 75, -14, 72, -16, 67, -8, 53, -14, 59,
     -9, 52, -11, 68, 9, -2, 30, -10, 31, -4, 33, -1, 33, 7, 31, 12, 37, 23, 31, 38, 20, 64],
    # I slices
    [20, -15, 2, 54, 3, 74, 20, -15, 2, 54, 3, 74, -28, 127, -23, 104, -6, 53, -1, 54, 7, 51, 0, 0, 0, 0, 0, 0, 0,
     0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
     0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
     0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 41, 0, 63, 0, 63, 0, 63, -9, 83, 4, 86, 0, 97,
     -7, 72, 13, 41, 3, 62, 0, 11, 1, 55, 0, 69, -17, 127, -13, 102, 0, 82, -7, 74, -21, 107, -27, 127, -31, 127,
     -24, 127, -18, 95, -27, 127, -21, 114, -30, 127, -17, 123, -12, 115, -16, 122, -11, 115, -12, 63, -2, 68,
     -15, 84, -13, 104, -3, 70, -8, 93, -10, 90, -30, 127, -1, 74, -6, 97, -7, 91, -20, 127, -4, 56, -5, 82, -7,
     76, -22, 125, -7, 93, -11, 87, -3, 77, -5, 71, -4, 63, -4, 68, -12, 84, -7, 62, -7, 65, 8, 61, 5, 56, -2, 66,
     1, 64, 0, 61, -2, 78, 1, 50, 7, 52, 10, 35, 0, 44, 11, 38, 1, 45, 0, 46, 5, 44, 31, 17, 1, 51, 7, 50, 28, 19,
     16, 33, 14, 62, -13, 108, -15, 100, -13, 101, -13, 91, -12, 94, -10, 88, -16, 84, -10, 86, -7, 83, -13, 87,
     -19, 94, 1, 70, 0, 72, -5, 74, 18, 59, -8, 102, -15, 100, 0, 95, -4, 75, 2, 72, -11, 75, -3, 71, 15, 46, -13,
     69, 0, 62, 0, 65, 21, 37, -15, 72, 9, 57, 16, 54, 0, 62, 12, 72, 24, 0, 15, 9, 8, 25, 13, 18, 15, 9, 13, 19,
     10, 37, 12, 18, 6, 29, 20, 33, 15, 30, 4, 45, 1, 58, 0, 62, 7, 61, 12, 38, 11, 45, 15, 39, 11, 42, 13, 44,
     16, 45, 12, 41, 10, 49, 30, 34, 18, 42, 10, 55, 17, 51, 17, 46, 0, 89, 26, -19, 22, -17, 26, -17, 30, -25,
     28, -20, 33, -23, 37, -27, 33, -23, 40, -28, 38, -17, 33, -11, 40, -15, 41, -6, 38, 1, 41, 17, 30, -6, 27, 3,
     26, 22, 37, -16, 35, -4, 38, -8, 38, -3, 37, 3, 38, 5, 42, 0, 35, 16, 39, 22, 14, 48, 27, 37, 21, 60, 12, 68,
     2, 97, -3, 71, -6, 42, -5, 50, -3, 54, -2, 62, 0, 58, 1, 63, -2, 72, -1, 74, -9, 91, -5, 67, -5, 27, -3, 39,
     -2, 44, 0, 46, -16, 64, -8, 68, -10, 78, -6, 77, -10, 86, -12, 92, -15, 55, -10, 60, -6, 62, -4, 65, -12, 73,
     -8, 76, -7, 80, -9, 88, -17, 110, -11, 97, -20, 84, -11, 79, -6, 73, -4, 74, -13, 86, -13, 96, -11, 97, -19,
     117, -8, 78, -5, 33, -4, 48, -2, 53, -3, 62, -13, 71, -10, 79, -12, 86, -13, 90, -14, 97, 0, 0, -6, 93, -6,
     84, -8, 79, 0, 66, -1, 71, 0, 62, -2, 60, -2, 59, -5, 75, -3, 62, -4, 58, -9, 66, -1, 79, 0, 71, 3, 68, 10,
     44, -7, 62, 15, 36, 14, 40, 16, 27, 12, 29, 1, 44, 20, 36, 18, 32, 5, 42, 1, 48, 10, 62, 17, 46, 9, 64, -12,
     104, -11, 97, -16, 96, -7, 88, -8, 85, -7, 85, -9, 85, -13, 88, 4, 66, -3, 77, -3, 76, -6, 76, 10, 58, -1,
     76, -1, 83, -7, 99, -14, 95, 2, 95, 0, 76, -5, 74, 0, 70, -11, 75, 1, 68, 0, 65, -14, 73, 3, 62, 4, 62, -1,
     68, -13, 75, 11, 55, 5, 64, 12, 70, 15, 6, 6, 19, 7, 16, 12, 14, 18, 13, 13, 11, 13, 15, 15, 16, 12, 23, 13,
     23, 15, 20, 14, 26, 14, 44, 17, 40, 17, 47, 24, 17, 21, 21, 25, 22, 31, 27, 22, 29, 19, 35, 14, 50, 10, 57,
     7, 63, -2, 77, -4, 82, -3, 94, 9, 69, -12, 109, 36, -35, 36, -34, 32, -26, 37, -30, 44, -32, 34, -18, 34,
     -15, 40, -15, 33, -7, 35, -5, 33, 0, 38, 2, 33, 13, 23, 35, 13, 58, 29, -3, 26, 0, 22, 30, 31, -7, 35, -15,
     34, -3, 34, 3, 36, -1, 34, 5, 32, 11, 35, 5, 34, 12, 39, 11, 30, 29, 34, 26, 29, 39, 19, 66, 31, 21, 31, 31,
     25, 50, -17, 120, -20, 112, -18, 114, -11, 85, -15, 92, -14, 89, -26, 71, -15, 81, -14, 80, 0, 68, -14, 70,
     -24, 56, -23, 68, -24, 50, -11, 74, 23, -13, 26, -13, 40, -15, 49, -14, 44, 3, 45, 6, 44, 34, 33, 54, 19, 82,
     -3, 75, -1, 23, 1, 34, 1, 43, 0, 54, -2, 55, 0, 61, 1, 64, 0, 68, -9, 92, -14, 106, -13, 97, -15, 90, -12,
     90, -18, 88, -10, 73, -9, 79, -14, 86, -10, 73, -10, 70, -10, 69, -5, 66, -9, 64, -5, 58, 2, 59, 21, -10, 24,
     -11, 28, -8, 28, -1, 29, 3, 29, 9, 35, 20, 29, 36, 14, 67],
]

# ctxIdxInc tables of significant_coeff_flag / last_significant_coeff_flag
# for 8x8 luma blocks in frame-coded macroblocks (Table 9-43)
_SIG8 = [0, 1, 2, 3, 4, 5, 5, 4, 4, 3, 3, 4, 4, 4, 5, 5, 4, 4, 4, 4, 3, 3, 6, 7, 7, 7, 8, 9, 10, 9, 8, 7, 7, 6, 11,
         12, 13, 11, 6, 7, 8, 9, 14, 10, 9, 8, 6, 11, 12, 13, 11, 6, 9, 14, 10, 9, 11, 12, 13, 11, 14, 10, 12]
_LAST8 = [0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 3, 3, 3,
          3, 3, 3, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5, 5, 5, 6, 6, 6, 6, 7, 7, 7, 7, 8, 8, 8]
# ctxIdxBlockCatOffset (Table 9-40) per ctxBlockCat 0..4
_CBF_OFF = [0, 4, 8, 12, 16]
_SIG_OFF = [0, 15, 29, 44, 47]
_ABS_OFF = [0, 10, 20, 30, 39]

# default scaling lists (Tables 7-3, 7-4), in zig-zag scan order
_DEF4_INTRA = [6, 13, 13, 20, 20, 20, 28, 28, 28, 28, 32, 32, 32, 37, 37, 42]
_DEF4_INTER = [10, 14, 14, 20, 20, 20, 24, 24, 24, 24, 27, 27, 27, 30, 30, 34]
_DEF8_INTRA = [6, 10, 10, 13, 11, 13, 16, 16, 16, 16, 18, 18, 18, 18, 18, 23, 23, 23, 23, 23, 23, 25, 25, 25, 25,
               25, 25, 25, 27, 27, 27, 27, 27, 27, 27, 27, 29, 29, 29, 29, 29, 29, 29, 31, 31, 31, 31, 31, 31, 33,
               33, 33, 33, 33, 36, 36, 36, 36, 38, 38, 38, 40, 40, 42]
_DEF8_INTER = [9, 13, 13, 15, 13, 15, 17, 17, 17, 17, 19, 19, 19, 19, 19, 21, 21, 21, 21, 21, 21, 22, 22, 22, 22,
               22, 22, 22, 24, 24, 24, 24, 24, 24, 24, 24, 25, 25, 25, 25, 25, 25, 25, 27, 27, 27, 27, 27, 27, 28,
               28, 28, 28, 28, 30, 30, 30, 30, 32, 32, 32, 33, 33, 35]


def _zigzag(n):
    """Raster index of each zig-zag scan position of an n x n block."""
    out = []
    for s in range(2 * n - 1):
        cells = [(s - j, j) for j in range(n) if 0 <= s - j < n]  # (x, y) on anti-diagonal s
        if s % 2 == 0:
            cells = [(y, x) for (x, y) in cells]
        out.extend(y * n + x for (x, y) in cells)
    return out


_ZZ4, _ZZ8 = _zigzag(4), _zigzag(8)
assert _ZZ4 == [0, 1, 4, 8, 5, 2, 3, 6, 9, 12, 13, 10, 7, 11, 14, 15]


def _raster(lst, zz):
    out = [0] * len(lst)
    for k, v in enumerate(lst):
        out[zz[k]] = v
    return out


class Cabac:
    """The arithmetic decoder of 9.3.3.2 (9-bit offset register, one bit per
    renormalisation step: exact bit position after a terminating bin)."""

    def __init__(self, data: bytes, bitpos: int, qp: int, table: int):
        self.data, self.nbits = data, len(data) * 8
        mn = _MN[table]
        q = max(0, min(51, qp))
        self.st = []
        for i in range(460):
            m, n = mn[2 * i], mn[2 * i + 1]
            pre = max(1, min(126, ((m * q) >> 4) + n))
            self.st.append(((63 - pre) << 1) if pre <= 63 else (((pre - 64) << 1) | 1))
        self.start(bitpos)

    def start(self, bitpos):
        self.pos, self.rng, self.off = bitpos, 510, 0
        for _ in range(9):
            self.off = (self.off << 1) | self.bit()

    def bit(self):
        p = self.pos
        self.pos = p + 1
        return (self.data[p >> 3] >> (7 - (p & 7))) & 1 if p < self.nbits else 0

    def dec(self, ci):
        s = self.st[ci]
        lps = _LPS_BY_STATE[s][(self.rng >> 6) & 3]
        rng = self.rng - lps
        if self.off < rng:
            b = s & 1
            self.st[ci] = _NEXT_MPS[s]
        else:
            self.off -= rng
            rng = lps
            b = (s & 1) ^ 1
            self.st[ci] = _NEXT_LPS[s]
        while rng < 256:
            rng <<= 1
            self.off = (self.off << 1) | self.bit()
        self.rng = rng
        return b

    def byp(self):
        self.off = (self.off << 1) | self.bit()
        if self.off >= self.rng:
            self.off -= self.rng
            return 1
        return 0

    def term(self):
        self.rng -= 2
        if self.off >= self.rng:
            return 1
        while self.rng < 256:
            self.rng <<= 1
            self.off = (self.off << 1) | self.bit()
        return 0

    def eg(self, k):
        v = 0
        while self.byp():
            v += 1 << k
            k += 1
        while k > 0:
            k -= 1
            v += self.byp() << k
        return v


# ---------------------------------------------------------------------------
# Parameter sets and slice headers (7.3.2, 7.3.3)
# ---------------------------------------------------------------------------
def _scaling_list(b: Bits, size):
    last, nxt, out, use_default = 8, 8, [], False
    for j in range(size):
        if nxt != 0:
            nxt = (last + b.se() + 256) % 256
            use_default = j == 0 and nxt == 0
        out.append(last if nxt == 0 else nxt)
        last = out[-1]
    return None if use_default else out


def _matrices(b: Bits, count, fallback):
    """count scaling lists (zig-zag order) with fall-back rule A (fallback
    None) or B (fallback = the sequence-level lists)."""
    defaults = [_DEF4_INTRA, _DEF4_INTRA, _DEF4_INTRA, _DEF4_INTER, _DEF4_INTER, _DEF4_INTER, _DEF8_INTRA,
                _DEF8_INTER]
    out = []
    for i in range(count):
        present = b.u(1)
        lst = _scaling_list(b, 16 if i < 6 else 64) if present else "absent"
        if lst is None:  # useDefaultScalingMatrixFlag
            lst = list(defaults[i])
        elif lst == "absent":
            if i in (0, 3, 6, 7):
                lst = list(defaults[i]) if fallback is None else list(fallback[i])
            else:
                lst = list(out[i - 1])
        out.append(lst)
    return out


def parse_sps(b: Bits) -> dict:
    s = {"profile_idc": b.u(8)}
    b.u(8)
    b.u(8)
    s["id"] = b.ue()
    s["scaling"] = None
    if s["profile_idc"] in (100, 110, 122, 244, 44, 83, 86, 118, 128, 138, 139, 134, 135):
        if b.ue() != 1:
            raise NotImplementedError("chroma format other than 4:2:0")
        if b.ue() != 0 or b.ue() != 0:
            raise NotImplementedError("bit depth above 8")
        if b.u(1):
            raise NotImplementedError("transform bypass")
        if b.u(1):
            s["scaling"] = _matrices(b, 8, None)
    s["log2_max_frame_num"] = b.ue() + 4
    s["poc_type"] = b.ue()
    if s["poc_type"] == 0:
        s["log2_max_poc_lsb"] = b.ue() + 4
    elif s["poc_type"] == 1:
        raise NotImplementedError("POC type 1")
    s["max_num_ref_frames"] = b.ue()
    b.u(1)
    s["mb_w"], s["mb_h"] = b.ue() + 1, b.ue() + 1
    if not b.u(1):
        raise NotImplementedError("field coding")
    s["direct_8x8_inference"] = b.u(1)
    s["crop"] = (0, 0, 0, 0)
    if b.u(1):
        s["crop"] = (b.ue(), b.ue(), b.ue(), b.ue())
    return s


def parse_pps(b: Bits, spss) -> dict:
    p = {"id": b.ue(), "sps_id": b.ue()}
    p["cabac"] = b.u(1)
    p["bottom_field_poc"] = b.u(1)
    if b.ue() != 0:
        raise NotImplementedError("slice groups")
    p["num_ref"] = (b.ue() + 1, b.ue() + 1)
    p["weighted_pred"] = b.u(1)
    p["weighted_bipred"] = b.u(2)
    p["init_qp"] = 26 + b.se()
    b.se()
    p["cqp"] = b.se()
    p["deblock_ctrl"] = b.u(1)
    p["constrained_intra"] = b.u(1)
    if b.u(1):
        raise NotImplementedError("redundant pictures")
    p["t8"] = 0
    p["cqp2"] = p["cqp"]
    p["scaling"] = None
    if b.more_rbsp_data():
        p["t8"] = b.u(1)
        if b.u(1):
            # absent lists fall back by rule A (the default lists) when the
            # SPS carries no matrices, else by rule B (the SPS's lists)
            seq = spss[p["sps_id"]]["scaling"]
            got = _matrices(b, 6 + 2 * p["t8"], seq)
            if len(got) < 8:
                got += [list(seq[6]), list(seq[7])] if seq else [list(_DEF8_INTRA), list(_DEF8_INTER)]
            p["scaling"] = got
        p["cqp2"] = b.se()
    return p


def parse_slice_header(b: Bits, nal_type, ref_idc, spss, ppss) -> dict:
    h = {"first_mb": b.ue(), "type": b.ue() % 5, "pps_id": b.ue()}  # type 0 P, 1 B, 2 I
    if h["type"] > 2:
        raise NotImplementedError("SP / SI slices")
    pps = ppss[h["pps_id"]]
    sps = spss[pps["sps_id"]]
    h["pps"], h["sps"] = pps, sps
    h["frame_num"] = b.u(sps["log2_max_frame_num"])
    h["idr"] = nal_type == 5
    h["ref_idc"] = ref_idc
    if h["idr"]:
        b.ue()
    h["poc_lsb"], h["delta_bottom"] = 0, 0
    if sps["poc_type"] == 0:
        h["poc_lsb"] = b.u(sps["log2_max_poc_lsb"])
        if pps["bottom_field_poc"]:
            h["delta_bottom"] = b.se()
    h["direct_spatial"] = b.u(1) if h["type"] == 1 else 0
    h["num_ref"] = [0, 0]
    if h["type"] != 2:
        h["num_ref"] = [pps["num_ref"][0], pps["num_ref"][1] if h["type"] == 1 else 0]
        if b.u(1):
            h["num_ref"][0] = b.ue() + 1
            if h["type"] == 1:
                h["num_ref"][1] = b.ue() + 1
    h["mods"] = [[], []]
    for l in range(2 if h["type"] == 1 else (1 if h["type"] == 0 else 0)):
        if b.u(1):
            while True:
                idc = b.ue()
                if idc == 3:
                    break
                if idc > 1:
                    raise NotImplementedError("long-term list modification")
                h["mods"][l].append((idc, b.ue() + 1))
    h["weights"] = None
    if (pps["weighted_pred"] and h["type"] == 0) or (pps["weighted_bipred"] == 1 and h["type"] == 1):
        lw, cw = b.ue(), b.ue()
        w = {"luma_log2": lw, "chroma_log2": cw, "l": []}
        for l in range(2 if h["type"] == 1 else 1):
            ents = []
            for _ in range(h["num_ref"][l]):
                yw, yo = 1 << lw, 0
                if b.u(1):
                    yw, yo = b.se(), b.se()
                cws, cos = [1 << cw, 1 << cw], [0, 0]
                if b.u(1):
                    for j in range(2):
                        cws[j], cos[j] = b.se(), b.se()
                ents.append((yw, yo, cws, cos))
            w["l"].append(ents)
        h["weights"] = w
    h["mmco"] = []
    if ref_idc:
        if h["idr"]:
            b.u(1)
            if b.u(1):
                raise NotImplementedError("long-term IDR")
        elif b.u(1):
            while True:
                op = b.ue()
                if op == 0:
                    break
                if op == 1:
                    h["mmco"].append((1, b.ue() + 1))
                elif op == 5:
                    h["mmco"].append((5, 0))
                else:
                    raise NotImplementedError(f"memory management operation {op}")
    h["cabac_init_idc"] = b.ue() if (pps["cabac"] and h["type"] != 2) else 0
    h["qp"] = pps["init_qp"] + b.se()
    h["deblock_idc"], h["alpha"], h["beta"] = 0, 0, 0
    if pps["deblock_ctrl"]:
        h["deblock_idc"] = b.ue()
        if h["deblock_idc"] != 1:
            h["alpha"], h["beta"] = b.se() * 2, b.se() * 2
    return h


# ---------------------------------------------------------------------------
# Decoding state
# ---------------------------------------------------------------------------
KIND_CODE = {"I4": 1, "I8": 2, "I16": 3, "PCM": 4}
# P partitions per mb_type 0..2; B partitions and their prediction lists
# (1 L0, 2 L1, 3 Bi) per mb_type 1..21 (Table 7-14)
_P_PARTS = {0: [(0, 0, 16, 16)], 1: [(0, 0, 16, 8), (0, 8, 16, 8)], 2: [(0, 0, 8, 16), (8, 0, 8, 16)]}
_B_TYPES = {1: (16, 16, (1,)), 2: (16, 16, (2,)), 3: (16, 16, (3,))}
for _i, (_a, _b) in enumerate([(1, 1), (2, 2), (1, 2), (2, 1), (1, 3), (2, 3), (3, 1), (3, 2), (3, 3)]):
    _B_TYPES[4 + 2 * _i] = (16, 8, (_a, _b))
    _B_TYPES[5 + 2 * _i] = (8, 16, (_a, _b))
# sub_mb_type: (width, height, prediction lists) -- P 0..3, B 1..12 (0 direct)
_P_SUB = {0: (8, 8, 1), 1: (8, 4, 1), 2: (4, 8, 1), 3: (4, 4, 1)}
_B_SUB = {1: (8, 8, 1), 2: (8, 8, 2), 3: (8, 8, 3), 4: (8, 4, 1), 5: (4, 8, 1), 6: (8, 4, 2), 7: (4, 8, 2),
          8: (8, 4, 3), 9: (4, 8, 3), 10: (4, 4, 1), 11: (4, 4, 2), 12: (4, 4, 3)}


class _Mb:
    __slots__ = ("slice", "kind", "skip", "direct16", "qp", "qpd", "cbp", "t8", "i16", "cmode", "modes", "ref",
                 "mv", "mvd", "direct", "cbf_dc", "cbf4", "cbfc", "levels", "dc", "luma_coded", "chroma_coded",
                 "nz", "wp", "btype", "syn")

    def __init__(self):
        self.slice = -1
        self.kind = None  # "I4" "I8" "I16" "PCM" "P" "B"
        self.skip = False
        self.direct16 = False  # B_Skip or B_Direct_16x16
        self.qp = self.qpd = self.cbp = self.t8 = self.i16 = self.cmode = 0
        self.modes = [2] * 16
        self.ref = [[-1] * 16, [-1] * 16]
        self.mv = [[(0, 0)] * 16, [(0, 0)] * 16]
        self.mvd = [[(0, 0)] * 16, [(0, 0)] * 16]
        self.direct = [False] * 16  # 4x4 blocks predicted in direct mode
        self.cbf_dc = 0
        self.cbf4 = [0] * 16
        self.cbfc = [[0] * 4, [0] * 4]
        self.levels = []
        self.dc = self.luma_coded = self.chroma_coded = self.nz = 0
        self.wp = [0xFF] * 4
        self.btype = -1  # B mb_type (0 B_Direct_16x16 .. 22 B_8x8)
        self.syn = None  # motion syntax: (shape, pred[4], sub[4]), RC_H264_MOTION_* / RC_H264_SUB_*


class Frame:
    """A decoded picture: identity, POC, DPB slot and what later pictures
    read of it (motion for the direct modes)."""

    def __init__(self, ident, frame_num, poc, slot):
        self.id, self.frame_num, self.poc, self.slot = ident, frame_num, poc, slot
        self.ref = True
        self.intra = None  # per MB
        self.ref_pic = None  # [list][mb][4x4] -> referenced Frame or None
        self.ref_idx = None  # [list][mb][4x4] -> index in the MB's slice list, -1 unused
        self.mv = None  # [list][mb][4x4]


class Decoder:
    """Parses a stream picture by picture into engine records."""

    def __init__(self, E, slots: int = 16):
        self.E = E
        self.spss, self.ppss = {}, {}
        self.refs: list[Frame] = []
        self.slots = slots
        self.count = 0
        self.pictures = []
        self.cur = None
        self.period = -1
        self.prev_ref_poc = (0, 0)  # (msb, lsb) of the previous reference picture

    # ---- stream -----------------------------------------------------------
    def decode(self, data: bytes):
        for ref_idc, t, rbsp in nal_units(data):
            b = Bits(rbsp)
            if t == 7:
                s = parse_sps(b)
                self.spss[s["id"]] = s
            elif t == 8:
                p = parse_pps(b, self.spss)
                self.ppss[p["id"]] = p
            elif t in (1, 5):
                h = parse_slice_header(b, t, ref_idc, self.spss, self.ppss)
                if not h["pps"]["cabac"]:
                    raise NotImplementedError("CAVLC (see h264_cavlc.py)")
                if h["first_mb"] == 0:
                    self._finish_picture()
                    self._start_picture(h)
                if h["mmco"]:
                    self.cur["mmco"] = h["mmco"]
                b.align()
                self._slice(h, rbsp, b.p)
            elif t in (6, 9, 10, 11, 12):
                continue
            else:
                raise NotImplementedError(f"NAL unit type {t}")
        self._finish_picture()
        return self.pictures

    # ---- picture ----------------------------------------------------------
    def _start_picture(self, h):
        sps, pps = h["sps"], h["pps"]
        self.sps, self.pps = sps, pps
        self.mb_w, self.mb_h = sps["mb_w"], sps["mb_h"]
        n = self.mb_w * self.mb_h
        self.mbs = [_Mb() for _ in range(n)]
        self.slices = []
        self.weights = []
        self.wkey = {}
        if h["idr"]:
            self.period += 1
            self.refs = []
            self.prev_ref_poc = (0, 0)
        # 8.2.1 picture order count (type 0)
        if sps["poc_type"] == 0:
            max_lsb = 1 << sps["log2_max_poc_lsb"]
            pmsb, plsb = self.prev_ref_poc
            lsb = h["poc_lsb"]
            if lsb < plsb and plsb - lsb >= max_lsb // 2:
                msb = pmsb + max_lsb
            elif lsb > plsb and lsb - plsb > max_lsb // 2:
                msb = pmsb - max_lsb
            else:
                msb = pmsb
            top = msb + lsb
            poc = min(top, top + h["delta_bottom"])
            if h["ref_idc"]:
                self.prev_ref_poc = (msb, lsb)
        else:  # type 2
            maxf = 1 << sps["log2_max_frame_num"]
            if h["idr"]:
                self.fn_offset = 0
            elif getattr(self, "prev_fn", 0) > h["frame_num"]:
                self.fn_offset = getattr(self, "fn_offset", 0) + maxf
            self.prev_fn = h["frame_num"]
            poc = 0 if h["idr"] else 2 * (getattr(self, "fn_offset", 0) + h["frame_num"]) - (0 if h["ref_idc"] else 1)
        used = {f.slot for f in self.refs}
        slot = next(s for s in range(self.slots) if s not in used)
        self.frame = Frame(self.count, h["frame_num"], poc, slot)
        self.cur = {"frame_num": h["frame_num"], "idr": h["idr"], "ref": bool(h["ref_idc"]), "mmco": None}

    def _finish_picture(self):
        if self.cur is None:
            return
        E = self.E
        f = self.frame
        n = len(self.mbs)
        recs = (E.H264Mb * n)()
        levels = []
        f.intra = [m.kind in ("I4", "I8", "I16", "PCM") for m in self.mbs]
        f.ref_pic = [[None] * n for _ in range(2)]
        f.ref_idx = [[None] * n for _ in range(2)]
        f.mv = [[None] * n for _ in range(2)]
        for a, m in enumerate(self.mbs):
            r = recs[a]
            if m.kind is None:
                r.kind = E.RC_H264_NONE
                continue
            r.kind = KIND_CODE.get(m.kind, E.RC_H264_INTER)
            r.transform_8x8 = m.t8
            r.qp = 0 if m.kind == "PCM" else m.qp
            r.qpc[0] = _QPC[max(0, min(51, r.qp + self.pps["cqp"]))]
            r.qpc[1] = _QPC[max(0, min(51, r.qp + self.pps["cqp2"]))]
            r.i16_mode, r.chroma_mode = m.i16, m.cmode
            r.dc_coded, r.slice, r.nz_mask = m.dc, m.slice, m.nz
            r.luma_coded, r.chroma_coded = m.luma_coded, m.chroma_coded
            r.coef_off = len(levels)
            levels.extend(m.levels)
            for i in range(16):
                r.intra_modes[i] = m.modes[i] if m.kind in ("I4", "I8") else 0
            inter = m.kind in ("P", "B")
            sl = self.slices[m.slice]
            for l in range(2):
                f.ref_pic[l][a] = [sl["list"][l][m.ref[l][k]] if (inter and m.ref[l][k] >= 0) else None
                                   for k in range(16)]
                f.ref_idx[l][a] = list(m.ref[l]) if inter else [-1] * 16
                f.mv[l][a] = list(m.mv[l]) if inter else [(0, 0)] * 16
            for b8 in range(4):
                k = (b8 >> 1) * 8 + (b8 & 1) * 2
                for l in range(2):
                    r.ref_idx[l][b8] = m.ref[l][k] if inter else -1
                r.wp[b8] = m.wp[b8] if inter else 0xFF
            for k in range(16):
                for l in range(2):
                    mx, my = m.mv[l][k] if (inter and m.ref[l][k] >= 0) else (0, 0)
                    r.mv[l][k][0], r.mv[l][k][1] = mx, my
        mos = (E.H264Motion * n)()
        for a, m in enumerate(self.mbs):
            if m.kind not in ("P", "B"):
                continue
            o = mos[a]
            o.shape = m.syn[0]
            for i in range(4):
                o.pred[i], o.sub[i] = m.syn[1][i], m.syn[2][i]
            for b8 in range(4):
                k = (b8 >> 1) * 8 + (b8 & 1) * 2
                for l in range(2):
                    o.ref_idx[l][b8] = -1 if (m.direct[k] or m.skip) else m.ref[l][k]
            for k in range(16):
                for l in range(2):
                    o.mvd[l][k][0], o.mvd[l][k][1] = m.mvd[l][k]
        smo = (E.H264SliceMotion * len(self.slices))()
        for i, s in enumerate(self.slices):
            for key, v in s["motion"].items():
                if isinstance(v, list):
                    arr = getattr(smo[i], key)
                    for j, x in enumerate(v):
                        arr[j] = x
                else:
                    setattr(smo[i], key, v)
        sl = (E.H264Slice * len(self.slices))()
        for i, s in enumerate(self.slices):
            sl[i].disable_deblocking_filter_idc = s["deblock_idc"]
            sl[i].alpha_offset, sl[i].beta_offset = s["alpha"], s["beta"]
            for l in range(2):
                sl[i].num_ref[l] = len(s["list"][l])
                for j, fr in enumerate(s["list"][l]):
                    sl[i].ref_slot[l][j] = fr.slot
                    sl[i].ref_id[l][j] = fr.id
        wts = (E.H264Weight * max(1, len(self.weights)))()
        for i, w in enumerate(self.weights):
            wts[i].explicit_mask = w["mask"]
            for c in range(3):
                wts[i].log_wd[c], wts[i].w0[c], wts[i].w1[c] = w["lwd"][c], w["w0"][c], w["w1"][c]
                wts[i].o0[c], wts[i].o1[c] = w["o0"][c], w["o1"][c]
        sc = self.pps["scaling"] or self.sps["scaling"]
        s4 = bytes(v for i in range(6) for v in _raster(sc[i], _ZZ4)) if sc else b""
        s8 = (bytes(v for i in (6, 7) for v in _raster(sc[i], _ZZ8)) + bytes([16] * 256)) if sc else b""
        self.pictures.append({
            "mbs": bytes(recs), "slices": bytes(sl), "weights": bytes(wts)[:64 * len(self.weights)],
            "motion": bytes(mos), "slice_motion": bytes(smo),
            "levels": array.array("h", levels).tobytes(), "scaling4": s4, "scaling8": s8,
            "num_slices": len(self.slices), "num_weights": len(self.weights), "slot": f.slot, "frame_id": f.id,
            "constrained_intra": self.pps["constrained_intra"], "mb_w": self.mb_w, "mb_h": self.mb_h,
            "crop": self.sps["crop"], "poc": f.poc, "period": self.period})
        # 8.2.5 reference marking
        if self.cur["ref"]:
            if self.cur["mmco"]:
                for op, diff in self.cur["mmco"]:
                    if op == 1:
                        pn = self.cur["frame_num"] - diff
                        self.refs = [g for g in self.refs if self._pic_num(g) != pn]
                    else:
                        raise NotImplementedError("memory management operation 5")
            elif not self.cur["idr"]:
                if len(self.refs) >= max(1, self.sps["max_num_ref_frames"]):
                    self.refs.remove(min(self.refs, key=self._pic_num))
            self.refs.append(f)
        self.count += 1
        self.cur = None

    def _pic_num(self, f):
        maxf = 1 << self.sps["log2_max_frame_num"]
        return f.frame_num - maxf if f.frame_num > self.cur["frame_num"] else f.frame_num

    def _ref_lists(self, h):
        """8.2.4: initial lists (P by PicNum, B by POC), then modifications."""
        lists = [[], []]
        if h["type"] == 0:
            lists[0] = sorted(self.refs, key=self._pic_num, reverse=True)
        elif h["type"] == 1:
            poc = self.frame.poc
            before = sorted((f for f in self.refs if f.poc < poc), key=lambda f: -f.poc)
            after = sorted((f for f in self.refs if f.poc > poc), key=lambda f: f.poc)
            lists[0], lists[1] = before + after, after + before
            if len(lists[1]) > 1 and lists[0] == lists[1]:
                lists[1][0], lists[1][1] = lists[1][1], lists[1][0]
        maxf = 1 << self.sps["log2_max_frame_num"]
        for l in range(2):
            n = h["num_ref"][l]
            # 8.2.4.3.1: the list is worked on with one spare entry; an inserted
            # picture removes only its later copies, so a picture may appear
            # more than once (explicit weighting gives each entry its own
            # weights); entries past the available references are "no
            # reference picture" and never used
            lst = (lists[l] + [None] * (n + 1))[: n + 1]
            pred, idx = self.cur["frame_num"], 0
            for idc, absdiff in h["mods"][l]:
                pn = pred - absdiff if idc == 0 else pred + absdiff
                pn = pn + maxf if pn < 0 else pn - maxf if pn >= maxf else pn
                pred = pn
                want = pn - maxf if pn > self.cur["frame_num"] else pn
                f = next(g for g in self.refs if self._pic_num(g) == want)
                lst = lst[:idx] + [f] + lst[idx:]
                idx += 1
                lst = (lst[:idx] + [x for x in lst[idx:] if x is not f] + [None] * (n + 1))[: n + 1]
            lst = lst[:n]
            while lst and lst[-1] is None:
                lst.pop()
            if None in lst:
                raise NotImplementedError("a missing reference inside the list")
            lists[l] = lst
        return lists

    # ---- slice data (7.3.4) ----------------------------------------------
    def _slice(self, h, rbsp, bitpos):
        self.h = h
        self.sid = len(self.slices)
        lists = self._ref_lists(h)
        self.lists = lists
        self.slices.append({"deblock_idc": h["deblock_idc"], "alpha": h["alpha"], "beta": h["beta"], "list": lists})
        self.slices[-1]["motion"] = self._slice_motion()
        table = 3 if h["type"] == 2 else h["cabac_init_idc"]
        c = Cabac(rbsp, bitpos, h["qp"], table)
        self.c = c
        qp = h["qp"]
        self.prev_addr = -1
        addr = h["first_mb"]
        n = len(self.mbs)
        while True:
            if addr >= n:
                raise ValueError("macroblock past the picture")
            m = self.mbs[addr]
            m.slice = self.sid
            skip = False
            if h["type"] != 2:
                base = 11 if h["type"] == 0 else 24
                inc = sum(1 for a in (self._mba(addr), self._mbb(addr)) if a >= 0 and not self.mbs[a].skip)
                skip = bool(c.dec(base + inc))
            if skip:
                m.skip = True
                m.qp = qp
                m.syn = (1, [0] * 4, [0] * 4)  # RC_H264_MOTION_SKIP
                if h["type"] == 0:
                    m.kind = "P"
                    self._p_skip(addr)
                else:
                    m.kind = "B"
                    m.direct16 = True
                    m.btype = 0
                    self._direct(addr, range(4))
                    self._weights_for(m)
            else:
                qp = self._macroblock(addr, qp)
            self.prev_addr = addr
            addr += 1
            if c.term():
                break
        # the slice data ends with its stop bit: the RBSP's last set bit lies
        # within the few flush bits after the terminating bin (encoders pad
        # the flush differently) and only zero bits follow
        last = len(rbsp) * 8 - 1
        while last >= 0 and not (rbsp[last >> 3] >> (7 - (last & 7))) & 1:
            last -= 1
        if not c.pos - 1 <= last <= c.pos + 15:
            raise ValueError(f"slice data ends at bit {c.pos}, its stop bit is at {last}")

    # ---- neighbours (6.4.9-6.4.11) ----------------------------------------
    def _avail(self, a, addr):
        return 0 <= a < addr and self.mbs[a].slice == self.sid

    def _mba(self, addr):
        return addr - 1 if addr % self.mb_w > 0 and self._avail(addr - 1, addr) else -1

    def _mbb(self, addr):
        return addr - self.mb_w if self._avail(addr - self.mb_w, addr) else -1

    def _nb(self, addr, dx, dy):
        x, y = addr % self.mb_w + dx, addr // self.mb_w + dy
        if x < 0 or y < 0 or x >= self.mb_w:
            return -1
        a = y * self.mb_w + x
        return a if self._avail(a, addr) else -1

    def _luma_nb(self, addr, x, y):
        """(MB, raster 4x4) of luma sample (x, y) relative to the MB, or (-1, 0)."""
        if y >= 16 or (x >= 16 and y >= 0):
            return -1, 0
        dx = -1 if x < 0 else 1 if x >= 16 else 0
        dy = -1 if y < 0 else 0
        a = addr if (dx == 0 and dy == 0) else self._nb(addr, dx, dy)
        if a < 0:
            return -1, 0
        return a, ((y % 16) >> 2) * 4 + ((x % 16) >> 2)

    # ---- macroblock layer (7.3.5) -----------------------------------------
    def _macroblock(self, addr, qp):
        c, h, m = self.c, self.h, self.mbs[addr]
        A, B = self._mba(addr), self._mbb(addr)
        if h["type"] == 2:
            mt = self._mb_type_i(3, A, B, True)
        elif h["type"] == 0:
            if c.dec(14):
                mt = self._mb_type_i(17, A, B, False)
            else:
                mt = ("P", (3 if c.dec(16) else 0) if not c.dec(15) else (1 if c.dec(17) else 2))
        else:
            mt = self._mb_type_b(A, B)
        kind, val = mt
        if kind == "PCM":
            at = (c.pos + 7) & ~7
            bb = Bits(c.data)
            bb.p = at
            m.kind, m.qp = "PCM", qp
            m.levels = [bb.u(8) for _ in range(384)]
            m.nz = 0xFFFF
            m.cbp = 0x2F
            m.cbf_dc = 7
            m.cbf4 = [1] * 16
            m.cbfc = [[1] * 4, [1] * 4]
            c.start(bb.p)
            return qp
        if kind == "I":
            return self._intra_mb(addr, val, qp)
        if kind == "P":
            self._inter_p(addr, val)
        else:
            self._inter_b(addr, val)
        cbp = self._cbp(addr)
        m.cbp = cbp
        if (cbp & 15) and self.pps["t8"] and self._no_sub_lt8(m):
            m.t8 = c.dec(399 + self._t8_inc(addr))
        return self._residual(addr, cbp, qp)

    def _mb_type_i(self, base, A, B, neighbours):
        """I mb_type binarization (Table 9-36), prefix-less; base 3 (I slice)
        or the suffix offsets 17 (P) / 32 (B)."""
        c = self.c
        if neighbours:
            inc = sum(1 for a in (A, B) if a >= 0 and self.mbs[a].kind != "I4" and self.mbs[a].kind != "I8")
            first = c.dec(base + inc)
            ctx = [base + 3, base + 4, base + 5, base + 6, base + 7]
        else:
            first = c.dec(base)
            ctx = [base + 1, base + 2, base + 2, base + 3, base + 3]
        if not first:
            return ("I", 0)
        if c.term():
            return ("PCM", 25)
        luma = c.dec(ctx[0])
        chroma = c.dec(ctx[1])
        if chroma:
            chroma = 1 + c.dec(ctx[2])
        p1 = c.dec(ctx[3])
        p0 = c.dec(ctx[4])
        return ("I", 1 + (p1 << 1 | p0) + 4 * chroma + 12 * luma)

    def _mb_type_b(self, A, B):
        c = self.c
        inc = sum(1 for a in (A, B) if a >= 0 and not self.mbs[a].direct16)
        if not c.dec(27 + inc):
            return ("B", 0)
        if not c.dec(27 + 3):
            return ("B", 1 + c.dec(27 + 5))
        bits = c.dec(27 + 4) << 3
        bits |= c.dec(27 + 5) << 2
        bits |= c.dec(27 + 5) << 1
        bits |= c.dec(27 + 5)
        if bits < 8:
            return ("B", bits + 3)
        if bits == 13:
            return self._mb_type_i(32, A, B, False)
        if bits == 14:
            return ("B", 11)
        if bits == 15:
            return ("B", 22)
        return ("B", ((bits << 1) | c.dec(27 + 5)) - 4)

    def _no_sub_lt8(self, m):
        if m.kind in ("P", "B") and self._subs is not None:
            for st in self._subs:
                if m.kind == "P" and st != 0:
                    return False
                if m.kind == "B" and st != 1 and st != 2 and st != 3 and not (st == 0 and self.sps["direct_8x8_inference"]):
                    return False
        if m.kind == "B" and m.direct16 and not self.sps["direct_8x8_inference"]:
            return False
        return True

    def _t8_inc(self, addr):
        return sum(1 for a in (self._mba(addr), self._mbb(addr)) if a >= 0 and self.mbs[a].t8)

    # ---- intra (7.3.5.1, 8.3.1.1, 8.3.2.1) ---------------------------------
    def _intra_mb(self, addr, mt, qp):
        c, m = self.c, self.mbs[addr]
        self._subs = None
        if mt == 0:
            m.t8 = c.dec(399 + self._t8_inc(addr)) if self.pps["t8"] else 0
            m.kind = "I8" if m.t8 else "I4"
            codes = []
            for _ in range(4 if m.t8 else 16):
                codes.append(-1 if c.dec(68) else (c.dec(69) | c.dec(69) << 1 | c.dec(69) << 2))
            self._intra_modes(addr, codes, 8 if m.t8 else 4)
        else:
            m.kind = "I16"
            m.i16 = (mt - 1) % 4
        m.cmode = self._chroma_mode(addr)
        if m.kind == "I16":
            cbp = (15 if mt >= 13 else 0) | ((((mt - 1) // 4) % 3) << 4)
        else:
            cbp = self._cbp(addr)
        m.cbp = cbp
        return self._residual(addr, cbp, qp)

    def _chroma_mode(self, addr):
        c = self.c
        inc = 0
        for a in (self._mba(addr), self._mbb(addr)):
            if a >= 0:
                n = self.mbs[a]
                if n.kind in ("I4", "I8", "I16") and n.cmode != 0:
                    inc += 1
        if not c.dec(64 + inc):
            return 0
        if not c.dec(67):
            return 1
        return 2 if not c.dec(67) else 3

    def _intra_modes(self, addr, codes, size):
        m = self.mbs[addr]
        cip = self.pps["constrained_intra"]
        order = _BLK_RASTER if size == 4 else [0, 2, 8, 10]
        for i, code in enumerate(codes):
            k = order[i]
            x, y = (k & 3) * 4, (k >> 2) * 4
            dc, modes = False, []
            for nx, ny in ((x - 1, y), (x, y - 1)):
                a, kk = self._luma_nb(addr, nx, ny)
                if a < 0:
                    dc = True
                    break
                n = self.mbs[a]
                if n.kind in ("P", "B") and cip:
                    dc = True
                    break
                if a == addr or n.kind in ("I4", "I8"):
                    modes.append(n.modes[kk])
                else:
                    modes.append(2)
            pred = 2 if dc else min(modes)
            mode = pred if code < 0 else (code if code < pred else code + 1)
            blocks = [k] if size == 4 else [k, k + 1, k + 4, k + 5]
            for kk in blocks:
                m.modes[kk] = mode

    # ---- coded_block_pattern, qp delta --------------------------------------
    def _cbp(self, addr):
        c, m = self.c, self.mbs[addr]
        luma = 0
        for b8 in range(4):
            x, y = (b8 & 1) * 8, (b8 >> 1) * 8
            conds = []
            for nx, ny in ((x - 1, y), (x, y - 1)):
                a, k = self._luma_nb(addr, nx, ny)
                if a < 0:
                    conds.append(0)
                    continue
                n = self.mbs[a]
                nb8 = ((k >> 2) >> 1) * 2 + ((k & 3) >> 1)
                if a == addr:
                    conds.append(0 if (luma >> nb8) & 1 else 1)
                elif n.kind == "PCM":
                    conds.append(0)
                elif not n.skip and (n.cbp >> nb8) & 1:
                    conds.append(0)
                else:
                    conds.append(1)
            luma |= c.dec(73 + conds[0] + 2 * conds[1]) << b8
        conds0, conds1 = [], []
        for a in (self._mba(addr), self._mbb(addr)):
            if a < 0:
                conds0.append(0)
                conds1.append(0)
                continue
            n = self.mbs[a]
            cc = 2 if n.kind == "PCM" else (0 if n.skip else n.cbp >> 4)
            conds0.append(1 if cc else 0)
            conds1.append(1 if cc == 2 else 0)
        chroma = 0
        if c.dec(77 + conds0[0] + 2 * conds0[1]):
            chroma = 1 + c.dec(77 + 4 + conds1[0] + 2 * conds1[1])
        return luma | chroma << 4

    def _qp_delta(self, addr):
        c = self.c
        inc = 0
        p = self.prev_addr
        if p >= 0:
            n = self.mbs[p]
            if not (n.skip or n.kind == "PCM" or (n.kind != "I16" and n.cbp == 0) or n.qpd == 0):
                inc = 1
        if not c.dec(60 + inc):
            return 0
        k = 1
        ctx = 62
        while c.dec(ctx):
            k += 1
            ctx = 63
            if k > 200:
                raise ValueError("mb_qp_delta too long")
        return (k + 1) // 2 if k & 1 else -(k // 2)

    # ---- residual (7.3.5.3, CABAC) ----------------------------------------
    def _residual(self, addr, cbp, qp):
        m = self.mbs[addr]
        intra = m.kind in ("I4", "I8", "I16")
        if cbp or m.kind == "I16":
            m.qpd = self._qp_delta(addr)
            qp = (qp + m.qpd + 52) % 52
        m.qp = qp
        payload = []
        if m.kind == "I16":
            inc = self._cbf_dc_inc(addr, 0, intra)
            lv = self._block(0, 16, inc)
            if lv is not None:
                m.cbf_dc |= 1
                m.dc |= 1
                payload.extend(lv)
        blocks = {}
        for b8 in range(4):
            if not (cbp >> b8) & 1:
                continue
            bx, by = (b8 & 1) * 2, (b8 >> 1) * 2
            if m.t8:
                lv = self._block(5, 64, None)
                for k in (by * 4 + bx, by * 4 + bx + 1, (by + 1) * 4 + bx, (by + 1) * 4 + bx + 1):
                    m.cbf4[k] = 1
                if lv is not None and any(lv):
                    blocks[b8] = lv
                    m.nz |= (3 << (by * 4 + bx)) | (3 << ((by + 1) * 4 + bx))
                continue
            for i4 in range(4):
                k = (by + (i4 >> 1)) * 4 + bx + (i4 & 1)
                inc = self._cbf_luma_inc(addr, k, intra)
                if m.kind == "I16":
                    lv = self._block(1, 15, inc)
                    lv = None if lv is None else [0] + lv
                else:
                    lv = self._block(2, 16, inc)
                if lv is not None:
                    m.cbf4[k] = 1
                    blocks[k] = lv
                    if any(lv):
                        m.nz |= 1 << k
        for k in sorted(blocks):
            m.luma_coded |= 1 << k
            payload.extend(blocks[k])
        chroma = cbp >> 4
        cdc = [None, None]
        if chroma:
            for comp in range(2):
                lv = self._block(3, 4, self._cbf_dc_inc(addr, 1 + comp, intra))
                if lv is not None:
                    m.cbf_dc |= 2 << comp
                    m.dc |= 2 << comp
                    cdc[comp] = lv
        for comp in range(2):
            if cdc[comp] is not None:
                payload.extend(cdc[comp])
        if chroma == 2:
            cac = {}
            for comp in range(2):
                for blk in range(4):
                    lv = self._block(4, 15, self._cbf_cac_inc(addr, comp, blk, intra))
                    if lv is not None:
                        m.cbfc[comp][blk] = 1
                        cac[comp * 4 + blk] = [0] + lv
            for bit in sorted(cac):
                m.chroma_coded |= 1 << bit
                payload.extend(cac[bit])
        m.levels = payload
        return qp

    def _cbf_cond(self, a, intra, get):
        """condTermFlagN of coded_block_flag (9.3.3.1.1.9) for neighbour MB a;
        get(n) -> the transform block's flag, or None when it has none."""
        if a < 0:
            return 1 if intra else 0
        n = self.mbs[a]
        if n.kind == "PCM":
            return 1
        if n.skip:
            return 0
        v = get(n)
        return 0 if v is None else v

    def _cbf_dc_inc(self, addr, bit, intra):
        def get(n):
            if bit == 0:
                return (n.cbf_dc & 1) if n.kind == "I16" else None
            return ((n.cbf_dc >> bit) & 1) if (n.cbp >> 4) else None
        return self._cbf_cond(self._mba(addr), intra, get) + 2 * self._cbf_cond(self._mbb(addr), intra, get)

    def _cbf_luma_inc(self, addr, k, intra):
        m = self.mbs[addr]
        x, y = (k & 3) * 4, (k >> 2) * 4
        out = []
        for nx, ny in ((x - 1, y), (x, y - 1)):
            a, kk = self._luma_nb(addr, nx, ny)
            nb8 = ((kk >> 2) >> 1) * 2 + ((kk & 3) >> 1)
            if a == addr:
                out.append(m.cbf4[kk] if (m.cbp >> nb8) & 1 else 0)
                continue

            def get(n, kk=kk, nb8=nb8):
                if not (n.cbp >> nb8) & 1:
                    return None
                return 1 if n.t8 else n.cbf4[kk]
            out.append(self._cbf_cond(a, intra, get))
        return out[0] + 2 * out[1]

    def _cbf_cac_inc(self, addr, comp, blk, intra):
        m = self.mbs[addr]
        x, y = blk & 1, blk >> 1
        out = []
        for nx, ny in ((x - 1, y), (x, y - 1)):
            if nx >= 0 and ny >= 0:
                out.append(m.cbfc[comp][ny * 2 + nx])
                continue
            a = self._mba(addr) if nx < 0 else self._mbb(addr)
            kk = (ny % 2) * 2 + (nx % 2)

            def get(n, kk=kk):
                return n.cbfc[comp][kk] if (n.cbp >> 4) == 2 else None
            out.append(self._cbf_cond(a, intra, get))
        return out[0] + 2 * out[1]

    def _block(self, cat, maxnum, cbf_inc):
        """residual_block_cabac: levels in scan order, or None when
        coded_block_flag is 0."""
        c = self.c
        if cat != 5:
            if not c.dec(85 + _CBF_OFF[cat] + cbf_inc):
                return None
            sig_b, last_b, abs_b = 105 + _SIG_OFF[cat], 166 + _SIG_OFF[cat], 227 + _ABS_OFF[cat]
        else:
            sig_b, last_b, abs_b = 402, 417, 426
        sig = []
        i = 0
        last_found = False
        while i < maxnum - 1:
            inc = _SIG8[i] if cat == 5 else (min(i, 2) if cat == 3 else i)
            if c.dec(sig_b + inc):
                sig.append(i)
                linc = _LAST8[i] if cat == 5 else (min(i, 2) if cat == 3 else i)
                if c.dec(last_b + linc):
                    last_found = True
                    break
            i += 1
        if not last_found:
            sig.append(maxnum - 1)
        out = [0] * maxnum
        gt1 = eq1 = 0
        cap = 4 - (1 if cat == 3 else 0)
        for pos in reversed(sig):
            if not c.dec(abs_b + (0 if gt1 else min(4, 1 + eq1))):
                v = 0
            else:
                v = 1
                while v < 14 and c.dec(abs_b + 5 + min(cap, gt1)):
                    v += 1
                if v == 14:
                    v += c.eg(0)
            lev = v + 1
            out[pos] = -lev if c.byp() else lev
            if v == 0:
                eq1 += 1
            else:
                gt1 += 1
        return out

    # ---- inter macroblocks -------------------------------------------------
    def _ref_idx(self, addr, X, x, y):
        c, m = self.c, self.mbs[addr]
        conds = []
        for nx, ny in ((x - 1, y), (x, y - 1)):
            a, k = self._luma_nb(addr, nx, ny)
            if a < 0:
                conds.append(0)
                continue
            n = self.mbs[a]
            if n.skip or n.kind not in ("P", "B") or n.direct[k] or n.ref[X][k] <= 0:
                conds.append(0)
            else:
                conds.append(1)
        r = 0
        if c.dec(54 + conds[0] + 2 * conds[1]):
            r = 1
            ctx = 58
            while c.dec(ctx):
                r += 1
                ctx = 59
                if r > 64:
                    raise ValueError("ref_idx too long")
        return r

    def _mvd(self, addr, X, x, y):
        c = self.c
        out = []
        for comp, base in ((0, 40), (1, 47)):
            s = 0
            for nx, ny in ((x - 1, y), (x, y - 1)):
                a, k = self._luma_nb(addr, nx, ny)
                if a < 0:
                    continue
                n = self.mbs[a]
                if n.skip or n.kind not in ("P", "B") or n.direct[k] or n.ref[X][k] < 0:
                    continue
                s += abs(n.mvd[X][k][comp])
            inc = 0 if s < 3 else (2 if s > 32 else 1)
            if not c.dec(base + inc):
                out.append(0)
                continue
            v, ctx = 1, base + 3
            while v < 9 and c.dec(ctx):
                if v < 4:
                    ctx += 1
                v += 1
            if v >= 9:
                v += c.eg(3)
            out.append(-v if c.byp() else v)
        return tuple(out)

    def _set(self, m, done, X, x, y, w, h, ref, mv, mvd):
        for yy in range(y >> 2, (y + h) >> 2):
            for xx in range(x >> 2, (x + w) >> 2):
                k = yy * 4 + xx
                m.ref[X][k], m.mv[X][k], m.mvd[X][k] = ref, mv, mvd
                done[X][k] = True

    def _mv_nb(self, addr, X, x, y, done):
        """(refIdxLX, mvLX) of the partition covering luma (x, y); ref -2 when
        not available (outside, other slice, or later in decoding order)."""
        a, k = self._luma_nb(addr, x, y)
        if a < 0:
            return -2, (0, 0)
        if a == addr and not done[X][k]:
            return -2, (0, 0)
        n = self.mbs[a]
        if n.kind not in ("P", "B") or n.ref[X][k] < 0:
            return -1, (0, 0)
        return n.ref[X][k], n.mv[X][k]

    def _mvp(self, addr, X, x, y, w, h, ref, done, shape):
        """8.4.1.3 motion vector prediction."""
        A = self._mv_nb(addr, X, x - 1, y, done)
        B = self._mv_nb(addr, X, x, y - 1, done)
        C = self._mv_nb(addr, X, x + w, y - 1, done)
        if C[0] == -2:
            C = self._mv_nb(addr, X, x - 1, y - 1, done)
        if B[0] == -2 and C[0] == -2 and A[0] != -2:
            B, C = A, A
        A, B, C = [((r if r >= -1 else -1), mv) for r, mv in (A, B, C)]
        if shape == "16x8":
            if y == 0 and B[0] == ref:
                return B[1]
            if y == 8 and A[0] == ref:
                return A[1]
        elif shape == "8x16":
            if x == 0 and A[0] == ref:
                return A[1]
            if x == 8 and C[0] == ref:
                return C[1]
        same = [nb for nb in (A, B, C) if nb[0] == ref]
        if len(same) == 1:
            return same[0][1]
        med = lambda p, q, r: max(min(p, q), min(max(p, q), r))
        return (med(A[1][0], B[1][0], C[1][0]), med(A[1][1], B[1][1], C[1][1]))

    def _p_skip(self, addr):
        """8.4.1.1 P_Skip motion."""
        m = self.mbs[addr]
        done = [[False] * 16, [False] * 16]
        a = self._mv_nb(addr, 0, -1, 0, done)
        b = self._mv_nb(addr, 0, 0, -1, done)
        if a[0] == -2 or b[0] == -2 or (a[0] == 0 and a[1] == (0, 0)) or (b[0] == 0 and b[1] == (0, 0)):
            mv = (0, 0)
        else:
            mv = self._mvp(addr, 0, 0, 0, 16, 16, 0, done, "16x16")
        self._set(m, done, 0, 0, 0, 16, 16, 0, mv, (0, 0))
        self._weights_for(m)

    def _inter_p(self, addr, mt):
        c, m, h = self.c, self.mbs[addr], self.h
        m.kind = "P"
        done = [[False] * 16, [False] * 16]
        nref = h["num_ref"][0]
        if mt < 3:
            self._subs = None
            parts = _P_PARTS[mt]
            shape = ("16x16", "16x8", "8x16")[mt]
            m.syn = (2 + mt, [1] * len(parts) + [0] * (4 - len(parts)), [0] * 4)
            refs = [self._ref_idx_at(addr, 0, x, y, w, hh, nref) for (x, y, w, hh) in parts]
            for (x, y, w, hh), r in zip(parts, refs):
                d = self._mvd(addr, 0, x, y)
                p = self._mvp(addr, 0, x, y, w, hh, r, done, shape)
                self._set(m, done, 0, x, y, w, hh, r, (p[0] + d[0], p[1] + d[1]), d)
        else:
            subs = []
            for _ in range(4):
                if c.dec(21):
                    subs.append(0)
                elif not c.dec(22):
                    subs.append(1)
                else:
                    subs.append(2 if c.dec(23) else 3)
            self._subs = subs
            m.syn = (5, [1] * 4, list(subs))  # P_8x8: sub shapes 0..3 as RC_H264_SUB_*
            refs = [self._ref_idx_at(addr, 0, (i & 1) * 8, (i >> 1) * 8, 8, 8, nref) for i in range(4)]
            for i8 in range(4):
                x8, y8 = (i8 & 1) * 8, (i8 >> 1) * 8
                sw, sh, _ = _P_SUB[subs[i8]]
                for yy in range(0, 8, sh):
                    for xx in range(0, 8, sw):
                        d = self._mvd(addr, 0, x8 + xx, y8 + yy)
                        p = self._mvp(addr, 0, x8 + xx, y8 + yy, sw, sh, refs[i8], done, "sub")
                        self._set(m, done, 0, x8 + xx, y8 + yy, sw, sh, refs[i8], (p[0] + d[0], p[1] + d[1]), d)
        self._weights_for(m)

    def _ref_idx_at(self, addr, X, x, y, w, h, nref):
        """ref_idx of the w x h partition at (x, y): parsed when the list has
        more than one entry, and stored over the whole partition at once,
        because the contexts of later ref_idx read it (its motion vector is
        set when its mvd is parsed)."""
        r = self._ref_idx(addr, X, x, y) if nref > 1 else 0
        if r >= nref:
            raise ValueError("ref_idx past the list")
        m = self.mbs[addr]
        for yy in range(y >> 2, (y + h) >> 2):
            for xx in range(x >> 2, (x + w) >> 2):
                m.ref[X][yy * 4 + xx] = r
        return r

    def _inter_b(self, addr, mt):
        c, m, h = self.c, self.mbs[addr], self.h
        m.kind = "B"
        m.btype = mt
        done = [[False] * 16, [False] * 16]
        nref = h["num_ref"]
        if mt == 0:
            self._subs = None
            m.direct16 = True
            m.syn = (1, [0] * 4, [0] * 4)
            self._direct(addr, range(4))
            self._weights_for(m)
            return
        if mt < 22:
            self._subs = None
            pw, ph, preds = _B_TYPES[mt]
            parts = [(0, 0)] if pw == 16 and ph == 16 else ([(0, 0), (0, 8)] if ph == 8 else [(0, 0), (8, 0)])
            shape = "16x16" if len(parts) == 1 else ("16x8" if ph == 8 else "8x16")
            m.syn = ({"16x16": 2, "16x8": 3, "8x16": 4}[shape], list(preds) + [0] * (4 - len(preds)), [0] * 4)
            refs = [[-1] * len(parts), [-1] * len(parts)]
            for X in range(2):
                for i, (x, y) in enumerate(parts):
                    if preds[i] & (1 << X):
                        refs[X][i] = self._ref_idx_at(addr, X, x, y, pw, ph, nref[X])
            for X in range(2):
                for i, (x, y) in enumerate(parts):
                    if preds[i] & (1 << X):
                        d = self._mvd(addr, X, x, y)
                        p = self._mvp(addr, X, x, y, pw, ph, refs[X][i], done, shape)
                        self._set(m, done, X, x, y, pw, ph, refs[X][i], (p[0] + d[0], p[1] + d[1]), d)
                    else:
                        self._set(m, done, X, x, y, pw, ph, -1, (0, 0), (0, 0))
            self._weights_for(m)
            return
        # B_8x8
        subs = []
        for _ in range(4):
            if not c.dec(36):
                subs.append(0)
            elif not c.dec(37):
                subs.append(1 + c.dec(39))
            else:
                t = 3
                if c.dec(38):
                    if c.dec(39):
                        subs.append(11 + c.dec(39))
                        continue
                    t += 4
                t += 2 * c.dec(39)
                t += c.dec(39)
                subs.append(t)
        self._subs = subs
        _subshape = {(8, 8): 0, (8, 4): 1, (4, 8): 2, (4, 4): 3}
        m.syn = (5, [_B_SUB[t][2] if t else 0 for t in subs],
                 [_subshape[_B_SUB[t][:2]] if t else 4 for t in subs])
        direct8 = [i for i in range(4) if subs[i] == 0]
        if direct8:
            self._direct(addr, direct8)
            for i8 in direct8:
                for k in self._b8_blocks(i8):
                    done[0][k] = done[1][k] = True
        refs = [[-1] * 4, [-1] * 4]
        for X in range(2):
            for i8 in range(4):
                if subs[i8] and _B_SUB[subs[i8]][2] & (1 << X):
                    refs[X][i8] = self._ref_idx_at(addr, X, (i8 & 1) * 8, (i8 >> 1) * 8, 8, 8, nref[X])
        for X in range(2):
            for i8 in range(4):
                if not subs[i8]:
                    continue
                x8, y8 = (i8 & 1) * 8, (i8 >> 1) * 8
                sw, sh, pred = _B_SUB[subs[i8]]
                for yy in range(0, 8, sh):
                    for xx in range(0, 8, sw):
                        if pred & (1 << X):
                            d = self._mvd(addr, X, x8 + xx, y8 + yy)
                            p = self._mvp(addr, X, x8 + xx, y8 + yy, sw, sh, refs[X][i8], done, "sub")
                            self._set(m, done, X, x8 + xx, y8 + yy, sw, sh, refs[X][i8], (p[0] + d[0], p[1] + d[1]),
                                      d)
                        else:
                            self._set(m, done, X, x8 + xx, y8 + yy, sw, sh, -1, (0, 0), (0, 0))
        self._weights_for(m)

    @staticmethod
    def _b8_blocks(i8):
        bx, by = (i8 & 1) * 2, (i8 >> 1) * 2
        return [by * 4 + bx, by * 4 + bx + 1, (by + 1) * 4 + bx, (by + 1) * 4 + bx + 1]

    # ---- direct prediction (8.4.1.2) ---------------------------------------
    def _colocated(self, addr, i8):
        """(refIdxCol, mvCol, referenced Frame) of the corner 4x4 block of 8x8
        i8 in the co-located picture RefPicList1[0] (direct_8x8_inference;
        8.4.1.2.1): its list-0 motion if it has some, else its list-1 motion;
        an intra block gives refIdxCol -1 and a zero vector."""
        col = self.lists[1][0]
        k = (0, 3, 12, 15)[i8]
        if col.intra[addr]:
            return -1, (0, 0), None
        L = 0 if col.ref_idx[0][addr][k] >= 0 else 1
        return col.ref_idx[L][addr][k], col.mv[L][addr][k], col.ref_pic[L][addr][k]

    def _direct(self, addr, parts):
        if not self.sps["direct_8x8_inference"]:
            raise NotImplementedError("direct prediction without direct_8x8_inference")
        m, h = self.mbs[addr], self.h
        col = self.lists[1][0]
        if h["direct_spatial"]:
            done = [[False] * 16, [False] * 16]
            refs, mvps = [-1, -1], [(0, 0), (0, 0)]
            for X in range(2):
                A = self._mv_nb(addr, X, -1, 0, done)
                B = self._mv_nb(addr, X, 0, -1, done)
                C = self._mv_nb(addr, X, 16, -1, done)
                if C[0] == -2:
                    C = self._mv_nb(addr, X, -1, -1, done)
                mp = lambda p, q: min(p, q) if (p >= 0 and q >= 0) else max(p, q)
                refs[X] = mp(max(A[0], -1), mp(max(B[0], -1), max(C[0], -1)))
            zero = refs[0] < 0 and refs[1] < 0
            if zero:
                refs = [0, 0]
            else:
                for X in range(2):
                    if refs[X] >= 0:
                        mvps[X] = self._mvp(addr, X, 0, 0, 16, 16, refs[X], done, "16x16")
            for i8 in parts:
                rc, mvc, _ = self._colocated(addr, i8)
                colzero = rc == 0 and abs(mvc[0]) <= 1 and abs(mvc[1]) <= 1
                for k in self._b8_blocks(i8):
                    for X in range(2):
                        if refs[X] < 0:
                            m.ref[X][k], m.mv[X][k] = -1, (0, 0)
                        elif zero or (refs[X] == 0 and colzero):
                            m.ref[X][k], m.mv[X][k] = refs[X], (0, 0)
                        else:
                            m.ref[X][k], m.mv[X][k] = refs[X], mvps[X]
                        m.mvd[X][k] = (0, 0)
                    m.direct[k] = True
        else:
            for i8 in parts:
                rc, mvc, fr = self._colocated(addr, i8)
                r0 = 0
                if rc >= 0:
                    r0 = next(i for i, f in enumerate(self.lists[0]) if f is fr)
                pic0, pic1 = self.lists[0][r0], self.lists[1][0]
                tb = max(-128, min(127, self.frame.poc - pic0.poc))
                td = max(-128, min(127, pic1.poc - pic0.poc))
                if td == 0:
                    mv0, mv1 = mvc, (0, 0)
                else:
                    tx = (16384 + abs(int(td / 2))) // abs(td) * (1 if td > 0 else -1)
                    dsf = max(-1024, min(1023, (tb * tx + 32) >> 6))
                    mv0 = tuple((dsf * v + 128) >> 8 for v in mvc)
                    mv1 = (mv0[0] - mvc[0], mv0[1] - mvc[1])
                for k in self._b8_blocks(i8):
                    m.ref[0][k], m.mv[0][k] = r0, mv0
                    m.ref[1][k], m.mv[1][k] = 0, mv1
                    m.mvd[0][k] = m.mvd[1][k] = (0, 0)
                    m.direct[k] = True

    # ---- weighted prediction (8.4.2.3) -------------------------------------
    def _weights_for(self, m):
        """The weight-table entry of each 8x8 partition: explicit tables of the
        slice, implicit weights from POC distances, or default (0xff)."""
        for b8 in range(4):
            k = (b8 >> 1) * 8 + (b8 & 1) * 2
            m.wp[b8] = self._wp_index(m.ref[0][k], m.ref[1][k])

    def _wp_index(self, r0, r1):
        """The weight-table entry for refIdxL0 = r0 and refIdxL1 = r1 in the
        current slice (-1: list unused), 0xff for the default."""
        h, pps = self.h, self.pps
        explicit = h["weights"] is not None
        implicit = h["type"] == 1 and pps["weighted_bipred"] == 2
        if not explicit and not (implicit and r0 >= 0 and r1 >= 0):
            return 0xFF
        if explicit:
            w = h["weights"]
            lw, cw = w["luma_log2"], w["chroma_log2"]
            e0 = w["l"][0][r0] if r0 >= 0 else None
            e1 = w["l"][1][r1] if r1 >= 0 else None
            ent = {"lwd": [lw, cw, cw],
                   "w0": [e0[0], e0[2][0], e0[2][1]] if e0 else [0, 0, 0],
                   "o0": [e0[1], e0[3][0], e0[3][1]] if e0 else [0, 0, 0],
                   "w1": [e1[0], e1[2][0], e1[2][1]] if e1 else [0, 0, 0],
                   "o1": [e1[1], e1[3][0], e1[3][1]] if e1 else [0, 0, 0]}
        else:
            p0, p1 = self.lists[0][r0], self.lists[1][r1]
            tb = max(-128, min(127, self.frame.poc - p0.poc))
            td = max(-128, min(127, p1.poc - p0.poc))
            w0 = w1 = 32
            if td != 0:
                tx = (16384 + abs(int(td / 2))) // abs(td) * (1 if td > 0 else -1)
                dsf = max(-1024, min(1023, (tb * tx + 32) >> 6))
                if -64 <= (dsf >> 2) <= 128:
                    w0, w1 = 64 - (dsf >> 2), dsf >> 2
            ent = {"lwd": [5, 5, 5], "w0": [w0] * 3, "w1": [w1] * 3, "o0": [0] * 3, "o1": [0] * 3}
        mask = 0
        for comp in range(3):
            unit0 = ent["w0"][comp] == 1 << ent["lwd"][comp] and ent["o0"][comp] == 0
            unit1 = ent["w1"][comp] == 1 << ent["lwd"][comp] and ent["o1"][comp] == 0
            plain = (unit0 or r0 < 0) and (unit1 or r1 < 0)
            if not plain:
                mask |= 1 << comp
        if mask == 0:
            return 0xFF
        ent["mask"] = mask
        key = (mask, tuple(ent["lwd"]), tuple(ent["w0"]), tuple(ent["w1"]), tuple(ent["o0"]), tuple(ent["o1"]))
        if key not in self.wkey:
            self.wkey[key] = len(self.weights)
            self.weights.append(ent)
        return self.wkey[key]

    def _slice_motion(self):
        """The slice's rc_h264_slice_motion fields: direct mode, co-located
        picture, temporal-direct scale factors per refIdxL0 (as
        SliceDecoder::new computes them) and the weight entry of every
        (refIdxL0, refIdxL1) pair."""
        h, lists = self.h, self.lists
        b = h["type"] == 1
        sm = {"b_slice": int(b), "direct_spatial": int(bool(h.get("direct_spatial"))),
              "direct_8x8_inference": int(bool(self.sps["direct_8x8_inference"])), "col_slot": -1,
              "col_short_term": 0, "dist_scale": [256] * 32, "direct_copy": [1] * 32, "wp_map": [0xFF] * (33 * 33)}
        if b and lists[1]:
            p1 = lists[1][0]
            sm["col_slot"], sm["col_short_term"] = p1.slot, 1
            for i, p0 in enumerate(lists[0][:32]):
                tb = max(-128, min(127, self.frame.poc - p0.poc))
                td = max(-128, min(127, p1.poc - p0.poc))
                if td != 0:
                    tx = (16384 + abs(int(td / 2))) // abs(td) * (1 if td > 0 else -1)
                    sm["dist_scale"][i] = max(-1024, min(1023, (tb * tx + 32) >> 6))
                    sm["direct_copy"][i] = 0
        n0, n1 = len(lists[0]), len(lists[1])
        for r0 in range(-1, min(n0, 32)):
            for r1 in range(-1, min(n1, 32)):
                sm["wp_map"][(r0 + 1) * 33 + (r1 + 1)] = self._wp_index(r0, r1)
        return sm
