"""H.264 Baseline-profile (CAVLC) parse into reconstruction records.

TEST INFRASTRUCTURE: this module turns a Baseline H.264 elementary stream
into the per-picture syntax records of include/pito_recon.h (rc_h264_mb,
rc_h264_slice, levels), so that the reference's golden streams can drive
the oracle and the GPU engine end to end.  It restates the parse half of
the reference decoder (src/h264/dec/cavlc.rs, mbtypes.rs, slicedec.rs
:473-937 and :1582-1862, src/syntax/h264/{params,slice,dpb}.rs) for the
tools a Baseline stream uses: I and P slices, CAVLC residuals, Intra4x4 /
Intra16x16 / I_PCM, P partitions down to 4x4 with motion-vector prediction,
P_Skip, several slices per picture, several reference frames with sliding-
window marking and short-term list modification.  Anything else raises
NotImplementedError.  Nothing in the engine imports it.
"""
from __future__ import annotations

import ctypes

# ---------------------------------------------------------------------------
# Variable-length code tables (ITU-T H.264 Tables 9-4, 9-5, 9-7, 9-8, 9-9,
# 9-10; the reference holds the same codes in src/h264/dec/cavlc_tables.rs
# and src/h264/dec/mbtypes.rs:195).
# ---------------------------------------------------------------------------
# coeff_token, per nC class (0: 0<=nC<2, 1: 2<=nC<4, 2: 4<=nC<8, 3: 8<=nC,
# 4: chroma DC 4:2:0), per TotalCoeff 0..16, the codes for TrailingOnes
# 0..3 (None where the combination does not exist).
_CT = [
    [  # 0 <= nC < 2
        ["1"], ["000101", "01"], ["00000111", "000100", "001"], ["000000111", "00000110", "0000101", "00011"],
        ["0000000111", "000000110", "00000101", "000011"], ["00000000111", "0000000110", "000000101", "0000100"],
        ["0000000001111", "00000000110", "0000000101", "00000100"],
        ["0000000001011", "0000000001110", "00000000101", "000000100"],
        ["0000000001000", "0000000001010", "0000000001101", "0000000100"],
        ["00000000001111", "00000000001110", "0000000001001", "00000000100"],
        ["00000000001011", "00000000001010", "00000000001101", "0000000001100"],
        ["000000000001111", "000000000001110", "00000000001001", "00000000001100"],
        ["000000000001011", "000000000001010", "000000000001101", "00000000001000"],
        ["0000000000001111", "000000000000001", "000000000001001", "000000000001100"],
        ["0000000000001011", "0000000000001110", "0000000000001101", "000000000001000"],
        ["0000000000000111", "0000000000001010", "0000000000001001", "0000000000001100"],
        ["0000000000000100", "0000000000000110", "0000000000000101", "0000000000001000"],
    ],
    [  # 2 <= nC < 4
        ["11"], ["001011", "10"], ["000111", "00111", "011"], ["0000111", "001010", "001001", "0101"],
        ["00000111", "000110", "000101", "0100"], ["00000100", "0000110", "0000101", "00110"],
        ["000000111", "00000110", "00000101", "001000"], ["00000001111", "000000110", "000000101", "000100"],
        ["00000001011", "00000001110", "00000001101", "0000100"],
        ["000000001111", "00000001010", "00000001001", "000000100"],
        ["000000001011", "000000001110", "000000001101", "00000001100"],
        ["000000001000", "000000001010", "000000001001", "00000001000"],
        ["0000000001111", "0000000001110", "0000000001101", "000000001100"],
        ["0000000001011", "0000000001010", "0000000001001", "0000000001100"],
        ["0000000000111", "00000000001011", "0000000000110", "0000000001000"],
        ["00000000001001", "00000000001000", "00000000001010", "0000000000001"],
        ["00000000000111", "00000000000110", "00000000000101", "00000000000100"],
    ],
    [  # 4 <= nC < 8
        ["1111"], ["001111", "1110"], ["001011", "01111", "1101"], ["001000", "01100", "01110", "1100"],
        ["0001111", "01010", "01011", "1011"], ["0001011", "01000", "01001", "1010"],
        ["0001001", "001110", "001101", "1001"], ["0001000", "001010", "001001", "1000"],
        ["00001111", "0001110", "0001101", "01101"], ["00001011", "00001110", "0001010", "001100"],
        ["000001111", "00001010", "00001101", "0001100"], ["000001011", "000001110", "00001001", "00001100"],
        ["000001000", "000001010", "000001101", "00001000"], ["0000001101", "000000111", "000001001", "000001100"],
        ["0000001001", "0000001100", "0000001011", "0000001010"],
        ["0000000101", "0000001000", "0000000111", "0000000110"],
        ["0000000001", "0000000100", "0000000011", "0000000010"],
    ],
    None,  # 8 <= nC: six-bit fixed-length code, see _coeff_token
    [  # nC == -1 (chroma DC, 4:2:0)
        ["01"], ["000111", "1"], ["000100", "000110", "001"], ["000011", "0000011", "0000010", "000101"],
        ["000010", "00000011", "00000010", "0000000"],
    ],
]

# total_zeros for 4x4 blocks: per TotalCoeff 1..15, codes for total_zeros 0..
_TZ4 = [
    ["1", "011", "010", "0011", "0010", "00011", "00010", "000011", "000010", "0000011", "0000010", "00000011",
     "00000010", "000000011", "000000010", "000000001"],
    ["111", "110", "101", "100", "011", "0101", "0100", "0011", "0010", "00011", "00010", "000011", "000010",
     "000001", "000000"],
    ["0101", "111", "110", "101", "0100", "0011", "100", "011", "0010", "00011", "00010", "000001", "00001",
     "000000"],
    ["00011", "111", "0101", "0100", "110", "101", "100", "0011", "011", "0010", "00010", "00001", "00000"],
    ["0101", "0100", "0011", "111", "110", "101", "100", "011", "0010", "00001", "0001", "00000"],
    ["000001", "00001", "111", "110", "101", "100", "011", "010", "0001", "001", "000000"],
    ["000001", "00001", "101", "100", "011", "11", "010", "0001", "001", "000000"],
    ["000001", "0001", "00001", "011", "11", "10", "010", "001", "000000"],
    ["000001", "000000", "0001", "11", "10", "001", "01", "00001"],
    ["00001", "00000", "001", "11", "10", "01", "0001"],
    ["0000", "0001", "001", "010", "1", "011"],
    ["0000", "0001", "01", "1", "001"],
    ["000", "001", "1", "01"],
    ["00", "01", "1"],
    ["0", "1"],
]
# total_zeros for the 2x2 chroma DC block: per TotalCoeff 1..3
_TZ2 = [["1", "01", "001", "000"], ["1", "01", "00"], ["1", "0"]]
# run_before: per zerosLeft 1..6 and >6, codes for run_before 0..
_RB = [
    ["1", "0"], ["1", "01", "00"], ["11", "10", "01", "00"], ["11", "10", "01", "001", "000"],
    ["11", "10", "011", "010", "001", "000"], ["11", "000", "001", "011", "010", "101", "100"],
    ["111", "110", "101", "100", "011", "010", "001", "0001", "00001", "000001", "0000001", "00000001", "000000001",
     "0000000001", "00000000001"],
]
# coded_block_pattern from codeNum (me(v), 4:2:0): (Intra_4x4, Inter),
# each luma bits 0..3 | chroma << 4
_CBP = [
    (47, 0), (31, 16), (15, 1), (0, 2), (23, 4), (27, 8), (29, 32), (30, 3), (7, 5), (11, 10), (13, 12), (14, 15),
    (39, 47), (43, 7), (45, 11), (46, 13), (16, 14), (3, 6), (5, 9), (10, 31), (12, 35), (19, 37), (21, 42),
    (26, 44), (28, 33), (35, 34), (37, 36), (42, 40), (44, 39), (1, 43), (2, 45), (4, 46), (8, 17), (17, 18),
    (18, 20), (20, 24), (24, 19), (6, 21), (9, 26), (22, 28), (25, 23), (32, 27), (33, 29), (34, 30), (36, 22),
    (40, 25), (38, 38), (41, 41),
]
# chroma QP from qPI (Table 8-15)
_QPC = list(range(30)) + [29, 30, 31, 32, 32, 33, 34, 34, 35, 35, 36, 36, 37, 37, 37, 38, 38, 38, 39, 39, 39, 39]


def _decoder(table):
    """code string -> value dicts, per code length (for bitwise matching)."""
    return {code: v for v, code in table}


_CT_DEC = []
for cls in _CT:
    if cls is None:
        _CT_DEC.append(None)
        continue
    d = {}
    for tc, codes in enumerate(cls):
        for t1, code in enumerate(codes):
            if code:
                d[code] = (t1, tc)
    _CT_DEC.append(d)
_TZ4_DEC = [{c: z for z, c in enumerate(row)} for row in _TZ4]
_TZ2_DEC = [{c: z for z, c in enumerate(row)} for row in _TZ2]
_RB_DEC = [{c: r for r, c in enumerate(row)} for row in _RB]

# luma4x4BlkIdx (decode order) -> raster 4x4 index by * 4 + bx
_BLK_RASTER = [0, 1, 4, 5, 2, 3, 6, 7, 8, 9, 12, 13, 10, 11, 14, 15]


# ---------------------------------------------------------------------------
# Bitstream
# ---------------------------------------------------------------------------
def nal_units(data: bytes):
    """(nal_ref_idc, nal_unit_type, rbsp) for every NAL unit (Annex B)."""
    starts = []
    i = 0
    while True:
        j = data.find(b"\x00\x00\x01", i)
        if j < 0:
            break
        starts.append(j + 3)
        i = j + 3
    out = []
    for n, s in enumerate(starts):
        e = starts[n + 1] - 3 if n + 1 < len(starts) else len(data)
        while e > s and data[e - 1] == 0:  # trailing zero bytes / 4-byte start codes
            e -= 1
        raw = data[s:e]
        rbsp = bytearray()
        zeros = 0
        for b in raw[1:]:
            if zeros >= 2 and b == 3:
                zeros = 0
                continue
            rbsp.append(b)
            zeros = zeros + 1 if b == 0 else 0
        out.append(((raw[0] >> 5) & 3, raw[0] & 31, bytes(rbsp)))
    return out


class Bits:
    def __init__(self, data: bytes):
        self.d = data
        self.p = 0
        self.n = len(data) * 8

    def u(self, n: int) -> int:
        v = 0
        for _ in range(n):
            if self.p >= self.n:
                raise ValueError("read past the end of the RBSP")
            v = (v << 1) | ((self.d[self.p >> 3] >> (7 - (self.p & 7))) & 1)
            self.p += 1
        return v

    def ue(self) -> int:
        z = 0
        while self.u(1) == 0:
            z += 1
            if z > 31:
                raise ValueError("bad exp-Golomb code")
        return (1 << z) - 1 + self.u(z)

    def se(self) -> int:
        k = self.ue()
        return (k + 1) >> 1 if k & 1 else -(k >> 1)

    def te(self, cmax: int) -> int:
        return 1 - self.u(1) if cmax == 1 else self.ue()

    def more_rbsp_data(self) -> bool:
        if self.p >= self.n:
            return False
        # the last set bit of the RBSP is the stop bit
        last = self.n - 1
        while last >= 0 and not ((self.d[last >> 3] >> (7 - (last & 7))) & 1):
            last -= 1
        return self.p < last

    def code(self, table: dict, maxlen: int = 16):
        s = ""
        while len(s) <= maxlen:
            s += "1" if self.u(1) else "0"
            if s in table:
                return table[s]
        raise ValueError("no code matches")

    def align(self):
        self.p = (self.p + 7) & ~7


# ---------------------------------------------------------------------------
# Parameter sets and slice header (src/syntax/h264/params.rs, slice.rs)
# ---------------------------------------------------------------------------
def parse_sps(b: Bits) -> dict:
    s = {"profile_idc": b.u(8)}
    b.u(8)
    s["level_idc"] = b.u(8)
    s["id"] = b.ue()
    if s["profile_idc"] in (100, 110, 122, 244, 44, 83, 86, 118, 128, 138, 139, 134, 135):
        raise NotImplementedError("High-profile SPS fields")
    s["log2_max_frame_num"] = b.ue() + 4
    s["poc_type"] = b.ue()
    if s["poc_type"] == 0:
        s["log2_max_poc_lsb"] = b.ue() + 4
    elif s["poc_type"] == 1:
        b.u(1)
        b.se()
        b.se()
        for _ in range(b.ue()):
            b.se()
    s["max_num_ref_frames"] = b.ue()
    b.u(1)  # gaps_in_frame_num_value_allowed_flag
    s["mb_w"] = b.ue() + 1
    s["mb_h"] = b.ue() + 1
    if not b.u(1):
        raise NotImplementedError("field coding")
    b.u(1)  # direct_8x8_inference_flag
    s["crop"] = (0, 0, 0, 0)
    if b.u(1):
        s["crop"] = (b.ue(), b.ue(), b.ue(), b.ue())  # left, right, top, bottom in 2-sample units
    return s


def parse_pps(b: Bits) -> dict:
    p = {"id": b.ue(), "sps_id": b.ue()}
    if b.u(1):
        raise NotImplementedError("CABAC")
    p["bottom_field_poc"] = b.u(1)
    if b.ue() != 0:
        raise NotImplementedError("slice groups")
    p["num_ref_l0"] = b.ue() + 1
    p["num_ref_l1"] = b.ue() + 1
    p["weighted_pred"] = b.u(1)
    p["weighted_bipred"] = b.u(2)
    p["init_qp"] = 26 + b.se()
    b.se()  # pic_init_qs
    p["chroma_qp_offset"] = b.se()
    p["deblock_ctrl"] = b.u(1)
    p["constrained_intra"] = b.u(1)
    p["redundant_pic_cnt"] = b.u(1)
    if b.more_rbsp_data():
        raise NotImplementedError("High-profile PPS fields")
    return p


def parse_slice_header(b: Bits, nal_type: int, nal_ref_idc: int, spss: dict, ppss: dict) -> dict:
    h = {"first_mb": b.ue(), "type": b.ue() % 5, "pps_id": b.ue()}
    if h["type"] not in (0, 2):
        raise NotImplementedError("B / SP / SI slices")
    pps = ppss[h["pps_id"]]
    sps = spss[pps["sps_id"]]
    h["frame_num"] = b.u(sps["log2_max_frame_num"])
    h["idr"] = nal_type == 5
    if h["idr"]:
        b.ue()  # idr_pic_id
    if sps["poc_type"] == 0:
        h["poc_lsb"] = b.u(sps["log2_max_poc_lsb"])
        if pps["bottom_field_poc"]:
            b.se()
    elif sps["poc_type"] == 1:
        raise NotImplementedError("POC type 1")
    if pps["redundant_pic_cnt"]:
        b.ue()
    h["num_ref"] = pps["num_ref_l0"]
    h["mods"] = []
    if h["type"] == 0:
        if b.u(1):  # num_ref_idx_active_override_flag
            h["num_ref"] = b.ue() + 1
        if b.u(1):  # ref_pic_list_modification_flag_l0
            while True:
                idc = b.ue()
                if idc == 3:
                    break
                if idc in (0, 1):
                    h["mods"].append((idc, b.ue() + 1))
                else:
                    raise NotImplementedError("long-term list modification")
    if pps["weighted_pred"] and h["type"] == 0:
        raise NotImplementedError("explicit weighted prediction")
    h["mmco"] = []
    if nal_ref_idc:
        if h["idr"]:
            b.u(1)  # no_output_of_prior_pics_flag
            if b.u(1):
                raise NotImplementedError("long-term IDR")
        elif b.u(1):  # adaptive_ref_pic_marking_mode_flag
            while True:
                op = b.ue()
                if op == 0:
                    break
                if op == 1:
                    h["mmco"].append((1, b.ue() + 1))
                else:
                    raise NotImplementedError(f"memory management operation {op}")
    h["qp"] = pps["init_qp"] + b.se()
    h["deblock_idc"], h["alpha"], h["beta"] = 0, 0, 0
    if pps["deblock_ctrl"]:
        h["deblock_idc"] = b.ue()
        if h["deblock_idc"] != 1:
            h["alpha"] = b.se() * 2
            h["beta"] = b.se() * 2
    return h


# ---------------------------------------------------------------------------
# CAVLC residual blocks (src/h264/dec/cavlc.rs)
# ---------------------------------------------------------------------------
def _coeff_token(b: Bits, nc: int):
    if nc >= 8:
        v = b.u(6)
        if v == 3:
            return 0, 0
        tc, t1 = (v >> 2) + 1, v & 3
        if t1 > tc:
            raise ValueError("bad fixed-length coeff_token")
        return t1, tc
    cls = 4 if nc < 0 else 0 if nc < 2 else 1 if nc < 4 else 2
    return b.code(_CT_DEC[cls])


def residual_block(b: Bits, nc: int, max_coeff: int):
    """Levels of one block in scan order (length max_coeff) and TotalCoeff."""
    t1, tc = _coeff_token(b, nc)
    coef = [0] * max_coeff
    if tc == 0:
        return coef, 0
    if tc > max_coeff:
        raise ValueError("TotalCoeff exceeds the block")
    levels = []
    suffix = 1 if (tc > 10 and t1 < 3) else 0
    for i in range(tc):
        if i < t1:
            levels.append(-1 if b.u(1) else 1)
            continue
        prefix = 0
        while b.u(1) == 0:
            prefix += 1
            if prefix > 32:
                raise ValueError("bad level_prefix")
        code = min(15, prefix) << suffix
        size = suffix
        if prefix == 14 and suffix == 0:
            size = 4
        if prefix >= 15:
            size = prefix - 3
        if size:
            code += b.u(size)
        if prefix >= 15 and suffix == 0:
            code += 15
        if prefix >= 16:
            code += (1 << (prefix - 3)) - 4096
        if i == t1 and t1 < 3:
            code += 2
        lev = (code + 2) >> 1 if code % 2 == 0 else (-code - 1) >> 1
        levels.append(lev)
        if suffix == 0:
            suffix = 1
        if abs(lev) > (3 << (suffix - 1)) and suffix < 6:
            suffix += 1
    if tc < max_coeff:
        tz = b.code((_TZ2_DEC if max_coeff == 4 else _TZ4_DEC)[tc - 1])
    else:
        tz = 0
    runs = []
    left = tz
    for i in range(tc - 1):
        r = b.code(_RB_DEC[min(left, 7) - 1]) if left > 0 else 0
        runs.append(r)
        left -= r
    runs.append(left)
    pos = -1
    for i in range(tc - 1, -1, -1):
        pos += runs[i] + 1
        if pos >= max_coeff:
            raise ValueError("coefficient run past the block")
        coef[pos] = levels[i]
    return coef, tc


# ---------------------------------------------------------------------------
# Picture decoding state
# ---------------------------------------------------------------------------
class _Mb:
    __slots__ = ("slice", "kind", "qp", "modes", "tc", "tcc", "ref", "mv", "cbp", "i16", "cmode", "levels",
                 "dc", "luma_coded", "chroma_coded", "nz", "shape", "subs", "mvd")

    def __init__(self):
        self.slice = -1
        self.kind = None   # "I4", "I16", "PCM", "P", "SKIP"
        self.modes = [2] * 16          # raster 4x4 Intra4x4 modes
        self.tc = [0] * 16             # TotalCoeff per luma 4x4 (raster), 16 for PCM
        self.tcc = [[0] * 4, [0] * 4]  # chroma AC TotalCoeff per component and 4x4
        self.ref = [-1] * 16           # list-0 ref_idx per 4x4 (raster)
        self.mv = [(0, 0)] * 16
        self.levels = []
        self.dc = 0
        self.luma_coded = 0
        self.chroma_coded = 0
        self.nz = 0
        self.i16 = 0
        self.cmode = 0
        self.qp = 0
        self.shape = 0            # motion syntax: RC_H264_MOTION_*
        self.subs = [0] * 4       # P_8x8 sub-partitions (RC_H264_SUB_*)
        self.mvd = [(0, 0)] * 16  # list-0 mvd per 4x4 (raster)


class Frame:
    def __init__(self, ident: int, frame_num: int, slot: int):
        self.id, self.frame_num, self.slot = ident, frame_num, slot


class Decoder:
    """Parses a Baseline stream picture by picture into engine records."""

    def __init__(self, E, slots: int = 8):
        self.E = E
        self.spss, self.ppss = {}, {}
        self.refs = []        # short-term reference frames
        self.slots = slots
        self.count = 0
        self.pictures = []    # per decoded picture: dict of records and metadata
        self.cur = None

    # ---- picture boundaries
    def _start_picture(self, h, sps, pps):
        self.sps, self.pps = sps, pps
        n = sps["mb_w"] * sps["mb_h"]
        self.mbs = [_Mb() for _ in range(n)]
        self.slices = []
        self.levels = []
        self.cur = {"frame_num": h["frame_num"], "idr": h["idr"], "ref": None, "mmco": None}
        self.cur_slot = self.count % self.slots
        used = {f.slot for f in self.refs}
        if self.cur_slot in used:
            raise RuntimeError("DPB slot still referenced")

    def _finish_picture(self):
        if self.cur is None:
            return
        E = self.E
        sps = self.sps
        recs = (E.H264Mb * len(self.mbs))()
        levels = []
        for a, m in enumerate(self.mbs):
            r = recs[a]
            if m.kind is None:
                r.kind = E.RC_H264_NONE
                continue
            r.kind = {"I4": E.RC_H264_I4x4, "I16": E.RC_H264_I16x16, "PCM": E.RC_H264_IPCM}.get(m.kind, E.RC_H264_INTER)
            r.transform_8x8 = 0
            r.qp = m.qp
            qc = _QPC[max(0, min(51, m.qp + self.pps["chroma_qp_offset"]))]
            r.qpc[0] = r.qpc[1] = qc
            r.i16_mode = m.i16
            r.chroma_mode = m.cmode
            r.dc_coded = m.dc
            r.slice = m.slice
            r.nz_mask = m.nz
            r.luma_coded = m.luma_coded
            r.chroma_coded = m.chroma_coded
            r.coef_off = len(levels)
            levels.extend(m.levels)
            for i in range(16):
                r.intra_modes[i] = m.modes[i] if m.kind == "I4" else 0
            for b8 in range(4):
                blk = (b8 >> 1) * 8 + (b8 & 1) * 2  # raster 4x4 index of the 8x8's top-left
                r.ref_idx[0][b8] = m.ref[blk] if m.kind in ("P", "SKIP") else -1
                r.ref_idx[1][b8] = -1
                r.wp[b8] = 0xFF
            for k in range(16):
                mx, my = m.mv[k] if m.kind in ("P", "SKIP") else (0, 0)
                r.mv[0][k][0], r.mv[0][k][1] = mx, my
                r.mv[1][k][0] = r.mv[1][k][1] = 0
        # motion syntax (P slices: list 0 only, no direct modes, no weights)
        mos = (E.H264Motion * len(self.mbs))()
        for a, m in enumerate(self.mbs):
            if m.kind not in ("P", "SKIP"):
                continue
            o = mos[a]
            o.shape = m.shape
            for i in range(4):
                o.pred[i] = 1 if m.kind == "P" and (m.shape == 5 or i < (1 if m.shape == 2 else 2)) else 0
                o.sub[i] = m.subs[i] if m.shape == 5 else 0
            for b8 in range(4):
                o.ref_idx[0][b8] = m.ref[(b8 >> 1) * 8 + (b8 & 1) * 2] if m.kind == "P" else -1
                o.ref_idx[1][b8] = -1
            for k in range(16):
                o.mvd[0][k][0], o.mvd[0][k][1] = m.mvd[k] if m.kind == "P" else (0, 0)
        smo = (E.H264SliceMotion * len(self.slices))()
        for i in range(len(self.slices)):
            smo[i].col_slot = -1
            for j in range(33 * 33):
                smo[i].wp_map[j] = 0xFF
        sl = (E.H264Slice * len(self.slices))()
        for i, s in enumerate(self.slices):
            sl[i].disable_deblocking_filter_idc = s["deblock_idc"]
            sl[i].alpha_offset = s["alpha"]
            sl[i].beta_offset = s["beta"]
            sl[i].num_ref[0] = len(s["list"])
            sl[i].num_ref[1] = 0
            for j, f in enumerate(s["list"]):
                sl[i].ref_slot[0][j] = f.slot
                sl[i].ref_id[0][j] = f.id
        import array
        lv = array.array("h", levels)
        self.pictures.append({"mbs": bytes(recs), "slices": bytes(sl), "weights": b"", "levels": lv.tobytes(),
                              "motion": bytes(mos), "slice_motion": bytes(smo),
                              "num_slices": len(self.slices), "slot": self.cur_slot, "frame_id": self.count,
                              "constrained_intra": self.pps["constrained_intra"],
                              "mb_w": sps["mb_w"], "mb_h": sps["mb_h"], "crop": sps["crop"]})
        # reference marking (src/syntax/h264/dpb.rs): IDR empties the DPB;
        # otherwise memory-management operations or the sliding window
        frame = Frame(self.count, self.cur["frame_num"], self.cur_slot)
        if self.cur["ref"]:
            if self.cur["idr"]:
                self.refs = []
            elif self.cur["mmco"]:
                for op, diff in self.cur["mmco"]:
                    pic_num = self.cur["frame_num"] - diff
                    self.refs = [f for f in self.refs if self._pic_num(f) != pic_num]
            else:
                if len(self.refs) >= max(1, self.sps["max_num_ref_frames"]):
                    oldest = min(self.refs, key=self._pic_num)
                    self.refs.remove(oldest)
            self.refs.append(frame)
        self.count += 1
        self.cur = None

    def _pic_num(self, f):
        maxf = 1 << self.sps["log2_max_frame_num"]
        return f.frame_num - maxf if f.frame_num > self.cur["frame_num"] else f.frame_num

    def _ref_list(self, h):
        lst = sorted(self.refs, key=self._pic_num, reverse=True)
        maxf = 1 << self.sps["log2_max_frame_num"]
        pred = self.cur["frame_num"]
        for i, (idc, absdiff) in enumerate(h["mods"]):
            pn = pred - absdiff if idc == 0 else pred + absdiff
            pn = pn + maxf if pn < 0 else pn - maxf if pn >= maxf else pn
            pred = pn
            want = pn - maxf if pn > self.cur["frame_num"] else pn
            f = next(f for f in self.refs if self._pic_num(f) == want)
            lst = [x for x in lst if x is not f]
            lst.insert(i, f)
        lst = lst[: h["num_ref"]]
        if len(lst) < h["num_ref"] and h["type"] == 0:
            raise RuntimeError("reference list shorter than num_ref_idx_active")
        return lst

    # ---- stream
    def decode(self, data: bytes):
        for ref_idc, t, rbsp in nal_units(data):
            b = Bits(rbsp)
            if t == 7:
                s = parse_sps(b)
                self.spss[s["id"]] = s
            elif t == 8:
                p = parse_pps(b)
                self.ppss[p["id"]] = p
            elif t in (1, 5):
                h = parse_slice_header(b, t, ref_idc, self.spss, self.ppss)
                pps = self.ppss[h["pps_id"]]
                sps = self.spss[pps["sps_id"]]
                if h["first_mb"] == 0:
                    self._finish_picture()
                    self._start_picture(h, sps, pps)
                self.cur["ref"] = bool(ref_idc)
                if h["mmco"]:
                    self.cur["mmco"] = h["mmco"]
                self._slice(b, h)
            elif t in (6, 9, 10, 11, 12):
                continue
            else:
                raise NotImplementedError(f"NAL unit type {t}")
        self._finish_picture()
        return self.pictures

    # ---- slice data (7.3.4)
    def _slice(self, b: Bits, h):
        sid = len(self.slices)
        lst = self._ref_list(h) if h["type"] == 0 else []
        self.slices.append({"deblock_idc": h["deblock_idc"], "alpha": h["alpha"], "beta": h["beta"], "list": lst})
        self.slice_first = h["first_mb"]
        self.slice_id = sid
        self.num_ref = h["num_ref"] if h["type"] == 0 else 0
        qp = h["qp"]
        addr = h["first_mb"]
        n = len(self.mbs)
        more = True
        while more:
            if h["type"] == 0:
                run = b.ue()
                for _ in range(run):
                    if addr >= n:
                        raise ValueError("skip run past the picture")
                    self._skip(addr, qp)
                    addr += 1
                if run > 0:
                    more = b.more_rbsp_data()
                    if not more:
                        break
            if addr >= n:
                raise ValueError("macroblock past the picture")
            qp = self._macroblock(b, addr, qp, h["type"] == 0)
            more = b.more_rbsp_data()
            addr += 1

    # ---- neighbours
    def _avail(self, a, addr):
        return 0 <= a < addr and self.mbs[a].slice == self.slice_id

    def _nb(self, addr, dx, dy):
        """MB address of the neighbour (dx, dy) in MB units, or -1."""
        mw = self.sps["mb_w"]
        x, y = addr % mw + dx, addr // mw + dy
        if x < 0 or y < 0 or x >= mw:
            return -1
        a = y * mw + x
        return a if self._avail(a, addr) else -1

    def _luma_nb(self, addr, x, y):
        """(MB address, raster 4x4 index) of the luma sample (x, y) relative to
        the current MB's top-left; -1 when not available."""
        if y >= 16 or (x >= 16 and y >= 0):
            return -1, 0
        dx = -1 if x < 0 else 1 if x >= 16 else 0
        dy = -1 if y < 0 else 0
        a = addr if (dx == 0 and dy == 0) else self._nb(addr, dx, dy)
        if a < 0:
            return -1, 0
        xx, yy = x % 16, y % 16
        return a, (yy >> 2) * 4 + (xx >> 2)

    def _nc_luma(self, addr, blk):
        x, y = (blk & 3) * 4, (blk >> 2) * 4
        vals = []
        for nx, ny in ((x - 1, y), (x, y - 1)):
            a, k = self._luma_nb(addr, nx, ny)
            if a >= 0:
                vals.append(self.mbs[a].tc[k])
        return (vals[0] + vals[1] + 1) >> 1 if len(vals) == 2 else vals[0] if vals else 0

    def _nc_chroma(self, addr, c, blk):
        x, y = (blk & 1) * 4, (blk >> 1) * 4
        vals = []
        for nx, ny in ((x - 1, y), (x, y - 1)):
            dx = -1 if nx < 0 else 0
            dy = -1 if ny < 0 else 0
            a = addr if (dx == 0 and dy == 0) else self._nb(addr, dx, dy)
            if a < 0:
                continue
            m = self.mbs[a]
            kk = ((ny % 8) >> 2) * 2 + ((nx % 8) >> 2)
            vals.append(16 if m.kind == "PCM" else m.tcc[c][kk])
        return (vals[0] + vals[1] + 1) >> 1 if len(vals) == 2 else vals[0] if vals else 0

    # ---- P_Skip (8.4.1.1)
    def _skip(self, addr, qp):
        m = self.mbs[addr]
        m.slice, m.kind, m.qp = self.slice_id, "SKIP", qp
        m.shape = 1  # RC_H264_MOTION_SKIP
        m.ref = [-1] * 16
        m.mv = [(0, 0)] * 16
        done = [False] * 16
        a = self._mv_nb(addr, -1, 0, done)
        bb = self._mv_nb(addr, 0, -1, done)
        if a[0] < -1 or bb[0] < -1 or (a[0] == 0 and a[1] == (0, 0)) or (bb[0] == 0 and bb[1] == (0, 0)):
            mv = (0, 0)
        else:
            mv = self._mvp(addr, 0, 0, 16, 16, 0, done, "16x16", 0)
        m.ref = [0] * 16
        m.mv = [mv] * 16

    # neighbour partition at luma (x, y): (ref_idx, mv); ref -2 = not available
    def _mv_nb(self, addr, x, y, done):
        a, k = self._luma_nb(addr, x, y)
        if a < 0:
            return -2, (0, 0)
        if a == addr and not done[k]:
            return -2, (0, 0)
        m = self.mbs[a]
        if m.kind not in ("P", "SKIP"):
            return -1, (0, 0)
        return m.ref[k], m.mv[k]

    def _mvp(self, addr, x, y, w, h, ref, done, shape, part):
        """Motion-vector predictor of the partition at (x, y), size w x h (8.4.1.3)."""
        A = self._mv_nb(addr, x - 1, y, done)
        B = self._mv_nb(addr, x, y - 1, done)
        C = self._mv_nb(addr, x + w, y - 1, done)
        if C[0] == -2:
            C = self._mv_nb(addr, x - 1, y - 1, done)
        if B[0] == -2 and C[0] == -2 and A[0] != -2:
            B, C = A, A
        A, B, C = [((r if r >= -1 else -1), mv) for r, mv in (A, B, C)]
        if shape == "16x8":
            if part == 0 and B[0] == ref:
                return B[1]
            if part == 1 and A[0] == ref:
                return A[1]
        elif shape == "8x16":
            if part == 0 and A[0] == ref:
                return A[1]
            if part == 1 and C[0] == ref:
                return C[1]
        same = [n for n in (A, B, C) if n[0] == ref]
        if len(same) == 1:
            return same[0][1]
        med = lambda p, q, r: max(min(p, q), min(max(p, q), r))
        return (med(A[1][0], B[1][0], C[1][0]), med(A[1][1], B[1][1], C[1][1]))

    # ---- macroblock_layer (7.3.5)
    def _macroblock(self, b: Bits, addr: int, qp: int, pslice: bool) -> int:
        m = self.mbs[addr]
        m.slice = self.slice_id
        t = b.ue()
        if pslice:
            if t < 5:
                return self._inter_mb(b, addr, t, qp)
            t -= 5
        if t == 25:
            b.align()
            samples = [b.u(8) for _ in range(384)]
            m.kind, m.qp = "PCM", 0
            m.tc = [16] * 16
            m.tcc = [[16] * 4, [16] * 4]
            m.levels = samples
            m.nz = 0xFFFF
            return qp  # QP_Y of I_PCM is the prediction (no mb_qp_delta); the loop filter uses 0
        if t == 0:
            m.kind = "I4"
            modes_dec = []
            for _ in range(16):
                flag = b.u(1)
                modes_dec.append(-1 if flag else b.u(3))
            m.cmode = b.ue()
            self._intra4_modes(addr, modes_dec)
            cbp = _CBP[b.ue()][0]
        elif 1 <= t <= 24:
            m.kind = "I16"
            m.i16 = (t - 1) % 4
            cbp = (15 if t >= 13 else 0) | ((((t - 1) // 4) % 3) << 4)
            m.cmode = b.ue()
        else:
            raise ValueError(f"mb_type {t}")
        return self._residual(b, addr, cbp, qp)

    def _intra4_modes(self, addr, modes_dec):
        m = self.mbs[addr]
        cip = self.pps["constrained_intra"]
        for i, code in enumerate(modes_dec):
            k = _BLK_RASTER[i]
            x, y = (k & 3) * 4, (k >> 2) * 4
            modes = []
            dc = False
            for nx, ny in ((x - 1, y), (x, y - 1)):
                a, kk = self._luma_nb(addr, nx, ny)
                if a < 0:
                    dc = True
                    break
                n = self.mbs[a]
                if n.kind in ("P", "SKIP") and cip:
                    dc = True
                    break
                modes.append(n.modes[kk] if (n.kind == "I4" and a != addr) or a == addr else 2)
            pred = 2 if dc else min(modes)
            m.modes[k] = pred if code < 0 else (code if code < pred else code + 1)

    def _inter_mb(self, b: Bits, addr: int, t: int, qp: int) -> int:
        m = self.mbs[addr]
        m.kind = "P"
        m.ref = [-1] * 16
        m.mv = [(0, 0)] * 16
        done = [False] * 16
        nref = self.num_ref
        if t <= 2:
            parts = {0: [(0, 0, 16, 16)], 1: [(0, 0, 16, 8), (0, 8, 16, 8)], 2: [(0, 0, 8, 16), (8, 0, 8, 16)]}[t]
            shape = {0: "16x16", 1: "16x8", 2: "8x16"}[t]
            refs = [b.te(nref - 1) if nref > 1 else 0 for _ in parts]
            m.shape = 2 + t
            m.mvd = [(0, 0)] * 16
            for pi, (x, y, w, h) in enumerate(parts):
                mvd = (b.se(), b.se())
                p = self._mvp(addr, x, y, w, h, refs[pi], done, shape, pi)
                mv = (p[0] + mvd[0], p[1] + mvd[1])
                self._fill(m, done, x, y, w, h, refs[pi], mv, mvd)
        else:
            subs = [b.ue() for _ in range(4)]
            refs = [b.te(nref - 1) if (nref > 1 and t == 3) else 0 for _ in range(4)]
            m.shape, m.subs = 5, list(subs)
            m.mvd = [(0, 0)] * 16
            for i8 in range(4):
                x8, y8 = (i8 & 1) * 8, (i8 >> 1) * 8
                st = subs[i8]
                sp = {0: [(0, 0, 8, 8)], 1: [(0, 0, 8, 4), (0, 4, 8, 4)], 2: [(0, 0, 4, 8), (4, 0, 4, 8)],
                      3: [(0, 0, 4, 4), (4, 0, 4, 4), (0, 4, 4, 4), (4, 4, 4, 4)]}[st]
                for (x, y, w, h) in sp:
                    mvd = (b.se(), b.se())
                    p = self._mvp(addr, x8 + x, y8 + y, w, h, refs[i8], done, "sub", 0)
                    mv = (p[0] + mvd[0], p[1] + mvd[1])
                    self._fill(m, done, x8 + x, y8 + y, w, h, refs[i8], mv, mvd)
        cbp = _CBP[b.ue()][1]
        return self._residual(b, addr, cbp, qp)

    @staticmethod
    def _fill(m, done, x, y, w, h, ref, mv, mvd):
        for yy in range(y >> 2, (y + h) >> 2):
            for xx in range(x >> 2, (x + w) >> 2):
                k = yy * 4 + xx
                m.ref[k], m.mv[k], m.mvd[k], done[k] = ref, mv, mvd, True

    # ---- residual (7.3.5.3), levels stored as the engine's payload
    def _residual(self, b: Bits, addr: int, cbp: int, qp: int) -> int:
        m = self.mbs[addr]
        i16 = m.kind == "I16"
        luma, chroma = cbp & 15, cbp >> 4
        if luma or chroma or i16:
            qp = (qp + b.se() + 52) % 52
        m.qp = qp
        m.cbp = cbp
        payload = []
        if i16:
            dc, tc = residual_block(b, self._nc_luma(addr, 0), 16)
            if tc:
                m.dc |= 1
                payload.extend(dc)
        blocks = {}
        for i in range(16):
            k = _BLK_RASTER[i]
            if not (luma >> (i // 4)) & 1:
                m.tc[k] = 0
                continue
            if i16:
                ac, tc = residual_block(b, self._nc_luma(addr, k), 15)
                coef = [0] + ac
            else:
                coef, tc = residual_block(b, self._nc_luma(addr, k), 16)
            m.tc[k] = tc
            if tc:
                blocks[k] = coef
        for k in sorted(blocks):  # the engine's payload: coded 4x4 blocks in raster order
            m.luma_coded |= 1 << k
            payload.extend(blocks[k])
        m.nz = sum(1 << k for k in range(16) if m.tc[k])
        cdc = [[0] * 4, [0] * 4]
        if chroma & 3:
            for c in range(2):
                cdc[c], tc = residual_block(b, -1, 4)
                if tc:
                    m.dc |= 2 << c
        for c in range(2):
            if m.dc >> (1 + c) & 1:
                payload.extend(cdc[c])
        cac = {}
        for c in range(2):
            for blk in range(4):
                if chroma & 2:
                    ac, tc = residual_block(b, self._nc_chroma(addr, c, blk), 15)
                    m.tcc[c][blk] = tc
                    if tc:
                        cac[c * 4 + blk] = [0] + ac
                else:
                    m.tcc[c][blk] = 0
        for bit in sorted(cac):
            m.chroma_coded |= 1 << bit
            payload.extend(cac[bit])
        m.levels = payload
        return qp
