"""HEVC Main / Main10 parse into reconstruction records.

TEST INFRASTRUCTURE: this module turns an HEVC elementary stream (Annex B)
into the per-picture syntax records of include/pito_recon.h (rc_hevc_ctb,
rc_hevc_blk, rc_hevc_mvf, rc_hevc_tu, rc_hevc_slice, levels, expanded
scaling factors), so that the reference's golden x265 streams
(tests/refs/hevc/*.hevc, sha256 of their reconstructions in
tests/refs/hevc/manifest.toml) can drive the oracle and the GPU engine end
to end.  It restates, in this project's own code, the parse half of the
reference decoder:

  parameter sets, slice headers, RPS and POC   src/syntax/hevc/{params,slice,dpb}.rs
  CABAC engine and context initialisation      src/hevc/cabac.rs
  CTU / CU / PU / TU / residual / SAO syntax   src/hevc/slicedec.rs:846-2203
  merge, AMVP and temporal MV prediction       src/hevc/mvpred.rs:82-301
  reference lists, DPB and output order        src/hevc/decoder.rs, src/syntax/hevc/dpb.rs

following ITU-T H.265 (v1) clauses 7.3, 7.4, 8.3, 8.4.2, 8.5.3, 8.6.1 and
9.3.  Tools outside Main / Main10 (range extensions, long-term reference
pictures, field coding) raise NotImplementedError.  Nothing in the engine
imports it.
"""
from __future__ import annotations

import ctypes

import numpy as np

# ---------------------------------------------------------------------------
# CABAC tables (H.265 9.3.2.2 Tables 9-5..9-37 initValue per context; 9.3.4.3
# Tables 9-46 rangeTabLps and 9-47 transIdxLps).  The reference holds the same
# standard values in src/hevc/spec_tables.rs:35-69 and src/syntax/cabac.rs.
# Per syntax element: (initType 0, initType 1, initType 2).
# ---------------------------------------------------------------------------
_INIT = {
    "sao_merge": ([153], [153], [153]),
    "sao_type": ([200], [185], [160]),
    "split_cu": ([139, 141, 157], [107, 139, 126], [107, 139, 126]),
    "transquant_bypass": ([154], [154], [154]),
    "cu_skip": ([154, 154, 154], [197, 185, 201], [197, 185, 201]),
    "pred_mode": ([154], [149], [134]),
    "part_mode": ([184, 154, 154, 154], [154, 139, 154, 154], [154, 139, 154, 154]),
    "prev_intra_luma": ([184], [154], [183]),
    "intra_chroma": ([63], [152], [152]),
    "rqt_root_cbf": ([154], [79], [79]),
    "merge_flag": ([154], [110], [154]),
    "merge_idx": ([154], [122], [137]),
    "inter_pred_idc": ([154] * 5, [95, 79, 63, 31, 31], [95, 79, 63, 31, 31]),
    "ref_idx": ([154, 154], [153, 153], [153, 153]),
    "mvp_flag": ([154], [168], [168]),
    "split_transform": ([153, 138, 138], [124, 138, 94], [224, 167, 122]),
    "cbf_luma": ([111, 141], [153, 111], [153, 111]),
    "cbf_chroma": ([94, 138, 182, 154], [149, 107, 167, 154], [149, 92, 167, 154]),
    "mvd_gt0": ([154], [140], [169]),
    "mvd_gt1": ([154], [198], [198]),
    "cu_qp_delta_abs": ([154, 154], [154, 154], [154, 154]),
    "transform_skip": ([139, 139], [139, 139], [139, 139]),
    "last_x_prefix": ([110, 110, 124, 125, 140, 153, 125, 127, 140, 109, 111, 143, 127, 111, 79, 108, 123, 63],
                      [125, 110, 94, 110, 95, 79, 125, 111, 110, 78, 110, 111, 111, 95, 94, 108, 123, 108],
                      [125, 110, 124, 110, 95, 94, 125, 111, 111, 79, 125, 126, 111, 111, 79, 108, 123, 93]),
    "last_y_prefix": ([110, 110, 124, 125, 140, 153, 125, 127, 140, 109, 111, 143, 127, 111, 79, 108, 123, 63],
                      [125, 110, 94, 110, 95, 79, 125, 111, 110, 78, 110, 111, 111, 95, 94, 108, 123, 108],
                      [125, 110, 124, 110, 95, 94, 125, 111, 111, 79, 125, 126, 111, 111, 79, 108, 123, 93]),
    "coded_sub_block": ([91, 171, 134, 141], [121, 140, 61, 154], [121, 140, 61, 154]),
    "sig_coeff": ([111, 111, 125, 110, 110, 94, 124, 108, 124, 107, 125, 141, 179, 153, 125, 107, 125, 141, 179,
                   153, 125, 107, 125, 141, 179, 153, 125, 140, 139, 182, 182, 152, 136, 152, 136, 153, 136, 139,
                   111, 136, 139, 111],
                  [155, 154, 139, 153, 139, 123, 123, 63, 153, 166, 183, 140, 136, 153, 154, 166, 183, 140, 136,
                   153, 154, 166, 183, 140, 136, 153, 154, 170, 153, 123, 123, 107, 121, 107, 121, 167, 151, 183,
                   140, 151, 183, 140],
                  [170, 154, 139, 153, 139, 123, 123, 63, 124, 166, 183, 140, 136, 153, 154, 166, 183, 140, 136,
                   153, 154, 166, 183, 140, 136, 153, 154, 170, 153, 138, 138, 122, 121, 122, 121, 167, 151, 183,
                   140, 151, 183, 140]),
    "gt1": ([140, 92, 137, 138, 140, 152, 138, 139, 153, 74, 149, 92, 139, 107, 122, 152, 140, 179, 166, 182, 140,
             227, 122, 197],
            [154, 196, 196, 167, 154, 152, 167, 182, 182, 134, 149, 136, 153, 121, 136, 137, 169, 194, 166, 167, 154,
             167, 137, 182],
            [154, 196, 167, 167, 154, 152, 167, 182, 182, 134, 149, 136, 153, 121, 136, 122, 169, 208, 166, 167, 154,
             152, 167, 182]),
    "gt2": ([138, 153, 136, 167, 152, 152], [107, 167, 91, 122, 107, 167], [107, 167, 91, 107, 107, 167]),
}
# context index of each element's first context, in this module's layout
CTX = {}
_n = 0
for _k, _v in _INIT.items():
    CTX[_k] = _n
    _n += len(_v[0])
NUM_CTX = _n
_INIT_FLAT = [sum((list(v[t]) for v in _INIT.values()), []) for t in range(3)]

_RANGE_LPS = [
    (128, 176, 208, 240), (128, 167, 197, 227), (128, 158, 187, 216), (123, 150, 178, 205), (116, 142, 169, 195),
    (111, 135, 160, 185), (105, 128, 152, 175), (100, 122, 144, 166), (95, 116, 137, 158), (90, 110, 130, 150),
    (85, 104, 123, 142), (81, 99, 117, 135), (77, 94, 111, 128), (73, 89, 105, 122), (69, 85, 100, 116),
    (66, 80, 95, 110), (62, 76, 90, 104), (59, 72, 86, 99), (56, 69, 81, 94), (53, 65, 77, 89), (51, 62, 73, 85),
    (48, 59, 69, 80), (46, 56, 66, 76), (43, 53, 63, 72), (41, 50, 59, 69), (39, 48, 56, 65), (37, 45, 54, 62),
    (35, 43, 51, 59), (33, 41, 48, 56), (32, 39, 46, 53), (30, 37, 43, 50), (29, 35, 41, 48), (27, 33, 39, 45),
    (26, 31, 37, 43), (24, 30, 35, 41), (23, 28, 33, 39), (22, 27, 32, 37), (21, 26, 30, 35), (20, 24, 29, 33),
    (19, 23, 27, 31), (18, 22, 26, 30), (17, 21, 25, 28), (16, 20, 23, 27), (15, 19, 22, 25), (14, 18, 21, 24),
    (14, 17, 20, 23), (13, 16, 19, 22), (12, 15, 18, 21), (12, 14, 17, 20), (11, 14, 16, 19), (11, 13, 15, 18),
    (10, 12, 15, 17), (10, 12, 14, 16), (9, 11, 13, 15), (9, 11, 12, 14), (8, 10, 12, 14), (8, 9, 11, 13),
    (7, 9, 11, 12), (7, 9, 10, 12), (7, 8, 10, 11), (6, 8, 9, 11), (6, 7, 9, 10), (6, 7, 8, 9), (2, 2, 2, 2),
]
_TRANS_LPS = [0, 0, 1, 2, 2, 4, 4, 5, 6, 7, 8, 9, 9, 11, 11, 12, 13, 13, 15, 15, 16, 16, 18, 18, 19, 19, 21, 21, 22,
              22, 23, 24, 24, 25, 26, 26, 27, 27, 28, 29, 29, 30, 30, 30, 31, 32, 32, 33, 33, 33, 34, 34, 35, 35, 35,
              36, 36, 36, 37, 37, 37, 38, 38, 63]
# state = pStateIdx << 1 | valMps
_NEXT_MPS = [(min((s >> 1) + 1, 62) << 1) | (s & 1) for s in range(128)]
_NEXT_LPS = [(_TRANS_LPS[s >> 1] << 1) | ((s & 1) ^ (1 if (s >> 1) == 0 else 0)) for s in range(128)]
_LPS_BY_STATE = [_RANGE_LPS[s >> 1] for s in range(128)]


def _init_state(v: int, qp: int) -> int:
    """9.3.2.2: context state from initValue and SliceQpY."""
    slope, offset = (v >> 4) * 5 - 45, ((v & 15) << 3) - 16
    pre = min(max(((slope * max(0, min(51, qp))) >> 4) + offset, 1), 126)
    return ((63 - pre) << 1) if pre <= 63 else (((pre - 64) << 1) | 1)


class Cabac:
    """The arithmetic decoder of 9.3.4.3 with the standard's 9-bit offset
    register, reading one bit per renormalisation step, so that the bit
    position after a terminating bin is exact (PCM samples and substream
    ends are located from it)."""

    def __init__(self, data: bytes, bitpos: int):
        self.data = data
        self.nbits = len(data) * 8
        self.st = [0] * NUM_CTX
        self.start(bitpos)

    def start(self, bitpos: int):
        self.pos = bitpos
        self.rng = 510
        self.off = self.bits(9)

    def bit(self) -> int:
        p = self.pos
        self.pos = p + 1
        if p >= self.nbits:
            return 0
        return (self.data[p >> 3] >> (7 - (p & 7))) & 1

    def bits(self, n: int) -> int:
        v = 0
        for _ in range(n):
            v = (v << 1) | self.bit()
        return v

    def init_contexts(self, qp: int, init_type: int):
        self.st = [_init_state(v, qp) for v in _INIT_FLAT[init_type]]

    def dec(self, ci: int) -> int:
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

    def byp(self) -> int:
        self.off = (self.off << 1) | self.bit()
        if self.off >= self.rng:
            self.off -= self.rng
            return 1
        return 0

    def byp_bits(self, n: int) -> int:
        v = 0
        for _ in range(n):
            v = (v << 1) | self.byp()
        return v

    def term(self) -> int:
        self.rng -= 2
        if self.off >= self.rng:
            return 1
        while self.rng < 256:
            self.rng <<= 1
            self.off = (self.off << 1) | self.bit()
        return 0


# ---------------------------------------------------------------------------
# Bitstream: NAL units and RBSP with the positions of removed emulation
# prevention bytes (entry points count them).
# ---------------------------------------------------------------------------
def nal_units(data: bytes):
    """Annex B byte stream -> NAL unit payloads (with emulation prevention)."""
    out, i, n = [], 0, len(data)
    starts = []
    while i + 3 <= n:
        if data[i] == 0 and data[i + 1] == 0 and data[i + 2] == 1:
            starts.append(i + 3)
            i += 3
        else:
            i += 1
    for k, s in enumerate(starts):
        e = starts[k + 1] - 3 if k + 1 < len(starts) else n
        while e > s and data[e - 1] == 0:
            e -= 1
        out.append(data[s:e])
    return out


def unescape(nal: bytes):
    """RBSP bytes and, for each removed 0x03, its index in the escaped NAL."""
    out, removed, zeros = bytearray(), [], 0
    for i, b in enumerate(nal):
        if zeros >= 2 and b == 3:
            removed.append(i)
            zeros = 0
            continue
        out.append(b)
        zeros = zeros + 1 if b == 0 else 0
    return bytes(out), removed


class Bits:
    def __init__(self, data: bytes, pos: int = 0):
        self.data, self.pos = data, pos

    def u(self, n: int) -> int:
        v = 0
        for _ in range(n):
            p = self.pos
            v = (v << 1) | ((self.data[p >> 3] >> (7 - (p & 7))) & 1 if p < len(self.data) * 8 else 0)
            self.pos = p + 1
        return v

    def ue(self) -> int:
        z = 0
        while self.u(1) == 0:
            z += 1
            if z > 32:
                raise ValueError("bad exp-Golomb code")
        return (1 << z) - 1 + self.u(z)

    def se(self) -> int:
        k = self.ue()
        return (k + 1) // 2 if k & 1 else -(k // 2)

    def align(self):
        self.pos = (self.pos + 7) & ~7


def _ceil_log2(v: int) -> int:
    n = 0
    while (1 << n) < v:
        n += 1
    return n


# ---------------------------------------------------------------------------
# Scans (6.5.3-6.5.5) and the scaling-list defaults (7.4.5 Table 7-6)
# ---------------------------------------------------------------------------
def _diag_scan(n: int):
    out, x, y = [], 0, 0
    while len(out) < n * n:
        while y >= 0:
            if x < n and y < n:
                out.append((x, y))
            y -= 1
            x += 1
        y, x = x, 0
    return out


SCAN = {}
for _s in (1, 2, 4, 8):
    SCAN[(_s, 0)] = _diag_scan(_s)
    SCAN[(_s, 1)] = [(x, y) for y in range(_s) for x in range(_s)]
    SCAN[(_s, 2)] = [(x, y) for x in range(_s) for y in range(_s)]

_DEF_INTRA8 = [16, 16, 16, 16, 16, 16, 16, 16, 16, 16, 17, 16, 17, 16, 17, 18, 17, 18, 18, 17, 18, 21, 19, 20, 21, 20,
               19, 21, 24, 22, 22, 24, 24, 22, 22, 24, 25, 25, 27, 30, 27, 25, 25, 29, 31, 35, 35, 31, 29, 36, 41, 44,
               41, 36, 47, 54, 54, 47, 65, 70, 65, 88, 88, 115]
_DEF_INTER8 = [16, 16, 16, 16, 16, 16, 16, 16, 16, 16, 17, 17, 17, 17, 17, 18, 18, 18, 18, 18, 18, 20, 20, 20, 20, 20,
               20, 20, 24, 24, 24, 24, 24, 24, 24, 24, 25, 25, 25, 25, 25, 25, 25, 28, 28, 28, 28, 28, 28, 33, 33, 33,
               33, 33, 41, 41, 41, 41, 54, 54, 54, 71, 71, 91]
_CTX_IDX_MAP = [0, 1, 4, 5, 2, 3, 4, 5, 6, 6, 8, 8, 7, 7, 8]


def _default_lists():
    """ScalingList[sizeId][matrixId] (coefficients in diagonal scan order) and
    the DC values of sizeId 2, 3."""
    lists = [[[16] * 16 for _ in range(6)]]
    for _ in range(3):
        lists.append([list(_DEF_INTRA8) if m < 3 else list(_DEF_INTER8) for m in range(6)])
    dc = {(s, m): 16 for s in (2, 3) for m in range(6)}
    return lists, dc


def parse_scaling_list_data(b: Bits):
    """7.3.4 scaling_list_data with the prediction rules of 7.4.5."""
    lists, dc = _default_lists()
    for size_id in range(4):
        step = 3 if size_id == 3 else 1
        for mid in range(0, 6, step):
            if not b.u(1):  # scaling_list_pred_mode_flag
                delta = b.ue()
                if delta:
                    ref = mid - delta * step
                    lists[size_id][mid] = list(lists[size_id][ref])
                    if size_id > 1:
                        dc[(size_id, mid)] = dc[(size_id, ref)]
                else:
                    d = _default_lists()
                    lists[size_id][mid] = list(d[0][size_id][mid])
                    if size_id > 1:
                        dc[(size_id, mid)] = 16
            else:
                nxt, n = 8, min(64, 1 << (4 + (size_id << 1)))
                if size_id > 1:
                    v = b.se() + 8
                    dc[(size_id, mid)] = v
                    nxt = v
                out = []
                for _ in range(n):
                    nxt = (nxt + b.se() + 256) % 256
                    out.append(nxt)
                lists[size_id][mid] = out
    # chroma 32x32 (matrixId 1, 2, 4, 5) are not coded for 4:2:0 and unused
    for mid in (1, 2, 4, 5):
        lists[3][mid] = list(lists[3][0 if mid < 3 else 3])
        dc[(3, mid)] = dc[(3, 0 if mid < 3 else 3)]
    return lists, dc


def scaling_factors(lists, dc) -> bytes:
    """ScalingFactor (7.4.5) as the engine's expanded table: per sizeId
    (4..32) and matrixId (intra Y Cb Cr, inter Y Cb Cr), n*n bytes, row-major."""
    out = bytearray()
    for size_id in range(4):
        n = 4 << size_id
        for mid in range(6):
            sl = lists[size_id][mid]
            m = [[0] * n for _ in range(n)]
            if size_id == 0:
                for i, (x, y) in enumerate(SCAN[(4, 0)]):
                    m[y][x] = sl[i]
            else:
                rep = n // 8
                for i, (x, y) in enumerate(SCAN[(8, 0)]):
                    for j in range(rep):
                        for k in range(rep):
                            m[y * rep + j][x * rep + k] = sl[i]
                if size_id > 1:
                    m[0][0] = dc[(size_id, mid)]
            for row in m:
                out.extend(row)
    return bytes(out)


# ---------------------------------------------------------------------------
# Parameter sets and slice headers (7.3.2, 7.3.6)
# ---------------------------------------------------------------------------
def _profile_tier_level(b: Bits, max_sub_layers_minus1: int):
    b.u(88)  # general profile space, tier, idc, compatibility flags, constraint flags
    b.u(8)   # general_level_idc
    sub_prof, sub_lvl = [], []
    for _ in range(max_sub_layers_minus1):
        sub_prof.append(b.u(1))
        sub_lvl.append(b.u(1))
    if max_sub_layers_minus1 > 0:
        for _ in range(max_sub_layers_minus1, 8):
            b.u(2)
    for i in range(max_sub_layers_minus1):
        if sub_prof[i]:
            b.u(88)
        if sub_lvl[i]:
            b.u(8)


def _st_ref_pic_set(b: Bits, idx: int, num: int, sets: list) -> dict:
    """7.3.7 st_ref_pic_set with the derivation of 7.4.8."""
    inter = b.u(1) if idx != 0 else 0
    if inter:
        delta_idx = b.ue() + 1 if idx == num else 1
        sign = b.u(1)
        abs_delta = b.ue() + 1
        delta_rps = (1 - 2 * sign) * abs_delta
        ref = sets[idx - delta_idx]
        nd = len(ref["s0"]) + len(ref["s1"])
        used, use_delta = [], []
        for _ in range(nd + 1):
            u = b.u(1)
            used.append(u)
            use_delta.append(1 if u else b.u(1))
        s0, s1 = [], []
        rs0, rs1 = ref["s0"], ref["s1"]
        nn = len(rs0)
        for j in range(len(rs1) - 1, -1, -1):
            d = rs1[j][0] + delta_rps
            if d < 0 and use_delta[nn + j]:
                s0.append((d, used[nn + j]))
        if delta_rps < 0 and use_delta[nd]:
            s0.append((delta_rps, used[nd]))
        for j in range(nn):
            d = rs0[j][0] + delta_rps
            if d < 0 and use_delta[j]:
                s0.append((d, used[j]))
        for j in range(nn - 1, -1, -1):
            d = rs0[j][0] + delta_rps
            if d > 0 and use_delta[j]:
                s1.append((d, used[j]))
        if delta_rps > 0 and use_delta[nd]:
            s1.append((delta_rps, used[nd]))
        for j in range(len(rs1)):
            d = rs1[j][0] + delta_rps
            if d > 0 and use_delta[nn + j]:
                s1.append((d, used[nn + j]))
        return {"s0": s0, "s1": s1}
    nneg, npos = b.ue(), b.ue()
    s0, s1, poc = [], [], 0
    for _ in range(nneg):
        poc -= b.ue() + 1
        s0.append((poc, b.u(1)))
    poc = 0
    for _ in range(npos):
        poc += b.ue() + 1
        s1.append((poc, b.u(1)))
    return {"s0": s0, "s1": s1}


def parse_sps(b: Bits) -> dict:
    s = {}
    b.u(4)
    msl = b.u(3)
    b.u(1)
    _profile_tier_level(b, msl)
    s["id"] = b.ue()
    s["chroma_format_idc"] = b.ue()
    if s["chroma_format_idc"] != 1:
        raise NotImplementedError("only 4:2:0")
    s["width"], s["height"] = b.ue(), b.ue()
    s["conf"] = (0, 0, 0, 0)
    if b.u(1):
        s["conf"] = (b.ue(), b.ue(), b.ue(), b.ue())  # left, right, top, bottom (chroma units)
    s["bit_depth"] = b.ue() + 8
    if b.ue() + 8 != s["bit_depth"]:
        raise NotImplementedError("luma and chroma bit depths differ")
    s["log2_max_poc_lsb"] = b.ue() + 4
    sub_info = b.u(1)
    for _ in range(0 if sub_info else msl, msl + 1):  # the highest sub-layer's values are kept
        s["max_dec_pic_buffering"] = b.ue() + 1
        s["max_num_reorder"] = b.ue()
        plus1 = b.ue()
        s["max_latency"] = s["max_num_reorder"] + plus1 - 1 if plus1 else 0
    s["log2_min_cb"] = b.ue() + 3
    s["log2_ctb"] = s["log2_min_cb"] + b.ue()
    s["log2_min_tb"] = b.ue() + 2
    s["log2_max_tb"] = s["log2_min_tb"] + b.ue()
    s["max_th_depth_inter"] = b.ue()
    s["max_th_depth_intra"] = b.ue()
    s["scaling_list_enabled"] = b.u(1)
    s["scaling"] = None
    if s["scaling_list_enabled"]:
        s["scaling"] = parse_scaling_list_data(b) if b.u(1) else _default_lists()
    s["amp"] = b.u(1)
    s["sao"] = b.u(1)
    s["pcm"] = b.u(1)
    if s["pcm"]:
        s["pcm_bd_y"] = b.u(4) + 1
        s["pcm_bd_c"] = b.u(4) + 1
        s["log2_min_pcm"] = b.ue() + 3
        s["log2_max_pcm"] = s["log2_min_pcm"] + b.ue()
        s["pcm_lf_disabled"] = b.u(1)
    n = b.ue()
    sets = []
    for i in range(n):
        sets.append(_st_ref_pic_set(b, i, n, sets))
    s["st_rps"] = sets
    s["lt_present"] = b.u(1)
    if s["lt_present"]:
        nlt = b.ue()
        s["lt_sps"] = [(b.u(s["log2_max_poc_lsb"]), b.u(1)) for _ in range(nlt)]
    else:
        s["lt_sps"] = []
    s["tmvp"] = b.u(1)
    s["strong_intra"] = b.u(1)
    return s


def parse_pps(b: Bits) -> dict:
    p = {}
    p["id"] = b.ue()
    p["sps_id"] = b.ue()
    p["dependent_slices"] = b.u(1)
    p["output_flag_present"] = b.u(1)
    p["extra_bits"] = b.u(3)
    p["sign_hiding"] = b.u(1)
    p["cabac_init_present"] = b.u(1)
    p["num_ref_default"] = (b.ue() + 1, b.ue() + 1)
    p["init_qp"] = 26 + b.se()
    p["constrained_intra"] = b.u(1)
    p["transform_skip"] = b.u(1)
    p["cu_qp_delta"] = b.u(1)
    p["diff_cu_qp_delta_depth"] = b.ue() if p["cu_qp_delta"] else 0
    p["cb_qp_offset"], p["cr_qp_offset"] = b.se(), b.se()
    p["slice_chroma_qp_offsets"] = b.u(1)
    p["weighted_pred"], p["weighted_bipred"] = b.u(1), b.u(1)
    p["transquant_bypass"] = b.u(1)
    p["tiles"] = b.u(1)
    p["wpp"] = b.u(1)
    p["tile_cols"], p["tile_rows"], p["uniform"] = 1, 1, 1
    p["col_widths"], p["row_heights"] = None, None
    p["lf_across_tiles"] = 1
    if p["tiles"]:
        p["tile_cols"], p["tile_rows"] = b.ue() + 1, b.ue() + 1
        p["uniform"] = b.u(1)
        if not p["uniform"]:
            p["col_widths"] = [b.ue() + 1 for _ in range(p["tile_cols"] - 1)]
            p["row_heights"] = [b.ue() + 1 for _ in range(p["tile_rows"] - 1)]
        p["lf_across_tiles"] = b.u(1)
    p["lf_across_slices"] = b.u(1)
    p["deblock_override_enabled"], p["deblock_disabled"], p["beta_offset"], p["tc_offset"] = 0, 0, 0, 0
    if b.u(1):  # deblocking_filter_control_present_flag
        p["deblock_override_enabled"] = b.u(1)
        p["deblock_disabled"] = b.u(1)
        if not p["deblock_disabled"]:
            p["beta_offset"], p["tc_offset"] = b.se() * 2, b.se() * 2
    p["scaling"] = parse_scaling_list_data(b) if b.u(1) else None
    p["lists_modification"] = b.u(1)
    p["log2_par_mrg"] = b.ue() + 2
    p["header_ext"] = b.u(1)
    return p


# NAL unit types (7.4.2.2)
TRAIL_N, TRAIL_R, RASL_N, RASL_R, BLA_W_LP, IDR_W_RADL, IDR_N_LP, CRA = 0, 1, 8, 9, 16, 19, 20, 21


def parse_slice_header(b: Bits, nal_type: int, spss: dict, ppss: dict, prev: dict | None) -> dict:
    h = {"nal_type": nal_type}
    h["first"] = b.u(1)
    h["no_output_of_prior_pics"] = b.u(1) if BLA_W_LP <= nal_type <= 23 else 0
    pps = ppss[b.ue()]
    sps = spss[pps["sps_id"]]
    h["pps"], h["sps"] = pps, sps
    wctb = (sps["width"] + (1 << sps["log2_ctb"]) - 1) >> sps["log2_ctb"]
    hctb = (sps["height"] + (1 << sps["log2_ctb"]) - 1) >> sps["log2_ctb"]
    h["dependent"] = 0
    h["segment_address"] = 0
    if not h["first"]:
        if pps["dependent_slices"]:
            h["dependent"] = b.u(1)
        h["segment_address"] = b.u(_ceil_log2(wctb * hctb))
    if h["dependent"]:
        if prev is None:
            raise ValueError("dependent slice segment without a slice")
        for k, v in prev.items():
            if k not in ("first", "dependent", "segment_address", "entry_points", "data_bit"):
                h.setdefault(k, v)
        h["dependent"] = 1
    else:
        b.u(pps["extra_bits"])
        h["type"] = b.ue()  # 0 B, 1 P, 2 I
        h["output"] = b.u(1) if pps["output_flag_present"] else 1
        h["poc_lsb"] = 0
        h["rps"] = {"s0": [], "s1": []}
        h["lt"] = []
        h["tmvp"] = 0
        if nal_type not in (IDR_W_RADL, IDR_N_LP):
            h["poc_lsb"] = b.u(sps["log2_max_poc_lsb"])
            if not b.u(1):  # short_term_ref_pic_set_sps_flag
                h["rps"] = _st_ref_pic_set(b, len(sps["st_rps"]), len(sps["st_rps"]), sps["st_rps"])
            else:
                idx = b.u(_ceil_log2(len(sps["st_rps"]))) if len(sps["st_rps"]) > 1 else 0
                h["rps"] = sps["st_rps"][idx]
            if sps["lt_present"]:
                nsps = b.ue() if sps["lt_sps"] else 0
                npics = b.ue()
                if nsps + npics:
                    raise NotImplementedError("long-term reference pictures")
            if sps["tmvp"]:
                h["tmvp"] = b.u(1)
        h["sao_luma"] = h["sao_chroma"] = 0
        if sps["sao"]:
            h["sao_luma"], h["sao_chroma"] = b.u(1), b.u(1)
        h["num_ref"] = [0, 0]
        h["mods"] = [None, None]
        h["mvd_l1_zero"] = 0
        h["cabac_init_flag"] = 0
        h["col_from_l0"] = 1
        h["col_ref_idx"] = 0
        h["weights"] = None
        h["max_merge"] = 5
        if h["type"] != 2:
            nrd = pps["num_ref_default"]
            h["num_ref"] = [nrd[0], nrd[1] if h["type"] == 0 else 0]
            if b.u(1):  # num_ref_idx_active_override_flag
                h["num_ref"][0] = b.ue() + 1
                if h["type"] == 0:
                    h["num_ref"][1] = b.ue() + 1
            total = sum(u for _, u in h["rps"]["s0"]) + sum(u for _, u in h["rps"]["s1"])
            if pps["lists_modification"] and total > 1:
                nb = _ceil_log2(total)
                for l in range(2 if h["type"] == 0 else 1):
                    if b.u(1):
                        h["mods"][l] = [b.u(nb) for _ in range(h["num_ref"][l])]
            if h["type"] == 0:
                h["mvd_l1_zero"] = b.u(1)
            if pps["cabac_init_present"]:
                h["cabac_init_flag"] = b.u(1)
            if h["tmvp"]:
                if h["type"] == 0:
                    h["col_from_l0"] = b.u(1)
                if (h["col_from_l0"] and h["num_ref"][0] > 1) or (not h["col_from_l0"] and h["num_ref"][1] > 1):
                    h["col_ref_idx"] = b.ue()
            if (pps["weighted_pred"] and h["type"] == 1) or (pps["weighted_bipred"] and h["type"] == 0):
                h["weights"] = _pred_weight_table(b, h)
            h["max_merge"] = 5 - b.ue()
        h["qp"] = pps["init_qp"] + b.se()
        h["cb_qp_offset"] = h["cr_qp_offset"] = 0
        if pps["slice_chroma_qp_offsets"]:
            h["cb_qp_offset"], h["cr_qp_offset"] = b.se(), b.se()
        override = b.u(1) if pps["deblock_override_enabled"] else 0
        h["deblock_disabled"] = pps["deblock_disabled"]
        h["beta_offset"], h["tc_offset"] = pps["beta_offset"], pps["tc_offset"]
        if override:
            h["deblock_disabled"] = b.u(1)
            if not h["deblock_disabled"]:
                h["beta_offset"], h["tc_offset"] = b.se() * 2, b.se() * 2
        h["lf_across"] = pps["lf_across_slices"]
        if pps["lf_across_slices"] and (h["sao_luma"] or h["sao_chroma"] or not h["deblock_disabled"]):
            h["lf_across"] = b.u(1)
    h["entry_points"] = []
    if pps["tiles"] or pps["wpp"]:
        n = b.ue()
        if n:
            bits = b.ue() + 1
            h["entry_points"] = [b.u(bits) + 1 for _ in range(n)]
    if pps["header_ext"]:
        for _ in range(b.ue()):
            b.u(8)
    # byte_alignment(): alignment_bit_equal_to_one, then zero bits
    if b.u(1) != 1:
        raise ValueError("slice header alignment bit")
    b.align()
    h["data_bit"] = b.pos
    return h


def _pred_weight_table(b: Bits, h) -> dict:
    """7.3.6.3 with the weights and offsets of 7.4.7.3 (8-bit units)."""
    lw = b.ue()
    cw = lw + b.se()
    out = {"luma_log2": lw, "chroma_log2": cw, "l": []}
    for l in range(2 if h["type"] == 0 else 1):
        n = h["num_ref"][l]
        lf = [b.u(1) for _ in range(n)]
        cf = [b.u(1) for _ in range(n)]
        ents = []
        for i in range(n):
            w, o = 1 << lw, 0
            if lf[i]:
                w += b.se()
                o = b.se()
            cws, cos = [1 << cw, 1 << cw], [0, 0]
            if cf[i]:
                for j in range(2):
                    cws[j] += b.se()
                    d = b.se()
                    cos[j] = max(-128, min(127, (128 - ((128 * cws[j]) >> cw)) + d))
            ents.append((w, o, cws, cos))
        out["l"].append(ents)
    return out


# ---------------------------------------------------------------------------
# Records (include/pito_recon.h)
# ---------------------------------------------------------------------------
F_INTRA, F_SKIP, F_NOFILTER, F_CBF, F_CODED = 1, 2, 4, 8, 16
E_TU_V, E_PU_V, E_TU_H, E_PU_H = 1, 2, 4, 8
TU_INTRA, TU_CBF, TU_SKIP, TU_BYPASS, TU_PCM = 1, 2, 4, 8, 16
TU_DTYPE = np.dtype([("x0", "<u2"), ("y0", "<u2"), ("log2", "u1"), ("c", "u1"), ("flags", "u1"), ("mode", "u1"),
                     ("qp", "i1"), ("max_x", "u1"), ("max_y", "u1"), ("reserved", "u1"), ("coef_off", "<u4")])
assert TU_DTYPE.itemsize == 16


class _Sao(ctypes.Structure):
    _fields_ = [("type_idx", ctypes.c_uint8 * 3), ("band_pos", ctypes.c_uint8 * 3), ("eo_class", ctypes.c_uint8 * 3),
                ("reserved", ctypes.c_uint8), ("offsets", (ctypes.c_int16 * 4) * 3)]


class _Ctb(ctypes.Structure):
    _fields_ = [("slice", ctypes.c_uint16), ("tile", ctypes.c_uint16), ("ts", ctypes.c_uint32), ("sao", _Sao),
                ("reserved", ctypes.c_uint16)]


class _Slice(ctypes.Structure):
    _fields_ = [("slice_addr", ctypes.c_uint32), ("deblock_disabled", ctypes.c_int32), ("beta_offset", ctypes.c_int32),
                ("tc_offset", ctypes.c_int32), ("lf_across", ctypes.c_int32), ("sao_luma", ctypes.c_int32),
                ("sao_chroma", ctypes.c_int32), ("weighted", ctypes.c_int32), ("luma_log2_denom", ctypes.c_int32),
                ("chroma_log2_denom", ctypes.c_int32), ("num_ref", ctypes.c_int32 * 2),
                ("ref_slot", (ctypes.c_int32 * 16) * 2), ("ref_id", (ctypes.c_uint32 * 16) * 2),
                ("luma_w", (ctypes.c_int16 * 16) * 2), ("luma_o", (ctypes.c_int16 * 16) * 2),
                ("chroma_w", ((ctypes.c_int16 * 2) * 16) * 2), ("chroma_o", ((ctypes.c_int16 * 2) * 16) * 2)]


assert ctypes.sizeof(_Ctb) == 44 and ctypes.sizeof(_Slice) == 688


# ---------------------------------------------------------------------------
# Decoded pictures
# ---------------------------------------------------------------------------
class Picture:
    """A decoded picture as motion prediction of later pictures sees it."""

    def __init__(self, ident, poc, slot, w4, h4):
        self.ident, self.poc, self.slot = ident, poc, slot
        self.ref = True
        # per 4x4 block: predFlag, mv, reference POC per list; intra
        self.pred = [[0] * (w4 * h4) for _ in range(2)]
        self.mv = [[(0, 0)] * (w4 * h4) for _ in range(2)]
        self.rpoc = [[0] * (w4 * h4) for _ in range(2)]
        self.intra = [True] * (w4 * h4)


_COMB = [(0, 1), (1, 0), (0, 2), (2, 0), (1, 2), (2, 1), (0, 3), (3, 0), (1, 3), (3, 1), (2, 3), (3, 2)]
_P2Nx2N, _P2NxN, _PNx2N, _PNxN, _P2NxnU, _P2NxnD, _PnLx2N, _PnRx2N = range(8)


class Decoder:
    """Parses a stream picture by picture; decode() returns one dict per
    picture in decoding order with its records, DPB slot, POC, output flag,
    coded-video-sequence index and crop rectangle."""

    def __init__(self, slots: int = 16):
        self.spss, self.ppss = {}, {}
        self.slots = slots
        self.dpb: list[Picture] = []
        self.next_id = 1
        self.cvs = -1
        self.prev_tid0_poc = 0
        self.pics = []
        self.cur = None
        self.skip_rasl = False
        self.first_pic = True

    # ---- stream level -----------------------------------------------------
    def decode(self, data: bytes):
        prev_slice = None
        for nal in nal_units(data):
            if len(nal) < 2:
                continue
            nal_type = (nal[0] >> 1) & 63
            tid = (nal[1] & 7) - 1
            rbsp, removed = unescape(nal)
            b = Bits(rbsp, 16)
            if nal_type == 33:
                s = parse_sps(b)
                self.spss[s["id"]] = s
            elif nal_type == 34:
                p = parse_pps(b)
                self.ppss[p["id"]] = p
            elif nal_type < 32:
                if nal_type > CRA and nal_type < 32:
                    continue
                h = parse_slice_header(b, nal_type, self.spss, self.ppss, prev_slice)
                h["tid"] = tid
                if h["first"]:
                    self._finish_picture()
                    if not self._start_picture(h):
                        prev_slice = None
                        continue
                elif self.cur is None:
                    continue
                if not h["dependent"]:
                    prev_slice = h
                self._slice(h, rbsp, removed)
                if not h["dependent"]:
                    prev_slice = h
            elif nal_type in (36, 37):  # end of sequence / bitstream
                self._finish_picture()
                self.first_pic = True
        self._finish_picture()
        return self.pics

    def _start_picture(self, h) -> bool:
        sps, pps = h["sps"], h["pps"]
        nt = h["nal_type"]
        irap = BLA_W_LP <= nt <= 23
        no_rasl_output = irap and (nt in (IDR_W_RADL, IDR_N_LP) or nt < IDR_W_RADL or self.first_pic)
        if irap:
            self.skip_rasl = no_rasl_output and nt in (CRA, BLA_W_LP, 17, 18)
        if nt in (RASL_N, RASL_R) and self.skip_rasl:
            return False
        self.first_pic = False
        # 8.3.1 picture order count
        max_lsb = 1 << sps["log2_max_poc_lsb"]
        lsb = h["poc_lsb"]
        if irap and no_rasl_output:
            msb = 0
        else:
            plsb, pmsb = self.prev_tid0_poc & (max_lsb - 1), self.prev_tid0_poc - (self.prev_tid0_poc & (max_lsb - 1))
            if lsb < plsb and plsb - lsb >= max_lsb // 2:
                msb = pmsb + max_lsb
            elif lsb > plsb and lsb - plsb > max_lsb // 2:
                msb = pmsb - max_lsb
            else:
                msb = pmsb
        poc = msb + lsb
        if h["tid"] == 0 and not (nt in (RASL_N, RASL_R, 6, 7) or (nt <= 14 and nt % 2 == 0)):
            self.prev_tid0_poc = poc
        self.new_sequence = bool(irap and no_rasl_output)
        self.unref = []
        if self.new_sequence:
            self.cvs += 1
            for p in self.dpb:
                p.ref = False
        # 8.3.2 reference picture set: the pictures it names stay references
        rps = h["rps"]
        keep = {poc + d for d, _ in rps["s0"]} | {poc + d for d, _ in rps["s1"]}
        for p in self.dpb:
            if p.ref and p.poc not in keep:
                p.ref = False
                self.unref.append(p.ident)
        self.dpb = [p for p in self.dpb if p.ref]
        self.st_before = [self._by_poc(poc + d) for d, u in rps["s0"] if u]
        self.st_after = [self._by_poc(poc + d) for d, u in rps["s1"] if u]
        used = {p.slot for p in self.dpb}
        slot = next(s for s in range(self.slots) if s not in used)
        W, H = sps["width"], sps["height"]
        self.W, self.H = W, H
        self.log2ctb = sps["log2_ctb"]
        self.wctb = (W + (1 << self.log2ctb) - 1) >> self.log2ctb
        self.hctb = (H + (1 << self.log2ctb) - 1) >> self.log2ctb
        self.w4, self.h4 = W // 4, H // 4
        self.bd = sps["bit_depth"]
        self.sps, self.pps = sps, pps
        self.cur = Picture(self.next_id, poc, slot, self.w4, self.h4)
        self.next_id += 1
        self._layout(pps)
        n4 = self.w4 * self.h4
        self.b_flags = [0] * n4
        self.b_edges = [0] * n4
        self.b_qp = [0] * n4
        self.b_ipm = [1] * n4
        self.b_depth = [0] * n4
        self.ctb_slice = [0xFFFF] * (self.wctb * self.hctb)
        self.ctb_sao = [None] * (self.wctb * self.hctb)
        self.tus = []
        self.levels = []
        self.slices = []
        self.slice_hdrs = []
        self.pic_hdr = h
        self.b_refidx = [[-1] * n4 for _ in range(2)]
        self.pcm_blocks = set()
        self.wpp_saved = {}
        self.saved_ds = None
        return True

    def _by_poc(self, poc):
        for p in self.dpb:
            if p.poc == poc:
                return p
        raise ValueError(f"missing reference picture POC {poc}")

    def _layout(self, pps):
        """6.5.1: tile columns / rows and the raster <-> tile scan maps."""
        wc, hc = self.wctb, self.hctb
        nc, nr = pps["tile_cols"], pps["tile_rows"]
        if pps["uniform"]:
            cw = [((i + 1) * wc) // nc - (i * wc) // nc for i in range(nc)]
            rh = [((j + 1) * hc) // nr - (j * hc) // nr for j in range(nr)]
        else:
            cw = pps["col_widths"] + [wc - sum(pps["col_widths"])]
            rh = pps["row_heights"] + [hc - sum(pps["row_heights"])]
        cb = [0]
        for v in cw:
            cb.append(cb[-1] + v)
        rb = [0]
        for v in rh:
            rb.append(rb[-1] + v)
        n = wc * hc
        self.rs2ts = [0] * n
        self.tile_id = [0] * n
        for rs in range(n):
            tbx, tby = rs % wc, rs // wc
            tx = max(i for i in range(nc) if tbx >= cb[i])
            ty = max(j for j in range(nr) if tby >= rb[j])
            v = 0
            for i in range(tx):
                v += rh[ty] * cw[i]
            for j in range(ty):
                v += wc * rh[j]
            v += (tby - rb[ty]) * cw[tx] + tbx - cb[tx]
            self.rs2ts[rs] = v
            self.tile_id[rs] = ty * nc + tx
        self.ts2rs = [0] * n
        for rs, ts in enumerate(self.rs2ts):
            self.ts2rs[ts] = rs
        self.col_bd, self.row_bd = cb, rb

    def _finish_picture(self):
        if self.cur is None:
            return
        pic = self.cur
        # every 4x4 block's slice-level data is final: build the records
        ctbs = (_Ctb * (self.wctb * self.hctb))()
        for rs in range(self.wctb * self.hctb):
            c = ctbs[rs]
            c.slice = self.ctb_slice[rs] if self.ctb_slice[rs] != 0xFFFF else 0
            c.tile = self.tile_id[rs]
            c.ts = self.rs2ts[rs]
            sao = self.ctb_sao[rs]
            if sao:
                for k in range(3):
                    c.sao.type_idx[k], c.sao.band_pos[k], c.sao.eo_class[k] = sao[k][0], sao[k][1], sao[k][2]
                    for j in range(4):
                        c.sao.offsets[k][j] = sao[k][3][j]
        blk = np.zeros((self.w4 * self.h4, 4), np.uint8)
        blk[:, 0] = self.b_flags
        blk[:, 1] = self.b_edges
        blk[:, 2] = np.array(self.b_qp, np.int8).view(np.uint8)
        blk[:, 3] = self.b_ipm
        mvf = np.zeros(self.w4 * self.h4, np.dtype([("mv", "<i2", (2, 2)), ("ref_idx", "i1", (2,)),
                                                     ("reserved", "<u2")]))
        mvf["ref_idx"][:] = -1
        for l in range(2):
            for i in range(self.w4 * self.h4):
                if pic.pred[l][i]:
                    mvf["mv"][i, l] = pic.mv[l][i]
                    mvf["ref_idx"][i, l] = self.b_refidx[l][i]
        tus = np.array(self.tus, TU_DTYPE) if self.tus else np.zeros(0, TU_DTYPE)
        sps, pps = self.sps, self.pps
        scaling = None
        if sps["scaling_list_enabled"]:
            lists, dc = pps["scaling"] if pps["scaling"] else sps["scaling"]
            scaling = scaling_factors(lists, dc)
        l, r, t, bm = sps["conf"]
        crop = (2 * l, 2 * t, self.W - 2 * (l + r), self.H - 2 * (t + bm))
        self.pics.append({
            "W": self.W, "H": self.H, "bit_depth": self.bd, "slot": pic.slot, "poc": pic.poc, "cvs": self.cvs,
            "output": self.pic_hdr["output"], "crop": crop, "frame_id": pic.ident,
            # the output process (DPB bumping): sequence start, the references
            # this picture's RPS dropped, and the SPS limits
            "new_sequence": self.new_sequence, "no_output_of_prior_pics": self.pic_hdr["no_output_of_prior_pics"],
            "unref": self.unref, "dpb": [sps["max_dec_pic_buffering"], sps["max_num_reorder"], sps["max_latency"]],
            "header": {"log2_ctb": self.log2ctb, "constrained_intra_pred": pps["constrained_intra"],
                       "strong_intra_smoothing": sps["strong_intra"], "loop_filter_across_tiles": pps["lf_across_tiles"],
                       "cb_qp_offset": pps["cb_qp_offset"], "cr_qp_offset": pps["cr_qp_offset"],
                       "num_slices": len(self.slices), "num_tus": len(tus), "frame_id": pic.ident},
            "bufs": {"ctbs": bytes(ctbs), "blk": blk.tobytes(), "mvf": mvf.tobytes(), "tus": tus.tobytes(),
                     "slices": b"".join(bytes(s) for s in self.slices),
                     "levels": np.array(self.levels, np.int16).tobytes(), "scaling": scaling or b""},
        })
        self.dpb.append(pic)
        self.cur = None

    # ---- slice level ------------------------------------------------------
    def _slice(self, h, rbsp, removed):
        """7.3.8.1 slice_segment_data with the context initialisation,
        WPP synchronisation and substream handling of 9.3.1."""
        pps = h["pps"]
        if not h["dependent"]:
            self._new_slice(h)
        hh = self.slice_hdrs[-1]
        self.h = hh
        sl_idx = len(self.slices) - 1
        self.slice_addr = hh["slice_addr"]
        t = hh["type"]
        if t == 2:
            init_type = 0
        elif t == 1:
            init_type = 2 if hh["cabac_init_flag"] else 1
        else:
            init_type = 1 if hh["cabac_init_flag"] else 2
        # substream starts (RBSP bytes) from the entry points, which count the
        # bytes of the slice segment data with emulation prevention included
        rem = sorted(removed)

        def esc(r):
            e = r
            for q in rem:
                if q <= e:
                    e += 1
                else:
                    break
            return e

        starts, e = [], esc(h["data_bit"] // 8)
        for off in h["entry_points"]:
            e += off
            starts.append(e - sum(1 for q in rem if q < e))
        c = Cabac(rbsp, h["data_bit"])
        self.c = c
        if not h["dependent"]:
            self.last_qp = hh["qp"]
        self.qp_delta, self.qp_delta_coded = 0, False
        ctb_ts = self.rs2ts[h["segment_address"]]
        first, sub = True, 0
        while True:
            rs = self.ts2rs[ctb_ts]
            rx, ry = rs % self.wctb, rs // self.wctb
            tc = self._tile_col(rx)
            tile_start = ctb_ts == 0 or self.tile_id[rs] != self.tile_id[self.ts2rs[ctb_ts - 1]]
            row_start = bool(pps["wpp"]) and rx == self.col_bd[tc]
            if not first and (tile_start or row_start):
                # end_of_subset_one_bit and byte_alignment() came before: the
                # next substream starts at the next byte boundary
                at = (c.pos + 7) & ~7
                if sub < len(starts) and starts[sub] * 8 != at:
                    raise ValueError(f"substream {sub + 1} starts at byte {at // 8}, entry point says {starts[sub]}")
                sub += 1
                c.start(at)
            if first or tile_start or row_start:
                if tile_start:
                    c.init_contexts(hh["qp"], init_type)
                elif row_start:
                    x0, y0 = rx << self.log2ctb, ry << self.log2ctb
                    src = None
                    if self.avail(x0, y0, x0 + (1 << self.log2ctb), y0 - (1 << self.log2ctb)):
                        src = self.wpp_saved.get(ry - 1)
                    if src is not None:
                        c.st = list(src)
                    else:
                        c.init_contexts(hh["qp"], init_type)
                elif h["dependent"] and self.saved_ds is not None:
                    c.st = list(self.saved_ds)
                else:
                    c.init_contexts(hh["qp"], init_type)
            if tile_start or row_start:
                self.last_qp = hh["qp"]
            first = False
            self.ctb_slice[rs] = sl_idx
            self._ctu(rx, ry, rs)
            if pps["wpp"]:
                width = self.col_bd[tc + 1] - self.col_bd[tc]
                if rx - self.col_bd[tc] == 1 or width == 1:
                    self.wpp_saved[ry] = list(c.st)
            end = c.term()
            ctb_ts += 1
            if end:
                break
            if ctb_ts >= self.wctb * self.hctb:
                raise ValueError("slice data runs past the picture")
            nrs = self.ts2rs[ctb_ts]
            nx = nrs % self.wctb
            if (pps["tiles"] and self.tile_id[nrs] != self.tile_id[rs]) or \
                    (pps["wpp"] and nx == self.col_bd[self._tile_col(nx)]):
                if c.term() != 1:
                    raise ValueError("end_of_subset_one_bit is not 1")
        if sub != len(starts):
            raise ValueError(f"{sub + 1} substreams decoded, {len(starts) + 1} signalled")
        if pps["dependent_slices"]:
            self.saved_ds = list(c.st)
        # the slice data ends with the stop bit: nothing but zero bits may follow
        for p in range(c.pos, len(rbsp) * 8):
            if (rbsp[p >> 3] >> (7 - (p & 7))) & 1:
                raise ValueError(f"slice data does not end where the NAL unit does (bit {c.pos} of {len(rbsp) * 8})")

    def _tile_col(self, rx):
        cb = self.col_bd
        for i in range(len(cb) - 1):
            if cb[i] <= rx < cb[i + 1]:
                return i
        return len(cb) - 2

    def _new_slice(self, h):
        hh = dict(h)
        hh["slice_addr"] = h["segment_address"]
        # 8.3.4 reference picture lists
        lists = [[], []]
        if hh["type"] != 2:
            before, after = self.st_before, self.st_after
            total = len(before) + len(after)
            if total == 0:
                raise ValueError("P/B slice without references")
            for l in range(2 if hh["type"] == 0 else 1):
                n = hh["num_ref"][l]
                temp = []
                order = before + after if l == 0 else after + before
                while len(temp) < max(n, total):
                    for p in order:
                        if len(temp) < max(n, total):
                            temp.append(p)
                mods = hh["mods"][l]
                lists[l] = [temp[mods[i]] if mods else temp[i] for i in range(n)]
        hh["lists"] = lists
        self.slice_hdrs.append(hh)
        s = _Slice()
        s.slice_addr = hh["slice_addr"]
        s.deblock_disabled = hh["deblock_disabled"]
        s.beta_offset, s.tc_offset = hh["beta_offset"], hh["tc_offset"]
        s.lf_across = hh["lf_across"]
        s.sao_luma, s.sao_chroma = hh["sao_luma"], hh["sao_chroma"]
        s.weighted = 1 if hh["weights"] else 0
        if hh["weights"]:
            s.luma_log2_denom = hh["weights"]["luma_log2"]
            s.chroma_log2_denom = hh["weights"]["chroma_log2"]
        for l in range(2):
            s.num_ref[l] = len(lists[l])
            for i, p in enumerate(lists[l]):
                s.ref_slot[l][i] = p.slot
                s.ref_id[l][i] = p.ident
                if hh["weights"]:
                    w, o, cws, cos = hh["weights"]["l"][l][i]
                    s.luma_w[l][i], s.luma_o[l][i] = w, o
                    for j in range(2):
                        s.chroma_w[l][i][j], s.chroma_o[l][i][j] = cws[j], cos[j]
        self.slices.append(s)
        hh["no_backward"] = all(p.poc <= self.cur.poc for l in range(2) for p in lists[l])

    # ---- availability (6.4.1) ---------------------------------------------
    def _zorder(self, x, y):
        m = (1 << self.log2ctb) - 1
        lx, ly = (x & m) >> 2, (y & m) >> 2
        r = 0
        for i in range(5):
            r |= ((lx >> i) & 1) << (2 * i) | ((ly >> i) & 1) << (2 * i + 1)
        return r

    def avail(self, xc, yc, xn, yn) -> bool:
        if xn < 0 or yn < 0 or xn >= self.W or yn >= self.H:
            return False
        s = self.log2ctb
        cn = (yn >> s) * self.wctb + (xn >> s)
        cc = (yc >> s) * self.wctb + (xc >> s)
        if cn != cc:
            if self.rs2ts[cn] > self.rs2ts[cc]:
                return False
            sn = self.ctb_slice[cn]
            if sn == 0xFFFF or self.slices[sn].slice_addr != self.slice_addr:
                return False
            return self.tile_id[cn] == self.tile_id[cc]
        return self._zorder(xn, yn) <= self._zorder(xc, yc)

    def _avail_ctb(self, rxn, ryn, rx, ry) -> bool:
        return self.avail(rx << self.log2ctb, ry << self.log2ctb, rxn << self.log2ctb, ryn << self.log2ctb)

    def _bi(self, x, y):
        return (y >> 2) * self.w4 + (x >> 2)

    def _fill(self, x0, y0, w, h):
        """4x4 block indices of a rectangle (clipped to the picture)."""
        out = []
        for by in range(y0 >> 2, min((y0 + h + 3) >> 2, self.h4)):
            base = by * self.w4
            for bx in range(x0 >> 2, min((x0 + w + 3) >> 2, self.w4)):
                out.append(base + bx)
        return out

    def _mark_edges(self, x0, y0, w, h, v, hz):
        if v:
            bx = x0 >> 2
            for by in range(y0 >> 2, min((y0 + h + 3) >> 2, self.h4)):
                self.b_edges[by * self.w4 + bx] |= v
        if hz:
            by = y0 >> 2
            for bx in range(x0 >> 2, min((x0 + w + 3) >> 2, self.w4)):
                self.b_edges[by * self.w4 + bx] |= hz

    # ---- CTU --------------------------------------------------------------
    def _ctu(self, rx, ry, rs):
        hh = self.h
        x0, y0 = rx << self.log2ctb, ry << self.log2ctb
        if hh["sao_luma"] or hh["sao_chroma"]:
            self._sao(rx, ry, rs)
        self._quadtree(x0, y0, self.log2ctb, 0)

    def _sao(self, rx, ry, rs):
        c, hh = self.c, self.h
        sao = None
        if rx > 0:
            lrs = rs - 1
            if self.ctb_slice[lrs] != 0xFFFF and self.slices[self.ctb_slice[lrs]].slice_addr == self.slice_addr and \
                    self.tile_id[lrs] == self.tile_id[rs]:
                if c.dec(CTX["sao_merge"]):
                    sao = self.ctb_sao[lrs]
        if sao is None and ry > 0:
            urs = rs - self.wctb
            if self.ctb_slice[urs] != 0xFFFF and self.slices[self.ctb_slice[urs]].slice_addr == self.slice_addr and \
                    self.tile_id[urs] == self.tile_id[rs]:
                if c.dec(CTX["sao_merge"]):
                    sao = self.ctb_sao[urs]
        if sao is None:
            sao = []
            cmax = (1 << (min(self.bd, 10) - 5)) - 1
            for k in range(3):
                if not ((k == 0 and hh["sao_luma"]) or (k > 0 and hh["sao_chroma"])):
                    sao.append((0, 0, 0, (0, 0, 0, 0)))
                    continue
                if k == 2:
                    t = sao[1][0]
                else:
                    t = 0
                    if c.dec(CTX["sao_type"]):
                        t = 2 if c.byp() else 1
                if t == 0:
                    sao.append((0, 0, 0, (0, 0, 0, 0)))
                    continue
                absv = []
                for _ in range(4):
                    v = 0
                    while v < cmax and c.byp():
                        v += 1
                    absv.append(v)
                if t == 1:
                    offs = [(-a if (a and c.byp()) else a) for a in absv]
                    band = c.byp_bits(5)
                    sao.append((1, band, 0, tuple(o << (self.bd - min(self.bd, 10)) for o in offs)))
                else:
                    eo = c.byp_bits(2) if k < 2 else sao[1][2]
                    offs = (absv[0], absv[1], -absv[2], -absv[3])
                    sao.append((2, 0, eo, tuple(o << (self.bd - min(self.bd, 10)) for o in offs)))
        self.ctb_sao[rs] = sao

    # ---- coding quadtree / unit (7.3.8.4-5) -------------------------------
    def _quadtree(self, x0, y0, log2, depth):
        c, sps, pps = self.c, self.sps, self.pps
        n = 1 << log2
        if x0 + n <= self.W and y0 + n <= self.H and log2 > sps["log2_min_cb"]:
            inc = 0
            if self.avail(x0, y0, x0 - 1, y0) and self.b_depth[self._bi(x0 - 1, y0)] > depth:
                inc += 1
            if self.avail(x0, y0, x0, y0 - 1) and self.b_depth[self._bi(x0, y0 - 1)] > depth:
                inc += 1
            split = c.dec(CTX["split_cu"] + inc)
        else:
            split = log2 > sps["log2_min_cb"]
        if pps["cu_qp_delta"] and log2 >= self.log2ctb - pps["diff_cu_qp_delta_depth"]:
            self.qp_delta_coded = False
            self.qp_delta = 0
        if split:
            h = n >> 1
            for dx, dy in ((0, 0), (h, 0), (0, h), (h, h)):
                if x0 + dx < self.W and y0 + dy < self.H:
                    self._quadtree(x0 + dx, y0 + dy, log2 - 1, depth + 1)
        else:
            self._cu(x0, y0, log2, depth)

    def _qp_pred(self, xq, yq):
        """8.6.1 qPY_PRED for the quantization group at (xq, yq)."""
        s = self.log2ctb
        same = lambda x, y: (x >> s) == (xq >> s) and (y >> s) == (yq >> s)
        qa = self.b_qp[self._bi(xq - 1, yq)] if self.avail(xq, yq, xq - 1, yq) and same(xq - 1, yq) else self.last_qp
        qb = self.b_qp[self._bi(xq, yq - 1)] if self.avail(xq, yq, xq, yq - 1) and same(xq, yq - 1) else self.last_qp
        self.qp_pred = (qa + qb + 1) >> 1

    def _update_qp(self):
        off = 6 * (self.bd - 8)
        self.qp_y = ((self.qp_pred + self.qp_delta + 52 + 2 * off) % (52 + off)) - off
        hh, pps = self.h, self.pps

        def qpc(q):
            return q if q < 30 else q - 6 if q > 43 else (29, 30, 31, 32, 33, 33, 34, 34, 35, 35, 36, 36, 37, 37)[q - 30]
        qi_cb = max(-off, min(57, self.qp_y + pps["cb_qp_offset"] + hh["cb_qp_offset"]))
        qi_cr = max(-off, min(57, self.qp_y + pps["cr_qp_offset"] + hh["cr_qp_offset"]))
        self.qp_cb, self.qp_cr = qpc(qi_cb) + off, qpc(qi_cr) + off

    def _cu(self, x0, y0, log2, depth):
        c, sps, pps, hh = self.c, self.sps, self.pps, self.h
        n = 1 << log2
        qg = (1 << (self.log2ctb - pps["diff_cu_qp_delta_depth"])) - 1
        if not pps["cu_qp_delta"]:
            qg = (1 << self.log2ctb) - 1
        if (x0 & qg) == 0 and (y0 & qg) == 0:
            self._qp_pred(x0, y0)
            if not pps["cu_qp_delta"]:
                self.qp_delta = 0
        self._update_qp()
        bypass = c.dec(CTX["transquant_bypass"]) if pps["transquant_bypass"] else 0
        self.bypass = bypass
        skip = 0
        if hh["type"] != 2:
            inc = 0
            if self.avail(x0, y0, x0 - 1, y0) and self.b_flags[self._bi(x0 - 1, y0)] & F_SKIP:
                inc += 1
            if self.avail(x0, y0, x0, y0 - 1) and self.b_flags[self._bi(x0, y0 - 1)] & F_SKIP:
                inc += 1
            skip = c.dec(CTX["cu_skip"] + inc)
        blocks = self._fill(x0, y0, n, n)
        fl = F_CODED | (F_SKIP if skip else 0) | (F_NOFILTER if bypass else 0)
        for i in blocks:
            self.b_depth[i] = depth
            self.b_flags[i] = fl
            self.b_qp[i] = self.qp_y
            self.b_ipm[i] = 1
            self.b_edges[i] = 0
            self.cur.intra[i] = False
        self._mark_edges(x0, y0, n, n, E_TU_V | E_PU_V, E_TU_H | E_PU_H)
        self.cu_intra = False
        self.cu_part = _P2Nx2N
        if skip:
            self._pu(x0, y0, n, x0, y0, n, n, 0, _P2Nx2N, True)
            self._finish_cu(blocks)
            return
        intra = c.dec(CTX["pred_mode"]) if hh["type"] != 2 else 1
        self.cu_intra = bool(intra)
        part = _P2Nx2N
        if not intra or log2 == sps["log2_min_cb"]:
            part = self._part_mode(intra, log2)
        self.cu_part = part
        if intra:
            for i in blocks:
                self.b_flags[i] |= F_INTRA
                self.cur.intra[i] = True
                for l in range(2):
                    self.cur.pred[l][i] = 0
                    self.b_refidx[l][i] = -1
            self.intra_split = part == _PNxN
            pcm = 0
            if part == _P2Nx2N and sps["pcm"] and sps["log2_min_pcm"] <= log2 <= sps["log2_max_pcm"]:
                pcm = c.term()
            if pcm:
                self.pcm_blocks.update(blocks)
                self._pcm(x0, y0, log2)
                if sps["pcm_lf_disabled"]:
                    for i in blocks:
                        self.b_flags[i] |= F_NOFILTER
                self._finish_cu(blocks)
                return
            self._intra_modes(x0, y0, n, part)
            self.max_trafo_depth = sps["max_th_depth_intra"] + (1 if self.intra_split else 0)
            self._transform_tree(x0, y0, x0, y0, log2, 0, 0, (1, 1))
        else:
            self.intra_split = False
            h, q = n // 2, n // 4
            parts = {
                _P2Nx2N: [(0, 0, n, n)], _P2NxN: [(0, 0, n, h), (0, h, n, h)], _PNx2N: [(0, 0, h, n), (h, 0, h, n)],
                _P2NxnU: [(0, 0, n, q), (0, q, n, n - q)], _P2NxnD: [(0, 0, n, n - q), (0, n - q, n, q)],
                _PnLx2N: [(0, 0, q, n), (q, 0, n - q, n)], _PnRx2N: [(0, 0, n - q, n), (n - q, 0, q, n)],
                _PNxN: [(0, 0, h, h), (h, 0, h, h), (0, h, h, h), (h, h, h, h)],
            }[part]
            merge2 = False
            for i, (px, py, pw, ph) in enumerate(parts):
                m = self._pu(x0, y0, n, x0 + px, y0 + py, pw, ph, i, part, False)
                if part == _P2Nx2N:
                    merge2 = m
                if px:
                    self._mark_edges(x0 + px, y0 + py, pw, ph, E_PU_V, 0)
                if py:
                    self._mark_edges(x0 + px, y0 + py, pw, ph, 0, E_PU_H)
            root = c.dec(CTX["rqt_root_cbf"]) if not merge2 else 1
            if root:
                self.max_trafo_depth = sps["max_th_depth_inter"]
                self._transform_tree(x0, y0, x0, y0, log2, 0, 0, (1, 1))
        self._finish_cu(blocks)

    def _finish_cu(self, blocks):
        for i in blocks:
            self.b_qp[i] = self.qp_y
        self.last_qp = self.qp_y

    def _part_mode(self, intra, log2):
        c, pm = self.c, CTX["part_mode"]
        if c.dec(pm):
            return _P2Nx2N
        if intra:
            return _PNxN
        if log2 == self.sps["log2_min_cb"]:
            if c.dec(pm + 1):
                return _P2NxN
            if log2 == 3:
                return _PNx2N
            return _PNx2N if c.dec(pm + 2) else _PNxN
        if not self.sps["amp"]:
            return _P2NxN if c.dec(pm + 1) else _PNx2N
        if c.dec(pm + 1):
            if c.dec(pm + 3):
                return _P2NxN
            return _P2NxnD if c.byp() else _P2NxnU
        if c.dec(pm + 3):
            return _PNx2N
        return _PnRx2N if c.byp() else _PnLx2N

    def _pcm(self, x0, y0, log2):
        """7.3.8.7 pcm_sample: byte-aligned raw samples after pcm_flag; the
        arithmetic decoder restarts after them (9.3.2.5)."""
        c, sps = self.c, self.sps
        at = (c.pos + 7) & ~7
        b = Bits(c.data, at)
        n, nc = 1 << log2, 1 << (log2 - 1)
        luma = [b.u(sps["pcm_bd_y"]) << (self.bd - sps["pcm_bd_y"]) for _ in range(n * n)]
        cb = [b.u(sps["pcm_bd_c"]) << (self.bd - sps["pcm_bd_c"]) for _ in range(nc * nc)]
        cr = [b.u(sps["pcm_bd_c"]) << (self.bd - sps["pcm_bd_c"]) for _ in range(nc * nc)]
        c.start(b.pos)
        for comp, xs, ys, l2, samples in ((0, x0, y0, log2, luma), (1, x0 // 2, y0 // 2, log2 - 1, cb),
                                          (2, x0 // 2, y0 // 2, log2 - 1, cr)):
            self.tus.append((xs, ys, l2, comp, TU_PCM, 0, 0, 0, 0, 0, len(self.levels)))
            self.levels.extend(samples)

    def _intra_modes(self, x0, y0, n, part):
        """7.3.8.5 + 8.4.2 / 8.4.3: luma modes by MPM, the chroma mode."""
        c = self.c
        pb = n // 2 if part == _PNxN else n
        cnt = 4 if part == _PNxN else 1
        offs = [(0, 0), (pb, 0), (0, pb), (pb, pb)][:cnt]
        prev = [c.dec(CTX["prev_intra_luma"]) for _ in offs]
        for k, (dx, dy) in enumerate(offs):
            if prev[k]:
                mpm = 0
                while mpm < 2 and c.byp():
                    mpm += 1
                rem = None
            else:
                rem = c.byp_bits(5)
            xp, yp = x0 + dx, y0 + dy
            cand = []
            for (xn, yn, is_b) in ((xp - 1, yp, False), (xp, yp - 1, True)):
                m = 1
                if self.avail(xp, yp, xn, yn):
                    i = self._bi(xn, yn)
                    if self.b_flags[i] & F_INTRA and not self.pcm_at(i):
                        if not (is_b and yn < ((yp >> self.log2ctb) << self.log2ctb)):
                            m = self.b_ipm[i]
                cand.append(m)
            a, b = cand
            if a == b:
                lst = [0, 1, 26] if a < 2 else [a, 2 + ((a + 29) % 32), 2 + ((a - 2 + 1) % 32)]
            else:
                cc = 0 if (a != 0 and b != 0) else (1 if (a != 1 and b != 1) else 26)
                lst = [a, b, cc]
            if rem is None:
                mode = lst[mpm]
            else:
                mode = rem
                for v in sorted(lst):
                    if mode >= v:
                        mode += 1
            for i in self._fill(xp, yp, pb, pb):
                self.b_ipm[i] = mode
        ic = 4
        if c.dec(CTX["intra_chroma"]):
            ic = c.byp_bits(2)
        lm = self.b_ipm[self._bi(x0, y0)]
        if ic == 4:
            cm = lm
        else:
            cm = (0, 26, 10, 1)[ic]
            if cm == lm:
                cm = 34
        self.chroma_mode = cm

    def pcm_at(self, i) -> bool:
        return i in self.pcm_blocks

    # ---- transform tree / unit (7.3.8.8-10) --------------------------------
    def _transform_tree(self, x0, y0, xb, yb, log2, depth, blk_idx, parent_cbf):
        c, sps = self.c, self.sps
        if log2 <= sps["log2_max_tb"] and log2 > sps["log2_min_tb"] and depth < self.max_trafo_depth and \
                not (self.intra_split and depth == 0):
            split = c.dec(CTX["split_transform"] + 5 - log2)
        else:
            inter_split = sps["max_th_depth_inter"] == 0 and not self.cu_intra and self.cu_part != _P2Nx2N and \
                depth == 0
            split = 1 if (log2 > sps["log2_max_tb"] or (self.intra_split and depth == 0) or inter_split) else 0
        cbf_c = [0, 0]
        if log2 > 2:
            for k in range(2):
                if depth == 0 or parent_cbf[k]:
                    cbf_c[k] = c.dec(CTX["cbf_chroma"] + depth)
        else:
            cbf_c = list(parent_cbf) if depth > 0 else [0, 0]
        if split:
            h = 1 << (log2 - 1)
            for k, (dx, dy) in enumerate(((0, 0), (h, 0), (0, h), (h, h))):
                self._transform_tree(x0 + dx, y0 + dy, x0, y0, log2 - 1, depth + 1, k, cbf_c)
            return
        cbf_l = 1
        if self.cu_intra or depth != 0 or cbf_c[0] or cbf_c[1]:
            cbf_l = c.dec(CTX["cbf_luma"] + (1 if depth == 0 else 0))
        n = 1 << log2
        if depth > 0:
            self._mark_edges(x0, y0, n, n, E_TU_V, E_TU_H)
        self._transform_unit(x0, y0, xb, yb, log2, blk_idx, cbf_l, cbf_c)

    def _transform_unit(self, x0, y0, xb, yb, log2, blk_idx, cbf_l, cbf_c):
        c, pps = self.c, self.pps
        chroma_here = log2 > 2 or blk_idx == 3
        if (cbf_l or cbf_c[0] or cbf_c[1]) and pps["cu_qp_delta"] and not self.qp_delta_coded:
            v = 0
            while v < 5 and c.dec(CTX["cu_qp_delta_abs"] + (0 if v == 0 else 1)):
                v += 1
            if v == 5:
                k = 0
                while c.byp():
                    v += 1 << k
                    k += 1
                v += c.byp_bits(k)
            if v and c.byp():
                v = -v
            self.qp_delta_coded = True
            self.qp_delta = v
            self._update_qp()
        n = 1 << log2
        if self.cu_intra or cbf_l:
            mode = self.b_ipm[self._bi(x0, y0)]
            self._tu_record(x0, y0, log2, 0, mode, cbf_l, self.qp_y + 6 * (self.bd - 8))
            if cbf_l:
                for i in self._fill(x0, y0, n, n):
                    self.b_flags[i] |= F_CBF
        if not chroma_here:
            return
        xc, yc, l2c = (x0 // 2, y0 // 2, log2 - 1) if log2 > 2 else (xb // 2, yb // 2, 2)
        for k in (1, 2):
            if self.cu_intra or cbf_c[k - 1]:
                self._tu_record(xc, yc, l2c, k, self.chroma_mode, cbf_c[k - 1], self.qp_cb if k == 1 else self.qp_cr)

    def _tu_record(self, x0, y0, log2, comp, mode, cbf, qp):
        flags = (TU_INTRA if self.cu_intra else 0)
        mx = my = 0
        off = len(self.levels)
        if cbf:
            flags |= TU_CBF
            if self.bypass:
                flags |= TU_BYPASS
            coeffs, ts = self._residual(log2, comp, mode if self.cu_intra else None)
            if ts:
                flags |= TU_SKIP
            mx = max(x for (x, y) in coeffs)
            my = max(y for (x, y) in coeffs)
            w = mx + 1
            lv = [0] * (w * (my + 1))
            for (x, y), v in coeffs.items():
                lv[y * w + x] = v
            self.levels.extend(lv)
        self.tus.append((x0, y0, log2, comp, flags, mode if self.cu_intra else 0, qp if not self.bypass else 0,
                         mx, my, 0, off))

    # ---- residual_coding (7.3.8.11) ---------------------------------------
    def _residual(self, log2, comp, intra_mode):
        c, pps = self.c, self.pps
        ts = 0
        if pps["transform_skip"] and not self.bypass and log2 <= 2:
            ts = c.dec(CTX["transform_skip"] + (1 if comp else 0))
        # last significant position
        cmax = (log2 << 1) - 1
        if comp == 0:
            off, shift = 3 * (log2 - 2) + ((log2 - 1) >> 2), (log2 + 1) >> 2
        else:
            off, shift = 15, log2 - 2
        px = 0
        while px < cmax and c.dec(CTX["last_x_prefix"] + off + (px >> shift)):
            px += 1
        py = 0
        while py < cmax and c.dec(CTX["last_y_prefix"] + off + (py >> shift)):
            py += 1
        lx = px if px <= 3 else (1 << ((px >> 1) - 1)) * (2 + (px & 1)) + c.byp_bits((px >> 1) - 1)
        ly = py if py <= 3 else (1 << ((py >> 1) - 1)) * (2 + (py & 1)) + c.byp_bits((py >> 1) - 1)
        scan_idx = 0
        if intra_mode is not None and (log2 == 2 or (log2 == 3 and comp == 0)):
            if 6 <= intra_mode <= 14:
                scan_idx = 2
            elif 22 <= intra_mode <= 30:
                scan_idx = 1
        if scan_idx == 2:
            lx, ly = ly, lx
        nsb = 1 << (log2 - 2)
        sb_scan = SCAN[(nsb, scan_idx)]
        pos_scan = SCAN[(4, scan_idx)]
        # subblock and position of the last coefficient
        last_sb = next(i for i, (xs, ys) in enumerate(sb_scan) if xs == lx >> 2 and ys == ly >> 2)
        last_pos = next(i for i, (xp, yp) in enumerate(pos_scan) if xp == lx & 3 and yp == ly & 3)
        csbf = {}
        coeffs = {}
        greater1_ctx = 1
        sig_base = CTX["sig_coeff"] + (0 if comp == 0 else 27)
        for i in range(last_sb, -1, -1):
            xs, ys = sb_scan[i]
            infer_dc = False
            if last_sb > i > 0:
                ctxv = 0
                if xs < nsb - 1:
                    ctxv += csbf.get((xs + 1, ys), 0)
                if ys < nsb - 1:
                    ctxv += csbf.get((xs, ys + 1), 0)
                flag = c.dec(CTX["coded_sub_block"] + min(ctxv, 1) + (0 if comp == 0 else 2))
                csbf[(xs, ys)] = flag
                infer_dc = True
            else:
                csbf[(xs, ys)] = 1
            prev_csbf = 0
            if xs < nsb - 1:
                prev_csbf += csbf.get((xs + 1, ys), 0)
            if ys < nsb - 1:
                prev_csbf += csbf.get((xs, ys + 1), 0) << 1
            sig = []  # scan positions n (descending) with sig_coeff_flag 1
            if i == last_sb:
                sig.append(last_pos)
                start = last_pos - 1
            else:
                start = 15
            if csbf[(xs, ys)]:
                for n in range(start, -1, -1):
                    xp, yp = pos_scan[n]
                    xc, yc = (xs << 2) + xp, (ys << 2) + yp
                    if n > 0 or not infer_dc:
                        if log2 == 2:
                            sc = _CTX_IDX_MAP[(yc << 2) + xc]
                        elif xc + yc == 0:
                            sc = 0
                        else:
                            if prev_csbf == 0:
                                sc = 2 if xp + yp == 0 else 1 if xp + yp < 3 else 0
                            elif prev_csbf == 1:
                                sc = 2 if yp == 0 else 1 if yp == 1 else 0
                            elif prev_csbf == 2:
                                sc = 2 if xp == 0 else 1 if xp == 1 else 0
                            else:
                                sc = 2
                            if comp == 0 and (xs > 0 or ys > 0):
                                sc += 3
                            if log2 == 3:
                                sc += 9 if scan_idx == 0 else 15
                            else:
                                sc += 21 if comp == 0 else 12
                        if c.dec(sig_base + sc):
                            sig.append(n)
                            infer_dc = False
                    else:
                        sig.append(0)  # inferred DC of a coded subblock
            if not sig:
                continue
            # greater1 / greater2 flags
            ctx_set = 0 if (i == 0 or comp > 0) else 2
            if i != last_sb and greater1_ctx == 0:
                ctx_set += 1
            greater1_ctx = 1
            gt1 = {}
            first_g1 = -1
            for k, n in enumerate(sig[:8]):
                f = c.dec(CTX["gt1"] + ctx_set * 4 + greater1_ctx + (16 if comp else 0))
                gt1[n] = f
                if f:
                    greater1_ctx = 0
                    if first_g1 < 0:
                        first_g1 = n
                elif 0 < greater1_ctx < 3:
                    greater1_ctx += 1
            gt2 = {}
            if first_g1 >= 0:
                gt2[first_g1] = c.dec(CTX["gt2"] + ctx_set + (4 if comp else 0))
            hidden = pps["sign_hiding"] and not self.bypass and (sig[0] - sig[-1] > 3)
            signs = {}
            for n in sig:
                if not (hidden and n == sig[-1]):
                    signs[n] = c.byp()
                else:
                    signs[n] = 0
            num_sig, sum_abs, rice = 0, 0, 0
            for n in sig:
                base = 1 + gt1.get(n, 0) + gt2.get(n, 0)
                thresh = (3 if n == first_g1 else 2) if num_sig < 8 else 1
                level = base
                if base == thresh:
                    # coeff_abs_level_remaining (9.3.3.11)
                    prefix = 0
                    while prefix < 32 and c.byp():
                        prefix += 1
                    if prefix <= 3:
                        rem = (prefix << rice) + c.byp_bits(rice)
                    else:
                        rem = (((1 << (prefix - 3)) + 2) << rice) + c.byp_bits(prefix - 3 + rice)
                    level = base + rem
                    if level > 3 * (1 << rice):
                        rice = min(rice + 1, 4)
                v = -level if signs[n] else level
                if hidden:
                    sum_abs += level
                    if n == sig[-1] and sum_abs & 1:
                        v = -v
                xp, yp = pos_scan[n]
                coeffs[((xs << 2) + xp, (ys << 2) + yp)] = max(-32768, min(32767, v))
                num_sig += 1
        return coeffs, ts

    # ---- prediction units (7.3.8.6) and motion (8.5.3) ---------------------
    def _pu(self, xc, yc, nc, xp, yp, w, h, part_idx, part, skip):
        c, hh = self.c, self.h
        mm = hh["max_merge"]
        if skip:
            merge, midx = True, 0
            if mm > 1:
                midx = self._merge_idx(mm)
        else:
            merge = bool(c.dec(CTX["merge_flag"]))
            midx = self._merge_idx(mm) if (merge and mm > 1) else 0
        if merge:
            pf, mv, ri = self._merge(xc, yc, nc, xp, yp, w, h, part_idx, part, midx)
        else:
            idc = 0  # 0 L0, 1 L1, 2 BI
            if hh["type"] == 0:
                if w + h != 12:
                    depth = self.b_depth[self._bi(xp, yp)]
                    if c.dec(CTX["inter_pred_idc"] + depth):
                        idc = 2
                    else:
                        idc = c.dec(CTX["inter_pred_idc"] + 4)
                else:
                    idc = c.dec(CTX["inter_pred_idc"] + 4)
            pf, mv, ri = [0, 0], [(0, 0), (0, 0)], [-1, -1]
            mvd = [None, None]
            mvp = [0, 0]
            for l in range(2):
                if (l == 0 and idc == 1) or (l == 1 and idc == 0):
                    continue
                r = 0
                nr = hh["num_ref"][l]
                if nr > 1:
                    while r < nr - 1:
                        bit = c.dec(CTX["ref_idx"] + r) if r < 2 else c.byp()
                        if not bit:
                            break
                        r += 1
                ri[l] = r
                pf[l] = 1
                if l == 1 and hh["mvd_l1_zero"] and idc == 2:
                    mvd[1] = (0, 0)
                else:
                    mvd[l] = self._mvd()
                mvp[l] = c.dec(CTX["mvp_flag"])
            for l in range(2):
                if pf[l]:
                    px, py = self._amvp(xc, yc, nc, xp, yp, w, h, part_idx, l, ri[l])[mvp[l]]
                    mx = ((px + mvd[l][0] + 65536) & 0xFFFF)
                    my = ((py + mvd[l][1] + 65536) & 0xFFFF)
                    mv[l] = (mx - 65536 if mx >= 32768 else mx, my - 65536 if my >= 32768 else my)
        pic = self.cur
        lists = hh["lists"]
        for i in self._fill(xp, yp, w, h):
            for l in range(2):
                pic.pred[l][i] = pf[l]
                pic.mv[l][i] = mv[l] if pf[l] else (0, 0)
                pic.rpoc[l][i] = lists[l][ri[l]].poc if pf[l] else 0
                self.b_refidx[l][i] = ri[l] if pf[l] else -1
        return merge

    def _merge_idx(self, mm):
        c = self.c
        i = 0
        if c.dec(CTX["merge_idx"]):
            i = 1
            while i < mm - 1 and c.byp():
                i += 1
        return i

    def _mvd(self):
        c = self.c
        g0 = [c.dec(CTX["mvd_gt0"]), c.dec(CTX["mvd_gt0"])]
        g1 = [c.dec(CTX["mvd_gt1"]) if g0[0] else 0, 0]
        g1[1] = c.dec(CTX["mvd_gt1"]) if g0[1] else 0
        out = []
        for k in range(2):
            v = 0
            if g0[k]:
                v = 1
                if g1[k]:
                    # abs_mvd_minus2: EG1
                    kk, a = 1, 0
                    while c.byp():
                        a += 1 << kk
                        kk += 1
                    a += c.byp_bits(kk)
                    v = a + 2
                if c.byp():
                    v = -v
            out.append(v)
        return tuple(out)

    def _nb(self, xc, yc, nc, xp, yp, w, h, part_idx, xn, yn):
        """6.4.2 availability of a neighbouring prediction block (inter only)."""
        same_cb = xc <= xn < xc + nc and yc <= yn < yc + nc
        if not same_cb:
            ok = self.avail(xp, yp, xn, yn)
        elif (w << 1) == nc and (h << 1) == nc and part_idx == 1 and yc + h <= yn and xc + w > xn:
            ok = False
        else:
            ok = True
        if ok and self.cur.intra[self._bi(xn, yn)]:
            ok = False
        return ok

    def _motion(self, i):
        p = self.cur
        return ((p.pred[0][i], p.mv[0][i] if p.pred[0][i] else (0, 0), self.b_refidx[0][i] if p.pred[0][i] else -1),
                (p.pred[1][i], p.mv[1][i] if p.pred[1][i] else (0, 0), self.b_refidx[1][i] if p.pred[1][i] else -1))

    def _merge(self, xc, yc, nc, xp, yp, w, h, part_idx, part, midx):
        hh = self.h
        ow, oh = w, h
        if self.pps["log2_par_mrg"] > 2 and nc == 8:
            xp, yp, w, h, part_idx = xc, yc, nc, nc, 0
            part_for_rules = _P2Nx2N
        else:
            part_for_rules = part
        L = self.pps["log2_par_mrg"]

        def diff_region(xn, yn):
            return not ((xp >> L) == (xn >> L) and (yp >> L) == (yn >> L))

        def cand_at(xn, yn):
            if not diff_region(xn, yn):
                return None
            if not self._nb(xc, yc, nc, xp, yp, w, h, part_idx, xn, yn):
                return None
            return self._motion(self._bi(xn, yn))

        # motion of each neighbour that is available (6.4.2, the merge region
        # and the second-partition rules); pruning compares against these,
        # whether or not that neighbour became a candidate itself
        ma1 = None
        if not (part_for_rules in (_PNx2N, _PnLx2N, _PnRx2N) and part_idx == 1):
            ma1 = cand_at(xp - 1, yp + h - 1)
        mb1 = None
        if not (part_for_rules in (_P2NxN, _P2NxnU, _P2NxnD) and part_idx == 1):
            mb1 = cand_at(xp + w - 1, yp - 1)
        mb0 = cand_at(xp + w, yp - 1)
        ma0 = cand_at(xp - 1, yp + h)
        mb2 = cand_at(xp - 1, yp - 1)
        a1 = ma1
        b1 = mb1 if (mb1 is not None and not (ma1 is not None and mb1 == ma1)) else None
        b0 = mb0 if (mb0 is not None and not (mb1 is not None and mb0 == mb1)) else None
        a0 = ma0 if (ma0 is not None and not (ma1 is not None and ma0 == ma1)) else None
        b2 = mb2
        if b2 is not None and ((ma1 is not None and b2 == ma1) or (mb1 is not None and b2 == mb1)):
            b2 = None
        if sum(x is not None for x in (a0, a1, b0, b1)) == 4:
            b2 = None
        lst = [x for x in (a1, b1, b0, a0, b2) if x is not None]
        mm = hh["max_merge"]
        if len(lst) < mm and hh["tmvp"]:
            col = []
            ok0, mv0 = self._tmvp(xp, yp, w, h, 0, 0)
            ok1, mv1 = (self._tmvp(xp, yp, w, h, 1, 0) if hh["type"] == 0 else (False, (0, 0)))
            if ok0 or ok1:
                lst.append(((1, mv0, 0) if ok0 else (0, (0, 0), -1), (1, mv1, 0) if ok1 else (0, (0, 0), -1)))
        lst = lst[:mm]
        if hh["type"] == 0 and 1 < len(lst) < mm:
            orig = len(lst)
            for ci in range(orig * (orig - 1)):
                if len(lst) >= mm:
                    break
                i0, i1 = _COMB[ci]
                c0, c1 = lst[i0], lst[i1]
                if c0[0][0] and c1[1][0]:
                    p0 = hh["lists"][0][c0[0][2]].poc
                    p1 = hh["lists"][1][c1[1][2]].poc
                    if p0 != p1 or c0[0][1] != c1[1][1]:
                        lst.append((c0[0], c1[1]))
        nref = hh["num_ref"][0] if hh["type"] == 1 else min(hh["num_ref"][0], hh["num_ref"][1])
        z = 0
        while len(lst) < mm:
            r = z if z < nref else 0
            if hh["type"] == 1:
                lst.append(((1, (0, 0), r), (0, (0, 0), -1)))
            else:
                lst.append(((1, (0, 0), r), (1, (0, 0), r)))
            z += 1
        m = lst[midx]
        pf = [m[0][0], m[1][0]]
        mv = [m[0][1], m[1][1]]
        ri = [m[0][2], m[1][2]]
        if pf[0] and pf[1] and ow + oh == 12:
            pf[1], ri[1], mv[1] = 0, -1, (0, 0)
        return pf, mv, ri

    def _scale(self, mv, td, tb):
        td = max(-128, min(127, td))
        tb = max(-128, min(127, tb))
        num = 16384 + (abs(td) >> 1)
        tx = num // abs(td) if td > 0 else -(num // abs(td))
        f = max(-4096, min(4095, (tb * tx + 32) >> 6))
        out = []
        for v in mv:
            p = f * v
            s = -1 if p < 0 else 1
            out.append(max(-32768, min(32767, s * ((abs(p) + 127) >> 8))))
        return tuple(out)

    def _amvp(self, xc, yc, nc, xp, yp, w, h, part_idx, X, ref_idx):
        hh = self.h
        lists = hh["lists"]
        Y = 1 - X
        target = lists[X][ref_idx]
        cur_poc = self.cur.poc

        def nb(xn, yn):
            return self._nb(xc, yc, nc, xp, yp, w, h, part_idx, xn, yn)

        def same_pic(i):
            p = self.cur
            for L in (X, Y):
                if p.pred[L][i] and lists[L][self.b_refidx[L][i]].poc == target.poc:
                    return p.mv[L][i]
            return None

        def scaled(i):
            p = self.cur
            for L in (X, Y):
                if p.pred[L][i]:
                    rp = lists[L][self.b_refidx[L][i]]
                    mv = p.mv[L][i]
                    if rp.poc != target.poc:
                        mv = self._scale(mv, cur_poc - rp.poc, cur_poc - target.poc)
                    return mv
            return None

        a_pos = [(xp - 1, yp + h), (xp - 1, yp + h - 1)]
        a_ok = [nb(*q) for q in a_pos]
        is_scaled = a_ok[0] or a_ok[1]
        mva = None
        for q, ok in zip(a_pos, a_ok):
            if ok and mva is None:
                mva = same_pic(self._bi(*q))
        if mva is None:
            for q, ok in zip(a_pos, a_ok):
                if ok and mva is None:
                    mva = scaled(self._bi(*q))
        b_pos = [(xp + w, yp - 1), (xp + w - 1, yp - 1), (xp - 1, yp - 1)]
        b_ok = [nb(*q) for q in b_pos]
        mvb = None
        for q, ok in zip(b_pos, b_ok):
            if ok and mvb is None:
                mvb = same_pic(self._bi(*q))
        if not is_scaled and mvb is not None and mva is None:
            mva = mvb
        if not is_scaled:
            mvb = None
            for q, ok in zip(b_pos, b_ok):
                if ok and mvb is None:
                    mvb = scaled(self._bi(*q))
        cands = []
        if mva is not None:
            cands.append(mva)
        if mvb is not None and (mva is None or mva != mvb):
            cands.append(mvb)
        if len(cands) < 2 and hh["tmvp"]:
            ok, mvc = self._tmvp(xp, yp, w, h, X, ref_idx)
            if ok:
                cands.append(mvc)
        while len(cands) < 2:
            cands.append((0, 0))
        return cands[:2]

    def _tmvp(self, xp, yp, w, h, X, ref_idx):
        """8.5.3.2.8 temporal luma motion vector prediction."""
        hh = self.h
        lists = hh["lists"]
        colpic = lists[0 if (hh["type"] == 1 or hh["col_from_l0"]) else 1][hh["col_ref_idx"]]
        xbr, ybr = xp + w, yp + h
        if (yp >> self.log2ctb) == (ybr >> self.log2ctb) and ybr < self.H and xbr < self.W:
            ok, mv = self._col(colpic, ((xbr >> 4) << 4), ((ybr >> 4) << 4), X, ref_idx)
            if ok:
                return ok, mv
        xm, ym = xp + (w >> 1), yp + (h >> 1)
        return self._col(colpic, ((xm >> 4) << 4), ((ym >> 4) << 4), X, ref_idx)

    def _col(self, colpic, x, y, X, ref_idx):
        i = self._bi(x, y)
        if colpic.intra[i]:
            return False, (0, 0)
        hh = self.h
        if not colpic.pred[0][i]:
            L = 1
        elif not colpic.pred[1][i]:
            L = 0
        else:  # bi-predicted: list X when no reference follows the picture, else list collocated_from_l0_flag
            L = X if hh["no_backward"] else hh["col_from_l0"]
        mv = colpic.mv[L][i]
        col_ref_poc = colpic.rpoc[L][i]
        target = hh["lists"][X][ref_idx]
        col_diff = colpic.poc - col_ref_poc
        cur_diff = self.cur.poc - target.poc
        if col_diff == cur_diff or col_diff == 0:
            return True, mv
        return True, self._scale(mv, col_diff, cur_diff)
