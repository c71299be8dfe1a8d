// synth_h264.cpp — seeded synthetic H.264 syntax records (the stand-in for
// the host CAVLC/CABAC parse of src/h264/dec/slicedec.rs:1582-1751).
//
// Integer-only: the same seed gives the same records on x86 and Arm.
#include <cstdlib>
#include <cstring>
#include <array>
#include <vector>

#include "synth.h"

namespace {

// QPC_TABLE, the chroma QP mapping of src/h264/dec/tables.rs:3-14.
int qpc_of(int q) {
    static const unsigned char tail[22] = {29, 30, 31, 32, 32, 33, 34, 34, 35, 35, 36,
                                           36, 37, 37, 37, 38, 38, 38, 39, 39, 39, 39};
    q = q < 0 ? 0 : q > 51 ? 51 : q;
    return q < 30 ? q : tail[q - 30];
}

struct Rng {
    uint64_t s;
    uint64_t next() {  // splitmix64
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    uint32_t u32() { return (uint32_t)(next() >> 32); }
    int below(int n) { return n <= 0 ? 0 : (int)((next() >> 16) % (uint64_t)n); }
    bool chance(int permille) { return below(1000) < permille; }
    // Rounded Laplacian(0, b=2): P(|v| >= 1) = e^-1/4, each further step e^-1/2.
    int laplace2() {
        if (u32() >= 3344923893u) return 0;
        int m = 1;
        while (m < 2047 && u32() < 2605029347u) m++;
        return (next() & 1) ? m : -m;
    }
};

struct Pic {
    rc_h264_picture pic;
    std::vector<rc_h264_motion> motion;
    std::vector<rc_h264_slice_motion> smotion;
    std::vector<rc_h264_mb> mbs;
    std::vector<rc_h264_slice> slices;
    std::vector<rc_h264_weight> weights;
    std::vector<int16_t> levels;
    uint8_t scaling4[6][16];
    uint8_t scaling8[6][64];
};

bool is_intra(int k) { return k >= RC_H264_I4x4 && k <= RC_H264_IPCM; }

struct Gen {
    const rc_synth_h264_opts &o;
    Rng r;
    Pic &p;
    std::vector<int> part_of;            // per MB: the inter partition drawn (0 16x16 .. 3 8x8)
    std::vector<std::array<int, 4>> subs_of;  // 8x8: the sub-partition drawn per 8x8
    Gen(const rc_synth_h264_opts &o_, Pic &p_) : o(o_), r{o_.seed}, p(p_) {}

    // availability of neighbour n (0 L, 1 T, 2 TR, 3 TL) for intra prediction
    bool nb(int mbx, int mby, int n) {
        static const int dx[4] = {-1, 0, 1, -1}, dy[4] = {0, -1, -1, -1};
        int x = mbx + dx[n], y = mby + dy[n];
        if (x < 0 || y < 0 || x >= o.mb_w) return false;
        const rc_h264_mb &q = p.mbs[mby * o.mb_w + mbx], &m = p.mbs[y * o.mb_w + x];
        if (m.kind == RC_H264_NONE || m.slice != q.slice) return false;
        return !o.constrained_intra_pred || is_intra(m.kind);
    }
    void avail4(int mbx, int mby, int bx, int by, bool &l, bool &t, bool &tl) {
        bool a = nb(mbx, mby, 0), b = nb(mbx, mby, 1), d = nb(mbx, mby, 3);
        l = bx > 0 ? true : a;
        t = by > 0 ? true : b;
        tl = (bx > 0 && by > 0) ? true : by > 0 ? a : bx > 0 ? b : d;
    }
    // uniform over the 4x4/8x8 modes whose reference samples exist
    int nxn_mode(bool l, bool t, bool tl) {
        int cand[9], n = 0;
        cand[n++] = 2;
        if (t) { cand[n++] = 0; cand[n++] = 3; cand[n++] = 7; }
        if (l) { cand[n++] = 1; cand[n++] = 8; }
        if (l && t && tl) { cand[n++] = 4; cand[n++] = 5; cand[n++] = 6; }
        return cand[r.below(n)];
    }
    int mode4(bool l, bool t, bool tl, int vert, int horiz) {  // 16x16 / chroma
        int cand[4], n = 0;
        cand[n++] = vert == 0 ? 2 : 0;  // DC: mode 2 for 16x16 (V = 0), mode 0 for chroma (V = 2)
        if (t) cand[n++] = vert;
        if (l) cand[n++] = horiz;
        if (l && t && tl) cand[n++] = 3;
        return cand[r.below(n)];
    }

    void put_levels(int n, int first, uint16_t &nzbits, uint16_t bitmask, bool coded) {
        size_t at = p.levels.size();
        p.levels.resize(at + n, 0);
        if (!coded) return;
        bool any = false;
        for (int k = first; k < n; k++) {
            int v = r.laplace2();
            p.levels[at + k] = (int16_t)v;
            any |= v != 0;
        }
        if (!any) p.levels[at + first] = (int16_t)((r.next() & 1) ? 1 : -1);
        nzbits |= bitmask;
    }

    void residual(rc_h264_mb &m, bool allow_t8) {
        int keep = 1000 - o.zero_permille;
        m.coef_off = (uint32_t)p.levels.size();
        uint16_t nz = 0;
        if (m.kind == RC_H264_I16x16) {
            m.dc_coded |= 1;
            size_t at = p.levels.size();
            p.levels.resize(at + 16, 0);
            if (r.chance(keep))
                for (int k = 0; k < 16; k++) p.levels[at + k] = (int16_t)r.laplace2();
        }
        bool t8 = m.kind == RC_H264_I8x8 || (allow_t8 && r.chance(o.t8_permille));
        if (t8) {
            for (int b8 = 0; b8 < 4; b8++)
                if (r.chance(keep)) m.luma_coded |= 1 << b8;
            if (m.kind == RC_H264_INTER && !m.luma_coded) t8 = false;
        }
        m.transform_8x8 = t8;
        if (t8) {
            for (int b8 = 0; b8 < 4; b8++) {
                if (!(m.luma_coded >> b8 & 1)) continue;
                int bx = (b8 & 1) * 2, by = (b8 >> 1) * 2;
                uint16_t bits = (uint16_t)((3u << (by * 4 + bx)) | (3u << ((by + 1) * 4 + bx)));
                put_levels(64, 0, nz, bits, true);
            }
        } else {
            m.luma_coded = 0;
            for (int b = 0; b < 16; b++)
                if (r.chance(keep)) m.luma_coded |= 1 << b;
            int first = m.kind == RC_H264_I16x16 ? 1 : 0;
            for (int b = 0; b < 16; b++)
                if (m.luma_coded >> b & 1) put_levels(16, first, nz, (uint16_t)(1u << b), true);
        }
        for (int b = 0; b < 8; b++)
            if (r.chance(keep)) m.chroma_coded |= 1 << b;
        if (m.chroma_coded || r.chance(keep)) m.dc_coded |= 6;
        for (int c = 0; c < 2; c++)
            if (m.dc_coded >> (1 + c) & 1) {
                size_t at = p.levels.size();
                p.levels.resize(at + 4, 0);
                for (int k = 0; k < 4; k++) p.levels[at + k] = (int16_t)r.laplace2();
            }
        uint16_t dummy = 0;
        for (int b = 0; b < 8; b++)
            if (m.chroma_coded >> b & 1) put_levels(16, 1, dummy, 0, true);
        m.nz_mask = nz;
    }

    void intra_mb(rc_h264_mb &m, int mbx, int mby) {
        if (r.chance(o.pcm_permille)) {
            m.kind = RC_H264_IPCM;
            m.qp = 0;
            m.qpc[0] = m.qpc[1] = (uint8_t)qpc_of(o.chroma_qp_offset);
            m.nz_mask = 0xffff;
            m.coef_off = (uint32_t)p.levels.size();
            for (int i = 0; i < 384; i++) p.levels.push_back((int16_t)r.below(256));
            return;
        }
        m.kind = (uint8_t)(RC_H264_I4x4 + r.below(3));
        bool l, t, tl;
        if (m.kind == RC_H264_I4x4) {
            for (int by = 0; by < 4; by++)
                for (int bx = 0; bx < 4; bx++) {
                    avail4(mbx, mby, bx, by, l, t, tl);
                    m.intra_modes[by * 4 + bx] = (uint8_t)nxn_mode(l, t, tl);
                }
        } else if (m.kind == RC_H264_I8x8) {
            for (int b8 = 0; b8 < 4; b8++) {
                int bx = (b8 & 1) * 2, by = (b8 >> 1) * 2;
                avail4(mbx, mby, bx, by, l, t, tl);
                uint8_t md = (uint8_t)nxn_mode(l, t, tl);
                m.intra_modes[by * 4 + bx] = m.intra_modes[by * 4 + bx + 1] = md;
                m.intra_modes[(by + 1) * 4 + bx] = m.intra_modes[(by + 1) * 4 + bx + 1] = md;
            }
        } else {
            for (int i = 0; i < 16; i++) m.intra_modes[i] = 2;
            m.i16_mode = (uint8_t)mode4(nb(mbx, mby, 0), nb(mbx, mby, 1), nb(mbx, mby, 3), 0, 1);
        }
        if (m.kind != RC_H264_I16x16) m.i16_mode = 0;
        m.chroma_mode = (uint8_t)mode4(nb(mbx, mby, 0), nb(mbx, mby, 1), nb(mbx, mby, 3), 2, 1);
        // chroma: 0 DC, 1 H (left), 2 V (top), 3 plane
        residual(m, false);
    }

    int16_t mv_comp(int pos, int size, int extent, bool outside, bool &used_out) {
        int R = o.mv_range;
        if (outside) {
            used_out = true;
            int d = 8 + r.below(48);
            int target = r.below(2) ? -(size + d) : extent + d;
            int v = (target - pos) * 4 + r.below(4);
            return (int16_t)(v < -32768 ? -32768 : v > 32767 ? 32767 : v);
        }
        return (int16_t)(r.below(8 * R) - 4 * R);
    }

    void inter_mb(rc_h264_mb &m, int mbx, int mby, bool wp) {
        m.kind = RC_H264_INTER;
        struct Rect { int x, y, w, h; };
        Rect rects[16];
        int nr = 0;
        int part = r.below(4);
        bool sub8 = false;
        int rect_b8[16];
        const int a = mby * o.mb_w + mbx;
        part_of[a] = part;
        if (part == 0) rects[nr++] = {0, 0, 4, 4};
        else if (part == 1) { rects[nr++] = {0, 0, 4, 2}; rects[nr++] = {0, 2, 4, 2}; }
        else if (part == 2) { rects[nr++] = {0, 0, 2, 4}; rects[nr++] = {2, 0, 2, 4}; }
        else
            for (int b8 = 0; b8 < 4; b8++) {
                int x8 = (b8 & 1) * 2, y8 = (b8 >> 1) * 2, s = r.below(4);
                subs_of[a][b8] = s;
                sub8 |= s != 0;
                if (s == 0) rects[nr++] = {x8, y8, 2, 2};
                else if (s == 1) { rects[nr++] = {x8, y8, 2, 1}; rects[nr++] = {x8, y8 + 1, 2, 1}; }
                else if (s == 2) { rects[nr++] = {x8, y8, 1, 2}; rects[nr++] = {x8 + 1, y8, 1, 2}; }
                else
                    for (int k = 0; k < 4; k++) rects[nr++] = {x8 + (k & 1), y8 + (k >> 1), 1, 1};
            }
        for (int i = 0; i < nr; i++) rect_b8[i] = (rects[i].y >> 1) * 2 + (rects[i].x >> 1);
        // reference choice per 8x8 (shared by its sub-partitions)
        int use[4][2];
        int8_t ref[4][2];
        for (int b8 = 0; b8 < 4; b8++) { use[b8][0] = use[b8][1] = 0; ref[b8][0] = ref[b8][1] = -1; }
        for (int i = 0; i < nr; i++) {
            int b8 = rect_b8[i];
            if (ref[b8][0] >= 0 || ref[b8][1] >= 0) continue;  // decided by an earlier sub-partition
            bool both = o.num_ref[0] > 0 && o.num_ref[1] > 0 && r.chance(o.bipred_permille);
            int l0 = o.num_ref[0] > 0 ? 1 : 0, l1 = o.num_ref[1] > 0 ? 1 : 0;
            if (!both && l0 && l1) { if (r.below(2)) l1 = 0; else l0 = 0; }
            int8_t r0 = l0 ? (int8_t)r.below(o.num_ref[0]) : -1, r1 = l1 ? (int8_t)r.below(o.num_ref[1]) : -1;
            // a 16x16 / 16x8 / 8x16 partition covers several 8x8 blocks
            const Rect &R = rects[i];
            for (int y = R.y; y < R.y + R.h; y++)
                for (int x = R.x; x < R.x + R.w; x++) {
                    int b = (y >> 1) * 2 + (x >> 1);
                    ref[b][0] = r0; ref[b][1] = r1;
                }
        }
        for (int b8 = 0; b8 < 4; b8++) {
            m.ref_idx[0][b8] = ref[b8][0];
            m.ref_idx[1][b8] = ref[b8][1];
            use[b8][0] = ref[b8][0] >= 0;
            use[b8][1] = ref[b8][1] >= 0;
        }
        int W = o.mb_w * 16, H = o.mb_h * 16;
        for (int i = 0; i < nr; i++) {
            const Rect &R = rects[i];
            int b8 = rect_b8[i];
            for (int l = 0; l < 2; l++) {
                int16_t mx = 0, my = 0;
                if (use[b8][l]) {
                    bool out = r.chance(o.outside_permille), used = false;
                    int px = mbx * 16 + R.x * 4, py = mby * 16 + R.y * 4;
                    if (out && r.below(2)) {
                        mx = mv_comp(px, R.w * 4, W, true, used);
                        my = mv_comp(py, R.h * 4, H, false, used);
                    } else if (out) {
                        mx = mv_comp(px, R.w * 4, W, false, used);
                        my = mv_comp(py, R.h * 4, H, true, used);
                    } else {
                        mx = mv_comp(px, R.w * 4, W, false, used);
                        my = mv_comp(py, R.h * 4, H, false, used);
                    }
                }
                for (int y = R.y; y < R.y + R.h; y++)
                    for (int x = R.x; x < R.x + R.w; x++) {
                        m.mv[l][y * 4 + x][0] = mx;
                        m.mv[l][y * 4 + x][1] = my;
                    }
            }
        }
        uint8_t e = wp && !p.weights.empty() ? (uint8_t)r.below((int)p.weights.size()) : 0xff;
        for (int b8 = 0; b8 < 4; b8++) m.wp[b8] = e;
        residual(m, !sub8);
    }

    void weights() {
        for (int i = 0; i < 4; i++) {
            rc_h264_weight w;
            memset(&w, 0, sizeof w);
            w.explicit_mask = (uint8_t)(r.chance(800) ? 7 : 1 + r.below(7));
            for (int c = 0; c < 3; c++) {
                int lw = r.below(8);
                w.log_wd[c] = lw;
                int *ws[2] = {&w.w0[c], &w.w1[c]}, *os[2] = {&w.o0[c], &w.o1[c]};
                for (int l = 0; l < 2; l++) {
                    int wt = (1 << lw) + r.below(65) - 32;
                    wt = wt < -128 ? -128 : wt > 127 ? 127 : wt;
                    int off = r.below(41) - 20;
                    if (wt == (1 << lw) && off == 0) off = 1;  // never a unit weighting
                    *ws[l] = wt;
                    *os[l] = off;
                }
            }
            p.weights.push_back(w);
        }
    }

    // Motion syntax for the generated inter MBs (a separate random stream, so
    // the records are the same with and without it): the partitions and refs
    // drawn, small random mvd, 20% of single-reference list-0 16x16 MBs as
    // P_Skip in pictures without list 1; per slice a weight entry per
    // (refIdxL0, refIdxL1) pair.  Pictures with list 1 are B slices whose
    // co-located picture is RefPicList1[0] (no direct modes are drawn).
    void motion_syntax() {
        Rng q{o.seed ^ 0x5bd1e9955bd1e995ull};
        const int n = o.mb_w * o.mb_h;
        p.motion.assign(n, rc_h264_motion());
        memset(p.motion.data(), 0, sizeof(rc_h264_motion) * n);
        const bool b = o.num_ref[1] > 0;
        for (auto &sl : p.slices) {
            rc_h264_slice_motion sm;
            memset(&sm, 0, sizeof sm);
            sm.b_slice = b;
            sm.direct_spatial = 1;
            sm.direct_8x8_inference = 1;
            sm.col_slot = b ? sl.ref_slot[1][0] : -1;
            sm.col_short_term = 1;
            for (int i = 0; i < RC_H264_MAX_REFS; i++) {
                sm.dist_scale[i] = 256;
                sm.direct_copy[i] = 1;
            }
            memset(sm.wp_map, 0xff, sizeof sm.wp_map);
            for (int r0 = -1; r0 < sl.num_ref[0]; r0++)
                for (int r1 = -1; r1 < sl.num_ref[1]; r1++)
                    if ((r0 >= 0 || r1 >= 0) && !p.weights.empty() && q.chance(o.wp_permille))
                        sm.wp_map[(r0 + 1) * (RC_H264_MAX_REFS + 1) + (r1 + 1)] = (uint8_t)q.below((int)p.weights.size());
            p.smotion.push_back(sm);
        }
        for (int a = 0; a < n; a++) {
            const rc_h264_mb &m = p.mbs[a];
            rc_h264_motion &mo = p.motion[a];
            if (m.kind != RC_H264_INTER) continue;
            const int part = part_of[a];
            for (int l = 0; l < 2; l++)
                for (int b8 = 0; b8 < 4; b8++) mo.ref_idx[l][b8] = m.ref_idx[l][b8];
            auto pred_of = [&](int b8) { return (uint8_t)((m.ref_idx[0][b8] >= 0) | (m.ref_idx[1][b8] >= 0) << 1); };
            if (part == 0 && !b && m.ref_idx[0][0] == 0 && q.chance(200)) {
                mo.shape = RC_H264_MOTION_SKIP;
                continue;
            }
            if (part < 3) {
                mo.shape = (uint8_t)(RC_H264_MOTION_16x16 + part);
                mo.pred[0] = pred_of(0);
                if (part) mo.pred[1] = pred_of(part == 1 ? 2 : 1);
            } else {
                mo.shape = RC_H264_MOTION_8x8;
                for (int b8 = 0; b8 < 4; b8++) {
                    mo.sub[b8] = (uint8_t)subs_of[a][b8];
                    mo.pred[b8] = pred_of(b8);
                }
            }
            // one mvd per (sub-)partition, held by each of its blocks
            for (int l = 0; l < 2; l++) {
                int16_t d[16][2];
                for (int k = 0; k < 16; k++) {
                    d[k][0] = (int16_t)(q.below(33) - 16);
                    d[k][1] = (int16_t)(q.below(33) - 16);
                }
                for (int k = 0; k < 16; k++) {
                    const int x = k & 3, y = k >> 2;
                    int sx = 0, sy = 0;  // the partition's first block
                    if (part == 1) sy = y & 2;
                    else if (part == 2) sx = x & 2;
                    else if (part == 3) {
                        const int b8 = (y >> 1) * 2 + (x >> 1), st = subs_of[a][b8];
                        sx = (x & 2) | (st == 2 || st == 3 ? (x & 1) : 0);
                        sy = (y & 2) | (st == 1 || st == 3 ? (y & 1) : 0);
                    }
                    mo.mvd[l][k][0] = d[sy * 4 + sx][0];
                    mo.mvd[l][k][1] = d[sy * 4 + sx][1];
                }
            }
        }
        p.pic.motion = p.motion.data();
        p.pic.slice_motion = p.smotion.data();
    }

    void run() {
        int n = o.mb_w * o.mb_h, ns = o.num_slices < 1 ? 1 : o.num_slices;
        part_of.assign(n, 0);
        subs_of.assign(n, std::array<int, 4>{0, 0, 0, 0});
        p.mbs.assign(n, rc_h264_mb());
        memset(p.mbs.data(), 0, sizeof(rc_h264_mb) * n);
        for (int s = 0; s < ns; s++) {
            rc_h264_slice sl;
            memset(&sl, 0, sizeof sl);
            sl.disable_deblocking_filter_idc = o.deblock_idc;
            sl.alpha_offset = o.alpha_offset;
            sl.beta_offset = o.beta_offset;
            for (int l = 0; l < 2; l++) {
                sl.num_ref[l] = o.num_ref[l];
                for (int i = 0; i < o.num_ref[l] && i < 4; i++) {
                    sl.ref_slot[l][i] = o.ref_slot[l][i];
                    sl.ref_id[l][i] = o.ref_id[l][i];
                }
            }
            p.slices.push_back(sl);
        }
        if (!o.intra_only) weights();
        if (o.custom_scaling) {
            for (int l = 0; l < 6; l++) {
                for (int i = 0; i < 16; i++) p.scaling4[l][i] = (uint8_t)(4 + r.below(60));
                for (int i = 0; i < 64; i++) p.scaling8[l][i] = (uint8_t)(4 + r.below(60));
            }
        }
        for (int a = 0; a < n; a++) {
            rc_h264_mb &m = p.mbs[a];
            int mbx = a % o.mb_w, mby = a / o.mb_w;
            m.slice = (uint16_t)((long long)a * ns / n);
            for (int l = 0; l < 2; l++)
                for (int b = 0; b < 4; b++) m.ref_idx[l][b] = -1;
            for (int b = 0; b < 4; b++) m.wp[b] = 0xff;
            for (int i = 0; i < 16; i++) m.intra_modes[i] = 2;
            int qp = o.qp_min + r.below(o.qp_max - o.qp_min + 1);
            m.qp = (uint8_t)qp;
            m.qpc[0] = m.qpc[1] = (uint8_t)qpc_of(qp + o.chroma_qp_offset);
            bool intra = o.intra_only || (o.num_ref[0] == 0 && o.num_ref[1] == 0) || r.chance(o.intra_permille);
            if (intra) intra_mb(m, mbx, mby);
            else inter_mb(m, mbx, mby, r.chance(o.wp_permille));
        }
        rc_h264_picture &pc = p.pic;
        memset(&pc, 0, sizeof pc);
        pc.mem = RC_MEM_HOST;
        pc.constrained_intra_pred = o.constrained_intra_pred;
        pc.frame_id = o.frame_id;
        pc.num_slices = (int)p.slices.size();
        pc.num_weights = (int)p.weights.size();
        pc.num_levels = p.levels.size();
        pc.mbs = p.mbs.data();
        pc.slices = p.slices.data();
        pc.weights = p.weights.empty() ? nullptr : p.weights.data();
        pc.levels = p.levels.empty() ? nullptr : p.levels.data();
        pc.scaling4 = o.custom_scaling ? &p.scaling4[0][0] : nullptr;
        pc.scaling8 = o.custom_scaling ? &p.scaling8[0][0] : nullptr;
        if (o.motion_syntax) motion_syntax();
    }
};

}  // namespace

extern "C" {

void rc_synth_h264_defaults(rc_synth_h264_opts *o) {
    memset(o, 0, sizeof *o);
    o->seed = 1;
    o->mb_w = 120;
    o->mb_h = 68;
    o->intra_permille = 300;
    o->wp_permille = 200;
    o->zero_permille = 800;
    o->outside_permille = 50;
    o->mv_range = 128;
    o->t8_permille = 500;
    o->qp_min = 20;
    o->qp_max = 40;
    o->num_slices = 1;
}

void *rc_synth_h264_new(const rc_synth_h264_opts *o) {
    if (!o || o->mb_w <= 0 || o->mb_h <= 0 || o->qp_max < o->qp_min || o->qp_min < 0 || o->qp_max > 51)
        return nullptr;
    for (int l = 0; l < 2; l++)
        if (o->num_ref[l] < 0 || o->num_ref[l] > 4) return nullptr;
    Pic *p = new Pic();
    memset(p->scaling4, 16, sizeof p->scaling4);
    memset(p->scaling8, 16, sizeof p->scaling8);
    Gen g(*o, *p);
    g.run();
    return p;
}

const rc_h264_picture *rc_synth_h264_picture(void *h) { return h ? &static_cast<Pic *>(h)->pic : nullptr; }

size_t rc_synth_h264_bytes(void *h) {
    if (!h) return 0;
    Pic *p = static_cast<Pic *>(h);
    return p->mbs.size() * sizeof(rc_h264_mb) + p->slices.size() * sizeof(rc_h264_slice) +
           p->weights.size() * sizeof(rc_h264_weight) + p->levels.size() * sizeof(int16_t);
}

void rc_synth_h264_free(void *h) { delete static_cast<Pic *>(h); }

}  // extern "C"
