// synth_hevc.cpp — seeded synthetic HEVC syntax records: the stand-in for
// the host CABAC parse of coding_quadtree / coding_unit / transform_tree
// (src/hevc/slicedec.rs:1139-1671).  It builds CTB quadtrees (CU 8..64),
// transform trees (TU 4..32), intra modes, inter partitions (incl. AMP) with
// motion fields, coefficient levels, per-CTB SAO and the block flags / edge
// marks the loop filters read, all in decode (tile-scan, z-) order.
//
// Integer-only: the same seed gives the same records on x86 and Arm.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "synth.h"

namespace {

struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    uint32_t u32() { return (uint32_t)(next() >> 32); }
    int below(int n) { return n <= 0 ? 0 : (int)((next() >> 16) % (uint64_t)n); }
    bool chance(int permille) { return below(1000) < permille; }
    // Rounded Laplacian(0, b=3): P(|v| >= 1) = e^-1/6, each further step e^-1/3.
    int laplace3() {
        if (u32() >= 3635611325u) return 0;
        int m = 1;
        while (m < 4095 && u32() < 3077478545u) m++;
        return (next() & 1) ? m : -m;
    }
};

int qpc_420(int q) {
    static const int t[14] = {29, 30, 31, 32, 33, 33, 34, 34, 35, 35, 36, 36, 37, 37};
    return q < 30 ? q : q > 43 ? q - 6 : t[q - 30];
}

struct Pic {
    rc_hevc_picture pic;
    std::vector<rc_hevc_ctb> ctbs;
    std::vector<rc_hevc_blk> blk;
    std::vector<rc_hevc_mvf> mvf;
    std::vector<rc_hevc_tu> tus;
    std::vector<rc_hevc_slice> slices;
    std::vector<int16_t> levels;
    std::vector<uint8_t> scaling;
};

struct Gen {
    const rc_synth_hevc_opts &o;
    Rng r;
    Pic &p;
    int W, H, w4, h4, ctb, wctb, hctb, bd;
    // per-CU state
    int cu_qp = 30, cu_intra = 0, cu_bypass = 0, chroma_mode = 0;
    int luma_mode[4] = {0, 0, 0, 0};  // per NxN PU (or all the same)
    int cu_x = 0, cu_y = 0, cu_log2 = 3, intra_split = 0;

    Gen(const rc_synth_hevc_opts &o_, Pic &p_) : o(o_), r{o_.seed}, p(p_) {
        W = o.width;
        H = o.height;
        w4 = W / 4;
        h4 = H / 4;
        ctb = 1 << o.log2_ctb;
        wctb = (W + ctb - 1) / ctb;
        hctb = (H + ctb - 1) / ctb;
        bd = o.bit_depth;
    }

    rc_hevc_blk &B(int x, int y) { return p.blk[(y >> 2) * w4 + (x >> 2)]; }

    void fill(int x0, int y0, int w, int h, int set_flags, int clear_flags = 0) {
        for (int y = y0; y < y0 + h && y < H; y += 4)
            for (int x = x0; x < x0 + w && x < W; x += 4) {
                rc_hevc_blk &b = B(x, y);
                b.flags = (uint8_t)((b.flags & ~clear_flags) | set_flags);
            }
    }
    // mark_edges, src/hevc/slicedec.rs:1345-1363
    void mark_edges(int x0, int y0, int w, int h, int v, int hz) {
        if (v)
            for (int y = y0; y < y0 + h && y < H; y += 4) B(x0, y).edges |= (uint8_t)v;
        if (hz)
            for (int x = x0; x < x0 + w && x < W; x += 4) B(x, y0).edges |= (uint8_t)hz;
    }

    int luma_qp_dq() const { return cu_qp + 6 * (bd - 8); }
    int chroma_qp_dq(int c) const {
        int offc = 6 * (bd - 8);
        int qpi = cu_qp + (c == 1 ? o.cb_qp_offset : o.cr_qp_offset);
        qpi = qpi < -offc ? -offc : qpi > 57 ? 57 : qpi;
        return qpc_420(qpi) + offc;
    }

    void emit_tu(int x0, int y0, int log2, int c, int mode, bool cbf) {
        rc_hevc_tu t;
        memset(&t, 0, sizeof t);
        t.x0 = (uint16_t)x0;
        t.y0 = (uint16_t)y0;
        t.log2 = (uint8_t)log2;
        t.c = (uint8_t)c;
        t.mode = (uint8_t)mode;
        t.qp = (int8_t)(c == 0 ? luma_qp_dq() : chroma_qp_dq(c));
        t.flags = (uint8_t)((cu_intra ? RC_HEVC_TU_INTRA : 0) | (cbf ? RC_HEVC_TU_CBF : 0) |
                            (cu_bypass ? RC_HEVC_TU_BYPASS : 0));
        if (cbf && log2 == 2 && !cu_bypass && r.chance(o.transform_skip_permille)) t.flags |= RC_HEVC_TU_SKIP;
        if (cbf) {
            int n = 1 << log2;
            // last significant position: small regions are the common case
            int mx = r.chance(500) ? r.below(n < 8 ? n : 8) : r.below(n);
            int my = r.chance(500) ? r.below(n < 8 ? n : 8) : r.below(n);
            t.max_x = (uint8_t)mx;
            t.max_y = (uint8_t)my;
            t.coef_off = (uint32_t)p.levels.size();
            int cnt = (mx + 1) * (my + 1);
            bool any = false;
            for (int i = 0; i < cnt; i++) {
                int v = r.laplace3();
                any |= v != 0;
                p.levels.push_back((int16_t)v);
            }
            if (!any) p.levels[t.coef_off + cnt - 1] = (int16_t)((r.next() & 1) ? 1 : -1);
        }
        if (cu_intra || cbf) p.tus.push_back(t);
    }

    void emit_pcm(int x0, int y0, int log2) {
        for (int c = 0; c < 3; c++) {
            int lg = c ? log2 - 1 : log2, n = 1 << lg;
            rc_hevc_tu t;
            memset(&t, 0, sizeof t);
            t.x0 = (uint16_t)(c ? x0 / 2 : x0);
            t.y0 = (uint16_t)(c ? y0 / 2 : y0);
            t.log2 = (uint8_t)lg;
            t.c = (uint8_t)c;
            t.flags = RC_HEVC_TU_INTRA | RC_HEVC_TU_PCM;
            t.coef_off = (uint32_t)p.levels.size();
            for (int i = 0; i < n * n; i++) p.levels.push_back((int16_t)r.below(1 << bd));
            p.tus.push_back(t);
        }
    }

    // transform_tree, src/hevc/slicedec.rs:1545-1600 (structure only)
    void transform_tree(int x0, int y0, int xb, int yb, int log2, int depth, int blk_idx) {
        bool split = log2 > 5 || (intra_split && depth == 0) || (log2 > 2 && r.chance(o.split_permille / 2));
        if (split) {
            int h = 1 << (log2 - 1);
            transform_tree(x0, y0, x0, y0, log2 - 1, depth + 1, 0);
            transform_tree(x0 + h, y0, x0, y0, log2 - 1, depth + 1, 1);
            transform_tree(x0, y0 + h, x0, y0, log2 - 1, depth + 1, 2);
            transform_tree(x0 + h, y0 + h, x0, y0, log2 - 1, depth + 1, 3);
            return;
        }
        int n = 1 << log2;
        if (depth > 0) mark_edges(x0, y0, n, n, RC_HEVC_E_TU_V, RC_HEVC_E_TU_H);
        int keep = 1000 - o.zero_tu_permille;
        bool cbf_l = r.chance(keep);
        int lmode = 0;
        if (cu_intra) {
            int pu = intra_split ? ((y0 >= cu_y + 4) ? 2 : 0) + ((x0 >= cu_x + 4) ? 1 : 0) : 0;
            lmode = luma_mode[pu];
        }
        emit_tu(x0, y0, log2, 0, lmode, cbf_l);
        if (cbf_l) fill(x0, y0, n, n, RC_HEVC_F_CBF);
        bool chroma_here = log2 > 2 || blk_idx == 3;
        if (!chroma_here) return;
        int xc = log2 > 2 ? x0 / 2 : xb / 2, yc = log2 > 2 ? y0 / 2 : yb / 2, lc = log2 > 2 ? log2 - 1 : 2;
        for (int c = 1; c < 3; c++) emit_tu(xc, yc, lc, c, chroma_mode, r.chance(keep));
    }

    int16_t mv_comp() { return (int16_t)(r.below(8 * o.mv_range) - 4 * o.mv_range); }

    void prediction_unit(int x, int y, int w, int h) {
        rc_hevc_mvf f;
        memset(&f, 0, sizeof f);
        f.ref_idx[0] = f.ref_idx[1] = -1;
        bool l0 = o.num_ref[0] > 0, l1 = o.num_ref[1] > 0;
        bool both = l0 && l1 && r.chance(o.bipred_permille);
        if (!both && l0 && l1) {
            if (r.below(2)) l1 = false;
            else l0 = false;
        }
        if (l0) f.ref_idx[0] = (int8_t)r.below(o.num_ref[0]);
        if (l1) f.ref_idx[1] = (int8_t)r.below(o.num_ref[1]);
        for (int l = 0; l < 2; l++)
            if (f.ref_idx[l] >= 0) {
                f.mv[l][0] = mv_comp();
                f.mv[l][1] = mv_comp();
            }
        for (int yy = y; yy < y + h; yy += 4)
            for (int xx = x; xx < x + w; xx += 4) p.mvf[(yy >> 2) * w4 + (xx >> 2)] = f;
    }

    // coding_unit, src/hevc/slicedec.rs:1224-1337 (structure only)
    void coding_unit(int x0, int y0, int log2) {
        int n = 1 << log2;
        cu_x = x0;
        cu_y = y0;
        cu_log2 = log2;
        cu_qp = o.qp_min + r.below(o.qp_max - o.qp_min + 1);
        cu_bypass = r.chance(o.bypass_permille);
        cu_intra = o.intra_only || (o.num_ref[0] == 0 && o.num_ref[1] == 0) || r.chance(o.intra_permille);
        for (int y = y0; y < y0 + n; y += 4)
            for (int x = x0; x < x0 + n; x += 4) {
                rc_hevc_blk &b = B(x, y);
                b.flags = (uint8_t)(RC_HEVC_F_CODED | (cu_bypass ? RC_HEVC_F_NOFILTER : 0) |
                                    (cu_intra ? RC_HEVC_F_INTRA : 0));
                b.qp = (int8_t)cu_qp;
                b.ipm = 1;
                b.edges = 0;
            }
        mark_edges(x0, y0, n, n, RC_HEVC_E_TU_V | RC_HEVC_E_PU_V, RC_HEVC_E_TU_H | RC_HEVC_E_PU_H);
        if (cu_intra) {
            intra_split = log2 == 3 && r.chance(500);
            bool pcm = !intra_split && log2 <= 5 && r.chance(o.pcm_permille);
            if (pcm) {
                emit_pcm(x0, y0, log2);
                if (o.pcm_loop_filter_disabled) fill(x0, y0, n, n, RC_HEVC_F_NOFILTER);
                return;
            }
            int nparts = intra_split ? 4 : 1, pb = intra_split ? n / 2 : n;
            for (int i = 0; i < nparts; i++) {
                luma_mode[i] = r.below(35);
                int xp = x0 + (i & 1) * pb, yp = y0 + (i >> 1) * pb;
                for (int y = yp; y < yp + pb; y += 4)
                    for (int x = xp; x < xp + pb; x += 4) B(x, y).ipm = (uint8_t)luma_mode[i];
            }
            if (!intra_split)
                for (int i = 1; i < 4; i++) luma_mode[i] = luma_mode[0];
            // intra_chroma_pred_mode: 4 = derived from luma, else the list with the mode-34 rule
            int icpm = r.below(5);
            if (icpm == 4) chroma_mode = luma_mode[0];
            else {
                static const int m4[4] = {0, 26, 10, 1};
                chroma_mode = m4[icpm] == luma_mode[0] ? 34 : m4[icpm];
            }
            transform_tree(x0, y0, x0, y0, log2, 0, 0);
            return;
        }
        intra_split = 0;
        // partition: 2Nx2N, 2NxN, Nx2N, and the four AMP shapes above 8x8
        int nshapes = log2 > 3 ? 7 : 3, part = r.below(nshapes);
        int h = n / 2, q = n / 4;
        struct P { int x, y, w, hh; } parts[2];
        int np = 1;
        switch (part) {
        case 0: parts[0] = {0, 0, n, n}; break;
        case 1: parts[0] = {0, 0, n, h}; parts[1] = {0, h, n, h}; np = 2; break;
        case 2: parts[0] = {0, 0, h, n}; parts[1] = {h, 0, h, n}; np = 2; break;
        case 3: parts[0] = {0, 0, n, q}; parts[1] = {0, q, n, n - q}; np = 2; break;
        case 4: parts[0] = {0, 0, n, n - q}; parts[1] = {0, n - q, n, q}; np = 2; break;
        case 5: parts[0] = {0, 0, q, n}; parts[1] = {q, 0, n - q, n}; np = 2; break;
        default: parts[0] = {0, 0, n - q, n}; parts[1] = {n - q, 0, q, n}; np = 2; break;
        }
        for (int i = 0; i < np; i++) {
            prediction_unit(x0 + parts[i].x, y0 + parts[i].y, parts[i].w, parts[i].hh);
            if (parts[i].x) mark_edges(x0 + parts[i].x, y0 + parts[i].y, parts[i].w, parts[i].hh, RC_HEVC_E_PU_V, 0);
            if (parts[i].y) mark_edges(x0 + parts[i].x, y0 + parts[i].y, parts[i].w, parts[i].hh, 0, RC_HEVC_E_PU_H);
        }
        // rqt_root_cbf: a CU without residual has no transform tree
        if (r.chance(1000 - o.zero_tu_permille / 2)) transform_tree(x0, y0, x0, y0, log2, 0, 0);
    }

    // coding_quadtree with the implicit splits at the picture border
    void quadtree(int x0, int y0, int log2) {
        int n = 1 << log2;
        bool inside = x0 + n <= W && y0 + n <= H;
        bool split = log2 > 3 && (!inside || r.chance(o.split_permille));
        if (split) {
            int h = n / 2;
            for (int i = 0; i < 4; i++) {
                int x = x0 + (i & 1) * h, y = y0 + (i >> 1) * h;
                if (x < W && y < H) quadtree(x, y, log2 - 1);
            }
            return;
        }
        coding_unit(x0, y0, log2);
    }

    void sao_params(rc_hevc_sao &s) {
        memset(&s, 0, sizeof s);
        if (!o.sao) return;
        for (int c = 0; c < 3; c++) {
            if (c == 2) {  // Cr shares Cb's type and edge class
                s.type_idx[2] = s.type_idx[1];
                s.eo_class[2] = s.eo_class[1];
            } else {
                s.type_idx[c] = (uint8_t)r.below(3);
                s.eo_class[c] = (uint8_t)r.below(4);
            }
            s.band_pos[c] = (uint8_t)r.below(32);
            for (int k = 0; k < 4; k++) {
                int v = r.below(8);
                if (s.type_idx[c] == 1) v = (r.next() & 1) ? -v : v;
                else if (k >= 2) v = -v;  // edge categories 3 and 4 subtract
                s.offsets[c][k] = (int16_t)v;
            }
        }
    }

    void run() {
        int nctb = wctb * hctb;
        p.blk.assign((size_t)w4 * h4, rc_hevc_blk());
        memset(p.blk.data(), 0, sizeof(rc_hevc_blk) * p.blk.size());
        p.mvf.assign((size_t)w4 * h4, rc_hevc_mvf());
        for (auto &f : p.mvf) {
            memset(&f, 0, sizeof f);
            f.ref_idx[0] = f.ref_idx[1] = -1;
        }
        p.ctbs.assign(nctb, rc_hevc_ctb());
        memset(p.ctbs.data(), 0, sizeof(rc_hevc_ctb) * nctb);
        // tiles with uniform spacing, tile-scan order
        int tc = o.tile_cols < 1 ? 1 : o.tile_cols, tr = o.tile_rows < 1 ? 1 : o.tile_rows;
        std::vector<int> colb(tc + 1), rowb(tr + 1), ts_to_rs;
        for (int i = 0; i <= tc; i++) colb[i] = i * wctb / tc;
        for (int i = 0; i <= tr; i++) rowb[i] = i * hctb / tr;
        for (int ty = 0; ty < tr; ty++)
            for (int tx = 0; tx < tc; tx++)
                for (int y = rowb[ty]; y < rowb[ty + 1]; y++)
                    for (int x = colb[tx]; x < colb[tx + 1]; x++) {
                        int rs = y * wctb + x;
                        p.ctbs[rs].tile = (uint16_t)(ty * tc + tx);
                        p.ctbs[rs].ts = (uint32_t)ts_to_rs.size();
                        ts_to_rs.push_back(rs);
                    }
        int ns = o.num_slices < 1 ? 1 : o.num_slices;
        if (ns > nctb) ns = nctb;
        for (int s = 0; s < ns; s++) {
            rc_hevc_slice sl;
            memset(&sl, 0, sizeof sl);
            sl.slice_addr = (uint32_t)ts_to_rs[(size_t)s * nctb / ns];
            sl.deblock_disabled = o.deblock_disabled;
            sl.beta_offset = o.beta_offset;
            sl.tc_offset = o.tc_offset;
            sl.lf_across = o.lf_across_slices;
            sl.sao_luma = sl.sao_chroma = o.sao ? 1 : 0;
            sl.weighted = o.weighted;
            sl.luma_log2_denom = r.below(8);
            sl.chroma_log2_denom = r.below(8);
            for (int l = 0; l < 2; l++) {
                sl.num_ref[l] = o.num_ref[l];
                for (int i = 0; i < o.num_ref[l] && i < 4; i++) {
                    sl.ref_slot[l][i] = o.ref_slot[l][i];
                    sl.ref_id[l][i] = o.ref_id[l][i];
                }
                for (int i = 0; i < RC_HEVC_MAX_REFS; i++) {
                    sl.luma_w[l][i] = (int16_t)((1 << sl.luma_log2_denom) + r.below(41) - 20);
                    sl.luma_o[l][i] = (int16_t)(r.below(41) - 20);
                    for (int c = 0; c < 2; c++) {
                        sl.chroma_w[l][i][c] = (int16_t)((1 << sl.chroma_log2_denom) + r.below(41) - 20);
                        sl.chroma_o[l][i][c] = (int16_t)(r.below(41) - 20);
                    }
                }
            }
            p.slices.push_back(sl);
        }
        if (o.scaling_lists) {
            p.scaling.resize(6 * (16 + 64 + 256 + 1024));
            for (auto &v : p.scaling) v = (uint8_t)(4 + r.below(60));
        }
        for (int ts = 0; ts < nctb; ts++) {
            int rs = ts_to_rs[ts];
            p.ctbs[rs].slice = (uint16_t)((long long)ts * ns / nctb);
            sao_params(p.ctbs[rs].sao);
            quadtree((rs % wctb) * ctb, (rs / wctb) * ctb, o.log2_ctb);
        }
        rc_hevc_picture &pc = p.pic;
        memset(&pc, 0, sizeof pc);
        pc.mem = RC_MEM_HOST;
        pc.log2_ctb = o.log2_ctb;
        pc.constrained_intra_pred = o.constrained_intra_pred;
        pc.strong_intra_smoothing = o.strong_intra_smoothing;
        pc.loop_filter_across_tiles = o.loop_filter_across_tiles;
        pc.cb_qp_offset = o.cb_qp_offset;
        pc.cr_qp_offset = o.cr_qp_offset;
        pc.num_slices = (int)p.slices.size();
        pc.num_tus = (int)p.tus.size();
        pc.frame_id = o.frame_id;
        pc.num_levels = p.levels.size();
        pc.ctbs = p.ctbs.data();
        pc.blk = p.blk.data();
        pc.mvf = p.mvf.data();
        pc.tus = p.tus.empty() ? nullptr : p.tus.data();
        pc.slices = p.slices.data();
        pc.levels = p.levels.empty() ? nullptr : p.levels.data();
        pc.scaling = p.scaling.empty() ? nullptr : p.scaling.data();
    }
};

}  // namespace

extern "C" {

void rc_synth_hevc_defaults(rc_synth_hevc_opts *o) {
    memset(o, 0, sizeof *o);
    o->seed = 1;
    o->width = 1920;
    o->height = 1080;
    o->bit_depth = 8;
    o->log2_ctb = 6;
    o->intra_permille = 250;
    o->zero_tu_permille = 750;
    o->split_permille = 500;
    o->mv_range = 256;
    o->qp_min = 22;
    o->qp_max = 37;
    o->strong_intra_smoothing = 1;
    o->loop_filter_across_tiles = 1;
    o->lf_across_slices = 1;
    o->sao = 1;
}

void *rc_synth_hevc_new(const rc_synth_hevc_opts *o) {
    if (!o || o->width <= 0 || o->height <= 0 || (o->width & 7) || (o->height & 7)) return nullptr;
    if ((o->bit_depth != 8 && o->bit_depth != 10) || o->log2_ctb < 4 || o->log2_ctb > 6) return nullptr;
    if (o->qp_min > o->qp_max || o->qp_min < -6 * (o->bit_depth - 8) || o->qp_max > 51) return nullptr;
    for (int l = 0; l < 2; l++)
        if (o->num_ref[l] < 0 || o->num_ref[l] > 4) return nullptr;
    if (o->mv_range <= 0 || o->mv_range > 4096) return nullptr;
    Pic *p = new Pic();
    Gen g(*o, *p);
    g.run();
    return p;
}

const rc_hevc_picture *rc_synth_hevc_picture(void *h) { return h ? &static_cast<Pic *>(h)->pic : nullptr; }

size_t rc_synth_hevc_bytes(void *h) {
    if (!h) return 0;
    Pic *p = static_cast<Pic *>(h);
    return p->ctbs.size() * sizeof(rc_hevc_ctb) + p->blk.size() * sizeof(rc_hevc_blk) +
           p->mvf.size() * sizeof(rc_hevc_mvf) + p->tus.size() * sizeof(rc_hevc_tu) +
           p->slices.size() * sizeof(rc_hevc_slice) + p->levels.size() * sizeof(int16_t);
}

void rc_synth_hevc_free(void *h) { delete static_cast<Pic *>(h); }

}  // extern "C"
