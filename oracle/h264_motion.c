/*
 * h264_motion.c — CPU restatement of the reference's H.264 motion
 * derivation, for pictures submitted with motion syntax (rc_h264_motion).
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the checker for the engine's
 * h264_mv_kernel.  It follows the reference's slice decoder
 * (src/h264/dec/slicedec.rs): nb_motion :581-621, nb_abc :623-633, mvp
 * :635-662, median_pred :664-681, set_motion :683-716, colocated :718-731,
 * spatial_direct_base :733-752, derive_direct :754-852, derive_p_skip
 * :854-866, derive_inter_motion :868-935; the temporal-direct tables of
 * SliceDecoder::new :371-384 arrive precomputed per slice.  Co-located
 * motion is what Frame::publish stores per MB (src/h264/dec/picture.rs:492).
 */
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

typedef struct {
    int avail, ref;
    int16_t mv[2];
} Nb;

static const Nb NB_NA = {0, -1, {0, 0}};

typedef struct {
    int mb_w, mb_h, addr;
    int nb[4]; /* A (left), B (above), C (above right), D (above left); -1 unavailable */
    uint32_t done; /* 4x4 blocks of the current MB whose motion is set */
    const rc_h264_picture *pic;
    const rc_h264_slice *sl;
    const rc_h264_slice_motion *sm;
    const rc_h264_motion *mo;
    rc_h264_mb *mbs;
    const oracle_h264_colmb *col; /* the co-located MB, or NULL */
} Mctx;

static int16_t wrap16(int v) { return (int16_t)(uint16_t)(v & 0xffff); }

static int median3(int a, int b, int c) {
    int lo = a < b ? a : b, hi = a < b ? b : a;
    return lo > (hi < c ? hi : c) ? lo : (hi < c ? hi : c);
}

/* nb_motion, slicedec.rs:581-621 (x, y in 4x4 blocks relative to the MB) */
static Nb nb_motion(const Mctx *c, int l, int x, int y) {
    int mb, bx, by;
    if (x < 0) {
        if (y < 0) { mb = c->nb[3]; bx = 3; by = 3; }
        else if (y > 3) return NB_NA;
        else { mb = c->nb[0]; bx = 3; by = y; }
    } else if (x > 3) {
        if (y < 0) { mb = c->nb[2]; bx = 0; by = 3; }
        else return NB_NA;
    } else if (y < 0) {
        mb = c->nb[1]; bx = x; by = 3;
    } else {
        if (!(c->done >> (y * 4 + x) & 1)) return NB_NA;
        mb = c->addr; bx = x; by = y;
    }
    if (mb < 0) return NB_NA;
    const rc_h264_mb *m = &c->mbs[mb];
    const int r = m->ref_idx[l][(by >> 1) * 2 + (bx >> 1)];
    Nb n = {1, -1, {0, 0}};
    if (r < 0) return n;
    n.ref = r;
    n.mv[0] = m->mv[l][by * 4 + bx][0];
    n.mv[1] = m->mv[l][by * 4 + bx][1];
    return n;
}

static void nb_abc(const Mctx *c, int l, int x, int y, int w, Nb *a, Nb *b, Nb *cc) {
    *a = nb_motion(c, l, x - 1, y);
    *b = nb_motion(c, l, x, y - 1);
    *cc = nb_motion(c, l, x + w, y - 1);
    if (!cc->avail) *cc = nb_motion(c, l, x - 1, y - 1);
}

/* median_pred, slicedec.rs:664-681 */
static void median_pred(Nb a, Nb b, Nb c, int ref, int16_t out[2]) {
    if (!b.avail && !c.avail && a.avail) {
        b = a;
        c = a;
    }
    const int ma = a.ref == ref, mb = b.ref == ref, mc = c.ref == ref;
    if (ma && !mb && !mc) { out[0] = a.mv[0]; out[1] = a.mv[1]; return; }
    if (!ma && mb && !mc) { out[0] = b.mv[0]; out[1] = b.mv[1]; return; }
    if (!ma && !mb && mc) { out[0] = c.mv[0]; out[1] = c.mv[1]; return; }
    out[0] = (int16_t)median3(a.mv[0], b.mv[0], c.mv[0]);
    out[1] = (int16_t)median3(a.mv[1], b.mv[1], c.mv[1]);
}

/* mvp, slicedec.rs:635-662: shape 1 = 16x8, 2 = 8x16 (directional rules) */
static void mvp(const Mctx *c, int l, int x, int y, int w, int ref, int shape, int part, int16_t out[2]) {
    Nb a, b, cc;
    nb_abc(c, l, x, y, w, &a, &b, &cc);
    if (shape == 1) {
        if (part == 0 && b.ref == ref) { out[0] = b.mv[0]; out[1] = b.mv[1]; return; }
        if (part == 1 && a.ref == ref) { out[0] = a.mv[0]; out[1] = a.mv[1]; return; }
    } else if (shape == 2) {
        if (part == 0 && a.ref == ref) { out[0] = a.mv[0]; out[1] = a.mv[1]; return; }
        if (part == 1 && cc.ref == ref) { out[0] = cc.mv[0]; out[1] = cc.mv[1]; return; }
    }
    median_pred(a, b, cc, ref, out);
}

/* set_motion, slicedec.rs:683-716 (x, y, w, h in 4x4 blocks) */
static void set_motion(Mctx *c, int x, int y, int w, int h, const int refs[2], int16_t mvs[2][2]) {
    rc_h264_mb *st = &c->mbs[c->addr];
    for (int l = 0; l < 2; l++) {
        const int16_t mx = refs[l] >= 0 ? mvs[l][0] : 0, my = refs[l] >= 0 ? mvs[l][1] : 0;
        for (int yy = y; yy < y + h; yy++)
            for (int xx = x; xx < x + w; xx++) {
                st->mv[l][yy * 4 + xx][0] = mx;
                st->mv[l][yy * 4 + xx][1] = my;
            }
        for (int by = y >> 1; by <= (y + h - 1) >> 1; by++)
            for (int bx = x >> 1; bx <= (x + w - 1) >> 1; bx++) st->ref_idx[l][by * 2 + bx] = (int8_t)refs[l];
    }
    for (int yy = y; yy < y + h; yy++)
        for (int xx = x; xx < x + w; xx++) c->done |= 1u << (yy * 4 + xx);
}

/* colocated, slicedec.rs:718-731 */
static void colocated(const Mctx *c, int raster, int16_t mv[2], int *ref, uint32_t *id) {
    if (c->sm->direct_8x8_inference) {
        const int bx = raster & 3, by = raster >> 2;
        raster = (by >= 2 ? 12 : 0) + (bx >= 2 ? 3 : 0);
    }
    const oracle_h264_colmb *m = c->col;
    if (!m || m->intra) {
        mv[0] = mv[1] = 0;
        *ref = -1;
        *id = 0xffffffffu;
        return;
    }
    const int b8 = (raster >> 3) * 2 + ((raster & 3) >> 1);
    const int l = m->ref_idx[0][b8] >= 0 ? 0 : 1;
    mv[0] = m->mv[l][raster][0];
    mv[1] = m->mv[l][raster][1];
    *ref = m->ref_idx[l][b8];
    *id = m->ref_id[l][b8];
}

static int min_pos(int x, int y) { return (x >= 0 && y >= 0) ? (x < y ? x : y) : (x > y ? x : y); }

static int small_mv(const int16_t mv[2]) { return mv[0] >= -1 && mv[0] <= 1 && mv[1] >= -1 && mv[1] <= 1; }

/* derive_direct, slicedec.rs:754-852, with spatial_direct_base :733-752 */
static int derive_direct(Mctx *c, int b8_mask) {
    const int spatial = c->sm->direct_spatial, d8i = c->sm->direct_8x8_inference;
    int base_refs[2] = {0, 0}, direct_zero = 0;
    int16_t base_mvs[2][2] = {{0, 0}, {0, 0}};
    if (spatial) {
        Nb nbs[2][3];
        for (int l = 0; l < 2; l++) {
            nb_abc(c, l, 0, 0, 4, &nbs[l][0], &nbs[l][1], &nbs[l][2]);
            base_refs[l] = min_pos(nbs[l][0].ref, min_pos(nbs[l][1].ref, nbs[l][2].ref));
        }
        if (base_refs[0] < 0 && base_refs[1] < 0) {
            base_refs[0] = base_refs[1] = 0;
            direct_zero = 1;
        } else {
            for (int l = 0; l < 2; l++)
                if (base_refs[l] >= 0) median_pred(nbs[l][0], nbs[l][1], nbs[l][2], base_refs[l], base_mvs[l]);
        }
    }
    const int col_short_term = c->sm->col_short_term;
    const int need_col = !direct_zero && col_short_term && (base_refs[0] == 0 || base_refs[1] == 0);
    if (spatial && (!need_col || d8i)) {
        for (int b8 = 0; b8 < 4; b8++) {
            if (!(b8_mask >> b8 & 1)) continue;
            int zero = 0;
            if (need_col) {
                int16_t mv[2];
                int r;
                uint32_t id;
                colocated(c, (b8 >> 1) * 8 + (b8 & 1) * 2, mv, &r, &id);
                zero = r == 0 && small_mv(mv);
            }
            int16_t mvs[2][2];
            for (int l = 0; l < 2; l++) {
                const int z = direct_zero || base_refs[l] < 0 || (base_refs[l] == 0 && zero);
                mvs[l][0] = z ? 0 : base_mvs[l][0];
                mvs[l][1] = z ? 0 : base_mvs[l][1];
            }
            set_motion(c, (b8 & 1) * 2, (b8 >> 1) * 2, 2, 2, base_refs, mvs);
        }
        return 0;
    }
    for (int b8 = 0; b8 < 4; b8++) {
        if (!(b8_mask >> b8 & 1)) continue;
        const int x8 = (b8 & 1) * 2, y8 = (b8 >> 1) * 2, unit = d8i ? 2 : 1;
        for (int sub = 0; sub < (unit == 1 ? 4 : 1); sub++) {
            const int x = x8 + (sub & 1), y = y8 + (sub >> 1);
            int16_t mv_col[2];
            int ref_col;
            uint32_t id_col;
            colocated(c, y * 4 + x, mv_col, &ref_col, &id_col);
            int refs[2];
            int16_t mvs[2][2];
            if (spatial) {
                const int col_zero = col_short_term && ref_col == 0 && small_mv(mv_col);
                for (int l = 0; l < 2; l++) {
                    const int z = direct_zero || base_refs[l] < 0 || (base_refs[l] == 0 && col_zero);
                    mvs[l][0] = z ? 0 : base_mvs[l][0];
                    mvs[l][1] = z ? 0 : base_mvs[l][1];
                    refs[l] = base_refs[l];
                }
            } else {
                int ref0 = 0;
                if (ref_col >= 0)
                    for (int i = 0; i < c->sl->num_ref[0] && i < RC_H264_MAX_REFS; i++)
                        if (c->sl->ref_id[0][i] == id_col) { ref0 = i; break; }
                const int copy = ref0 < c->sl->num_ref[0] ? c->sm->direct_copy[ref0] : 1;
                const int dsf = ref0 < c->sl->num_ref[0] ? c->sm->dist_scale[ref0] : 256;
                if (copy) {
                    mvs[0][0] = mv_col[0]; mvs[0][1] = mv_col[1];
                    mvs[1][0] = mvs[1][1] = 0;
                } else {
                    for (int i = 0; i < 2; i++) {
                        mvs[0][i] = (int16_t)((dsf * mv_col[i] + 128) >> 8);
                        mvs[1][i] = wrap16(mvs[0][i] - mv_col[i]);
                    }
                }
                refs[0] = ref0;
                refs[1] = 0;
            }
            set_motion(c, x, y, unit, unit, refs, mvs);
        }
    }
    return 0;
}

/* derive_p_skip, slicedec.rs:854-866 */
static void derive_p_skip(Mctx *c) {
    const Nb a = nb_motion(c, 0, -1, 0), b = nb_motion(c, 0, 0, -1);
    int16_t mvs[2][2] = {{0, 0}, {0, 0}};
    if (!(c->nb[0] < 0 || c->nb[1] < 0 || (a.ref == 0 && a.mv[0] == 0 && a.mv[1] == 0) ||
          (b.ref == 0 && b.mv[0] == 0 && b.mv[1] == 0)))
        mvp(c, 0, 0, 0, 4, 0, 0, 0, mvs[0]);
    const int refs[2] = {0, -1};
    set_motion(c, 0, 0, 4, 4, refs, mvs);
}

/* derive_inter_motion, slicedec.rs:868-935 */
static int derive_inter(Mctx *c) {
    const rc_h264_motion *mo = c->mo;
    const int n[2] = {c->sl->num_ref[0], c->sl->num_ref[1]};
    if (mo->shape == RC_H264_MOTION_SKIP) {
        if (c->sm->b_slice) return derive_direct(c, 0xf);
        if (n[0] < 1) return RC_EINVAL;
        derive_p_skip(c);
        return 0;
    }
    if (mo->shape != RC_H264_MOTION_8x8) {
        const int np = mo->shape == RC_H264_MOTION_16x16 ? 1 : 2;
        const int shape = mo->shape == RC_H264_MOTION_16x8 ? 1 : mo->shape == RC_H264_MOTION_8x16 ? 2 : 0;
        for (int p = 0; p < np; p++) {
            const int x = shape == 2 ? 2 * p : 0, y = shape == 1 ? 2 * p : 0;
            const int w = shape == 2 ? 2 : 4, h = shape == 1 ? 2 : 4;
            const int b8 = (y >> 1) * 2 + (x >> 1);
            int refs[2] = {-1, -1};
            int16_t mvs[2][2] = {{0, 0}, {0, 0}};
            for (int l = 0; l < 2; l++) {
                if (!(mo->pred[p] >> l & 1)) continue;
                const int r = mo->ref_idx[l][b8];
                if (r < 0 || r >= n[l]) return RC_EINVAL;
                int16_t p_mv[2];
                mvp(c, l, x, y, w, r, shape, p, p_mv);
                refs[l] = r;
                mvs[l][0] = wrap16(p_mv[0] + mo->mvd[l][y * 4 + x][0]);
                mvs[l][1] = wrap16(p_mv[1] + mo->mvd[l][y * 4 + x][1]);
            }
            set_motion(c, x, y, w, h, refs, mvs);
        }
        return 0;
    }
    for (int p = 0; p < 4; p++) {
        const int x8 = (p & 1) * 2, y8 = (p >> 1) * 2, sub = mo->sub[p];
        if (sub == RC_H264_SUB_DIRECT) {
            if (!c->sm->b_slice) return RC_EINVAL;
            const int rc = derive_direct(c, 1 << p);
            if (rc) return rc;
            continue;
        }
        if (sub > RC_H264_SUB_4x4) return RC_EINVAL;
        int refs[2] = {-1, -1};
        for (int l = 0; l < 2; l++) {
            if (!(mo->pred[p] >> l & 1)) continue;
            const int v = mo->ref_idx[l][p];
            if (v < 0 || v >= n[l]) return RC_EINVAL;
            refs[l] = v;
        }
        const int sw = (sub == RC_H264_SUB_8x8 || sub == RC_H264_SUB_8x4) ? 2 : 1;
        const int sh = (sub == RC_H264_SUB_8x8 || sub == RC_H264_SUB_4x8) ? 2 : 1;
        for (int sy = 0; sy < 2; sy += sh)
            for (int sx = 0; sx < 2; sx += sw) {
                const int x = x8 + sx, y = y8 + sy;
                int16_t mvs[2][2] = {{0, 0}, {0, 0}};
                for (int l = 0; l < 2; l++) {
                    if (refs[l] < 0) continue;
                    int16_t p_mv[2];
                    mvp(c, l, x, y, sw, refs[l], 0, 0, p_mv);
                    mvs[l][0] = wrap16(p_mv[0] + mo->mvd[l][y * 4 + x][0]);
                    mvs[l][1] = wrap16(p_mv[1] + mo->mvd[l][y * 4 + x][1]);
                }
                set_motion(c, x, y, sw, sh, refs, mvs);
            }
    }
    return 0;
}

int oracle_h264_derive_motion(int mb_w, int mb_h, const rc_h264_picture *pic,
                              const oracle_h264_colmb *const *col, int slots, rc_h264_mb *mbs,
                              oracle_h264_colmb *out_col) {
    if (!pic || !pic->motion || !pic->slice_motion || !mbs || !out_col) return RC_EINVAL;
    const int n = mb_w * mb_h;
    Mctx c;
    memset(&c, 0, sizeof c);
    c.mb_w = mb_w;
    c.mb_h = mb_h;
    c.pic = pic;
    c.mbs = mbs;
    for (int a = 0; a < n; a++) {
        rc_h264_mb *m = &mbs[a];
        const rc_h264_motion *mo = &pic->motion[a];
        const int inter = m->kind == RC_H264_INTER;
        if (inter != (mo->shape != RC_H264_MOTION_NONE) || mo->shape > RC_H264_MOTION_8x8) return RC_EINVAL;
        if (!inter) {
            memset(m->ref_idx, -1, sizeof m->ref_idx);
            memset(m->mv, 0, sizeof m->mv);
            memset(m->wp, 0xff, sizeof m->wp);
            continue;
        }
        if (m->slice >= pic->num_slices) return RC_EINVAL;
        c.addr = a;
        c.sl = &pic->slices[m->slice];
        c.sm = &pic->slice_motion[m->slice];
        c.mo = mo;
        c.done = 0;
        const int x = a % mb_w, y = a / mb_w;
        const int dx[4] = {-1, 0, 1, -1}, dy[4] = {0, -1, -1, -1};
        for (int i = 0; i < 4; i++) {
            const int nx = x + dx[i], ny = y + dy[i];
            const int na = ny * mb_w + nx;
            c.nb[i] = (nx >= 0 && ny >= 0 && nx < mb_w && mbs[na].kind != RC_H264_NONE && mbs[na].slice == m->slice)
                          ? na
                          : -1;
        }
        c.col = NULL;
        if (c.sm->b_slice) {
            if (c.sm->col_slot < 0 || c.sm->col_slot >= slots || !col[c.sm->col_slot]) return RC_EINVAL;
            c.col = &col[c.sm->col_slot][a];
        }
        memset(m->ref_idx, -1, sizeof m->ref_idx);
        memset(m->mv, 0, sizeof m->mv);
        const int rc = derive_inter(&c);
        if (rc) return rc;
        for (int b8 = 0; b8 < 4; b8++) {
            const int r0 = m->ref_idx[0][b8], r1 = m->ref_idx[1][b8];
            m->wp[b8] = c.sm->wp_map[(r0 + 1) * (RC_H264_MAX_REFS + 1) + (r1 + 1)];
        }
    }
    /* the picture's co-located motion (Frame::publish, picture.rs:492) */
    for (int a = 0; a < n; a++) {
        const rc_h264_mb *m = &mbs[a];
        oracle_h264_colmb *o = &out_col[a];
        memset(o, 0, sizeof *o);
        o->intra = m->kind != RC_H264_INTER;
        memcpy(o->mv, m->mv, sizeof o->mv);
        for (int l = 0; l < 2; l++)
            for (int b8 = 0; b8 < 4; b8++) {
                const int r = o->intra ? -1 : m->ref_idx[l][b8];
                o->ref_idx[l][b8] = (int8_t)r;
                o->ref_id[l][b8] = r >= 0 && r < RC_H264_MAX_REFS ? pic->slices[m->slice].ref_id[l][r] : 0xffffffffu;
            }
    }
    return 0;
}

int oracle_h264_recon_motion(int mb_w, int mb_h, const rc_h264_picture *pic,
                             const oracle_h264_colmb *const *col, int slots, oracle_h264_colmb *out_col,
                             const uint8_t *const *ry, const uint8_t *const *ru, const uint8_t *const *rv,
                             uint8_t *y, uint8_t *u, uint8_t *v, int filter) {
    if (!pic || !pic->mbs || !out_col || mb_w <= 0 || mb_h <= 0) return RC_EINVAL;
    const size_t n = (size_t)mb_w * mb_h;
    rc_h264_mb *mbs = (rc_h264_mb *)malloc(n * sizeof(rc_h264_mb));
    if (!mbs) return RC_ENOMEM;
    memcpy(mbs, pic->mbs, n * sizeof(rc_h264_mb));
    rc_h264_picture q = *pic;
    int rc = 0;
    if (pic->motion) {
        rc = oracle_h264_derive_motion(mb_w, mb_h, pic, col, slots, mbs, out_col);
        q.mbs = mbs;
        q.motion = NULL;
        q.slice_motion = NULL;
    } else {
        /* resolved records: their motion is the co-located motion */
        for (size_t a = 0; a < n; a++) {
            const rc_h264_mb *m = &pic->mbs[a];
            oracle_h264_colmb *o = &out_col[a];
            memset(o, 0, sizeof *o);
            o->intra = m->kind != RC_H264_INTER;
            memcpy(o->mv, m->mv, sizeof o->mv);
            for (int l = 0; l < 2; l++)
                for (int b8 = 0; b8 < 4; b8++) {
                    const int r = o->intra ? -1 : m->ref_idx[l][b8];
                    o->ref_idx[l][b8] = (int8_t)r;
                    o->ref_id[l][b8] = r >= 0 && r < RC_H264_MAX_REFS && m->slice < pic->num_slices
                                           ? pic->slices[m->slice].ref_id[l][r]
                                           : 0xffffffffu;
                }
        }
    }
    if (rc == 0)
        rc = filter ? oracle_h264_recon(mb_w, mb_h, &q, ry, ru, rv, y, u, v)
                    : oracle_h264_recon_nofilter(mb_w, mb_h, &q, ry, ru, rv, y, u, v);
    free(mbs);
    return rc;
}
