/*
 * hevc_recon.c — CPU restatement (C11) of pito-codecs' HEVC block
 * reconstruction: dequantisation (flat / scaling lists), 4..32 inverse DCT,
 * 4x4 DST, transform skip, DC-only shortcut, transquant bypass, residual add;
 * intra prediction (z-scan availability, substitution, [1 2 1] and strong
 * smoothing, planar / DC / 33 angular with edge filters); 8-tap / 4-tap
 * motion compensation with i16 intermediates, default and explicit weighted
 * prediction; deblocking (bS, luma strong / normal, chroma) and SAO.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Follows the reference's scalar
 * functions, which its tests pin to the AVX2 path (src/hevc/simd/tests.rs,
 * src/hevc/tests.rs:420-438).  Samples are uint16_t for every bit depth.
 *
 * Whole-picture order: inter prediction of every inter block, then every TU
 * in decode order (intra prediction + residual), then all vertical edges,
 * then all horizontal edges, then SAO from the deblocked picture.  This is
 * the order the reference's row pipeline is equivalent to: intra prediction
 * reads pre-deblock samples (save_bottom, src/hevc/slicedec.rs:1024), edges
 * 8 samples apart do not interact within a direction, and SAO reads
 * deblocked, pre-SAO neighbours (sao_edges, src/hevc/filter.rs:548-552).
 */
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ---- tables: src/hevc/spec_tables.rs, src/hevc/tables.rs --------------- */
static const int8_t TRANS[32][32] = {
#include "hevc_trans_matrix.inc"
};
static const int8_t DST[4][4] = {{29, 55, 74, 84}, {74, 74, 0, -74}, {84, -29, -74, 55}, {55, -84, 74, -29}};
static const int LEVEL_SCALE[6] = {40, 45, 51, 57, 64, 72};
static const int8_t ANGLE[35] = {0,  0,  32, 26, 21, 17, 13, 9,  5,  2,   0,   -2,  -5,  -9,  -13, -17, -21, -26,
                                 -32, -26, -21, -17, -13, -9, -5, -2, 0, 2, 5, 9, 13, 17, 21, 26, 32};
static const int16_t INV_ANGLE[15] = {-4096, -1638, -910, -630, -482, -390, -315, -256,
                                      -315,  -390,  -482, -630, -910, -1638, -4096};
static const uint8_t QPC_30_43[14] = {29, 30, 31, 32, 33, 33, 34, 34, 35, 35, 36, 36, 37, 37};
static const uint8_t BETA_TABLE[52] = {0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  6,  7,
                                       8,  9,  10, 11, 12, 13, 14, 15, 16, 17, 18, 20, 22, 24, 26, 28, 30, 32,
                                       34, 36, 38, 40, 42, 44, 46, 48, 50, 52, 54, 56, 58, 60, 62, 64};
static const uint8_t TC_TABLE[54] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                     2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 5, 5, 6, 6, 7, 8, 9, 10, 11, 13, 14, 16, 18, 20, 22, 24};
static const int8_t LUMA_FILTER[4][8] = {
    {0, 0, 0, 64, 0, 0, 0, 0}, {-1, 4, -10, 58, 17, -5, 1, 0}, {-1, 4, -11, 40, 40, -11, 4, -1}, {0, 1, -5, 17, 58, -10, 4, -1}};
static const int8_t CHROMA_FILTER[8][4] = {{0, 64, 0, 0},    {-2, 58, 10, -2}, {-4, 54, 16, -2}, {-6, 46, 28, -4},
                                           {-4, 36, 36, -4}, {-4, 28, 46, -6}, {-2, 16, 54, -4}, {-2, 10, 58, -2}};

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }
static inline int absi(int v) { return v < 0 ? -v : v; }
static inline int sgn(int v) { return (v > 0) - (v < 0); }

/* qpc_420, src/hevc/tables.rs:6-15 */
static int qpc_420(int q) { return q < 30 ? q : q > 43 ? q - 6 : QPC_30_43[q - 30]; }

typedef struct {
    const rc_hevc_picture *pic;
    int W, H, CW, CH, bd, w4, h4, log2ctb, wctb, hctb;
    uint16_t *pl[3];
    const uint16_t *const *ref[3];
} HCtx;

static int pw_of(const HCtx *c, int comp) { return comp ? c->CW : c->W; }
static int ph_of(const HCtx *c, int comp) { return comp ? c->CH : c->H; }
static const rc_hevc_blk *blk_at(const HCtx *c, int x, int y) { return &c->pic->blk[(y >> 2) * c->w4 + (x >> 2)]; }
static int ctb_of(const HCtx *c, int x, int y) { return (y >> c->log2ctb) * c->wctb + (x >> c->log2ctb); }
static uint32_t slice_addr_of_ctb(const HCtx *c, int ctb) { return c->pic->slices[c->pic->ctbs[ctb].slice].slice_addr; }

/* ---- a17-a20: dequant and inverse transforms, src/hevc/transform.rs ---- */
/* dequant, transform.rs:84-108 */
static void dequant(int16_t *co, int n, int max_x, int max_y, const uint8_t *m, int64_t scale, int64_t round,
                    int bd_shift) {
    for (int y = 0; y <= max_y; y++)
        for (int x = 0; x <= max_x; x++) {
            int v = co[y * n + x];
            if (!v) continue;
            int64_t f = m ? m[y * n + x] : 16;
            int64_t r = ((int64_t)v * f * scale + round) >> bd_shift;
            co[y * n + x] = (int16_t)(r < -32768 ? -32768 : r > 32767 ? 32767 : r);
        }
}

/* inverse::<N>, transform.rs:26-66: columns (+64 >> 7, clamp), then rows */
static void inverse(int16_t *co, int n, int dst, int max_x, int max_y, int bd_shift) {
    int32_t col[32][32];
    int step = 32 / n;
    int mx = max_x < n - 1 ? max_x : n - 1, my = max_y < n - 1 ? max_y : n - 1;
    memset(col, 0, sizeof col);
    for (int x = 0; x <= mx; x++) {
        int32_t *acc = col[x];
        for (int j = 0; j <= my; j++) {
            int d = co[j * n + x];
            if (!d) continue;
            for (int i = 0; i < n; i++) acc[i] += (dst ? DST[j][i] : TRANS[j * step][i]) * d;
        }
        for (int i = 0; i < n; i++) acc[i] = clampi((acc[i] + 64) >> 7, -32768, 32767);
    }
    int round = 1 << (bd_shift - 1);
    for (int y = 0; y < n; y++) {
        int32_t out[32];
        for (int i = 0; i < n; i++) out[i] = round;
        for (int j = 0; j <= mx; j++) {
            int g = col[j][y];
            if (!g) continue;
            for (int i = 0; i < n; i++) out[i] += (dst ? DST[j][i] : TRANS[j * step][i]) * g;
        }
        for (int i = 0; i < n; i++) co[y * n + i] = (int16_t)clampi(out[i] >> bd_shift, -32768, 32767);
    }
}

/* inverse_dc, transform.rs:68-71 */
static int inverse_dc(int dc, int bd_shift) {
    int e = clampi((64 * dc + 64) >> 7, -32768, 32767);
    return (64 * e + (1 << (bd_shift - 1))) >> bd_shift;
}

/* transform_skip, transform.rs:73-81 */
static void transform_skip(int16_t *co, int n, int log2, int bd_shift) {
    int ts_shift = 5 + log2, round = 1 << (bd_shift - 1);
    for (int i = 0; i < n * n; i++) co[i] = (int16_t)clampi((((int)co[i] << ts_shift) + round) >> bd_shift, -32768, 32767);
}

static const uint8_t *scaling_table(const rc_hevc_picture *p, int size_id, int matrix_id) {
    static const int off[4] = {0, 6 * 16, 6 * (16 + 64), 6 * (16 + 64 + 256)};
    static const int sz[4] = {16, 64, 256, 1024};
    return p->scaling + off[size_id] + matrix_id * sz[size_id];
}

/* reconstruct, src/hevc/slicedec.rs:2004-2049, into residual r[n*n] */
static void residual_of(const HCtx *c, const rc_hevc_tu *t, int16_t *co) {
    int n = 1 << t->log2, log2 = t->log2;
    int bd = c->bd;
    int intra = t->flags & RC_HEVC_TU_INTRA, ts = (t->flags & RC_HEVC_TU_SKIP) != 0;
    memset(co, 0, sizeof(int16_t) * n * n);
    const int16_t *lv = c->pic->levels + t->coef_off;
    for (int y = 0; y <= t->max_y; y++)
        for (int x = 0; x <= t->max_x; x++) co[y * n + x] = lv[y * (t->max_x + 1) + x];
    if (t->flags & RC_HEVC_TU_BYPASS) return;
    int qp = t->qp;
    int bd_shift = bd + log2 - 5;
    int64_t round = (int64_t)1 << (bd_shift - 1);
    int64_t scale = (int64_t)LEVEL_SCALE[qp % 6] << (qp / 6);
    const uint8_t *m = NULL;
    if (c->pic->scaling && !(ts && n > 4)) m = scaling_table(c->pic, log2 - 2, intra ? t->c : 3 + t->c);
    dequant(co, n, t->max_x, t->max_y, m, scale, round, bd_shift);
    int bs2 = 20 - bd;
    if (ts) transform_skip(co, n, log2, bs2);
    else if (t->max_x == 0 && t->max_y == 0 && !(intra && t->c == 0 && n == 4)) {
        int v = clampi(inverse_dc(co[0], bs2), -32768, 32767);
        for (int i = 0; i < n * n; i++) co[i] = (int16_t)v;
    } else inverse(co, n, intra && t->c == 0 && n == 4, t->max_x, t->max_y, bs2);
}

/* ---- a21: intra prediction ------------------------------------------- */
static uint32_t morton(uint32_t x, uint32_t y) {
    uint32_t r = 0;
    for (int i = 0; i < 16; i++) r |= ((x >> i) & 1u) << (2 * i) | ((y >> i) & 1u) << (2 * i + 1);
    return r;
}

/* zavail, src/hevc/slicedec.rs:625-643 (luma coordinates) */
static int zavail(const HCtx *c, int xc, int yc, int xn, int yn) {
    if (xn < 0 || yn < 0 || xn >= c->W || yn >= c->H) return 0;
    int s = c->log2ctb;
    int cn = (yn >> s) * c->wctb + (xn >> s), cc = (yc >> s) * c->wctb + (xc >> s);
    if (cn != cc) {
        const rc_hevc_ctb *n = &c->pic->ctbs[cn], *q = &c->pic->ctbs[cc];
        return n->ts < q->ts && slice_addr_of_ctb(c, cn) == slice_addr_of_ctb(c, cc) && n->tile == q->tile;
    }
    int m = (1 << s) - 1;
    return morton((xn & m) >> 2, (yn & m) >> 2) <= morton((xc & m) >> 2, (yc & m) >> 2);
}

typedef struct { uint16_t left[129], top[129]; } Refs;

/* substitute, src/hevc/intra.rs:19-65 */
static void substitute(Refs *r, const uint8_t *al, const uint8_t *at, int n, int bd) {
    int n2 = 2 * n, any = 0;
    for (int i = 0; i <= n2; i++) any |= al[i];
    for (int i = 1; i <= n2; i++) any |= at[i];
    if (!any) {
        for (int i = 0; i <= n2; i++) r->left[i] = r->top[i] = (uint16_t)(1 << (bd - 1));
        return;
    }
    if (!al[n2]) {
        int found = -1;
        for (int y = n2 - 1; y >= 0 && found < 0; y--)
            if (al[y]) found = r->left[y];
        for (int x = 1; x <= n2 && found < 0; x++)
            if (at[x]) found = r->top[x];
        r->left[n2] = (uint16_t)(found < 0 ? 0 : found);
    }
    for (int y = n2 - 1; y >= 0; y--)
        if (!al[y]) r->left[y] = r->left[y + 1];
    r->top[0] = r->left[0];
    for (int x = 1; x <= n2; x++)
        if (!at[x]) r->top[x] = r->top[x - 1];
}

/* filter, src/hevc/intra.rs:67-111 */
static void filter_refs(Refs *r, int mode, int n, int strong_enabled, int is_luma, int bd) {
    if (mode == 1 || n == 4) return;
    int md = absi(mode - 26) < absi(mode - 10) ? absi(mode - 26) : absi(mode - 10);
    int thres = n == 8 ? 7 : n == 16 ? 1 : 0;
    if (md <= thres) return;
    int n2 = 2 * n, cc = r->left[0];
    if (strong_enabled && is_luma && n == 32) {
        int bl = r->left[n2], tr = r->top[n2], thr = 1 << (bd - 5);
        if (absi(cc + tr - 2 * r->top[n]) < thr && absi(cc + bl - 2 * r->left[n]) < thr) {
            for (int i = 0; i < 63; i++) {
                r->left[1 + i] = (uint16_t)(((63 - i) * cc + (i + 1) * bl + 32) >> 6);
                r->top[1 + i] = (uint16_t)(((63 - i) * cc + (i + 1) * tr + 32) >> 6);
            }
            return;
        }
    }
    Refs o = *r;
    uint16_t corner = (uint16_t)((o.left[1] + 2 * cc + o.top[1] + 2) >> 2);
    for (int i = 1; i < n2; i++) {
        r->left[i] = (uint16_t)((o.left[i - 1] + 2 * o.left[i] + o.left[i + 1] + 2) >> 2);
        r->top[i] = (uint16_t)((o.top[i - 1] + 2 * o.top[i] + o.top[i + 1] + 2) >> 2);
    }
    r->left[0] = r->top[0] = corner;
}

/* predict, src/hevc/intra.rs:113-222 (into pred[n*n]) */
static void predict(const Refs *r, int mode, int n, int edge_filters, int bd, int *out) {
    int max = (1 << bd) - 1, log2 = 0;
    while ((1 << log2) < n) log2++;
    if (mode == 0) {
        int tr = r->top[1 + n], bl = r->left[1 + n];
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++)
                out[y * n + x] = ((n - 1 - x) * r->left[1 + y] + (x + 1) * tr + (n - 1 - y) * r->top[1 + x] + (y + 1) * bl + n) >> (log2 + 1);
        return;
    }
    if (mode == 1) {
        uint32_t sum = 0;
        for (int i = 1; i <= n; i++) sum += r->top[i] + r->left[i];
        int dc = (int)((sum + n) >> (log2 + 1));
        for (int i = 0; i < n * n; i++) out[i] = dc;
        if (edge_filters && n < 32) {
            out[0] = (r->left[1] + 2 * dc + r->top[1] + 2) >> 2;
            for (int x = 1; x < n; x++) out[x] = (r->top[1 + x] + 3 * dc + 2) >> 2;
            for (int y = 1; y < n; y++) out[y * n] = (r->left[1 + y] + 3 * dc + 2) >> 2;
        }
        return;
    }
    int angle = ANGLE[mode], refa[3 * 64 + 1], base = n;
    memset(refa, 0, sizeof refa);
    const uint16_t *main_ = mode >= 18 ? r->top : r->left, *side = mode >= 18 ? r->left : r->top;
    for (int x = 0; x <= n; x++) refa[base + x] = main_[x];
    if (angle < 0) {
        int lim = (n * angle) >> 5;
        if (lim < -1) {
            int inv = INV_ANGLE[mode - 11];
            for (int x = lim; x <= -1; x++) refa[base + x] = side[-1 + ((x * inv + 128) >> 8) + 1];
        }
    } else
        for (int x = n + 1; x <= 2 * n; x++) refa[base + x] = main_[x];
    int horizontal = mode < 18;
    for (int j = 0; j < n; j++) {
        int pos = (j + 1) * angle, idx = pos >> 5, fact = pos & 31;
        for (int i = 0; i < n; i++) {
            int k = base + i + idx + 1;
            int v = fact ? ((32 - fact) * refa[k] + fact * refa[k + 1] + 16) >> 5 : refa[k];
            if (horizontal) out[i * n + j] = v;
            else out[j * n + i] = v;
        }
    }
    if (edge_filters && n < 32) {
        if (mode == 26)
            for (int y = 0; y < n; y++) out[y * n] = clampi(r->top[1] + ((r->left[1 + y] - r->left[0]) >> 1), 0, max);
        else if (mode == 10)
            for (int x = 0; x < n; x++) out[x] = clampi(r->left[1] + ((r->top[1 + x] - r->top[0]) >> 1), 0, max);
    }
}

/* intra_predict, src/hevc/slicedec.rs:1673-1738 (whole-picture plane as
 * the pre-deblock source), writing the prediction into pred[n*n] */
static void intra_predict(const HCtx *c, int x0, int y0, int log2, int comp, int mode, int *pred) {
    int n = 1 << log2, sc = comp ? 2 : 1, xl = x0 * sc, yl = y0 * sc, unit = 4 / sc;
    int stride = pw_of(c, comp);
    const uint16_t *pl = c->pl[comp];
    uint8_t al[129], at[129];
    Refs r;
    memset(al, 0, sizeof al);
    memset(at, 0, sizeof at);
    memset(&r, 0, sizeof r);
#define AV(xn, yn) (zavail(c, xl, yl, (xn), (yn)) && (!c->pic->constrained_intra_pred || (blk_at(c, (xn), (yn))->flags & RC_HEVC_F_INTRA)))
    if (AV(xl - 1, yl - 1)) {
        al[0] = at[0] = 1;
        r.left[0] = r.top[0] = pl[(y0 - 1) * stride + x0 - 1];
    }
    for (int k = 0; k < 2 * n; k += unit) {
        int yn = y0 + k;
        if (AV(xl - 1, yn * sc))
            for (int i = 0; i < unit; i++) {
                al[1 + k + i] = 1;
                r.left[1 + k + i] = pl[(yn + i) * stride + x0 - 1];
            }
        int xn = x0 + k;
        if (AV(xn * sc, yl - 1))
            for (int i = 0; i < unit; i++) {
                at[1 + k + i] = 1;
                r.top[1 + k + i] = pl[(y0 - 1) * stride + xn + i];
            }
    }
#undef AV
    substitute(&r, al, at, n, c->bd);
    if (comp == 0) filter_refs(&r, mode, n, c->pic->strong_intra_smoothing, 1, c->bd);
    predict(&r, mode, n, comp == 0, c->bd, pred);
}

/* ---- a22-a24: inter prediction, src/hevc/inter.rs -------------------- */
static inline int rsamp(const HCtx *c, int comp, const uint16_t *p, int x, int y) {
    return p[clampi(y, 0, ph_of(c, comp) - 1) * pw_of(c, comp) + clampi(x, 0, pw_of(c, comp) - 1)];
}

/* interpolate, inter.rs:86-133, for one sample: window origin (x0w, y0w),
 * T taps; returns the i16 intermediate prediction */
static int interp_sample(const HCtx *c, int comp, const uint16_t *p, int xi, int yi, int fx, int fy) {
    int T = comp ? 4 : 8, m = T / 2 - 1, bd = c->bd;
    int shift1 = (bd < 12 ? bd : 12) - 8, shift3 = 14 - bd;
    const int8_t *hf = comp ? CHROMA_FILTER[fx] : LUMA_FILTER[fx];
    const int8_t *vf = comp ? CHROMA_FILTER[fy] : LUMA_FILTER[fy];
    if (fx == 0 && fy == 0) return (int16_t)(rsamp(c, comp, p, xi, yi) << shift3);
    if (fy == 0) {
        int s = 0;
        for (int k = 0; k < T; k++) s += hf[k] * rsamp(c, comp, p, xi - m + k, yi);
        return (int16_t)(s >> shift1);
    }
    if (fx == 0) {
        int s = 0;
        for (int k = 0; k < T; k++) s += vf[k] * rsamp(c, comp, p, xi, yi - m + k);
        return (int16_t)(s >> shift1);
    }
    int v = 0;
    for (int r = 0; r < T; r++) {
        int s = 0;
        for (int k = 0; k < T; k++) s += hf[k] * rsamp(c, comp, p, xi - m + k, yi - m + r);
        v += vf[r] * (int16_t)(s >> shift1);
    }
    return (int16_t)(v >> 6);
}

/* motion_compensate + put_*, src/hevc/slicedec.rs:2205-2280, inter.rs:207-301,
 * for sample (x, y) of component comp in an inter block */
static int mc_sample(const HCtx *c, int comp, int x, int y, const rc_hevc_mvf *f, const rc_hevc_slice *sl) {
    int bd = c->bd, max = (1 << bd) - 1, pv[2] = {0, 0}, use[2];
    for (int l = 0; l < 2; l++) {
        use[l] = f->ref_idx[l] >= 0;
        if (!use[l]) continue;
        int slot = sl->ref_slot[l][f->ref_idx[l]];
        const uint16_t *p = c->ref[comp][slot];
        int mvx = f->mv[l][0], mvy = f->mv[l][1];
        if (comp == 0) pv[l] = interp_sample(c, 0, p, x + (mvx >> 2), y + (mvy >> 2), mvx & 3, mvy & 3);
        else pv[l] = interp_sample(c, comp, p, x + (mvx >> 3), y + (mvy >> 3), mvx & 7, mvy & 7);
    }
    int bi = use[0] && use[1];
    if (!sl->weighted) {
        if (bi) {
            int shift = 15 - bd;
            return clampi((pv[0] + pv[1] + (1 << (shift - 1))) >> shift, 0, max);
        }
        int shift = 14 - bd, off = shift > 0 ? 1 << (shift - 1) : 0;
        return clampi((pv[use[0] ? 0 : 1] + off) >> shift, 0, max);
    }
    int log2wd = (comp ? sl->chroma_log2_denom : sl->luma_log2_denom) + 14 - bd;
    int w[2], o[2];
    for (int l = 0; l < 2; l++) {
        if (!use[l]) { w[l] = o[l] = 0; continue; }
        int ri = f->ref_idx[l];
        w[l] = comp ? sl->chroma_w[l][ri][comp - 1] : sl->luma_w[l][ri];
        o[l] = (comp ? sl->chroma_o[l][ri][comp - 1] : sl->luma_o[l][ri]) * (1 << (bd - 8));
    }
    if (bi) return clampi((pv[0] * w[0] + pv[1] * w[1] + ((o[0] + o[1] + 1) << log2wd)) >> (log2wd + 1), 0, max);
    int l = use[0] ? 0 : 1, v = pv[l] * w[l];
    v = log2wd >= 1 ? ((v + (1 << (log2wd - 1))) >> log2wd) + o[l] : v + o[l];
    return clampi(v, 0, max);
}

/* ---- a26-a27: deblocking, src/hevc/filter.rs:75-519 ------------------- */
static uint32_t h_ref_id(const HCtx *c, int ctb, const rc_hevc_mvf *f, int l) {
    const rc_hevc_slice *sl = &c->pic->slices[c->pic->ctbs[ctb].slice];
    int r = f->ref_idx[l];
    return (r >= 0 && r < sl->num_ref[l]) ? sl->ref_id[l][r] : 0xfffffffeu;
}
static int far_mv(const int16_t a[2], const int16_t b[2]) { return absi(a[0] - b[0]) >= 4 || absi(a[1] - b[1]) >= 4; }

/* motion_bs, filter.rs:112-144 */
static int motion_bs(const HCtx *c, int pctb, const rc_hevc_mvf *p, int qctb, const rc_hevc_mvf *q) {
    int np = (p->ref_idx[0] >= 0) + (p->ref_idx[1] >= 0), nq = (q->ref_idx[0] >= 0) + (q->ref_idx[1] >= 0);
    if (np != nq) return 1;
    if (np == 1) {
        int lp = p->ref_idx[0] >= 0 ? 0 : 1, lq = q->ref_idx[0] >= 0 ? 0 : 1;
        if (h_ref_id(c, pctb, p, lp) != h_ref_id(c, qctb, q, lq)) return 1;
        return far_mv(p->mv[lp], q->mv[lq]);
    }
    uint32_t p0 = h_ref_id(c, pctb, p, 0), p1 = h_ref_id(c, pctb, p, 1);
    uint32_t q0 = h_ref_id(c, qctb, q, 0), q1 = h_ref_id(c, qctb, q, 1);
    if (!((p0 == q0 && p1 == q1) || (p0 == q1 && p1 == q0))) return 1;
    if (p0 != p1) {
        if (p0 == q0) return far_mv(p->mv[0], q->mv[0]) || far_mv(p->mv[1], q->mv[1]);
        return far_mv(p->mv[0], q->mv[1]) || far_mv(p->mv[1], q->mv[0]);
    }
    return (far_mv(p->mv[0], q->mv[0]) || far_mv(p->mv[1], q->mv[1])) &&
           (far_mv(p->mv[0], q->mv[1]) || far_mv(p->mv[1], q->mv[0]));
}

/* boundary_strength, filter.rs:84-100 (p, q: 4x4 block indices) */
static int boundary_strength(const HCtx *c, int pi, int qi, int tu_edge, int pctb, int qctb) {
    const rc_hevc_blk *p = &c->pic->blk[pi], *q = &c->pic->blk[qi];
    if ((p->flags | q->flags) & RC_HEVC_F_INTRA) return 2;
    if (tu_edge && ((p->flags | q->flags) & RC_HEVC_F_CBF)) return 1;
    return motion_bs(c, pctb, &c->pic->mvf[pi], qctb, &c->pic->mvf[qi]);
}

/* edge_params, filter.rs:146-176: 0 = edge not filtered */
static int edge_params(const HCtx *c, int px, int py, int qx, int qy, int *tc_off, int *beta_off) {
    int pc = ctb_of(c, px, py), qc = ctb_of(c, qx, qy);
    const rc_hevc_slice *sq = &c->pic->slices[c->pic->ctbs[qc].slice];
    if (sq->deblock_disabled) return 0;
    if (pc != qc) {
        if (slice_addr_of_ctb(c, pc) != slice_addr_of_ctb(c, qc) && !sq->lf_across) return 0;
        if (!c->pic->loop_filter_across_tiles && c->pic->ctbs[pc].tile != c->pic->ctbs[qc].tile) return 0;
    }
    *tc_off = sq->tc_offset;
    *beta_off = sq->beta_offset;
    return 1;
}

/* tc_beta, filter.rs:74-82 */
static void tc_beta(int q, int bs, int tc_off, int beta_off, int bd, int *tc, int *beta) {
    int qb = clampi(q + beta_off, 0, 51), qt = clampi(q + 2 * (bs - 1) + tc_off, 0, 53);
    *tc = TC_TABLE[qt] << (bd - 8);
    *beta = BETA_TABLE[qb] << (bd - 8);
}

/* filter_luma, filter.rs:409-492: o = q0 of line 0, step across the edge,
 * along = between lines */
static void filter_luma(uint16_t *s, long o, long step, long along, int tc, int beta, int nfp, int nfq, int bd) {
#define PX(k, i) ((int)s[o + (k) * along - ((i) + 1) * step])
#define QX(k, i) ((int)s[o + (k) * along + (i) * step])
    int dp0 = absi(PX(0, 2) - 2 * PX(0, 1) + PX(0, 0)), dp3 = absi(PX(3, 2) - 2 * PX(3, 1) + PX(3, 0));
    int dq0 = absi(QX(0, 2) - 2 * QX(0, 1) + QX(0, 0)), dq3 = absi(QX(3, 2) - 2 * QX(3, 1) + QX(3, 0));
    int dpq0 = dp0 + dq0, dpq3 = dp3 + dq3, dp = dp0 + dp3, dq = dq0 + dq3, d = dpq0 + dpq3;
    if (d >= beta) return;
#define DSAM(k, dpq) ((dpq) < (beta >> 2) && absi(PX(k, 3) - PX(k, 0)) + absi(QX(k, 0) - QX(k, 3)) < (beta >> 3) && absi(PX(k, 0) - QX(k, 0)) < ((5 * tc + 1) >> 1))
    int strong = DSAM(0, 2 * dpq0) && DSAM(3, 2 * dpq3);
#undef DSAM
    int dep = dp < ((beta + (beta >> 1)) >> 3), deq = dq < ((beta + (beta >> 1)) >> 3);
    int max = (1 << bd) - 1;
    for (int k = 0; k < 4; k++) {
        long b = o + k * along;
        int p0 = s[b - step], p1 = s[b - 2 * step], p2 = s[b - 3 * step], p3 = s[b - 4 * step];
        int q0 = s[b], q1 = s[b + step], q2 = s[b + 2 * step], q3 = s[b + 3 * step];
        if (strong) {
            int t2 = 2 * tc;
            if (!nfp) {
                s[b - step] = (uint16_t)clampi((p2 + 2 * p1 + 2 * p0 + 2 * q0 + q1 + 4) >> 3, p0 - t2, p0 + t2);
                s[b - 2 * step] = (uint16_t)clampi((p2 + p1 + p0 + q0 + 2) >> 2, p1 - t2, p1 + t2);
                s[b - 3 * step] = (uint16_t)clampi((2 * p3 + 3 * p2 + p1 + p0 + q0 + 4) >> 3, p2 - t2, p2 + t2);
            }
            if (!nfq) {
                s[b] = (uint16_t)clampi((p1 + 2 * p0 + 2 * q0 + 2 * q1 + q2 + 4) >> 3, q0 - t2, q0 + t2);
                s[b + step] = (uint16_t)clampi((p0 + q0 + q1 + q2 + 2) >> 2, q1 - t2, q1 + t2);
                s[b + 2 * step] = (uint16_t)clampi((p0 + q0 + q1 + 3 * q2 + 2 * q3 + 4) >> 3, q2 - t2, q2 + t2);
            }
        } else {
            int delta = (9 * (q0 - p0) - 3 * (q1 - p1) + 8) >> 4;
            if (absi(delta) >= tc * 10) continue;
            delta = clampi(delta, -tc, tc);
            if (!nfp) s[b - step] = (uint16_t)clampi(p0 + delta, 0, max);
            if (!nfq) s[b] = (uint16_t)clampi(q0 - delta, 0, max);
            if (dep && !nfp) {
                int dpv = clampi((((p2 + p0 + 1) >> 1) - p1 + delta) >> 1, -(tc >> 1), tc >> 1);
                s[b - 2 * step] = (uint16_t)clampi(p1 + dpv, 0, max);
            }
            if (deq && !nfq) {
                int dqv = clampi((((q2 + q0 + 1) >> 1) - q1 - delta) >> 1, -(tc >> 1), tc >> 1);
                s[b + step] = (uint16_t)clampi(q1 + dqv, 0, max);
            }
        }
    }
#undef PX
#undef QX
}

/* filter_chroma, filter.rs:494-519 */
static void filter_chroma(uint16_t *s, long o, long step, long along, int tc, int nfp, int nfq, int bd) {
    int max = (1 << bd) - 1;
    for (int k = 0; k < 4; k++) {
        long b = o + k * along;
        int p0 = s[b - step], p1 = s[b - 2 * step], q0 = s[b], q1 = s[b + step];
        int delta = clampi((((q0 - p0) << 2) + p1 - q1 + 4) >> 3, -tc, tc);
        if (!nfp) s[b - step] = (uint16_t)clampi(p0 + delta, 0, max);
        if (!nfq) s[b] = (uint16_t)clampi(q0 - delta, 0, max);
    }
}

/* deblock_row, filter.rs:243-406, picture-wide: all vertical edges
 * (luma, then chroma), then all horizontal edges (luma, then chroma) */
static void deblock(HCtx *c) {
    int w4 = c->w4, h4 = c->h4, bd = c->bd, W = c->W, CW = c->CW;
    int8_t *bsv = (int8_t *)calloc((size_t)w4 * h4, 1), *bsh = (int8_t *)calloc((size_t)w4 * h4, 1);
    const rc_hevc_blk *B = c->pic->blk;
    for (int by = 0; by < h4; by++)
        for (int bx = 2; bx < w4; bx += 2) {
            int qi = by * w4 + bx, x = bx * 4, y = by * 4;
            const rc_hevc_blk *q = &B[qi];
            if (!(q->edges & (RC_HEVC_E_TU_V | RC_HEVC_E_PU_V)) || !(q->flags & RC_HEVC_F_CODED)) continue;
            int tco, bo;
            if (!edge_params(c, x - 1, y, x, y, &tco, &bo)) continue;
            int bs = boundary_strength(c, qi - 1, qi, (q->edges & RC_HEVC_E_TU_V) != 0, ctb_of(c, x - 1, y), ctb_of(c, x, y));
            bsv[qi] = (int8_t)bs;
            if (!bs) continue;
            const rc_hevc_blk *p = &B[qi - 1];
            int tc, beta;
            tc_beta((p->qp + q->qp + 1) >> 1, bs, tco, bo, bd, &tc, &beta);
            filter_luma(c->pl[0], (long)y * W + x, 1, W, tc, beta, (p->flags & RC_HEVC_F_NOFILTER) != 0,
                        (q->flags & RC_HEVC_F_NOFILTER) != 0, bd);
        }
    for (int by = 0; by < h4; by += 2)
        for (int bx = 4; bx < w4; bx += 4) {
            int qi = by * w4 + bx, x = bx * 4, y = by * 4;
            if (bsv[qi] != 2) continue;
            int tco, bo;
            if (!edge_params(c, x - 1, y, x, y, &tco, &bo)) continue;
            const rc_hevc_blk *p = &B[qi - 1], *q = &B[qi];
            for (int k = 1; k < 3; k++) {
                int qpi = ((p->qp + q->qp + 1) >> 1) + (k == 1 ? c->pic->cb_qp_offset : c->pic->cr_qp_offset);
                int qt = clampi(qpc_420(qpi) + 2 + tco, 0, 53), tc = TC_TABLE[qt] << (bd - 8);
                filter_chroma(c->pl[k], (long)(y / 2) * CW + x / 2, 1, CW, tc, (p->flags & RC_HEVC_F_NOFILTER) != 0,
                              (q->flags & RC_HEVC_F_NOFILTER) != 0, bd);
            }
        }
    for (int by = 2; by < h4; by += 2)
        for (int bx = 0; bx < w4; bx++) {
            int qi = by * w4 + bx, x = bx * 4, y = by * 4;
            const rc_hevc_blk *q = &B[qi];
            if (!(q->edges & (RC_HEVC_E_TU_H | RC_HEVC_E_PU_H)) || !(q->flags & RC_HEVC_F_CODED)) continue;
            int tco, bo;
            if (!edge_params(c, x, y - 1, x, y, &tco, &bo)) continue;
            int pi = qi - w4;
            int bs = boundary_strength(c, pi, qi, (q->edges & RC_HEVC_E_TU_H) != 0, ctb_of(c, x, y - 1), ctb_of(c, x, y));
            bsh[qi] = (int8_t)bs;
            if (!bs) continue;
            const rc_hevc_blk *p = &B[pi];
            int tc, beta;
            tc_beta((p->qp + q->qp + 1) >> 1, bs, tco, bo, bd, &tc, &beta);
            filter_luma(c->pl[0], (long)y * W + x, W, 1, tc, beta, (p->flags & RC_HEVC_F_NOFILTER) != 0,
                        (q->flags & RC_HEVC_F_NOFILTER) != 0, bd);
        }
    for (int by = 4; by < h4; by += 4)
        for (int bx = 0; bx < w4; bx += 2) {
            int qi = by * w4 + bx, x = bx * 4, y = by * 4;
            if (bsh[qi] != 2) continue;
            int tco, bo;
            if (!edge_params(c, x, y - 1, x, y, &tco, &bo)) continue;
            const rc_hevc_blk *p = &B[qi - w4], *q = &B[qi];
            for (int k = 1; k < 3; k++) {
                int qpi = ((p->qp + q->qp + 1) >> 1) + (k == 1 ? c->pic->cb_qp_offset : c->pic->cr_qp_offset);
                int qt = clampi(qpc_420(qpi) + 2 + tco, 0, 53), tc = TC_TABLE[qt] << (bd - 8);
                filter_chroma(c->pl[k], (long)(y / 2) * CW + x / 2, CW, 1, tc, (p->flags & RC_HEVC_F_NOFILTER) != 0,
                              (q->flags & RC_HEVC_F_NOFILTER) != 0, bd);
            }
        }
    free(bsv);
    free(bsh);
}

/* ---- a28: SAO, src/hevc/filter.rs:521-894 ----------------------------- */
/* cross_ok, filter.rs:605-632 */
static int cross_ok(const HCtx *c, int comp, int rs, int xn, int yn) {
    int s = c->log2ctb - (comp ? 1 : 0);
    int nrs = (yn >> s) * c->wctb + (xn >> s);
    if (nrs == rs) return 1;
    const rc_hevc_ctb *n = &c->pic->ctbs[nrs], *q = &c->pic->ctbs[rs];
    if (n->slice >= c->pic->num_slices) return 0;
    if (slice_addr_of_ctb(c, nrs) != slice_addr_of_ctb(c, rs)) {
        if (n->ts < q->ts && !c->pic->slices[q->slice].lf_across) return 0;
        if (q->ts < n->ts && !c->pic->slices[n->slice].lf_across) return 0;
    }
    return c->pic->loop_filter_across_tiles || n->tile == q->tile;
}

static void sao(HCtx *c, uint16_t *const src[3]) {
    static const int HP[4][2] = {{-1, 1}, {0, 0}, {-1, 1}, {1, -1}}, VP[4][2] = {{0, 0}, {-1, 1}, {-1, 1}, {-1, 1}};
    for (int rs = 0; rs < c->wctb * c->hctb; rs++) {
        const rc_hevc_ctb *ct = &c->pic->ctbs[rs];
        const rc_hevc_slice *sl = &c->pic->slices[ct->slice];
        int rx = rs % c->wctb, ry = rs / c->wctb;
        for (int comp = 0; comp < 3; comp++) {
            if (!(comp ? sl->sao_chroma : sl->sao_luma) || ct->sao.type_idx[comp] == 0) continue;
            int cs = (1 << c->log2ctb) >> (comp ? 1 : 0), w = pw_of(c, comp), h = ph_of(c, comp);
            int x0 = rx * cs, y0 = ry * cs, x1 = x0 + cs < w ? x0 + cs : w, y1 = y0 + cs < h ? y0 + cs : h;
            int bd = c->bd, max = (1 << bd) - 1, sc = comp ? 1 : 0;
            const int16_t *offs = ct->sao.offsets[comp];
            const uint16_t *in = src[comp];
            uint16_t *out = c->pl[comp];
            int near[3][3];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    int xn = j == 0 ? x0 - 1 : j == 1 ? x0 : x1, yn = i == 0 ? y0 - 1 : i == 1 ? y0 : y1;
                    near[i][j] = xn >= 0 && yn >= 0 && yn < h && xn < w && cross_ok(c, comp, rs, xn, yn);
                }
            for (int y = y0; y < y1; y++)
                for (int x = x0; x < x1; x++) {
                    if (c->pic->blk[((y << sc) >> 2) * c->w4 + ((x << sc) >> 2)].flags & RC_HEVC_F_NOFILTER) continue;
                    int v = in[y * w + x];
                    if (ct->sao.type_idx[comp] == 1) {
                        int table[32] = {0};
                        for (int j = 0; j < 4; j++) table[(j + ct->sao.band_pos[comp]) & 31] = offs[j];
                        out[y * w + x] = (uint16_t)clampi(v + table[v >> (bd - 5)], 0, max);
                        continue;
                    }
                    int cls = ct->sao.eo_class[comp] & 3, sum = 0, ok = 1;
                    for (int j = 0; j < 2 && ok; j++) {
                        int xn = x + HP[cls][j], yn = y + VP[cls][j];
                        if (xn < 0 || yn < 0 || xn >= w || yn >= h) { ok = 0; break; }
                        int ni = yn < y0 ? 0 : yn >= y1 ? 2 : 1, nj = xn < x0 ? 0 : xn >= x1 ? 2 : 1;
                        if (!near[ni][nj]) { ok = 0; break; }
                        sum += sgn(v - in[yn * w + xn]);
                    }
                    if (!ok) continue;
                    static const int edge_map[5] = {1, 2, 0, 3, 4};
                    int e = edge_map[2 + sum];
                    out[y * w + x] = (uint16_t)clampi(v + (e ? offs[e - 1] : 0), 0, max);
                }
        }
    }
}

/* ---- driver ----------------------------------------------------------- */
int oracle_hevc_recon(int width, int height, int bit_depth, const rc_hevc_picture *pic,
                      const uint16_t *const *ref_y, const uint16_t *const *ref_u, const uint16_t *const *ref_v,
                      uint16_t *y, uint16_t *u, uint16_t *v, int stages) {
    if (!pic || width <= 0 || height <= 0 || (width & 7) || (height & 7) || (bit_depth != 8 && bit_depth != 10))
        return RC_EINVAL;
    HCtx c;
    memset(&c, 0, sizeof c);
    c.pic = pic;
    c.W = width; c.H = height; c.CW = width / 2; c.CH = height / 2;
    c.bd = bit_depth; c.w4 = width / 4; c.h4 = height / 4;
    c.log2ctb = pic->log2_ctb;
    c.wctb = (width + (1 << c.log2ctb) - 1) >> c.log2ctb;
    c.hctb = (height + (1 << c.log2ctb) - 1) >> c.log2ctb;
    c.pl[0] = y; c.pl[1] = u; c.pl[2] = v;
    c.ref[0] = ref_y; c.ref[1] = ref_u; c.ref[2] = ref_v;
    /* inter prediction of every inter block */
    for (int by = 0; by < c.h4; by++)
        for (int bx = 0; bx < c.w4; bx++) {
            const rc_hevc_blk *b = &pic->blk[by * c.w4 + bx];
            if (!(b->flags & RC_HEVC_F_CODED) || (b->flags & RC_HEVC_F_INTRA)) continue;
            const rc_hevc_mvf *f = &pic->mvf[by * c.w4 + bx];
            const rc_hevc_slice *sl = &pic->slices[pic->ctbs[ctb_of(&c, bx * 4, by * 4)].slice];
            for (int yy = 0; yy < 4; yy++)
                for (int xx = 0; xx < 4; xx++)
                    y[(by * 4 + yy) * c.W + bx * 4 + xx] = (uint16_t)mc_sample(&c, 0, bx * 4 + xx, by * 4 + yy, f, sl);
            for (int k = 1; k < 3; k++)
                for (int yy = 0; yy < 2; yy++)
                    for (int xx = 0; xx < 2; xx++) {
                        int cx = bx * 2 + xx, cy = by * 2 + yy;
                        c.pl[k][cy * c.CW + cx] = (uint16_t)mc_sample(&c, k, cx, cy, f, sl);
                    }
        }
    /* TUs in decode order */
    int16_t co[1024];
    int pred[1024];
    for (int i = 0; i < pic->num_tus; i++) {
        const rc_hevc_tu *t = &pic->tus[i];
        int n = 1 << t->log2, w = pw_of(&c, t->c), max = (1 << c.bd) - 1;
        uint16_t *pl = c.pl[t->c];
        if (t->flags & RC_HEVC_TU_PCM) {
            const int16_t *s = pic->levels + t->coef_off;
            for (int yy = 0; yy < n; yy++)
                for (int xx = 0; xx < n; xx++) pl[(t->y0 + yy) * w + t->x0 + xx] = (uint16_t)s[yy * n + xx];
            continue;
        }
        if (t->flags & RC_HEVC_TU_INTRA) {
            intra_predict(&c, t->x0, t->y0, t->log2, t->c, t->mode, pred);
            for (int yy = 0; yy < n; yy++)
                for (int xx = 0; xx < n; xx++) pl[(t->y0 + yy) * w + t->x0 + xx] = (uint16_t)pred[yy * n + xx];
        }
        if (t->flags & RC_HEVC_TU_CBF) {
            residual_of(&c, t, co);
            /* add_residual, transform.rs:110-122 */
            for (int yy = 0; yy < n; yy++)
                for (int xx = 0; xx < n; xx++) {
                    uint16_t *p = &pl[(t->y0 + yy) * w + t->x0 + xx];
                    *p = (uint16_t)clampi(*p + co[yy * n + xx], 0, max);
                }
        }
    }
    if (stages & 1) deblock(&c);
    if (stages & 2) {
        uint16_t *copy[3];
        for (int k = 0; k < 3; k++) {
            size_t nb = (size_t)pw_of(&c, k) * ph_of(&c, k);
            copy[k] = (uint16_t *)malloc(nb * sizeof(uint16_t));
            if (!copy[k]) return RC_ENOMEM;
            memcpy(copy[k], c.pl[k], nb * sizeof(uint16_t));
        }
        sao(&c, copy);
        for (int k = 0; k < 3; k++) free(copy[k]);
    }
    return 0;
}

/* Block-level helpers for the known-answer tests. */
void oracle_hevc_inverse(int16_t *co, int log2, int dst, int max_x, int max_y, int bd_shift) {
    inverse(co, 1 << log2, dst, max_x, max_y, bd_shift);
}
int oracle_hevc_inverse_dc(int dc, int bd_shift) { return inverse_dc(dc, bd_shift); }
void oracle_hevc_intra_predict_refs(const uint16_t *left, const uint16_t *top, int mode, int log2, int is_luma,
                                    int strong, int bd, int *out) {
    Refs r;
    memcpy(r.left, left, sizeof r.left);
    memcpy(r.top, top, sizeof r.top);
    if (is_luma) filter_refs(&r, mode, 1 << log2, strong, 1, bd);
    predict(&r, mode, 1 << log2, is_luma, bd, out);
}
