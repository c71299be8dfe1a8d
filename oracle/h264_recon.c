/*
 * h264_recon.c — CPU restatement (C11) of pito-codecs' H.264 block
 * reconstruction: dequantisation, inverse transforms, intra prediction,
 * motion compensation with edge extension and weighted prediction, and the
 * deblocking filter with its boundary-strength derivation.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  It follows the reference's scalar
 * twins, which the reference's own tests pin to its SIMD production path
 * (src/h264/dec/simd/mc.rs:611-733, src/h264/dec/deblock.rs:551-636).
 * Integer semantics follow Rust: wrapping multiplies and left shifts are done
 * in uint32_t, right shifts of negative values are arithmetic.
 */
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ---- tables: src/h264/dec/tables.rs, src/syntax/h264/tables.rs ---------- */

/* NORM_ADJUST4/8, src/h264/dec/tables.rs:14-29 */
static const uint16_t NORM4[6][3] = {{10, 16, 13}, {11, 18, 14}, {13, 20, 16},
                                     {14, 23, 18}, {16, 25, 20}, {18, 29, 23}};
static const uint16_t NORM8[6][6] = {
    {20, 18, 32, 19, 25, 24}, {22, 19, 35, 21, 28, 26},
    {26, 23, 42, 24, 33, 31}, {28, 25, 45, 26, 35, 33},
    {32, 28, 51, 30, 40, 38}, {36, 32, 58, 34, 46, 43}};

/* ALPHA / BETA / TC0, src/h264/dec/tables.rs:61-92 */
static const uint8_t ALPHA[52] = {
    0,  0,  0,  0,  0,  0,  0,  0,  0,   0,   0,   0,   0,   0,   0,   0,   4,  4,
    5,  6,  7,  8,  9,  10, 12, 13, 15,  17,  20,  22,  25,  28,  32,  36,  40, 45,
    50, 56, 63, 71, 80, 90, 101, 113, 127, 144, 162, 182, 203, 226, 255, 255};
static const uint8_t BETA[52] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0,  0,  0,  0,  0,  0,  0,  0,  2,  2,
    2, 3, 3, 3, 3, 4, 4, 4, 6,  6,  7,  7,  8,  8,  9,  9,  10, 10,
    11, 11, 12, 12, 13, 13, 14, 14, 15, 15, 16, 16, 17, 17, 18, 18};
static const uint8_t TC0[52][3] = {
    {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},   {0, 0, 0},
    {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},   {0, 0, 0},
    {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},   {0, 0, 1},
    {0, 0, 1},  {0, 0, 1},  {0, 0, 1},  {0, 1, 1},  {0, 1, 1},   {1, 1, 1},
    {1, 1, 1},  {1, 1, 1},  {1, 1, 1},  {1, 1, 2},  {1, 1, 2},   {1, 1, 2},
    {1, 1, 2},  {1, 2, 3},  {1, 2, 3},  {2, 2, 3},  {2, 2, 4},   {2, 3, 4},
    {2, 3, 4},  {3, 3, 5},  {3, 4, 6},  {3, 4, 6},  {4, 5, 7},   {4, 5, 8},
    {4, 6, 9},  {5, 7, 10}, {6, 8, 11}, {6, 8, 13}, {7, 10, 14}, {8, 11, 16},
    {9, 12, 18}, {10, 13, 20}, {11, 15, 23}, {13, 17, 25}};

/* BLK4_XY decode order and RASTER_TO_BLK4, src/h264/dec/tables.rs:94-114 */
static const uint8_t BLK4_XY[16][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1},
                                       {2, 0}, {3, 0}, {2, 1}, {3, 1},
                                       {0, 2}, {1, 2}, {0, 3}, {1, 3},
                                       {2, 2}, {3, 2}, {2, 3}, {3, 3}};
static const uint8_t RASTER_TO_BLK4[16] = {0, 1, 4, 5, 2, 3, 6, 7,
                                           8, 9, 12, 13, 10, 11, 14, 15};
/* ZIGZAG4, src/syntax/h264/tables.rs:12 */
static const uint8_t ZIGZAG4[16] = {0, 1, 4, 8, 5, 2, 3, 6, 9, 12, 13, 10, 7, 11, 14, 15};
/* ZIGZAG8 is generated by anti-diagonal walk, src/syntax/h264/tables.rs:14-33 */
static uint8_t ZIGZAG8[64];
static int zz8_ready;

static void init_zigzag8(void) {
    if (zz8_ready) return;
    int k = 0;
    for (int d = 0; d < 15; d++)
        for (int i = 0; i < 8; i++) {
            int row = (d % 2 == 0) ? d - i : i;
            int col = (d % 2 == 0) ? i : d - i;
            if (row >= 0 && row < 8 && col >= 0 && col < 8) ZIGZAG8[k++] = (uint8_t)(row * 8 + col);
        }
    zz8_ready = 1;
}

static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
static inline int32_t wshl(int32_t a, int s) { return (int32_t)((uint32_t)a << s); }
static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline uint8_t clip_u8(int32_t v) { return (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v); }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }

/* ---- a1: LevelScale::new, src/h264/dec/transform.rs:10-28 --------------- */
static uint16_t norm4(int m, int pos) {  /* tables.rs:33-42 */
    int i = pos / 4, j = pos % 4;
    if (i % 2 == 0 && j % 2 == 0) return NORM4[m][0];
    if (i % 2 == 1 && j % 2 == 1) return NORM4[m][1];
    return NORM4[m][2];
}
static uint16_t norm8(int m, int pos) {  /* tables.rs:44-60 */
    int i = pos / 8, j = pos % 8, k;
    if (i % 4 == 0 && j % 4 == 0) k = 0;
    else if (i % 2 == 1 && j % 2 == 1) k = 1;
    else if (i % 4 == 2 && j % 4 == 2) k = 2;
    else if ((i % 4 == 0 && j % 2 == 1) || (i % 2 == 1 && j % 4 == 0)) k = 3;
    else if ((i % 4 == 0 && j % 4 == 2) || (i % 4 == 2 && j % 4 == 0)) k = 4;
    else k = 5;
    return NORM8[m][k];
}

void oracle_h264_level_scale(const uint8_t *m4, const uint8_t *m8,
                             int32_t ls4[6][6][16], int32_t ls8[6][6][64]) {
    for (int l = 0; l < 6; l++)
        for (int q = 0; q < 6; q++) {
            for (int p = 0; p < 16; p++)
                ls4[l][q][p] = (int32_t)(m4 ? m4[l * 16 + p] : 16) * norm4(q, p);
            for (int p = 0; p < 64; p++)
                ls8[l][q][p] = (int32_t)(m8 ? m8[l * 64 + p] : 16) * norm8(q, p);
        }
}

/* ---- a2: scale4 / scale8, src/h264/dec/transform.rs:30-46 --------------- */
static int32_t scale4(int32_t c, int32_t ls, int qp) {
    if (qp >= 24) return wshl(wmul(c, ls), qp / 6 - 4);
    return wadd(wmul(c, ls), 1 << (3 - qp / 6)) >> (4 - qp / 6);
}
static int32_t scale8(int32_t c, int32_t ls, int qp) {
    if (qp >= 36) return wshl(wmul(c, ls), qp / 6 - 6);
    return wadd(wmul(c, ls), 1 << (5 - qp / 6)) >> (6 - qp / 6);
}

/* ---- a3: luma_dc_dequant, src/h264/dec/transform.rs:48-75 --------------- */
void oracle_h264_luma_dc_dequant(int32_t c[16], int qp, int32_t ls00) {
    int32_t t[16];
    for (int i = 0; i < 4; i++) {
        const int32_t *r = c + i * 4;
        int32_t s01 = r[0] + r[1], d01 = r[0] - r[1];
        int32_t s23 = r[2] + r[3], d23 = r[2] - r[3];
        t[i * 4] = s01 + s23;
        t[i * 4 + 1] = s01 - s23;
        t[i * 4 + 2] = d01 - d23;
        t[i * 4 + 3] = d01 + d23;
    }
    for (int j = 0; j < 4; j++) {
        int32_t s01 = t[j] + t[4 + j], d01 = t[j] - t[4 + j];
        int32_t s23 = t[8 + j] + t[12 + j], d23 = t[8 + j] - t[12 + j];
        int32_t f[4] = {s01 + s23, s01 - s23, d01 - d23, d01 + d23};
        for (int i = 0; i < 4; i++)
            c[i * 4 + j] = qp >= 36 ? wshl(wmul(f[i], ls00), qp / 6 - 6)
                                    : wadd(wmul(f[i], ls00), 1 << (5 - qp / 6)) >> (6 - qp / 6);
    }
}

/* ---- a4: chroma_dc_dequant_420, src/h264/dec/transform.rs:77-91 --------- */
void oracle_h264_chroma_dc_dequant(int32_t c[4], int qp, int32_t ls00) {
    int32_t s0 = wadd(c[0], c[1]), d0 = wsub(c[0], c[1]);
    int32_t s1 = wadd(c[2], c[3]), d1 = wsub(c[2], c[3]);
    int32_t f[4] = {wadd(s0, s1), wadd(d0, d1), wsub(s0, s1), wsub(d0, d1)};
    for (int k = 0; k < 4; k++) c[k] = wshl(wmul(f[k], ls00), qp / 6) >> 5;
}

/* ---- a5: idct4_add, src/h264/dec/transform.rs:98-130 -------------------- */
void oracle_h264_idct4_add(const int32_t d[16], uint8_t *dst, int stride) {
    int32_t t[4][4], o[4][4];
    for (int i = 0; i < 4; i++) {
        const int32_t *r = d + i * 4;
        int32_t e = r[0] + r[2], f = r[0] - r[2];
        int32_t g = (r[1] >> 1) - r[3], h = r[1] + (r[3] >> 1);
        t[i][0] = e + h; t[i][1] = f + g; t[i][2] = f - g; t[i][3] = e - h;
    }
    for (int j = 0; j < 4; j++) {
        int32_t e = t[0][j] + t[2][j], f = t[0][j] - t[2][j];
        int32_t g = (t[1][j] >> 1) - t[3][j], h = t[1][j] + (t[3][j] >> 1);
        o[0][j] = e + h; o[1][j] = f + g; o[2][j] = f - g; o[3][j] = e - h;
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            dst[i * stride + j] = clip_u8(dst[i * stride + j] + ((o[i][j] + 32) >> 6));
}

/* ---- a6: idct8_1d / idct8_add, src/h264/dec/transform.rs:132-185 -------- */
static void idct8_1d(const int32_t d[8], int32_t out[8]) {
    int32_t a0 = d[0] + d[4], a4 = d[0] - d[4];
    int32_t a2 = (d[2] >> 1) - d[6], a6 = d[2] + (d[6] >> 1);
    int32_t b0 = a0 + a6, b2 = a4 + a2, b4 = a4 - a2, b6 = a0 - a6;
    int32_t a1 = -d[3] + d[5] - d[7] - (d[7] >> 1);
    int32_t a3 = d[1] + d[7] - d[3] - (d[3] >> 1);
    int32_t a5 = -d[1] + d[7] + d[5] + (d[5] >> 1);
    int32_t a7 = d[3] + d[5] + d[1] + (d[1] >> 1);
    int32_t b1 = a1 + (a7 >> 2), b7 = a7 - (a1 >> 2);
    int32_t b3 = a3 + (a5 >> 2), b5 = (a3 >> 2) - a5;
    out[0] = b0 + b7; out[1] = b2 + b5; out[2] = b4 + b3; out[3] = b6 + b1;
    out[4] = b6 - b1; out[5] = b4 - b3; out[6] = b2 - b5; out[7] = b0 - b7;
}

void oracle_h264_idct8_add(const int32_t d[64], uint8_t *dst, int stride) {
    int32_t t[8][8], o[8][8], col[8], res[8];
    for (int i = 0; i < 8; i++) idct8_1d(d + i * 8, t[i]);
    for (int j = 0; j < 8; j++) {
        for (int i = 0; i < 8; i++) col[i] = t[i][j];
        idct8_1d(col, res);
        for (int i = 0; i < 8; i++) o[i][j] = res[i];
    }
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++)
            dst[i * stride + j] = clip_u8(dst[i * stride + j] + ((o[i][j] + 32) >> 6));
}

/* ---- a7: intra prediction, src/h264/dec/intra.rs ----------------------- */
typedef struct { int left, top, top_left, top_right; } Avail;
typedef struct { int32_t top[16], left[8], tl; } Edge;

static inline int32_t et(const Edge *e, int x) { return x < 0 ? e->tl : e->top[x]; }
static inline int32_t el(const Edge *e, int y) { return y < 0 ? e->tl : e->left[y]; }

/* load_edge, intra.rs:31-62 */
static Edge load_edge(const uint8_t *plane, int stride, int x, int y, int n, Avail a) {
    Edge e;
    for (int i = 0; i < 16; i++) e.top[i] = 128;
    for (int i = 0; i < 8; i++) e.left[i] = 128;
    e.tl = 128;
    if (a.top) {
        const uint8_t *row = plane + (y - 1) * stride + x;
        for (int i = 0; i < n; i++) e.top[i] = row[i];
        if (a.top_right)
            for (int i = n; i < 2 * n; i++) e.top[i] = row[i];
        else
            for (int i = n; i < 2 * n; i++) e.top[i] = e.top[n - 1];
    }
    if (a.left)
        for (int i = 0; i < n; i++) e.left[i] = plane[(y + i) * stride + x - 1];
    if (a.top_left) e.tl = plane[(y - 1) * stride + x - 1];
    return e;
}

/* pred_nxn, intra.rs:64-192 */
static void pred_nxn(int mode, const Edge *e, int n, Avail a, uint8_t *out, int stride) {
#define PUT(x, y, v) out[(y) * stride + (x)] = (uint8_t)(v)
    switch (mode) {
    case 0:
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) PUT(x, y, et(e, x));
        break;
    case 1:
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) PUT(x, y, el(e, y));
        break;
    case 2: {
        int shift = n == 4 ? 2 : 3, st = 0, sl = 0, dc;
        for (int i = 0; i < n; i++) { st += et(e, i); sl += el(e, i); }
        if (a.top && a.left) dc = (st + sl + n) >> (shift + 1);
        else if (!a.top && a.left) dc = (sl + (n >> 1)) >> shift;
        else if (a.top && !a.left) dc = (st + (n >> 1)) >> shift;
        else dc = 128;
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) PUT(x, y, dc);
        break;
    }
    case 3:
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) {
                int v = (x == n - 1 && y == n - 1)
                            ? (et(e, 2 * n - 2) + 3 * et(e, 2 * n - 1) + 2) >> 2
                            : (et(e, x + y) + 2 * et(e, x + y + 1) + et(e, x + y + 2) + 2) >> 2;
                PUT(x, y, v);
            }
        break;
    case 4:
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) {
                int v;
                if (x > y) v = (et(e, x - y - 2) + 2 * et(e, x - y - 1) + et(e, x - y) + 2) >> 2;
                else if (x < y) v = (el(e, y - x - 2) + 2 * el(e, y - x - 1) + el(e, y - x) + 2) >> 2;
                else v = (et(e, 0) + 2 * e->tl + el(e, 0) + 2) >> 2;
                PUT(x, y, v);
            }
        break;
    case 5:
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) {
                int z = 2 * x - y, v, i = x - (y >> 1);
                if (z >= 0 && z % 2 == 0) v = (et(e, i - 1) + et(e, i) + 1) >> 1;
                else if (z > 0) v = (et(e, i - 2) + 2 * et(e, i - 1) + et(e, i) + 2) >> 2;
                else if (z == -1) v = (el(e, 0) + 2 * e->tl + et(e, 0) + 2) >> 2;
                else v = (el(e, y - 2 * x - 1) + 2 * el(e, y - 2 * x - 2) + el(e, y - 2 * x - 3) + 2) >> 2;
                PUT(x, y, v);
            }
        break;
    case 6:
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) {
                int z = 2 * y - x, v, i = y - (x >> 1);
                if (z >= 0 && z % 2 == 0) v = (el(e, i - 1) + el(e, i) + 1) >> 1;
                else if (z > 0) v = (el(e, i - 2) + 2 * el(e, i - 1) + el(e, i) + 2) >> 2;
                else if (z == -1) v = (el(e, 0) + 2 * e->tl + et(e, 0) + 2) >> 2;
                else v = (et(e, x - 2 * y - 1) + 2 * et(e, x - 2 * y - 2) + et(e, x - 2 * y - 3) + 2) >> 2;
                PUT(x, y, v);
            }
        break;
    case 7:
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) {
                int i = x + (y >> 1), v;
                if (y % 2 == 0) v = (et(e, i) + et(e, i + 1) + 1) >> 1;
                else v = (et(e, i) + 2 * et(e, i + 1) + et(e, i + 2) + 2) >> 2;
                PUT(x, y, v);
            }
        break;
    default: {
        int zmax = 2 * n - 3;
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) {
                int z = x + 2 * y, i = y + (x >> 1), v;
                if (z < zmax && z % 2 == 0) v = (el(e, i) + el(e, i + 1) + 1) >> 1;
                else if (z < zmax) v = (el(e, i) + 2 * el(e, i + 1) + el(e, i + 2) + 2) >> 2;
                else if (z == zmax) v = (el(e, n - 2) + 3 * el(e, n - 1) + 2) >> 2;
                else v = el(e, n - 1);
                PUT(x, y, v);
            }
        break;
    }
    }
#undef PUT
}

/* pred4x4, intra.rs:194-197 */
static void pred4x4(uint8_t *plane, int stride, int x, int y, int mode, Avail a) {
    Edge e = load_edge(plane, stride, x, y, 4, a);
    pred_nxn(mode, &e, 4, a, plane + y * stride + x, stride);
}

/* pred8x8 with reference-sample smoothing, intra.rs:199-233 */
static void pred8x8(uint8_t *plane, int stride, int x, int y, int mode, Avail a) {
    Edge p = load_edge(plane, stride, x, y, 8, a), f = p;
    if (a.top) {
        f.top[0] = a.top_left ? (p.tl + 2 * p.top[0] + p.top[1] + 2) >> 2
                              : (3 * p.top[0] + p.top[1] + 2) >> 2;
        for (int i = 1; i < 15; i++) f.top[i] = (p.top[i - 1] + 2 * p.top[i] + p.top[i + 1] + 2) >> 2;
        f.top[15] = (p.top[14] + 3 * p.top[15] + 2) >> 2;
    }
    if (a.top_left) {
        if (a.top && a.left) f.tl = (p.top[0] + 2 * p.tl + p.left[0] + 2) >> 2;
        else if (a.top) f.tl = (3 * p.tl + p.top[0] + 2) >> 2;
        else if (a.left) f.tl = (3 * p.tl + p.left[0] + 2) >> 2;
        else f.tl = p.tl;
    }
    if (a.left) {
        f.left[0] = a.top_left ? (p.tl + 2 * p.left[0] + p.left[1] + 2) >> 2
                               : (3 * p.left[0] + p.left[1] + 2) >> 2;
        for (int i = 1; i < 7; i++) f.left[i] = (p.left[i - 1] + 2 * p.left[i] + p.left[i + 1] + 2) >> 2;
        f.left[7] = (p.left[6] + 3 * p.left[7] + 2) >> 2;
    }
    pred_nxn(mode, &f, 8, a, plane + y * stride + x, stride);
}

/* pred16x16, intra.rs:240-305 */
static void pred16x16(uint8_t *plane, int stride, int x, int y, int mode, Avail a) {
    int32_t top[16] = {0}, left[16] = {0};
    if (a.top)
        for (int i = 0; i < 16; i++) top[i] = plane[(y - 1) * stride + x + i];
    if (a.left)
        for (int i = 0; i < 16; i++) left[i] = plane[(y + i) * stride + x - 1];
    uint8_t *b = plane + y * stride + x;
    if (mode == 0) {
        for (int r = 0; r < 16; r++)
            for (int c = 0; c < 16; c++) b[r * stride + c] = (uint8_t)top[c];
    } else if (mode == 1) {
        for (int r = 0; r < 16; r++)
            for (int c = 0; c < 16; c++) b[r * stride + c] = (uint8_t)left[r];
    } else if (mode == 2) {
        int st = 0, sl = 0, dc;
        for (int i = 0; i < 16; i++) { st += top[i]; sl += left[i]; }
        if (a.top && a.left) dc = (st + sl + 16) >> 5;
        else if (!a.top && a.left) dc = (sl + 8) >> 4;
        else if (a.top && !a.left) dc = (st + 8) >> 4;
        else dc = 128;
        for (int r = 0; r < 16; r++)
            for (int c = 0; c < 16; c++) b[r * stride + c] = (uint8_t)dc;
    } else {
        int32_t tl = a.top_left ? plane[(y - 1) * stride + x - 1] : 128;
#define T16(i) ((i) < 0 ? tl : top[(i)])
#define L16(i) ((i) < 0 ? tl : left[(i)])
        int32_t h = 0, v = 0;
        for (int k = 0; k < 8; k++) {
            h += (k + 1) * (T16(8 + k) - T16(6 - k));
            v += (k + 1) * (L16(8 + k) - L16(6 - k));
        }
#undef T16
#undef L16
        int32_t aa = 16 * (left[15] + top[15]), bb = (5 * h + 32) >> 6, cc = (5 * v + 32) >> 6;
        for (int r = 0; r < 16; r++)
            for (int c = 0; c < 16; c++) b[r * stride + c] = clip_u8((aa + bb * (c - 7) + cc * (r - 7) + 16) >> 5);
    }
}

/* pred_chroma, intra.rs:307-395 */
static void pred_chroma(uint8_t *plane, int stride, int x, int y, int mode, Avail a) {
    int32_t top[8] = {0}, left[8] = {0};
    if (a.top)
        for (int i = 0; i < 8; i++) top[i] = plane[(y - 1) * stride + x + i];
    if (a.left)
        for (int i = 0; i < 8; i++) left[i] = plane[(y + i) * stride + x - 1];
    uint8_t *b = plane + y * stride + x;
    if (mode == 0) {
        for (int by = 0; by < 2; by++)
            for (int bx = 0; bx < 2; bx++) {
                int st = 0, sl = 0, dc;
                for (int i = 0; i < 4; i++) { st += top[bx * 4 + i]; sl += left[by * 4 + i]; }
                if ((bx == 0 && by == 0) || (bx > 0 && by > 0)) {
                    if (a.top && a.left) dc = (st + sl + 4) >> 3;
                    else if (!a.top && a.left) dc = (sl + 2) >> 2;
                    else if (a.top && !a.left) dc = (st + 2) >> 2;
                    else dc = 128;
                } else if (bx > 0) {
                    dc = a.top ? (st + 2) >> 2 : a.left ? (sl + 2) >> 2 : 128;
                } else {
                    dc = a.left ? (sl + 2) >> 2 : a.top ? (st + 2) >> 2 : 128;
                }
                for (int r = 0; r < 4; r++)
                    for (int c = 0; c < 4; c++) b[(by * 4 + r) * stride + bx * 4 + c] = (uint8_t)dc;
            }
    } else if (mode == 1) {
        for (int r = 0; r < 8; r++)
            for (int c = 0; c < 8; c++) b[r * stride + c] = (uint8_t)left[r];
    } else if (mode == 2) {
        for (int r = 0; r < 8; r++)
            for (int c = 0; c < 8; c++) b[r * stride + c] = (uint8_t)top[c];
    } else {
        int32_t tl = a.top_left ? plane[(y - 1) * stride + x - 1] : 128;
#define T8(i) ((i) < 0 ? tl : top[(i)])
#define L8(i) ((i) < 0 ? tl : left[(i)])
        int32_t h = 0, v = 0;
        for (int k = 0; k < 4; k++) {
            h += (k + 1) * (T8(4 + k) - T8(2 - k));
            v += (k + 1) * (L8(4 + k) - L8(2 - k));
        }
#undef T8
#undef L8
        int32_t aa = 16 * (left[7] + top[7]), bb = (34 * h + 32) >> 6, cc = (34 * v + 32) >> 6;
        for (int r = 0; r < 8; r++)
            for (int c = 0; c < 8; c++) b[r * stride + c] = clip_u8((aa + bb * (c - 3) + cc * (r - 3) + 16) >> 5);
    }
}

/* ---- a8-a10: motion compensation -------------------------------------- */
/* Edge extension by coordinate clamp: window / copy_clamped,
 * src/h264/dec/picture.rs:686-735; predict_block, slicedec.rs:299-340. */
static inline int32_t tap6(int32_t a, int32_t b, int32_t c, int32_t d, int32_t e, int32_t f) {
    return a - 5 * b + 20 * c + 20 * d - 5 * e + f;
}
static inline uint8_t avg2(int a, int b) { return (uint8_t)((a + b + 1) >> 1); }

typedef struct { const uint8_t *p; int stride, w, h, x0, y0; } Win;
/* S(dx, dy) of output sample (c, r): window sample at clamp(x0+c+dx), clamp(y0+r+dy) */
static inline int32_t ws(const Win *w, int x, int y) {
    return w->p[clampi(w->y0 + y, 0, w->h - 1) * w->stride + clampi(w->x0 + x, 0, w->w - 1)];
}
static inline int32_t htap(const Win *w, int c, int r) {  /* horizontal 6-tap centred between c and c+1 */
    return tap6(ws(w, c - 2, r), ws(w, c - 1, r), ws(w, c, r), ws(w, c + 1, r), ws(w, c + 2, r), ws(w, c + 3, r));
}
static inline int32_t vtap(const Win *w, int c, int r) {
    return tap6(ws(w, c, r - 2), ws(w, c, r - 1), ws(w, c, r), ws(w, c, r + 1), ws(w, c, r + 2), ws(w, c, r + 3));
}

/* mc_luma_win_scalar, src/h264/dec/inter.rs:73-213, one output sample */
static uint8_t luma_sample(const Win *w, int c, int r, int fx, int fy) {
    if (fx == 0 && fy == 0) return (uint8_t)ws(w, c, r);
    if (fy == 0) {
        uint8_t b = clip_u8((htap(w, c, r) + 16) >> 5);
        if (fx == 1) return avg2(ws(w, c, r), b);
        if (fx == 2) return b;
        return avg2(ws(w, c + 1, r), b);
    }
    if (fx == 0) {
        uint8_t h = clip_u8((vtap(w, c, r) + 16) >> 5);
        if (fy == 2) return h;
        return avg2(fy == 1 ? ws(w, c, r) : ws(w, c, r + 1), h);
    }
    if (fx == 2 || fy == 2) {
        /* b1 rows: horizontal taps of rows r-2..r+3, then vertical tap */
        int32_t b1[6];
        for (int j = 0; j < 6; j++) b1[j] = htap(w, c, r + j - 2);
        int32_t t = tap6(b1[0], b1[1], b1[2], b1[3], b1[4], b1[5]);
        uint8_t jv = clip_u8((t + 512) >> 10);
        if (fx == 2 && fy == 2) return jv;
        if (fx == 2) {
            int32_t bh = fy == 1 ? b1[2] : b1[3];
            return avg2(clip_u8((bh + 16) >> 5), jv);
        }
        int32_t v = vtap(w, c + (fx == 1 ? 0 : 1), r);
        return avg2(clip_u8((v + 16) >> 5), jv);
    }
    int32_t t = htap(w, c, r + (fy == 1 ? 0 : 1));
    int32_t v = vtap(w, c + (fx == 1 ? 0 : 1), r);
    return avg2(clip_u8((t + 16) >> 5), clip_u8((v + 16) >> 5));
}

void oracle_h264_mc_luma(const uint8_t *plane, int width, int height, int px, int py, int mvx,
                         int mvy, int bw, int bh, uint8_t *out, int os) {
    Win w = {plane, width, width, height, px + (mvx >> 2), py + (mvy >> 2)};
    for (int r = 0; r < bh; r++)
        for (int c = 0; c < bw; c++) out[r * os + c] = luma_sample(&w, c, r, mvx & 3, mvy & 3);
}

/* mc_chroma_win_scalar, src/h264/dec/inter.rs:217-247 */
void oracle_h264_mc_chroma(const uint8_t *plane, int cwidth, int cheight, int cpx, int cpy,
                           int mvx, int mvy, int bw, int bh, uint8_t *out, int os) {
    Win w = {plane, cwidth, cwidth, cheight, cpx + (mvx >> 3), cpy + (mvy >> 3)};
    int fx = mvx & 7, fy = mvy & 7;
    int w00 = (8 - fx) * (8 - fy), w10 = fx * (8 - fy), w01 = (8 - fx) * fy, w11 = fx * fy;
    for (int r = 0; r < bh; r++)
        for (int c = 0; c < bw; c++) {
            if (fx == 0 && fy == 0) { out[r * os + c] = (uint8_t)ws(&w, c, r); continue; }
            int v = w00 * ws(&w, c, r) + w10 * ws(&w, c + 1, r) + w01 * ws(&w, c, r + 1) + w11 * ws(&w, c + 1, r + 1);
            out[r * os + c] = (uint8_t)((v + 32) >> 6);
        }
}

/* a11: weighted_store_scalar, src/h264/dec/inter.rs:286-352, for one
 * resolved component weighting (after Weight::simplify). */
static void weighted_store(uint8_t *dst, int ds, const uint8_t *a, const uint8_t *b, int ps, int bw,
                           int bh, int explicit_, int log_wd, int w0, int w1, int o0, int o1) {
    for (int r = 0; r < bh; r++)
        for (int c = 0; c < bw; c++) {
            int x = a ? a[r * ps + c] : 0, y = b ? b[r * ps + c] : 0, v;
            if (a && b) {
                if (!explicit_) v = (x + y + 1) >> 1;
                else v = clip_u8(((x * w0 + y * w1 + (1 << log_wd)) >> (log_wd + 1)) + ((o0 + o1 + 1) >> 1));
            } else if (a || b) {
                int s = a ? x : y;
                if (!explicit_) v = s;
                else {
                    int wt = a ? w0 : w1, o = a ? o0 : o1;
                    int round = log_wd >= 1 ? 1 << (log_wd - 1) : 0;
                    v = clip_u8(((s * wt + round) >> log_wd) + o);
                }
            } else continue;
            dst[r * ds + c] = (uint8_t)v;
        }
}

/* ---- picture-level driver -------------------------------------------- */
typedef struct {
    int mb_w, mb_h, W, H, CW, CH;
    const rc_h264_picture *pic;
    const uint8_t *const *ry, *const *ru, *const *rv;
    uint8_t *y, *u, *v;
    int32_t ls4[6][6][16], ls8[6][6][64];
} Ctx;

static int is_intra(int kind) { return kind >= RC_H264_I4x4 && kind <= RC_H264_IPCM; }

/* neighbour availability for intra (start_mb nb[] + intra_nb,
 * src/h264/dec/slicedec.rs:489-508, 525-530). n: 0 left, 1 top, 2 top-right, 3 top-left */
static int intra_nb(const Ctx *cx, int mbx, int mby, int n) {
    static const int dx[4] = {-1, 0, 1, -1}, dy[4] = {0, -1, -1, -1};
    int x = mbx + dx[n], y = mby + dy[n];
    if (x < 0 || y < 0 || x >= cx->mb_w) return 0;
    const rc_h264_mb *q = &cx->pic->mbs[mby * cx->mb_w + mbx];
    const rc_h264_mb *p = &cx->pic->mbs[y * cx->mb_w + x];
    if (p->kind == RC_H264_NONE || p->slice != q->slice) return 0;
    return !cx->pic->constrained_intra_pred || is_intra(p->kind);
}

/* luma_avail4, src/h264/dec/slicedec.rs:1297-1323 */
static Avail luma_avail4(const Ctx *cx, int mbx, int mby, int bx, int by) {
    int a = intra_nb(cx, mbx, mby, 0), b = intra_nb(cx, mbx, mby, 1);
    int c = intra_nb(cx, mbx, mby, 2), d = intra_nb(cx, mbx, mby, 3);
    Avail av;
    av.left = bx > 0 ? 1 : a;
    av.top = by > 0 ? 1 : b;
    if (bx > 0 && by > 0) av.top_left = 1;
    else if (by > 0) av.top_left = a;
    else if (bx > 0) av.top_left = b;
    else av.top_left = d;
    if (by == 0) av.top_right = bx < 3 ? b : c;
    else if (bx == 3) av.top_right = 0;
    else av.top_right = RASTER_TO_BLK4[(by - 1) * 4 + bx + 1] < RASTER_TO_BLK4[by * 4 + bx];
    return av;
}

/* coefficient scratch of one MB (Scratch, slicedec.rs:216-224) */
typedef struct { int32_t coef[256], coef_c[2][64]; uint16_t blk_nz; uint8_t c_nz[2]; } Coefs;

/* put_luma4 / put_luma8 / put_luma_dc / put_chroma_dc / put_chroma_ac,
 * src/h264/dec/slicedec.rs:1462-1555, applied to the MB's level payload */
static int place_levels(const Ctx *cx, const rc_h264_mb *m, Coefs *s) {
    memset(s, 0, sizeof *s);
    const int16_t *lv = cx->pic->levels + m->coef_off;
    size_t used = 0;
    int intra = is_intra(m->kind), qp = m->qp;
#define NEED(n) do { if (m->coef_off + used + (n) > cx->pic->num_levels) return RC_EINVAL; } while (0)
    if (m->kind == RC_H264_I16x16 && (m->dc_coded & 1)) {
        NEED(16);
        int32_t c[16] = {0};
        for (int k = 0; k < 16; k++) c[ZIGZAG4[k]] = lv[used + k];
        used += 16;
        oracle_h264_luma_dc_dequant(c, qp, cx->ls4[0][qp % 6][0]);
        for (int r = 0; r < 16; r++)
            if (c[r] != 0) { s->coef[r * 16] = c[r]; s->blk_nz |= 1 << r; }
    }
    if (m->transform_8x8) {
        const int32_t *ls = cx->ls8[intra ? 0 : 1][qp % 6];
        for (int b8 = 0; b8 < 4; b8++) {
            if (!(m->luma_coded >> b8 & 1)) continue;
            NEED(64);
            int any = 0;
            for (int k = 0; k < 64; k++) {
                int32_t l = lv[used + k];
                if (l) { int p = ZIGZAG8[k]; s->coef[b8 * 64 + p] = scale8(l, ls[p], qp); any = 1; }
            }
            used += 64;
            if (any) s->blk_nz |= 1 << b8;
        }
    } else {
        const int32_t *ls = cx->ls4[intra ? 0 : 3][qp % 6];
        int ac_only = m->kind == RC_H264_I16x16;
        for (int r = 0; r < 16; r++) {
            if (!(m->luma_coded >> r & 1)) continue;
            NEED(16);
            int any = 0;
            for (int k = ac_only; k < 16; k++) {
                int32_t l = lv[used + k];
                if (l) { int p = ZIGZAG4[k]; s->coef[r * 16 + p] = scale4(l, ls[p], qp); any = 1; }
            }
            used += 16;
            if (any) s->blk_nz |= 1 << r;
        }
    }
    for (int c = 0; c < 2; c++) {
        if (!(m->dc_coded >> (1 + c) & 1)) continue;
        NEED(4);
        int qpc = m->qpc[c], list = intra ? 1 + c : 4 + c;
        int32_t v[4] = {lv[used], lv[used + 1], lv[used + 2], lv[used + 3]};
        used += 4;
        oracle_h264_chroma_dc_dequant(v, qpc, cx->ls4[list][qpc % 6][0]);
        for (int b = 0; b < 4; b++)
            if (v[b] != 0) { s->coef_c[c][b * 16] = v[b]; s->c_nz[c] |= 1 << b; }
    }
    for (int c = 0; c < 2; c++) {
        int qpc = m->qpc[c], list = intra ? 1 + c : 4 + c;
        const int32_t *ls = cx->ls4[list][qpc % 6];
        for (int b = 0; b < 4; b++) {
            if (!(m->chroma_coded >> (c * 4 + b) & 1)) continue;
            NEED(16);
            int any = 0;
            for (int k = 1; k < 16; k++) {
                int32_t l = lv[used + k];
                if (l) { int p = ZIGZAG4[k]; s->coef_c[c][b * 16 + p] = scale4(l, ls[p], qpc); any = 1; }
            }
            used += 16;
            if (any) s->c_nz[c] |= 1 << b;
        }
    }
#undef NEED
    return 0;
}

/* add_luma_block4 / add_luma_block8 / add_chroma, slicedec.rs:1229-1295 */
static void add_luma4(Ctx *cx, Coefs *s, int mbx, int mby, int r) {
    if (!(s->blk_nz >> r & 1)) return;
    int px = mbx * 16 + (r & 3) * 4, py = mby * 16 + (r >> 2) * 4;
    oracle_h264_idct4_add(s->coef + r * 16, cx->y + py * cx->W + px, cx->W);
}
static void add_luma8(Ctx *cx, Coefs *s, int mbx, int mby, int b8) {
    if (!(s->blk_nz >> b8 & 1)) return;
    int px = mbx * 16 + (b8 & 1) * 8, py = mby * 16 + (b8 >> 1) * 8;
    oracle_h264_idct8_add(s->coef + b8 * 64, cx->y + py * cx->W + px, cx->W);
}
static void add_chroma(Ctx *cx, Coefs *s, int mbx, int mby) {
    for (int c = 0; c < 2; c++)
        for (int b = 0; b < 4; b++) {
            if (!(s->c_nz[c] >> b & 1)) continue;
            int px = mbx * 8 + (b & 1) * 4, py = mby * 8 + (b >> 1) * 4;
            uint8_t *pl = c ? cx->v : cx->u;
            oracle_h264_idct4_add(s->coef_c[c] + b * 16, pl + py * cx->CW + px, cx->CW);
        }
}

/* reconstruct_intra, src/h264/dec/slicedec.rs:1325-1388 */
static void recon_intra(Ctx *cx, const rc_h264_mb *m, Coefs *s, int mbx, int mby) {
    int x0 = mbx * 16, y0 = mby * 16, W = cx->W;
    if (m->kind == RC_H264_I4x4) {
        for (int i = 0; i < 16; i++) {
            int bx = BLK4_XY[i][0], by = BLK4_XY[i][1];
            Avail av = luma_avail4(cx, mbx, mby, bx, by);
            pred4x4(cx->y, W, x0 + bx * 4, y0 + by * 4, m->intra_modes[by * 4 + bx], av);
            add_luma4(cx, s, mbx, mby, by * 4 + bx);
        }
    } else if (m->kind == RC_H264_I8x8) {
        for (int b8 = 0; b8 < 4; b8++) {
            int bx = (b8 & 1) * 2, by = (b8 >> 1) * 2;
            Avail av = luma_avail4(cx, mbx, mby, bx, by);
            av.top_right = b8 == 0 ? intra_nb(cx, mbx, mby, 1) : b8 == 1 ? intra_nb(cx, mbx, mby, 2) : b8 == 2;
            pred8x8(cx->y, W, x0 + bx * 4, y0 + by * 4, m->intra_modes[by * 4 + bx], av);
            add_luma8(cx, s, mbx, mby, b8);
        }
    } else if (m->kind == RC_H264_I16x16) {
        Avail av = {intra_nb(cx, mbx, mby, 0), intra_nb(cx, mbx, mby, 1), intra_nb(cx, mbx, mby, 3), 0};
        pred16x16(cx->y, W, x0, y0, m->i16_mode, av);
        for (int r = 0; r < 16; r++) add_luma4(cx, s, mbx, mby, r);
    }
    Avail av = {intra_nb(cx, mbx, mby, 0), intra_nb(cx, mbx, mby, 1), intra_nb(cx, mbx, mby, 3), 0};
    pred_chroma(cx->u, cx->CW, mbx * 8, mby * 8, m->chroma_mode, av);
    pred_chroma(cx->v, cx->CW, mbx * 8, mby * 8, m->chroma_mode, av);
    add_chroma(cx, s, mbx, mby);
}

/* mc_rect, src/h264/dec/slicedec.rs:996-1087, per 4x4 block (each sample's
 * prediction depends only on its block's vector, reference and weights) */
static void predict_inter(Ctx *cx, const rc_h264_mb *m, int mbx, int mby) {
    const rc_h264_slice *sl = &cx->pic->slices[m->slice];
    for (int k = 0; k < 16; k++) {
        int x4 = k & 3, y4 = k >> 2, b8 = (y4 >> 1) * 2 + (x4 >> 1);
        int px = mbx * 16 + x4 * 4, py = mby * 16 + y4 * 4;
        uint8_t pl[2][16], pc[2][2][4];
        int use[2] = {0, 0};
        for (int l = 0; l < 2; l++) {
            int ri = m->ref_idx[l][b8];
            if (ri < 0) continue;
            use[l] = 1;
            int slot = sl->ref_slot[l][ri];
            int mvx = m->mv[l][k][0], mvy = m->mv[l][k][1];
            oracle_h264_mc_luma(cx->ry[slot], cx->W, cx->H, px, py, mvx, mvy, 4, 4, pl[l], 4);
            oracle_h264_mc_chroma(cx->ru[slot], cx->CW, cx->CH, px / 2, py / 2, mvx, mvy, 2, 2, pc[l][0], 2);
            oracle_h264_mc_chroma(cx->rv[slot], cx->CW, cx->CH, px / 2, py / 2, mvx, mvy, 2, 2, pc[l][1], 2);
        }
        const rc_h264_weight *wt = m->wp[b8] == 0xff ? NULL : &cx->pic->weights[m->wp[b8]];
        for (int comp = 0; comp < 3; comp++) {
            int ex = wt && (wt->explicit_mask >> comp & 1);
            int lw = ex ? wt->log_wd[comp] : 0, w0 = ex ? wt->w0[comp] : 0, w1 = ex ? wt->w1[comp] : 0;
            int o0 = ex ? wt->o0[comp] : 0, o1 = ex ? wt->o1[comp] : 0;
            if (comp == 0)
                weighted_store(cx->y + py * cx->W + px, cx->W, use[0] ? pl[0] : NULL, use[1] ? pl[1] : NULL, 4, 4, 4, ex, lw, w0, w1, o0, o1);
            else {
                uint8_t *dst = (comp == 1 ? cx->u : cx->v) + (py / 2) * cx->CW + px / 2;
                weighted_store(dst, cx->CW, use[0] ? pc[0][comp - 1] : NULL, use[1] ? pc[1][comp - 1] : NULL, 2, 2, 2, ex, lw, w0, w1, o0, o1);
            }
        }
    }
}

/* write_pcm, src/h264/dec/slicedec.rs:1404-1424 */
static void write_pcm(Ctx *cx, const rc_h264_mb *m, int mbx, int mby) {
    const int16_t *s = cx->pic->levels + m->coef_off;
    for (int r = 0; r < 16; r++)
        for (int c = 0; c < 16; c++) cx->y[(mby * 16 + r) * cx->W + mbx * 16 + c] = (uint8_t)s[r * 16 + c];
    for (int p = 0; p < 2; p++)
        for (int r = 0; r < 8; r++)
            for (int c = 0; c < 8; c++)
                (p ? cx->v : cx->u)[(mby * 8 + r) * cx->CW + mbx * 8 + c] = (uint8_t)s[256 + p * 64 + r * 8 + c];
}

/* ---- a14-a15: deblocking, src/h264/dec/deblock.rs ---------------------- */
#define ID_NONE 0xffffffffu

/* ref_ids8, deblock.rs:7-21 */
static void ref_ids8(const Ctx *cx, const rc_h264_mb *m, uint32_t ids[2][4]) {
    const rc_h264_slice *sl = &cx->pic->slices[m->slice];
    for (int l = 0; l < 2; l++)
        for (int b = 0; b < 4; b++) {
            int r = m->ref_idx[l][b];
            ids[l][b] = r >= 0 ? (r < sl->num_ref[l] ? sl->ref_id[l][r] : ID_NONE - 1) : ID_NONE;
        }
}

typedef struct { uint32_t ids[2]; int32_t mv[2][2]; } Blk;

/* blk, deblock.rs:29-41 */
static Blk blk_of(const rc_h264_mb *m, uint32_t ids[2][4], int raster) {
    int b8 = (raster >> 3) * 2 + ((raster & 3) >> 1);
    Blk b;
    for (int l = 0; l < 2; l++) {
        b.ids[l] = ids[l][b8];
        int keep = b.ids[l] != ID_NONE;
        b.mv[l][0] = keep ? m->mv[l][raster][0] : 0;
        b.mv[l][1] = keep ? m->mv[l][raster][1] : 0;
    }
    return b;
}

/* near_mv / motion_bs, deblock.rs:43-59 */
static int near_mv(const int32_t a[2], const int32_t b[2]) {
    return (uint32_t)(a[0] - b[0] + 3) < 7 && (uint32_t)(a[1] - b[1] + 3) < 7;
}
static int motion_bs(Blk p, Blk q) {
    int same = p.ids[0] == q.ids[0] && p.ids[1] == q.ids[1] && near_mv(p.mv[0], q.mv[0]) && near_mv(p.mv[1], q.mv[1]);
    int cross = p.ids[0] == q.ids[1] && p.ids[1] == q.ids[0] && near_mv(p.mv[0], q.mv[1]) && near_mv(p.mv[1], q.mv[0]);
    return !(same || cross);
}

typedef struct { uint8_t bs[4]; int32_t tc0[4]; int32_t alpha, beta; } EdgeParams;

/* filter_lanes, deblock.rs:146-229.  s[k][i]: k = p3..q3, i = lane */
static void filter_lanes(int n, int16_t s[8][16], const EdgeParams *ep, int chroma) {
    int per = n / 4;
    int16_t alpha = (int16_t)ep->alpha, beta = (int16_t)ep->beta;
    int on[16], bs_on[16];
    int16_t tc0[16];
    int any = 0;
    for (int k = 0; k < 4; k++)
        for (int i = k * per; i < (k + 1) * per; i++) { bs_on[i] = ep->bs[k] != 0; tc0[i] = (int16_t)ep->tc0[k]; }
    for (int i = 0; i < n; i++) {
        on[i] = bs_on[i] && abs(s[3][i] - s[4][i]) < alpha && abs(s[2][i] - s[3][i]) < beta && abs(s[5][i] - s[4][i]) < beta;
        any |= on[i];
    }
    if (!any) return;
    int strong_edge = ep->bs[0] >= 4;
    if (chroma) {
        for (int i = 0; i < n; i++) {
            int p1 = s[2][i], p0 = s[3][i], q0 = s[4][i], q1 = s[5][i], np0, nq0;
            if (strong_edge) {
                np0 = (2 * p1 + p0 + q1 + 2) >> 2;
                nq0 = (2 * q1 + q0 + p1 + 2) >> 2;
            } else {
                int tc = tc0[i] + 1;
                int delta = clampi((((q0 - p0) << 2) + (p1 - q1) + 4) >> 3, -tc, tc);
                np0 = clampi(p0 + delta, 0, 255);
                nq0 = clampi(q0 - delta, 0, 255);
            }
            if (on[i]) { s[3][i] = (int16_t)np0; s[4][i] = (int16_t)nq0; }
        }
        return;
    }
    if (strong_edge) {
        int lim = (alpha >> 2) + 2;
        for (int i = 0; i < n; i++) {
            int a = s[0][i], b = s[1][i], c = s[2][i], d = s[3][i], e = s[4][i], f = s[5][i], g = s[6][i], h = s[7][i];
            int strong = abs(d - e) < lim;
            int sp = on[i] && abs(b - d) < beta && strong;
            int sq = on[i] && abs(g - e) < beta && strong;
            int wp0 = (2 * c + d + f + 2) >> 2, wq0 = (2 * f + e + c + 2) >> 2;
            int sp0 = (b + 2 * c + 2 * d + 2 * e + f + 4) >> 3, sq0 = (c + 2 * d + 2 * e + 2 * f + g + 4) >> 3;
            s[3][i] = (int16_t)(sp ? sp0 : on[i] ? wp0 : d);
            s[2][i] = (int16_t)(sp ? (b + c + d + e + 2) >> 2 : c);
            s[1][i] = (int16_t)(sp ? (2 * a + 3 * b + c + d + e + 4) >> 3 : b);
            s[4][i] = (int16_t)(sq ? sq0 : on[i] ? wq0 : e);
            s[5][i] = (int16_t)(sq ? (d + e + f + g + 2) >> 2 : f);
            s[6][i] = (int16_t)(sq ? (2 * h + 3 * g + f + e + d + 4) >> 3 : g);
        }
    } else {
        for (int i = 0; i < n; i++) {
            int p2 = s[1][i], p1 = s[2][i], p0 = s[3][i], q0 = s[4][i], q1 = s[5][i], q2 = s[6][i];
            int ap = abs(p2 - p0) < beta, aq = abs(q2 - q0) < beta;
            int t0 = tc0[i], tc = t0 + ap + aq;
            int delta = clampi((((q0 - p0) << 2) + (p1 - q1) + 4) >> 3, -tc, tc);
            int avg = (p0 + q0 + 1) >> 1;
            int np1 = p1 + clampi((p2 + avg - (p1 << 1)) >> 1, -t0, t0);
            int nq1 = q1 + clampi((q2 + avg - (q1 << 1)) >> 1, -t0, t0);
            if (on[i]) {
                s[3][i] = (int16_t)clampi(p0 + delta, 0, 255);
                s[4][i] = (int16_t)clampi(q0 - delta, 0, 255);
                if (ap) s[2][i] = (int16_t)np1;
                if (aq) s[5][i] = (int16_t)nq1;
            }
        }
    }
}

/* filter_vertical, deblock.rs:231-262 (edge between columns x-1 and x) */
static void filter_vertical(int n, uint8_t *pix, int stride, int x, int y, const EdgeParams *ep, int chroma) {
    int16_t s[8][16];
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 8; k++) s[k][i] = pix[(y + i) * stride + x - 4 + k];
    filter_lanes(n, s, ep, chroma);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 8; k++) pix[(y + i) * stride + x - 4 + k] = (uint8_t)s[k][i];
}

/* filter_horizontal, deblock.rs:264-299 (edge between rows y-1 and y) */
static void filter_horizontal(int n, uint8_t *pix, int stride, int x, int y, const EdgeParams *ep, int chroma) {
    int16_t s[8][16];
    for (int k = 0; k < 8; k++)
        for (int i = 0; i < n; i++) s[k][i] = pix[(y - 4 + k) * stride + x + i];
    filter_lanes(n, s, ep, chroma);
    int k0 = chroma ? 3 : 1, k1 = chroma ? 5 : 7;
    for (int k = k0; k < k1; k++)
        for (int i = 0; i < n; i++) pix[(y - 4 + k) * stride + x + i] = (uint8_t)s[k][i];
}

static EdgeParams edge_params(int qpp, int qpq, const uint8_t b[4], int alpha_off, int beta_off) {
    EdgeParams ep;
    int qpav = (qpp + qpq + 1) >> 1;
    int ia = clampi(qpav + alpha_off, 0, 51), ib = clampi(qpav + beta_off, 0, 51);
    for (int k = 0; k < 4; k++) {
        ep.bs[k] = b[k];
        ep.tc0[k] = (b[k] >= 1 && b[k] < 4) ? TC0[ia][b[k] - 1] : 0;
    }
    ep.alpha = ALPHA[ia];
    ep.beta = BETA[ib];
    return ep;
}

/* deblock_mb, deblock.rs:301-495 */
static void deblock_mb(Ctx *cx, int addr) {
    const rc_h264_picture *pic = cx->pic;
    const rc_h264_mb *q = &pic->mbs[addr];
    if (q->kind == RC_H264_NONE) return;
    const rc_h264_slice *sq = &pic->slices[q->slice];
    if (sq->disable_deblocking_filter_idc == 1) return;
    int mb_w = cx->mb_w, mx = addr % mb_w, my = addr / mb_w;
    const rc_h264_mb *nbs[2] = {NULL, NULL};
    if (mx > 0) nbs[0] = &pic->mbs[addr - 1];
    if (my > 0) nbs[1] = &pic->mbs[addr - mb_w];
    for (int d = 0; d < 2; d++)
        if (nbs[d] && (nbs[d]->kind == RC_H264_NONE ||
                       (sq->disable_deblocking_filter_idc == 2 && nbs[d]->slice != q->slice)))
            nbs[d] = NULL;
    int t8 = q->transform_8x8;
    uint8_t bs[2][4][4];
    memset(bs, 0, sizeof bs);
    if (is_intra(q->kind)) {
        for (int d = 0; d < 2; d++) {
            if (nbs[d]) memset(bs[d][0], 4, 4);
            for (int e = 1; e < 4; e++)
                if (!(t8 && e % 2 == 1)) memset(bs[d][e], 3, 4);
        }
    } else {
        const rc_h264_mb *ext[2] = {NULL, NULL};
        int intra_nb_[2] = {0, 0};
        for (int d = 0; d < 2; d++) {
            if (!nbs[d]) continue;
            if (is_intra(nbs[d]->kind)) intra_nb_[d] = 1;
            else ext[d] = nbs[d];
        }
        /* motion_lanes_scalar, deblock.rs:89-108 */
        uint32_t qids[2][4], pids[2][2][4];
        ref_ids8(cx, q, qids);
        for (int d = 0; d < 2; d++)
            if (ext[d]) ref_ids8(cx, ext[d], pids[d]);
        uint16_t mot[2] = {0, 0};
        for (int d = 0; d < 2; d++)
            for (int r = 0; r < 16; r++) {
                int first, rp;
                if (d == 0) { first = (r & 3) == 0; rp = first ? r + 3 : r - 1; }
                else { first = r < 4; rp = (r + 12) % 16; }
                Blk pb, qb = blk_of(q, qids, r);
                if (first) {
                    if (!ext[d]) continue;
                    pb = blk_of(ext[d], pids[d], rp);
                } else pb = blk_of(q, qids, rp);
                mot[d] |= (uint16_t)(motion_bs(pb, qb) << r);
            }
        uint16_t nzq = q->nz_mask, nz[2], keep[2];
        nz[0] = (uint16_t)(nzq | ((nzq << 1) & 0xeeee) | (ext[0] ? (ext[0]->nz_mask >> 3) & 0x1111 : 0));
        nz[1] = (uint16_t)(nzq | (nzq << 4) | (ext[1] ? ext[1]->nz_mask >> 12 : 0));
        uint16_t odd0 = t8 ? 0xaaaa : 0, odd1 = t8 ? 0xf0f0 : 0;
        keep[0] = (uint16_t)(~odd0 & (ext[0] ? 0xffff : ~0x1111));
        keep[1] = (uint16_t)(~odd1 & (ext[1] ? 0xffff : ~0x000f));
        /* bs_bytes_scalar, deblock.rs:61-78 */
        for (int d = 0; d < 2; d++)
            for (int e = 0; e < 4; e++)
                for (int k = 0; k < 4; k++) {
                    int r = d == 0 ? k * 4 + e : e * 4 + k;
                    if ((nz[d] >> r) & (keep[d] >> r) & 1) bs[d][e][k] = 2;
                    else bs[d][e][k] = (uint8_t)((mot[d] >> r) & (keep[d] >> r) & 1);
                }
        for (int d = 0; d < 2; d++)
            if (intra_nb_[d]) memset(bs[d][0], 4, 4);
    }
    int allzero = 1;
    for (int i = 0; i < 32; i++) allzero &= ((uint8_t *)bs)[i] == 0;
    if (allzero) return;
#define QP_OF(m) ((m)->kind == RC_H264_IPCM ? 0 : (int)(m)->qp)
    int q_qp = QP_OF(q);
    for (int d = 0; d < 2; d++)
        for (int e = 0; e < 4; e++) {
            if (!(bs[d][e][0] | bs[d][e][1] | bs[d][e][2] | bs[d][e][3])) continue;
            int qpp = (e == 0 && nbs[d]) ? QP_OF(nbs[d]) : q_qp;
            EdgeParams ep = edge_params(qpp, q_qp, bs[d][e], sq->alpha_offset, sq->beta_offset);
            if (ep.alpha == 0 || ep.beta == 0) continue;
            if (d == 0) filter_vertical(16, cx->y, cx->W, mx * 16 + e * 4, my * 16, &ep, 0);
            else filter_horizontal(16, cx->y, cx->W, mx * 16, my * 16 + e * 4, &ep, 0);
        }
#undef QP_OF
    for (int d = 0; d < 2; d++)
        for (int ce = 0; ce < 2; ce++) {
            int e = ce * 2;
            if (!(bs[d][e][0] | bs[d][e][1] | bs[d][e][2] | bs[d][e][3])) continue;
            EdgeParams ep[2];
            for (int c = 0; c < 2; c++) {
                int qpp = (e == 0 && nbs[d]) ? nbs[d]->qpc[c] : q->qpc[c];
                ep[c] = edge_params(qpp, q->qpc[c], bs[d][e], sq->alpha_offset, sq->beta_offset);
            }
            int off0 = ep[0].alpha == 0 || ep[0].beta == 0, off1 = ep[1].alpha == 0 || ep[1].beta == 0;
            if (off0 && off1) continue;
            int y = my * 8 + d * ce * 4, x = mx * 8 + (1 - d) * ce * 4;
            for (int c = 0; c < 2; c++) {
                if (c == 0 ? off0 : off1) continue;
                uint8_t *pl = c ? cx->v : cx->u;
                if (d == 0) filter_vertical(8, pl, cx->CW, x, y, &ep[c], 1);
                else filter_horizontal(8, pl, cx->CW, x, y, &ep[c], 1);
            }
        }
}

static int validate(int mb_w, int mb_h, const rc_h264_picture *pic) {
    if (!pic || !pic->mbs || mb_w <= 0 || mb_h <= 0) return RC_EINVAL;
    for (int a = 0; a < mb_w * mb_h; a++) {
        const rc_h264_mb *m = &pic->mbs[a];
        if (m->kind > RC_H264_INTER) return RC_EINVAL;
        if (m->kind == RC_H264_NONE) continue;
        if (m->slice >= pic->num_slices) return RC_EINVAL;
        if (m->kind == RC_H264_INTER) {
            const rc_h264_slice *sl = &pic->slices[m->slice];
            for (int l = 0; l < 2; l++)
                for (int b = 0; b < 4; b++) {
                    int r = m->ref_idx[l][b];
                    if (r >= sl->num_ref[l]) return RC_EINVAL;
                }
            for (int b = 0; b < 4; b++)
                if (m->wp[b] != 0xff && m->wp[b] >= pic->num_weights) return RC_EINVAL;
        }
        if (m->kind == RC_H264_IPCM && m->coef_off + 384 > pic->num_levels) return RC_EINVAL;
    }
    return 0;
}

static int recon(int mb_w, int mb_h, const rc_h264_picture *pic, const uint8_t *const *ry,
                 const uint8_t *const *ru, const uint8_t *const *rv, uint8_t *y, uint8_t *u,
                 uint8_t *v, int filter) {
    int rc = validate(mb_w, mb_h, pic);
    if (rc) return rc;
    init_zigzag8();
    Ctx *cx = (Ctx *)malloc(sizeof(Ctx));
    if (!cx) return RC_ENOMEM;
    cx->mb_w = mb_w; cx->mb_h = mb_h; cx->W = mb_w * 16; cx->H = mb_h * 16;
    cx->CW = mb_w * 8; cx->CH = mb_h * 8; cx->pic = pic;
    cx->ry = ry; cx->ru = ru; cx->rv = rv; cx->y = y; cx->u = u; cx->v = v;
    oracle_h264_level_scale(pic->scaling4, pic->scaling8, cx->ls4, cx->ls8);
    Coefs s;
    for (int a = 0; a < mb_w * mb_h && !rc; a++) {
        const rc_h264_mb *m = &pic->mbs[a];
        int mbx = a % mb_w, mby = a / mb_w;
        switch (m->kind) {
        case RC_H264_NONE: break;
        case RC_H264_IPCM: write_pcm(cx, m, mbx, mby); break;
        case RC_H264_INTER:
            rc = place_levels(cx, m, &s);
            if (rc) break;
            predict_inter(cx, m, mbx, mby);
            /* reconstruct_inter_residual, slicedec.rs:1390-1402 */
            if (m->transform_8x8)
                for (int b8 = 0; b8 < 4; b8++) add_luma8(cx, &s, mbx, mby, b8);
            else
                for (int r = 0; r < 16; r++) add_luma4(cx, &s, mbx, mby, r);
            add_chroma(cx, &s, mbx, mby);
            break;
        default:
            rc = place_levels(cx, m, &s);
            if (!rc) recon_intra(cx, m, &s, mbx, mby);
        }
    }
    if (!rc && filter)
        for (int a = 0; a < mb_w * mb_h; a++) deblock_mb(cx, a);
    free(cx);
    return rc;
}

int oracle_h264_recon(int mb_w, int mb_h, const rc_h264_picture *pic, const uint8_t *const *ry,
                      const uint8_t *const *ru, const uint8_t *const *rv, uint8_t *y, uint8_t *u,
                      uint8_t *v) {
    return recon(mb_w, mb_h, pic, ry, ru, rv, y, u, v, 1);
}

int oracle_h264_recon_nofilter(int mb_w, int mb_h, const rc_h264_picture *pic,
                               const uint8_t *const *ry, const uint8_t *const *ru,
                               const uint8_t *const *rv, uint8_t *y, uint8_t *u, uint8_t *v) {
    return recon(mb_w, mb_h, pic, ry, ru, rv, y, u, v, 0);
}

void oracle_h264_deblock(int mb_w, int mb_h, const rc_h264_picture *pic, uint8_t *y, uint8_t *u,
                         uint8_t *v) {
    Ctx *cx = (Ctx *)malloc(sizeof(Ctx));
    if (!cx) return;
    init_zigzag8();
    cx->mb_w = mb_w; cx->mb_h = mb_h; cx->W = mb_w * 16; cx->H = mb_h * 16;
    cx->CW = mb_w * 8; cx->CH = mb_h * 8; cx->pic = pic; cx->y = y; cx->u = u; cx->v = v;
    for (int a = 0; a < mb_w * mb_h; a++) deblock_mb(cx, a);
    free(cx);
}
