// h264_kernels.cu — H.264 block reconstruction on sm_103a.
//
// Three launches per picture:
//
//  h264_mb_kernel       one CTA (256 threads) per macroblock, all in parallel.
//                       Inter MBs: dequantisation (scale4/scale8, chroma DC
//                       Hadamard), 4x4/8x8 inverse transforms, 6-tap luma and
//                       bilinear chroma motion compensation with edge
//                       extension by coordinate clamp, default / explicit
//                       weighted prediction, residual add and clip, fused.
//                       I_PCM MBs are copied.  Every MB also gets its
//                       loop-filter parameters (boundary strengths, QPs),
//                       which depend on syntax only.
//  h264_intra_kernel    persistent; one warp per intra MB in anti-diagonal
//                       order (key x + 2y); a warp waits (acquire loads,
//                       capped spin) for its intra neighbours L, T, TR, TL,
//                       then predicts and adds the residual block by block
//                       in decode order on a shared-memory canvas.
//  h264_deblock_kernel  one warp per MB row, walking the row left to right
//                       on a shared-memory tile (the reference's MB-raster
//                       filter order, src/h264/dec/slicedec.rs:184-208): row
//                       y filters MB x once row y-1 has published MBs 0..x,
//                       so every edge sees exactly the samples it would in
//                       raster order.
//
// Arithmetic follows src/h264/dec/{transform,intra,inter,deblock}.rs and the
// reconstruction half of slicedec.rs; citations at each function.
#include <stdint.h>
#include <string.h>

#include "recon_internal.h"

namespace {

// ---- tables --------------------------------------------------------------
__constant__ uint8_t cZZ4[16] = {0, 1, 4, 8, 5, 2, 3, 6, 9, 12, 13, 10, 7, 11, 14, 15};
__constant__ uint8_t cZZ8[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                                 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                                 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                                 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
__constant__ uint8_t cALPHA[52] = {0,  0,  0,  0,  0,  0,  0,  0,   0,   0,   0,   0,   0,   0,
                                   0,  0,  4,  4,  5,  6,  7,  8,   9,   10,  12,  13,  15,  17,
                                   20, 22, 25, 28, 32, 36, 40, 45,  50,  56,  63,  71,  80,  90,
                                   101, 113, 127, 144, 162, 182, 203, 226, 255, 255};
__constant__ uint8_t cBETA[52] = {0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  2,  2,
                                  2,  3,  3,  3,  3,  4,  4,  4,  6,  6,  7,  7,  8,  8,  9,  9,  10, 10,
                                  11, 11, 12, 12, 13, 13, 14, 14, 15, 15, 16, 16, 17, 17, 18, 18};
__constant__ uint8_t cTC0[52][3] = {
    {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},   {0, 0, 0},   {0, 0, 0},
    {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 0},   {0, 0, 0},   {0, 0, 0},
    {0, 0, 0},  {0, 0, 0},  {0, 0, 0},  {0, 0, 1},  {0, 0, 1},   {0, 0, 1},   {0, 0, 1},
    {0, 1, 1},  {0, 1, 1},  {1, 1, 1},  {1, 1, 1},  {1, 1, 1},   {1, 1, 1},   {1, 1, 2},
    {1, 1, 2},  {1, 1, 2},  {1, 1, 2},  {1, 2, 3},  {1, 2, 3},   {2, 2, 3},   {2, 2, 4},
    {2, 3, 4},  {2, 3, 4},  {3, 3, 5},  {3, 4, 6},  {3, 4, 6},   {4, 5, 7},   {4, 5, 8},
    {4, 6, 9},  {5, 7, 10}, {6, 8, 11}, {6, 8, 13}, {7, 10, 14}, {8, 11, 16}, {9, 12, 18},
    {10, 13, 20}, {11, 15, 23}, {13, 17, 25}};
// decode order of 4x4 blocks (BLK4_XY) and its inverse (RASTER_TO_BLK4)
__constant__ uint8_t cBLK4X[16] = {0, 1, 0, 1, 2, 3, 2, 3, 0, 1, 0, 1, 2, 3, 2, 3};
__constant__ uint8_t cBLK4Y[16] = {0, 0, 1, 1, 0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 3, 3};
__constant__ uint8_t cR2B[16] = {0, 1, 4, 5, 2, 3, 6, 7, 8, 9, 12, 13, 10, 11, 14, 15};

constexpr uint32_t ID_NONE = 0xffffffffu;

// ---- small helpers -------------------------------------------------------
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }
__device__ __forceinline__ int clip255(int v) { return min(max(v, 0), 255); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
__device__ __forceinline__ int32_t wshl(int32_t a, int s) { return (int32_t)((uint32_t)a << s); }
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ bool is_intra(int k) { return k >= RC_H264_I4x4 && k <= RC_H264_IPCM; }
// kinds reconstructed by the wavefront (everything else is done by h264_mb_kernel)
__device__ __forceinline__ bool wave_intra(int k) { return k >= RC_H264_I4x4 && k <= RC_H264_I16x16; }

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ bool aborted(const uint32_t *err) {
    return (*(const volatile uint32_t *)err & RC_DEV_ERR_TIMEOUT) != 0;
}
// Wait until *f == epoch; false after `limit` polls or once another warp has
// recorded a timeout (the caller then abandons the launch instead of
// spinning for ever).
__device__ bool wait_flag(const uint32_t *f, uint32_t epoch, uint32_t limit, const uint32_t *err) {
    uint32_t it = 0;
    while (ld_acquire(f) != epoch) {
        if (++it > limit) return false;
        if ((it & 63) == 0 && aborted(err)) return false;
        __nanosleep(it < 32 ? 32 : 256);
    }
    return true;
}

// scale4 / scale8, src/h264/dec/transform.rs:30-46
__device__ __forceinline__ int32_t scale4(int32_t c, int32_t ls, int qp) {
    return qp >= 24 ? wshl(wmul(c, ls), qp / 6 - 4) : (wadd(wmul(c, ls), 1 << (3 - qp / 6)) >> (4 - qp / 6));
}
__device__ __forceinline__ int32_t scale8(int32_t c, int32_t ls, int qp) {
    return qp >= 36 ? wshl(wmul(c, ls), qp / 6 - 6) : (wadd(wmul(c, ls), 1 << (5 - qp / 6)) >> (6 - qp / 6));
}

// luma_dc_dequant, src/h264/dec/transform.rs:48-75 (one thread)
__device__ void luma_dc_dequant(int32_t c[16], int qp, int32_t ls00) {
    int32_t t[16];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int32_t s01 = c[i * 4] + c[i * 4 + 1], d01 = c[i * 4] - c[i * 4 + 1];
        int32_t s23 = c[i * 4 + 2] + c[i * 4 + 3], d23 = c[i * 4 + 2] - c[i * 4 + 3];
        t[i * 4] = s01 + s23; t[i * 4 + 1] = s01 - s23; t[i * 4 + 2] = d01 - d23; t[i * 4 + 3] = d01 + d23;
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        int32_t s01 = t[j] + t[4 + j], d01 = t[j] - t[4 + j];
        int32_t s23 = t[8 + j] + t[12 + j], d23 = t[8 + j] - t[12 + j];
        int32_t f[4] = {s01 + s23, s01 - s23, d01 - d23, d01 + d23};
#pragma unroll
        for (int i = 0; i < 4; i++)
            c[i * 4 + j] = qp >= 36 ? wshl(wmul(f[i], ls00), qp / 6 - 6)
                                    : (wadd(wmul(f[i], ls00), 1 << (5 - qp / 6)) >> (6 - qp / 6));
    }
}

// chroma_dc_dequant_420, src/h264/dec/transform.rs:77-91 (one thread)
__device__ void chroma_dc_dequant(int32_t c[4], int qp, int32_t ls00) {
    int32_t s0 = wadd(c[0], c[1]), d0 = wsub(c[0], c[1]), s1 = wadd(c[2], c[3]), d1 = wsub(c[2], c[3]);
    int32_t f[4] = {wadd(s0, s1), wadd(d0, d1), wsub(s0, s1), wsub(d0, d1)};
#pragma unroll
    for (int k = 0; k < 4; k++) c[k] = wshl(wmul(f[k], ls00), qp / 6) >> 5;
}

// One pass of the 4x4 inverse transform over 4 values with stride st
// (idct4_add, src/h264/dec/transform.rs:98-118).
__device__ __forceinline__ void idct4_1d(int32_t *d, int st) {
    int32_t r0 = d[0], r1 = d[st], r2 = d[2 * st], r3 = d[3 * st];
    int32_t e = r0 + r2, f = r0 - r2, g = (r1 >> 1) - r3, h = r1 + (r3 >> 1);
    d[0] = e + h; d[st] = f + g; d[2 * st] = f - g; d[3 * st] = e - h;
}
// idct8_1d, src/h264/dec/transform.rs:132-160, in place with stride st
__device__ __forceinline__ void idct8_1d(int32_t *d, int st) {
    int32_t x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = d[i * st];
    int32_t a0 = x[0] + x[4], a4 = x[0] - x[4], a2 = (x[2] >> 1) - x[6], a6 = x[2] + (x[6] >> 1);
    int32_t b0 = a0 + a6, b2 = a4 + a2, b4 = a4 - a2, b6 = a0 - a6;
    int32_t a1 = -x[3] + x[5] - x[7] - (x[7] >> 1);
    int32_t a3 = x[1] + x[7] - x[3] - (x[3] >> 1);
    int32_t a5 = -x[1] + x[7] + x[5] + (x[5] >> 1);
    int32_t a7 = x[3] + x[5] + x[1] + (x[1] >> 1);
    int32_t b1 = a1 + (a7 >> 2), b7 = a7 - (a1 >> 2), b3 = a3 + (a5 >> 2), b5 = (a3 >> 2) - a5;
    d[0] = b0 + b7; d[st] = b2 + b5; d[2 * st] = b4 + b3; d[3 * st] = b6 + b1;
    d[4 * st] = b6 - b1; d[5 * st] = b4 - b3; d[6 * st] = b2 - b5; d[7 * st] = b0 - b7;
}

// ---- motion compensation (src/h264/dec/inter.rs) ------------------------
struct Ref {
    const uint8_t *p;
    int pitch, w, h;
};
// window sample with edge extension by coordinate clamp (copy_clamped,
// src/h264/dec/picture.rs:723-735)
__device__ __forceinline__ int rs(const Ref &r, int x, int y) {
    return __ldg(r.p + clampi(y, 0, r.h - 1) * r.pitch + clampi(x, 0, r.w - 1));
}
__device__ __forceinline__ int tap6(int a, int b, int c, int d, int e, int f) { return a - 5 * b + 20 * c + 20 * d - 5 * e + f; }
__device__ __forceinline__ int avg2(int a, int b) { return (a + b + 1) >> 1; }
__device__ __forceinline__ int htap(const Ref &r, int x, int y) {
    return tap6(rs(r, x - 2, y), rs(r, x - 1, y), rs(r, x, y), rs(r, x + 1, y), rs(r, x + 2, y), rs(r, x + 3, y));
}
__device__ __forceinline__ int vtap(const Ref &r, int x, int y) {
    return tap6(rs(r, x, y - 2), rs(r, x, y - 1), rs(r, x, y), rs(r, x, y + 1), rs(r, x, y + 2), rs(r, x, y + 3));
}
// mc_luma_win_scalar, inter.rs:73-213, for the sample at integer position (x, y)
__device__ int luma_sample(const Ref &r, int x, int y, int fx, int fy) {
    if (fx == 0 && fy == 0) return rs(r, x, y);
    if (fy == 0) {
        int b = clip255((htap(r, x, y) + 16) >> 5);
        return fx == 1 ? avg2(rs(r, x, y), b) : fx == 2 ? b : avg2(rs(r, x + 1, y), b);
    }
    if (fx == 0) {
        int h = clip255((vtap(r, x, y) + 16) >> 5);
        return fy == 2 ? h : avg2(fy == 1 ? rs(r, x, y) : rs(r, x, y + 1), h);
    }
    if (fx == 2 || fy == 2) {
        int b1[6];
#pragma unroll
        for (int j = 0; j < 6; j++) b1[j] = htap(r, x, y + j - 2);
        int j = clip255((tap6(b1[0], b1[1], b1[2], b1[3], b1[4], b1[5]) + 512) >> 10);
        if (fx == 2 && fy == 2) return j;
        if (fx == 2) return avg2(clip255(((fy == 1 ? b1[2] : b1[3]) + 16) >> 5), j);
        return avg2(clip255((vtap(r, x + (fx == 1 ? 0 : 1), y) + 16) >> 5), j);
    }
    int t = htap(r, x, y + (fy == 1 ? 0 : 1));
    int v = vtap(r, x + (fx == 1 ? 0 : 1), y);
    return avg2(clip255((t + 16) >> 5), clip255((v + 16) >> 5));
}
// mc_chroma_win_scalar, inter.rs:217-247, one sample at integer position (x, y)
__device__ __forceinline__ int chroma_sample(const Ref &r, int x, int y, int fx, int fy) {
    if ((fx | fy) == 0) return rs(r, x, y);
    int v = (8 - fx) * (8 - fy) * rs(r, x, y) + fx * (8 - fy) * rs(r, x + 1, y) + (8 - fx) * fy * rs(r, x, y + 1) +
            fx * fy * rs(r, x + 1, y + 1);
    return (v + 32) >> 6;
}
// weighted_store_scalar, inter.rs:286-352, one sample of one resolved
// component weighting (after Weight::simplify)
__device__ __forceinline__ int weigh(int a, int b, bool u0, bool u1, bool ex, int lw, int w0, int w1, int o0, int o1) {
    if (u0 && u1)
        return ex ? clip255(((a * w0 + b * w1 + (1 << lw)) >> (lw + 1)) + ((o0 + o1 + 1) >> 1)) : (a + b + 1) >> 1;
    int s = u0 ? a : b;
    if (!ex) return s;
    int wt = u0 ? w0 : w1, o = u0 ? o0 : o1;
    int round = lw >= 1 ? 1 << (lw - 1) : 0;
    return clip255(((s * wt + round) >> lw) + o);
}

__device__ __forceinline__ void set_error(uint32_t *e, uint32_t code) { atomicOr(e, code); }

__device__ void compute_db(const H264Launch &P, const rc_h264_mb &q, const rc_h264_mb &left, const rc_h264_mb &top,
                           int addr, int lane, DbMb *out);

// ===========================================================================
// Kernel 1: inter MBs (prediction + residual) and I_PCM, one CTA per MB.
// ===========================================================================
__global__ void __launch_bounds__(256) h264_mb_kernel(H264Launch P) {
    __shared__ __align__(16) rc_h264_mb m;
    __shared__ int32_t coef[256];
    __shared__ int32_t coefc[128];
    __shared__ uint8_t predy[256];
    __shared__ uint8_t predc[128];
    __shared__ __align__(16) rc_h264_mb nbr[2];  // left, top (loop-filter parameters)
    __shared__ uint32_t nzl, nzc;
    const int t = threadIdx.x, addr = blockIdx.x;
    const int mbx = addr % P.mb_w, mby = addr / P.mb_w;
    constexpr int RW = (int)(sizeof(rc_h264_mb) / 4);
    if (t < RW) ((uint32_t *)&m)[t] = __ldg((const uint32_t *)(P.mbs + addr) + t);
    else if (t < 2 * RW) {
        if (mbx > 0) ((uint32_t *)&nbr[0])[t - RW] = __ldg((const uint32_t *)(P.mbs + addr - 1) + t - RW);
    } else if (t < 3 * RW) {
        if (mby > 0) ((uint32_t *)&nbr[1])[t - 2 * RW] = __ldg((const uint32_t *)(P.mbs + addr - P.mb_w) + t - 2 * RW);
    }
    if (t == 0) { nzl = 0; nzc = 0; }
    coef[t] = 0;
    if (t < 128) coefc[t] = 0;
    __syncthreads();
    if (t < 32) compute_db(P, m, nbr[0], nbr[1], addr, t, P.db + addr);
    const int kind = m.kind;
    if (kind == RC_H264_NONE || kind > RC_H264_INTER) return;
    uint8_t *Y = P.dpb + (size_t)P.out_slot * P.slot_bytes;
    uint8_t *U = Y + P.u_off, *V = Y + P.v_off;
    if (kind == RC_H264_IPCM) {  // write_pcm, src/h264/dec/slicedec.rs:1404-1424
        if (m.coef_off + 384ull > P.num_levels) { if (t == 0) set_error(P.error, RC_DEV_ERR_RECORD); return; }
        const int16_t *s = P.levels + m.coef_off;
        Y[(size_t)(mby * 16 + (t >> 4)) * P.pitch + mbx * 16 + (t & 15)] = (uint8_t)s[t];
        if (t < 128) {
            int c = t >> 6, x = t & 7, y = (t >> 3) & 7;
            (c ? V : U)[(size_t)(mby * 8 + y) * P.cpitch + mbx * 8 + x] = (uint8_t)s[256 + t];
        }
        return;
    }
    if (m.slice >= P.num_slices) { if (t == 0) set_error(P.error, RC_DEV_ERR_RECORD); return; }
    const rc_h264_slice *sl = P.slices + m.slice;
    const bool intra = kind != RC_H264_INTER;
    const int t8 = m.transform_8x8, i16 = kind == RC_H264_I16x16;
    const int nl = __popc(m.luma_coded & (t8 ? 0xf : 0xffff)), ndc = __popc(m.dc_coded & 6);
    const int nlum = (i16 && (m.dc_coded & 1)) ? 16 : 0;
    const unsigned long long need =
        nlum + (unsigned long long)nl * (t8 ? 64 : 16) + ndc * 4 + __popc(m.chroma_coded) * 16;
    if (m.coef_off + need > P.num_levels) { if (t == 0) set_error(P.error, RC_DEV_ERR_RECORD); return; }
    __shared__ uint32_t ibits;  // intra: availability (bits 0..3) and waits (bits 4..7)
    if (intra) {
        if (t == 0) ibits = 0;
        __syncthreads();
        if (t < 4) {
            // start_mb neighbour availability + intra_nb, slicedec.rs:489-508, 525-530
            const int dx = t == 0 ? -1 : t == 2 ? 1 : t == 3 ? -1 : 0, dy = t == 0 ? 0 : -1;
            const int nx = mbx + dx, ny = mby + dy;
            if (nx >= 0 && ny >= 0 && nx < P.mb_w) {
                const rc_h264_mb *pm = P.mbs + ny * P.mb_w + nx;
                const int nk = __ldg(&pm->kind);
                const bool a = nk != RC_H264_NONE && __ldg(&pm->slice) == m.slice && (!P.constrained_intra || is_intra(nk));
                // the top-right MB is read only by Intra4x4 block (3,0) in modes 3 / 7 (diagonal down-left,
                // vertical-left) and by the top-using modes of Intra8x8 block 1 (intra.rs:31-62, 199-233)
                bool uses = true;
                if (t == 2)
                    uses = kind == RC_H264_I4x4 ? (m.intra_modes[3] == 3 || m.intra_modes[3] == 7)
                           : kind == RC_H264_I8x8 ? (m.intra_modes[2] != 1 && m.intra_modes[2] != 8) : false;
                uint32_t b = a ? (1u << t) : 0;
                if (a && uses && wave_intra(nk)) b |= 16u << t;
                atomicOr(&ibits, b);
            }
        }
    }
    if (!intra) {
    // ---- prediction (mc_rect, slicedec.rs:996-1087), one luma sample per thread
    {
        const int x = t & 15, y = t >> 4, k = (y >> 2) * 4 + (x >> 2), b8 = (y >> 3) * 2 + (x >> 3);
        int v[2] = {0, 0};
        bool u[2] = {false, false};
#pragma unroll
        for (int l = 0; l < 2; l++) {
            int ri = m.ref_idx[l][b8];
            if (ri < 0) continue;
            int slot = ri < min(__ldg(&sl->num_ref[l]), RC_H264_MAX_REFS) ? __ldg(&sl->ref_slot[l][ri]) : -1;
            if (slot < 0 || slot >= P.dpb_slots) { set_error(P.error, RC_DEV_ERR_RECORD); continue; }
            u[l] = true;
            Ref r{P.dpb + (size_t)slot * P.slot_bytes, P.pitch, P.W, P.H};
            int mvx = m.mv[l][k][0], mvy = m.mv[l][k][1];
            v[l] = luma_sample(r, mbx * 16 + x + (mvx >> 2), mby * 16 + y + (mvy >> 2), mvx & 3, mvy & 3);
        }
        int wi = m.wp[b8];
        const rc_h264_weight *w = (wi != 0xff && wi < P.num_weights) ? P.weights + wi : nullptr;
        bool ex = w && (w->explicit_mask & 1);
        predy[t] = (uint8_t)weigh(v[0], v[1], u[0], u[1], ex, ex ? w->log_wd[0] : 0, ex ? w->w0[0] : 0,
                                  ex ? w->w1[0] : 0, ex ? w->o0[0] : 0, ex ? w->o1[0] : 0);
    }
    if (t < 128) {
        const int c = t >> 6, x = t & 7, y = (t >> 3) & 7, k = (y >> 1) * 4 + (x >> 1), b8 = (y >> 2) * 2 + (x >> 2);
        int v[2] = {0, 0};
        bool u[2] = {false, false};
#pragma unroll
        for (int l = 0; l < 2; l++) {
            int ri = m.ref_idx[l][b8];
            if (ri < 0) continue;
            int slot = ri < min(__ldg(&sl->num_ref[l]), RC_H264_MAX_REFS) ? __ldg(&sl->ref_slot[l][ri]) : -1;
            if (slot < 0 || slot >= P.dpb_slots) continue;
            u[l] = true;
            Ref r{P.dpb + (size_t)slot * P.slot_bytes + (c ? P.v_off : P.u_off), P.cpitch, P.CW, P.CH};
            int mvx = m.mv[l][k][0], mvy = m.mv[l][k][1];
            v[l] = chroma_sample(r, mbx * 8 + x + (mvx >> 3), mby * 8 + y + (mvy >> 3), mvx & 7, mvy & 7);
        }
        int wi = m.wp[b8];
        const rc_h264_weight *w = (wi != 0xff && wi < P.num_weights) ? P.weights + wi : nullptr;
        int cc = 1 + c;
        bool ex = w && (w->explicit_mask >> cc & 1);
        predc[t] = (uint8_t)weigh(v[0], v[1], u[0], u[1], ex, ex ? w->log_wd[cc] : 0, ex ? w->w0[cc] : 0,
                                  ex ? w->w1[cc] : 0, ex ? w->o0[cc] : 0, ex ? w->o1[cc] : 0);
    }
    }

    // ---- level placement + dequantisation (put_luma4/8, put_luma_dc,
    // put_chroma_dc/ac, slicedec.rs:1462-1555); lists: luma4 intra 0 / inter 3,
    // luma8 intra 0 / inter 1, chroma intra 1+c / inter 4+c
    const int16_t *lv = P.levels + m.coef_off;
    const int qp = m.qp, l4 = intra ? 0 : 3, l8 = intra ? 0 : 1, lc = intra ? 1 : 4;
    if (nlum && t == 0) {  // put_luma_dc, slicedec.rs:1501-1515
        int32_t c[16];
        for (int k = 0; k < 16; k++) c[cZZ4[k]] = lv[k];
        luma_dc_dequant(c, qp, __ldg(P.ls4 + (0 * 6 + qp % 6) * 16));
        uint32_t bits = 0;
        for (int r = 0; r < 16; r++)
            if (c[r]) { coef[r * 16] = c[r]; bits |= 1u << r; }
        atomicOr(&nzl, bits);
    }
    if (t8) {
        int b8 = t >> 6, kk = t & 63;
        if (m.luma_coded >> b8 & 1) {
            int l = lv[nlum + __popc(m.luma_coded & ((1u << b8) - 1)) * 64 + kk];
            if (l) {
                int p = cZZ8[kk];
                coef[b8 * 64 + p] = scale8(l, __ldg(P.ls8 + (l8 * 6 + qp % 6) * 64 + p), qp);
                atomicOr(&nzl, 1u << b8);
            }
        }
    } else {
        int r = t >> 4, kk = t & 15;
        if (kk >= i16 && (m.luma_coded >> r & 1)) {
            int l = lv[nlum + __popc(m.luma_coded & ((1u << r) - 1)) * 16 + kk];
            if (l) {
                int p = cZZ4[kk];
                coef[r * 16 + p] = scale4(l, __ldg(P.ls4 + (l4 * 6 + qp % 6) * 16 + p), qp);
                atomicOr(&nzl, 1u << r);
            }
        }
    }
    const int off_dc = nlum + nl * (t8 ? 64 : 16), off_ac = off_dc + ndc * 4;
    if (t < 2 && (m.dc_coded >> (1 + t) & 1)) {
        int c = t, at = off_dc + ((c == 1 && (m.dc_coded & 2)) ? 4 : 0), qpc = m.qpc[c];
        int32_t d[4] = {lv[at], lv[at + 1], lv[at + 2], lv[at + 3]};
        chroma_dc_dequant(d, qpc, __ldg(P.ls4 + ((lc + c) * 6 + qpc % 6) * 16));
        for (int b = 0; b < 4; b++)
            if (d[b]) { coefc[c * 64 + b * 16] = d[b]; atomicOr(&nzc, 1u << (c * 4 + b)); }
    }
    if (t < 128) {
        int c = t >> 6, b = (t >> 4) & 3, kk = t & 15, bit = c * 4 + b;
        if (kk >= 1 && (m.chroma_coded >> bit & 1)) {
            int l = lv[off_ac + __popc(m.chroma_coded & ((1u << bit) - 1)) * 16 + kk];
            if (l) {
                int qpc = m.qpc[c], p = cZZ4[kk];
                coefc[c * 64 + b * 16 + p] = scale4(l, __ldg(P.ls4 + ((lc + c) * 6 + qpc % 6) * 16 + p), qpc);
                atomicOr(&nzc, 1u << bit);
            }
        }
    }
    __syncthreads();
    // ---- inverse transforms: rows, then columns
    if (t8) {
        if (t < 32 && (nzl >> (t >> 3) & 1)) idct8_1d(coef + (t >> 3) * 64 + (t & 7) * 8, 1);
    } else if (t < 64 && (nzl >> (t >> 2) & 1)) idct4_1d(coef + (t >> 2) * 16 + (t & 3) * 4, 1);
    if (t >= 64 && t < 96 && (nzc >> ((t - 64) >> 2) & 1)) idct4_1d(coefc + ((t - 64) >> 2) * 16 + (t & 3) * 4, 1);
    __syncthreads();
    if (t8) {
        if (t < 32 && (nzl >> (t >> 3) & 1)) idct8_1d(coef + (t >> 3) * 64 + (t & 7), 8);
    } else if (t < 64 && (nzl >> (t >> 2) & 1)) idct4_1d(coef + (t >> 2) * 16 + (t & 3), 4);
    if (t >= 64 && t < 96 && (nzc >> ((t - 64) >> 2) & 1)) idct4_1d(coefc + ((t - 64) >> 2) * 16 + (t & 3), 4);
    __syncthreads();
    if (intra) {
        // residual samples ((v + 32) >> 6, idct4_add / idct8_add) and the
        // prediction parameters for the intra wavefront
        int16_t *res = P.ires + (size_t)addr * 384;
        {
            const int x = t & 15, y = t >> 4;
            int r = 0;
            if (t8) {
                int b8 = (y >> 3) * 2 + (x >> 3);
                if (nzl >> b8 & 1) r = (coef[b8 * 64 + (y & 7) * 8 + (x & 7)] + 32) >> 6;
            } else {
                int b = (y >> 2) * 4 + (x >> 2);
                if (nzl >> b & 1) r = (coef[b * 16 + (y & 3) * 4 + (x & 3)] + 32) >> 6;
            }
            res[t] = (int16_t)max(-32768, min(32767, r));
        }
        if (t < 128) {
            const int c = t >> 6, x = t & 7, y = (t >> 3) & 7, blk = c * 4 + (y >> 2) * 2 + (x >> 2);
            int r = (nzc >> blk & 1) ? (coefc[blk * 16 + (y & 3) * 4 + (x & 3)] + 32) >> 6 : 0;
            res[256 + t] = (int16_t)max(-32768, min(32767, r));
        }
        if (t == 0) {
            IntraInfo in;
            in.kind = (uint8_t)kind;
            in.t8 = (uint8_t)t8;
            in.i16_mode = m.i16_mode;
            in.chroma_mode = m.chroma_mode;
            in.nb = (uint8_t)(ibits & 15);
            in.wait = (uint8_t)(ibits >> 4);
            in.pad0 = in.pad1 = 0;
            for (int i = 0; i < 16; i++) in.modes[i] = m.intra_modes[i];
            in.pad2[0] = in.pad2[1] = 0;
            P.iinfo[addr] = in;
        }
        return;
    }
    // ---- residual add + clip, store
    {
        const int x = t & 15, y = t >> 4;
        int v = predy[t];
        if (t8) {
            int b8 = (y >> 3) * 2 + (x >> 3);
            if (nzl >> b8 & 1) v = clip255(v + ((coef[b8 * 64 + (y & 7) * 8 + (x & 7)] + 32) >> 6));
        } else {
            int r = (y >> 2) * 4 + (x >> 2);
            if (nzl >> r & 1) v = clip255(v + ((coef[r * 16 + (y & 3) * 4 + (x & 3)] + 32) >> 6));
        }
        Y[(size_t)(mby * 16 + y) * P.pitch + mbx * 16 + x] = (uint8_t)v;
    }
    if (t < 128) {
        const int c = t >> 6, x = t & 7, y = (t >> 3) & 7, blk = c * 4 + (y >> 2) * 2 + (x >> 2);
        int v = predc[t];
        if (nzc >> blk & 1) v = clip255(v + ((coefc[blk * 16 + (y & 3) * 4 + (x & 3)] + 32) >> 6));
        (c ? V : U)[(size_t)(mby * 8 + y) * P.cpitch + mbx * 8 + x] = (uint8_t)v;
    }
}

// ===========================================================================
// Kernel 2: intra + deblocking wavefront, one warp per task.
// ===========================================================================
struct __align__(16) WarpSmem {
    IntraInfo q;          // the task's MB (modes, availability)
    int16_t res[384];     // residual samples: 16x16 luma, then 8x8 Cb, 8x8 Cr
    uint8_t cy[17 * 32];  // luma canvas: rows -1..15, cols -1..30 -> [(r+1)*32 + c+1]
    uint8_t cc[2][9 * 12];  // chroma canvas: rows -1..7, cols -1..10
    int32_t e[32];       // reference samples: top 0..15, left 16..23, corner 24
    int32_t f[32];       // smoothed reference samples (8x8)
};

__device__ __forceinline__ int cvy(const WarpSmem &S, int r, int c) { return S.cy[(r + 1) * 32 + c + 1]; }

struct Avail {
    bool left, top, tl, tr;
};

// pred_nxn, src/h264/dec/intra.rs:64-192, one sample (x, y) of an n x n block
// with reference samples top[0..2n), left[0..n), corner tl
__device__ int pred_nxn_px(int mode, const int32_t *top, const int32_t *left, int tl, int n, Avail a, int x, int y) {
#define ET(i) ((i) < 0 ? tl : top[(i)])
#define EL(i) ((i) < 0 ? tl : left[(i)])
    switch (mode) {
    case 0: return ET(x);
    case 1: return EL(y);
    case 2: {
        int shift = n == 4 ? 2 : 3, st = 0, sl = 0;
        for (int i = 0; i < n; i++) { st += top[i]; sl += left[i]; }
        if (a.top && a.left) return (st + sl + n) >> (shift + 1);
        if (a.left) return (sl + (n >> 1)) >> shift;
        if (a.top) return (st + (n >> 1)) >> shift;
        return 128;
    }
    case 3:
        if (x == n - 1 && y == n - 1) return (ET(2 * n - 2) + 3 * ET(2 * n - 1) + 2) >> 2;
        return (ET(x + y) + 2 * ET(x + y + 1) + ET(x + y + 2) + 2) >> 2;
    case 4:
        if (x > y) return (ET(x - y - 2) + 2 * ET(x - y - 1) + ET(x - y) + 2) >> 2;
        if (x < y) return (EL(y - x - 2) + 2 * EL(y - x - 1) + EL(y - x) + 2) >> 2;
        return (ET(0) + 2 * tl + EL(0) + 2) >> 2;
    case 5: {
        int z = 2 * x - y, i = x - (y >> 1);
        if (z >= 0 && (z & 1) == 0) return (ET(i - 1) + ET(i) + 1) >> 1;
        if (z > 0) return (ET(i - 2) + 2 * ET(i - 1) + ET(i) + 2) >> 2;
        if (z == -1) return (EL(0) + 2 * tl + ET(0) + 2) >> 2;
        return (EL(y - 2 * x - 1) + 2 * EL(y - 2 * x - 2) + EL(y - 2 * x - 3) + 2) >> 2;
    }
    case 6: {
        int z = 2 * y - x, i = y - (x >> 1);
        if (z >= 0 && (z & 1) == 0) return (EL(i - 1) + EL(i) + 1) >> 1;
        if (z > 0) return (EL(i - 2) + 2 * EL(i - 1) + EL(i) + 2) >> 2;
        if (z == -1) return (EL(0) + 2 * tl + ET(0) + 2) >> 2;
        return (ET(x - 2 * y - 1) + 2 * ET(x - 2 * y - 2) + ET(x - 2 * y - 3) + 2) >> 2;
    }
    case 7: {
        int i = x + (y >> 1);
        if ((y & 1) == 0) return (ET(i) + ET(i + 1) + 1) >> 1;
        return (ET(i) + 2 * ET(i + 1) + ET(i + 2) + 2) >> 2;
    }
    default: {
        int zmax = 2 * n - 3, z = x + 2 * y, i = y + (x >> 1);
        if (z < zmax && (z & 1) == 0) return (EL(i) + EL(i + 1) + 1) >> 1;
        if (z < zmax) return (EL(i) + 2 * EL(i + 1) + EL(i + 2) + 2) >> 2;
        if (z == zmax) return (EL(n - 2) + 3 * EL(n - 1) + 2) >> 2;
        return EL(n - 1);
    }
    }
#undef ET
#undef EL
}

// load_edge, src/h264/dec/intra.rs:31-62, into S.e (lanes 0..24)
__device__ __forceinline__ void load_edge(WarpSmem &S, int lane, int bx0, int by0, int n, Avail a) {
    if (lane < 16) {
        int v = 128;
        if (a.top && lane < 2 * n) v = cvy(S, by0 - 1, bx0 + ((lane < n || a.tr) ? lane : n - 1));
        S.e[lane] = v;
    } else if (lane < 24) {
        int j = lane - 16;
        S.e[lane] = (a.left && j < n) ? cvy(S, by0 + j, bx0 - 1) : 128;
    } else if (lane == 24) {
        S.e[24] = a.tl ? cvy(S, by0 - 1, bx0 - 1) : 128;
    }
}

// pred8x8 reference-sample smoothing, src/h264/dec/intra.rs:199-231, S.e -> S.f
__device__ __forceinline__ void smooth8(WarpSmem &S, int lane, Avail a) {
    const int32_t *pt = S.e, *pl = S.e + 16;
    int ptl = S.e[24];
    if (lane < 16) {
        int v = pt[lane];
        if (a.top) {
            if (lane == 0) v = a.tl ? (ptl + 2 * pt[0] + pt[1] + 2) >> 2 : (3 * pt[0] + pt[1] + 2) >> 2;
            else if (lane == 15) v = (pt[14] + 3 * pt[15] + 2) >> 2;
            else v = (pt[lane - 1] + 2 * pt[lane] + pt[lane + 1] + 2) >> 2;
        }
        S.f[lane] = v;
    } else if (lane < 24) {
        int j = lane - 16, v = pl[j];
        if (a.left) {
            if (j == 0) v = a.tl ? (ptl + 2 * pl[0] + pl[1] + 2) >> 2 : (3 * pl[0] + pl[1] + 2) >> 2;
            else if (j == 7) v = (pl[6] + 3 * pl[7] + 2) >> 2;
            else v = (pl[j - 1] + 2 * pl[j] + pl[j + 1] + 2) >> 2;
        }
        S.f[lane] = v;
    } else if (lane == 24) {
        int v = ptl;
        if (a.tl) {
            if (a.top && a.left) v = (pt[0] + 2 * ptl + pl[0] + 2) >> 2;
            else if (a.top) v = (3 * ptl + pt[0] + 2) >> 2;
            else if (a.left) v = (3 * ptl + pl[0] + 2) >> 2;
        }
        S.f[24] = v;
    }
}

// reconstruct_intra, src/h264/dec/slicedec.rs:1325-1388, one warp.
// nb: availability of neighbours L, T, TR, TL for intra prediction.
__device__ void intra_mb(WarpSmem &S, const H264Launch &P, int lane, int mbx, int mby, const bool nb[4], uint8_t *Y,
                         uint8_t *U, uint8_t *V) {
    const IntraInfo &m = S.q;
    const int x0 = mbx * 16, y0 = mby * 16, cx0 = mbx * 8, cy0 = mby * 8;
    // canvas: neighbour samples
    if (mby > 0) {
        int gx = x0 + lane - 1;
        S.cy[lane] = (gx >= 0 && gx < P.W) ? __ldcg(Y + (size_t)(y0 - 1) * P.pitch + gx) : 0;
        if (lane < 20) {
            int c = lane / 10, gxc = cx0 + lane % 10 - 1;
            S.cc[c][lane % 10] = (gxc >= 0 && gxc < P.CW) ? __ldcg((c ? V : U) + (size_t)(cy0 - 1) * P.cpitch + gxc) : 0;
        }
    }
    if (mbx > 0) {
        if (lane < 16) S.cy[(lane + 1) * 32] = __ldcg(Y + (size_t)(y0 + lane) * P.pitch + x0 - 1);
        int c = lane >> 3, r = lane & 7;
        if (lane < 16) S.cc[c][(r + 1) * 12] = __ldcg((c ? V : U) + (size_t)(cy0 + r) * P.cpitch + cx0 - 1);
    }
    __syncwarp();
    // ---- luma
    if (m.kind == RC_H264_I4x4) {
        for (int i = 0; i < 16; i++) {
            const int bx = cBLK4X[i], by = cBLK4Y[i];
            Avail a;  // luma_avail4, slicedec.rs:1297-1323
            a.left = bx > 0 ? true : nb[0];
            a.top = by > 0 ? true : nb[1];
            a.tl = (bx > 0 && by > 0) ? true : by > 0 ? nb[0] : bx > 0 ? nb[1] : nb[3];
            a.tr = by == 0 ? (bx < 3 ? nb[1] : nb[2]) : bx == 3 ? false : cR2B[(by - 1) * 4 + bx + 1] < cR2B[by * 4 + bx];
            load_edge(S, lane, bx * 4, by * 4, 4, a);
            __syncwarp();
            if (lane < 16) {
                int x = lane & 3, y = lane >> 2;
                int v = pred_nxn_px(m.modes[by * 4 + bx], S.e, S.e + 16, S.e[24], 4, a, x, y);
                v = clip255(v + S.res[(by * 4 + y) * 16 + bx * 4 + x]);
                S.cy[(by * 4 + y + 1) * 32 + bx * 4 + x + 1] = (uint8_t)v;
            }
            __syncwarp();
        }
    } else if (m.kind == RC_H264_I8x8) {
        for (int b8 = 0; b8 < 4; b8++) {
            const int bx = (b8 & 1) * 2, by = (b8 >> 1) * 2;
            Avail a;
            a.left = bx > 0 ? true : nb[0];
            a.top = by > 0 ? true : nb[1];
            a.tl = (bx > 0 && by > 0) ? true : by > 0 ? nb[0] : bx > 0 ? nb[1] : nb[3];
            a.tr = b8 == 0 ? nb[1] : b8 == 1 ? nb[2] : b8 == 2;
            load_edge(S, lane, bx * 4, by * 4, 8, a);
            __syncwarp();
            smooth8(S, lane, a);
            __syncwarp();
#pragma unroll
            for (int h = 0; h < 2; h++) {
                int idx = lane + 32 * h, x = idx & 7, y = idx >> 3;
                int v = pred_nxn_px(m.modes[by * 4 + bx], S.f, S.f + 16, S.f[24], 8, a, x, y);
                v = clip255(v + S.res[(by * 4 + y) * 16 + bx * 4 + x]);
                S.cy[(by * 4 + y + 1) * 32 + bx * 4 + x + 1] = (uint8_t)v;
            }
            __syncwarp();
        }
    } else {
        // pred16x16, src/h264/dec/intra.rs:240-305
        const bool al = nb[0], at = nb[1], atl = nb[3];
        const int mode = m.i16_mode;
        int topv = at ? cvy(S, -1, lane & 15) : 0, leftv = al ? cvy(S, lane & 15, -1) : 0;
        int tl = atl ? cvy(S, -1, -1) : 128;
        int st = __reduce_add_sync(0xffffffffu, (unsigned)(lane < 16 ? topv : 0));
        int sl = __reduce_add_sync(0xffffffffu, (unsigned)(lane < 16 ? leftv : 0));
        int hterm = 0, vterm = 0;
        if (lane < 8) {
            int k = lane;
            int t8k = at ? cvy(S, -1, 8 + k) : 0;
            int t6k = (6 - k) < 0 ? tl : (at ? cvy(S, -1, 6 - k) : 0);
            int l8k = al ? cvy(S, 8 + k, -1) : 0;
            int l6k = (6 - k) < 0 ? tl : (al ? cvy(S, 6 - k, -1) : 0);
            hterm = (k + 1) * (t8k - t6k);
            vterm = (k + 1) * (l8k - l6k);
        }
        int H = (int)__reduce_add_sync(0xffffffffu, (unsigned)hterm);
        int Vv = (int)__reduce_add_sync(0xffffffffu, (unsigned)vterm);
        int dc;
        if (at && al) dc = (st + sl + 16) >> 5;
        else if (al) dc = (sl + 8) >> 4;
        else if (at) dc = (st + 8) >> 4;
        else dc = 128;
        int aa = 16 * ((al ? cvy(S, 15, -1) : 0) + (at ? cvy(S, -1, 15) : 0));
        int bb = (5 * H + 32) >> 6, cc = (5 * Vv + 32) >> 6;
        // all reads of the canvas edge are done before any write below
        __syncwarp();
#pragma unroll
        for (int h = 0; h < 8; h++) {
            int idx = lane + 32 * h, x = idx & 15, y = idx >> 4, v;
            if (mode == 0) v = at ? cvy(S, -1, x) : 0;
            else if (mode == 1) v = al ? cvy(S, y, -1) : 0;
            else if (mode == 2) v = dc;
            else v = clip255((aa + bb * (x - 7) + cc * (y - 7) + 16) >> 5);
            v = clip255(v + S.res[y * 16 + x]);
            // rows 0..15 of the canvas are not read again by this MB's prediction
            S.cy[(y + 1) * 32 + x + 1] = (uint8_t)v;
        }
        __syncwarp();
    }
    // ---- chroma, pred_chroma, src/h264/dec/intra.rs:307-395
    {
        const bool al = nb[0], at = nb[1], atl = nb[3];
        const int mode = m.chroma_mode;
        int outv[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            int idx = lane + 32 * h, c = idx >> 6, x = idx & 7, y = (idx >> 3) & 7;
            const uint8_t *cv = S.cc[c];
#define CT(i) (at ? (int)cv[(i) + 1] : 0)
#define CL(i) (al ? (int)cv[((i) + 1) * 12] : 0)
            int v;
            if (mode == 0) {
                int bx = x >> 2, by = y >> 2, st = 0, sl = 0;
                for (int i = 0; i < 4; i++) { st += CT(bx * 4 + i); sl += CL(by * 4 + i); }
                if ((bx == 0 && by == 0) || (bx > 0 && by > 0)) {
                    v = (at && al) ? (st + sl + 4) >> 3 : al ? (sl + 2) >> 2 : at ? (st + 2) >> 2 : 128;
                } else if (bx > 0) {
                    v = at ? (st + 2) >> 2 : al ? (sl + 2) >> 2 : 128;
                } else {
                    v = al ? (sl + 2) >> 2 : at ? (st + 2) >> 2 : 128;
                }
            } else if (mode == 1) v = CL(y);
            else if (mode == 2) v = CT(x);
            else {
                int tl = atl ? cv[0] : 128, hh = 0, vv = 0;
                for (int k = 0; k < 4; k++) {
                    int tm = (2 - k) < 0 ? tl : CT(2 - k), lm = (2 - k) < 0 ? tl : CL(2 - k);
                    hh += (k + 1) * (CT(4 + k) - tm);
                    vv += (k + 1) * (CL(4 + k) - lm);
                }
                int aa = 16 * (CL(7) + CT(7)), bb = (34 * hh + 32) >> 6, cc2 = (34 * vv + 32) >> 6;
                v = clip255((aa + bb * (x - 3) + cc2 * (y - 3) + 16) >> 5);
            }
#undef CT
#undef CL
            v = clip255(v + S.res[256 + c * 64 + y * 8 + x]);
            outv[h] = v;
        }
        __syncwarp();
#pragma unroll
        for (int h = 0; h < 4; h++) {
            int idx = lane + 32 * h, c = idx >> 6, x = idx & 7, y = (idx >> 3) & 7;
            S.cc[c][(y + 1) * 12 + x + 1] = (uint8_t)outv[h];
        }
    }
    __syncwarp();
    // ---- store the MB
    {
        int r = lane >> 1, half = lane & 1;
        const uint8_t *s = S.cy + (r + 1) * 32 + 1 + half * 8;
        uint32_t lo = s[0] | s[1] << 8 | s[2] << 16 | (uint32_t)s[3] << 24;
        uint32_t hi = s[4] | s[5] << 8 | s[6] << 16 | (uint32_t)s[7] << 24;
        *(uint2 *)(Y + (size_t)(y0 + r) * P.pitch + x0 + half * 8) = make_uint2(lo, hi);
        if (lane < 16) {
            int c = lane >> 3, rr = lane & 7;
            const uint8_t *q = S.cc[c] + (rr + 1) * 12 + 1;
            uint32_t a0 = q[0] | q[1] << 8 | q[2] << 16 | (uint32_t)q[3] << 24;
            uint32_t a1 = q[4] | q[5] << 8 | q[6] << 16 | (uint32_t)q[7] << 24;
            *(uint2 *)((c ? V : U) + (size_t)(cy0 + rr) * P.cpitch + cx0) = make_uint2(a0, a1);
        }
    }
}

// ---- deblocking (src/h264/dec/deblock.rs) -------------------------------
// ref_ids8, deblock.rs:7-21, for one 8x8 block and list
__device__ __forceinline__ uint32_t ref_id(const H264Launch &P, const rc_h264_mb &m, int l, int b8) {
    int r = m.ref_idx[l][b8];
    if (r < 0) return ID_NONE;
    if (m.slice >= P.num_slices) return ID_NONE - 1;
    const rc_h264_slice *sl = P.slices + m.slice;
    return r < min(__ldg(&sl->num_ref[l]), RC_H264_MAX_REFS) ? __ldg(&sl->ref_id[l][r]) : ID_NONE - 1;
}
__device__ __forceinline__ bool near_mv(int ax, int ay, int bx, int by) {
    return (uint32_t)(ax - bx + 3) < 7u && (uint32_t)(ay - by + 3) < 7u;
}
// motion_bs of blk(p, rp) vs blk(q, rq), deblock.rs:29-59
__device__ int motion_bs(const H264Launch &P, const rc_h264_mb &p, int rp, const rc_h264_mb &q, int rq) {
    int pb = (rp >> 3) * 2 + ((rp & 3) >> 1), qb = (rq >> 3) * 2 + ((rq & 3) >> 1);
    uint32_t pi0 = ref_id(P, p, 0, pb), pi1 = ref_id(P, p, 1, pb), qi0 = ref_id(P, q, 0, qb), qi1 = ref_id(P, q, 1, qb);
    int p0x = pi0 != ID_NONE ? p.mv[0][rp][0] : 0, p0y = pi0 != ID_NONE ? p.mv[0][rp][1] : 0;
    int p1x = pi1 != ID_NONE ? p.mv[1][rp][0] : 0, p1y = pi1 != ID_NONE ? p.mv[1][rp][1] : 0;
    int q0x = qi0 != ID_NONE ? q.mv[0][rq][0] : 0, q0y = qi0 != ID_NONE ? q.mv[0][rq][1] : 0;
    int q1x = qi1 != ID_NONE ? q.mv[1][rq][0] : 0, q1y = qi1 != ID_NONE ? q.mv[1][rq][1] : 0;
    bool same = pi0 == qi0 && pi1 == qi1 && near_mv(p0x, p0y, q0x, q0y) && near_mv(p1x, p1y, q1x, q1y);
    bool cross = pi0 == qi1 && pi1 == qi0 && near_mv(p0x, p0y, q1x, q1y) && near_mv(p1x, p1y, q0x, q0y);
    return !(same || cross);
}

// Loop-filter parameters of one MB (the boundary-strength and QP part of
// deblock_mb, deblock.rs:301-403); one warp, lane = dir*16 + edge*4 + segment.
__device__ void compute_db(const H264Launch &P, const rc_h264_mb &q, const rc_h264_mb &left, const rc_h264_mb &top,
                           int addr, int lane, DbMb *out) {
    const int mx = addr % P.mb_w, my = addr / P.mb_w;
    int bs = 0;
    bool filt = q.kind != RC_H264_NONE && q.slice < P.num_slices;
    int idc = 1, aoff = 0, boff = 0;
    if (filt) {
        const rc_h264_slice *sq = P.slices + q.slice;
        idc = __ldg(&sq->disable_deblocking_filter_idc);
        aoff = __ldg(&sq->alpha_offset);
        boff = __ldg(&sq->beta_offset);
        filt = idc != 1;
    }
    bool usable[2];
    usable[0] = mx > 0 && left.kind != RC_H264_NONE && !(idc == 2 && left.slice != q.slice);
    usable[1] = my > 0 && top.kind != RC_H264_NONE && !(idc == 2 && top.slice != q.slice);
    if (filt) {
        const bool t8 = q.transform_8x8;
        const int dir = lane >> 4, e = (lane >> 2) & 3, k = lane & 3;
        const rc_h264_mb &p = dir == 0 ? left : top;
        if (is_intra(q.kind)) {
            bs = e == 0 ? (usable[dir] ? 4 : 0) : ((t8 && (e & 1)) ? 0 : 3);
        } else {
            const int r = dir == 0 ? k * 4 + e : e * 4 + k;
            const bool first = e == 0;
            if (first && usable[dir] && is_intra(p.kind)) bs = 4;
            else if (first && !usable[dir]) bs = 0;
            else if (t8 && (e & 1)) bs = 0;
            else {
                const int nzq = q.nz_mask;
                int nz;
                if (dir == 0) nz = (nzq >> r & 1) | (e > 0 ? (nzq >> (r - 1) & 1) : (p.nz_mask >> (r + 3) & 1));
                else nz = (nzq >> r & 1) | (e > 0 ? (nzq >> (r - 4) & 1) : (p.nz_mask >> (r + 12) & 1));
                if (nz) bs = 2;
                else {
                    int rp = dir == 0 ? (first ? r + 3 : r - 1) : (first ? r + 12 : r - 4);
                    bs = first ? motion_bs(P, p, rp, q, r) : motion_bs(P, q, rp, q, r);
                }
            }
        }
    }
    const bool any = __ballot_sync(0xffffffffu, bs != 0) != 0;
    out->bs[lane] = (uint8_t)bs;
    if (lane == 0) {
        const int qq = q.kind == RC_H264_IPCM ? 0 : q.qp;
        out->qp[0] = (uint8_t)qq;
        out->qp[1] = (uint8_t)(usable[0] ? (left.kind == RC_H264_IPCM ? 0 : left.qp) : qq);
        out->qp[2] = (uint8_t)(usable[1] ? (top.kind == RC_H264_IPCM ? 0 : top.qp) : qq);
        for (int c = 0; c < 2; c++) {
            out->qpc[0][c] = q.qpc[c];
            out->qpc[1][c] = usable[0] ? left.qpc[c] : q.qpc[c];
            out->qpc[2][c] = usable[1] ? top.qpc[c] : q.qpc[c];
        }
        out->flags = (filt && any) ? 1 : 0;
        out->aoff = (int8_t)aoff;
        out->boff = (int8_t)boff;
    }
}

// filter_lanes, deblock.rs:146-229, for one line of 8 samples s[0..7] = p3..q3
__device__ __forceinline__ void filt_luma(int *s, int bsv, bool strong_edge, int alpha, int beta, int tc0) {
    int p3 = s[0], p2 = s[1], p1 = s[2], p0 = s[3], q0 = s[4], q1 = s[5], q2 = s[6], q3 = s[7];
    bool on = bsv != 0 && abs(p0 - q0) < alpha && abs(p1 - p0) < beta && abs(q1 - q0) < beta;
    if (!on) return;
    if (strong_edge) {
        bool strong = abs(p0 - q0) < ((alpha >> 2) + 2);
        bool sp = abs(p2 - p0) < beta && strong, sq = abs(q2 - q0) < beta && strong;
        if (sp) {
            s[3] = (p2 + 2 * p1 + 2 * p0 + 2 * q0 + q1 + 4) >> 3;
            s[2] = (p2 + p1 + p0 + q0 + 2) >> 2;
            s[1] = (2 * p3 + 3 * p2 + p1 + p0 + q0 + 4) >> 3;
        } else s[3] = (2 * p1 + p0 + q1 + 2) >> 2;
        if (sq) {
            s[4] = (p1 + 2 * p0 + 2 * q0 + 2 * q1 + q2 + 4) >> 3;
            s[5] = (p0 + q0 + q1 + q2 + 2) >> 2;
            s[6] = (2 * q3 + 3 * q2 + q1 + q0 + p0 + 4) >> 3;
        } else s[4] = (2 * q1 + q0 + p1 + 2) >> 2;
    } else {
        bool ap = abs(p2 - p0) < beta, aq = abs(q2 - q0) < beta;
        int tc = tc0 + ap + aq;
        int delta = clampi((((q0 - p0) << 2) + (p1 - q1) + 4) >> 3, -tc, tc);
        int avg = (p0 + q0 + 1) >> 1;
        s[3] = clip255(p0 + delta);
        s[4] = clip255(q0 - delta);
        if (ap) s[2] = p1 + clampi((p2 + avg - (p1 << 1)) >> 1, -tc0, tc0);
        if (aq) s[5] = q1 + clampi((q2 + avg - (q1 << 1)) >> 1, -tc0, tc0);
    }
}
__device__ __forceinline__ void filt_chroma(int *s, int bsv, bool strong_edge, int alpha, int beta, int tc0) {
    int p1 = s[2], p0 = s[3], q0 = s[4], q1 = s[5];
    bool on = bsv != 0 && abs(p0 - q0) < alpha && abs(p1 - p0) < beta && abs(q1 - q0) < beta;
    if (!on) return;
    if (strong_edge) {
        s[3] = (2 * p1 + p0 + q1 + 2) >> 2;
        s[4] = (2 * q1 + q0 + p1 + 2) >> 2;
    } else {
        int tc = tc0 + 1;
        int delta = clampi((((q0 - p0) << 2) + (p1 - q1) + 4) >> 3, -tc, tc);
        s[3] = clip255(p0 + delta);
        s[4] = clip255(q0 - delta);
    }
}

// edge parameters (params closure of deblock_mb, deblock.rs:386-403)
__device__ __forceinline__ void edge_consts(int qpp, int qpq, int bsv, int aoff, int boff, int &alpha, int &beta,
                                            int &tc0) {
    int qpav = (qpp + qpq + 1) >> 1;
    int ia = clampi(qpav + aoff, 0, 51), ib = clampi(qpav + boff, 0, 51);
    alpha = cALPHA[ia];
    beta = cBETA[ib];
    tc0 = (bsv >= 1 && bsv < 4) ? cTC0[ia][bsv - 1] : 0;
}

__device__ __forceinline__ void load_record(rc_h264_mb &dst, const rc_h264_mb *src, int lane) {
    const uint32_t *s = (const uint32_t *)src;
    uint32_t *d = (uint32_t *)&dst;
    for (int i = lane; i < (int)(sizeof(rc_h264_mb) / 4); i += 32) d[i] = __ldg(s + i);
}

// ===========================================================================
// Kernel 3: loop filter, one warp per MB row walking left to right.
// ===========================================================================
// Tile of the current MB: luma rows -4..15 x cols -4..15, chroma rows -4..7 x
// cols -4..7 per component.  Columns -4..-1 hold the left MB's columns after
// its own filtering; rows -4..-1 the MB above, read once row y-1 has
// published it.
struct __align__(16) RowTile {
    uint8_t y[20][20];
    uint8_t c[2][12][12];
    DbMb db;
};

__global__ void __launch_bounds__(32) h264_deblock_kernel(H264Launch P) {
    __shared__ RowTile T;
    const int lane = threadIdx.x, my = blockIdx.x;
    uint8_t *Y = P.dpb + (size_t)P.out_slot * P.slot_bytes;
    uint8_t *U = Y + P.u_off, *V = Y + P.v_off;
    const uint32_t tag = (P.epoch & 0xffffu) << 16;
    const bool luma = lane < 16;
    const int cc = (lane - 16) >> 3, li = luma ? lane : (lane - 16) & 7;
    // prefetched (pre-deblock) samples of the next MB: one row per lane
    uint4 pre_y = make_uint4(0, 0, 0, 0);
    uint2 pre_c = make_uint2(0, 0);
    uint32_t pre_db = 0;
    auto prefetch = [&](int x) {
        if (luma) pre_y = __ldcg((const uint4 *)(Y + (size_t)(my * 16 + lane) * P.pitch + x * 16));
        else pre_c = __ldcg((const uint2 *)((cc ? V : U) + (size_t)(my * 8 + li) * P.cpitch + x * 8));
        if (lane < 12) pre_db = __ldcg((const uint32_t *)(P.db + (size_t)my * P.mb_w + x) + lane);
    };
    prefetch(0);
    for (int x = 0; x < P.mb_w; x++) {
        // ---- stage the MB (rows 0..15 / 0..7, columns 0..15 / 0..7)
        if (luma) {
            uint32_t w[4] = {pre_y.x, pre_y.y, pre_y.z, pre_y.w};
#pragma unroll
            for (int i = 0; i < 4; i++) *(uint32_t *)&T.y[lane + 4][4 + 4 * i] = w[i];
        } else {
            *(uint32_t *)&T.c[cc][li + 4][4] = pre_c.x;
            *(uint32_t *)&T.c[cc][li + 4][8] = pre_c.y;
        }
        if (lane < 12) ((uint32_t *)&T.db)[lane] = pre_db;
        // ---- the MB above must be final: row y-1 has published MBs 0..x
        if (my > 0) {
            bool ok = true;
            if (lane == 0) {
                const uint32_t need = (uint32_t)min(x + 1, P.mb_w);
                const uint32_t *f = P.rowprog + my - 1;
                uint32_t it = 0, v;
                while (((v = ld_acquire(f)) & 0xffff0000u) != tag || (v & 0xffffu) < need) {
                    if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) { ok = false; break; }
                    if (it > 256) __nanosleep(64);
                }
            }
            if (!__shfl_sync(0xffffffffu, ok, 0)) {
                if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT);
                return;
            }
            // rows -4..-1: luma lanes 0..3 (16 bytes), chroma lanes 4..11 (8 bytes)
            if (lane < 4) {
                uint4 v = __ldcg((const uint4 *)(Y + (size_t)(my * 16 - 4 + lane) * P.pitch + x * 16));
                uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int i = 0; i < 4; i++) *(uint32_t *)&T.y[lane][4 + 4 * i] = w[i];
            } else if (lane < 12) {
                int c = (lane - 4) >> 2, r = (lane - 4) & 3;
                uint2 v = __ldcg((const uint2 *)((c ? V : U) + (size_t)(my * 8 - 4 + r) * P.cpitch + x * 8));
                *(uint32_t *)&T.c[c][r][4] = v.x;
                *(uint32_t *)&T.c[c][r][8] = v.y;
            }
        }
        __syncwarp();
        if (x + 1 < P.mb_w) prefetch(x + 1);
        const DbMb &db = T.db;
        if (db.flags) {
            const int aoff = db.aoff, boff = db.boff;
            // ---- vertical edges, one row per lane
            {
                int s[20];
                uint8_t *row = luma ? T.y[lane + 4] : T.c[cc][li + 4];
                const int n = luma ? 20 : 12;
#pragma unroll
                for (int i = 0; i < 20; i++) s[i] = i < n ? row[i] : 0;
                const int k = luma ? li >> 2 : li >> 1;
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int bsv = db.bs[(e << 2) | k];
                    const bool strong = db.bs[e << 2] >= 4;
                    int alpha, beta, tc0;
                    if (luma) {
                        edge_consts(e == 0 ? db.qp[1] : db.qp[0], db.qp[0], bsv, aoff, boff, alpha, beta, tc0);
                        filt_luma(s + 4 * e, bsv, strong, alpha, beta, tc0);
                    } else if ((e & 1) == 0) {
                        edge_consts(e == 0 ? db.qpc[1][cc] : db.qpc[0][cc], db.qpc[0][cc], bsv, aoff, boff, alpha,
                                    beta, tc0);
                        filt_chroma(s + 2 * e, bsv, strong, alpha, beta, tc0);
                    }
                }
#pragma unroll
                for (int i = 0; i < 20; i++)
                    if (i < n) row[i] = (uint8_t)s[i];
            }
            __syncwarp();
            // ---- horizontal edges, one column per lane
            {
                int s[20];
                const int n = luma ? 20 : 12;
#pragma unroll
                for (int i = 0; i < 20; i++) s[i] = i < n ? (luma ? T.y[i][lane + 4] : T.c[cc][i][li + 4]) : 0;
                const int k = luma ? li >> 2 : li >> 1;
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int bsv = db.bs[16 | (e << 2) | k];
                    const bool strong = db.bs[16 | (e << 2)] >= 4;
                    int alpha, beta, tc0;
                    if (luma) {
                        edge_consts(e == 0 ? db.qp[2] : db.qp[0], db.qp[0], bsv, aoff, boff, alpha, beta, tc0);
                        filt_luma(s + 4 * e, bsv, strong, alpha, beta, tc0);
                    } else if ((e & 1) == 0) {
                        edge_consts(e == 0 ? db.qpc[2][cc] : db.qpc[0][cc], db.qpc[0][cc], bsv, aoff, boff, alpha,
                                    beta, tc0);
                        filt_chroma(s + 2 * e, bsv, strong, alpha, beta, tc0);
                    }
                }
#pragma unroll
                for (int i = 0; i < 20; i++)
                    if (i < n) {
                        if (luma) T.y[i][lane + 4] = (uint8_t)s[i];
                        else T.c[cc][i][li + 4] = (uint8_t)s[i];
                    }
            }
            __syncwarp();
        }
        // ---- write back what is final: this MB's columns 0..11 (chroma 0..3),
        // the left MB's columns 12..15 (chroma 4..7), and the rows of the MB
        // above that this MB's top edge modified
        if (luma) {
            uint8_t *dst = Y + (size_t)(my * 16 + lane) * P.pitch + x * 16;
            const uint8_t *r = T.y[lane + 4];
            *(uint32_t *)(dst + 0) = *(const uint32_t *)(r + 4);
            *(uint32_t *)(dst + 4) = *(const uint32_t *)(r + 8);
            *(uint32_t *)(dst + 8) = *(const uint32_t *)(r + 12);
            if (x > 0) *(uint32_t *)(dst - 4) = *(const uint32_t *)(r + 0);
            if (x == P.mb_w - 1) *(uint32_t *)(dst + 12) = *(const uint32_t *)(r + 16);
        } else {
            uint8_t *dst = (cc ? V : U) + (size_t)(my * 8 + li) * P.cpitch + x * 8;
            const uint8_t *r = T.c[cc][li + 4];
            *(uint32_t *)(dst + 0) = *(const uint32_t *)(r + 4);
            if (x > 0) *(uint32_t *)(dst - 4) = *(const uint32_t *)(r + 0);
            if (x == P.mb_w - 1) *(uint32_t *)(dst + 4) = *(const uint32_t *)(r + 8);
        }
        if (my > 0 && db.flags) {
            if (lane < 3) {  // luma rows -3..-1
                uint8_t *dst = Y + (size_t)(my * 16 - 3 + lane) * P.pitch + x * 16;
                const uint8_t *r = T.y[lane + 1] + 4;
                *(uint4 *)dst = make_uint4(*(const uint32_t *)(r), *(const uint32_t *)(r + 4),
                                           *(const uint32_t *)(r + 8), *(const uint32_t *)(r + 12));
            } else if (lane < 5) {  // chroma row -1
                int c = lane - 3;
                uint8_t *dst = (c ? V : U) + (size_t)(my * 8 - 1) * P.cpitch + x * 8;
                const uint8_t *r = T.c[c][3] + 4;
                *(uint2 *)dst = make_uint2(*(const uint32_t *)(r), *(const uint32_t *)(r + 4));
            }
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(P.rowprog + my, tag | (uint32_t)(x == P.mb_w - 1 ? P.mb_w : x));
        // ---- shift: this MB's columns 12..15 become the next MB's left columns
        if (luma) {
            *(uint32_t *)&T.y[lane + 4][0] = *(const uint32_t *)&T.y[lane + 4][16];
        } else {
            *(uint32_t *)&T.c[cc][li + 4][0] = *(const uint32_t *)&T.c[cc][li + 4][8];
        }
        __syncwarp();
    }
}

// Loop-filter parameters of every MB on their own (one warp per MB); the
// allocation-free deblocking entry point needs them without the MB kernel.
__global__ void __launch_bounds__(128) h264_db_params_kernel(H264Launch P) {
    __shared__ __align__(16) rc_h264_mb rec[4][3];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int addr = blockIdx.x * 4 + w;
    if (addr >= P.mb_w * P.mb_h) return;
    const int mbx = addr % P.mb_w, mby = addr / P.mb_w;
    load_record(rec[w][0], P.mbs + addr, lane);
    if (mbx > 0) load_record(rec[w][1], P.mbs + addr - 1, lane);
    if (mby > 0) load_record(rec[w][2], P.mbs + addr - P.mb_w, lane);
    __syncwarp();
    compute_db(P, rec[w][0], rec[w][1], rec[w][2], addr, lane, P.db + addr);
}


// ===========================================================================
// Wave kernel: intra reconstruction and the loop filter in one cooperative
// launch.  CTAs [0, intra_blocks) take intra MBs in anti-diagonal order, one
// warp per MB; the remaining CTAs each filter a band of WAVE_WARPS MB rows,
// one warp per row walking left to right.  Inside a band the MB above comes
// through shared memory (a ring of final bottom rows per row); across bands
// through global memory and a per-row progress word.  A row filters MB x once
// the intra MBs among (x-1..x+1, y..y+1) are reconstructed and the row above
// has finished MBs 0..x.
// ===========================================================================
constexpr int WAVE_WARPS = 8;
constexpr int RING = 8;

struct __align__(16) BandRow {
    RowTile T;
    uint8_t ring[RING][128];  // bottom rows 12..15 of each final MB: luma 4x16, Cb 4x8, Cr 4x8
};
struct __align__(16) BandSmem {
    BandRow r[WAVE_WARPS];
    volatile int prog[WAVE_WARPS];  // MBs of each row that are final (in this CTA's rows)
    volatile int icol;              // columns whose intra MBs (band rows + the row below) are reconstructed
    volatile int above;             // MBs of the row above the band that are final
};
union __align__(16) WaveSmem {
    WarpSmem iw[WAVE_WARPS];
    BandSmem band;
};

__device__ void wave_intra_worker(const H264Launch &P, WarpSmem &S, int lane) {
    uint8_t *Y = P.dpb + (size_t)P.out_slot * P.slot_bytes;
    uint8_t *U = Y + P.u_off, *V = Y + P.v_off;
    for (;;) {
        unsigned ti = 0;
        if (lane == 0) ti = aborted(P.error) ? 0xffffffffu : atomicAdd(P.counter, 1u);
        ti = __shfl_sync(0xffffffffu, ti, 0);
        if (ti >= (unsigned)P.ntasks) return;
        const int addr = __ldg(P.tasks + ti) & 0x7fffffffu;
        if (!wave_intra(__ldg(&P.mbs[addr].kind))) continue;
        const int mbx = addr % P.mb_w, mby = addr / P.mb_w;
        // prediction parameters and residual (independent of the neighbours)
        if (lane < 8) ((uint32_t *)&S.q)[lane] = __ldcg((const uint32_t *)(P.iinfo + addr) + lane);
        {
            const uint4 *src = (const uint4 *)(P.ires + (size_t)addr * 384);
            uint4 *dst = (uint4 *)S.res;
            dst[lane] = __ldcg(src + lane);
            if (lane < 16) dst[32 + lane] = __ldcg(src + 32 + lane);
        }
        __syncwarp();
        // wait for the intra neighbours whose samples the modes read
        bool ok = true;
        const int waits = S.q.wait;
        if (lane < 4 && (waits >> lane & 1)) {
            const int dx = lane == 0 ? -1 : lane == 2 ? 1 : lane == 3 ? -1 : 0, dy = lane == 0 ? 0 : -1;
            const int nx = mbx + dx, ny = mby + dy;
            if (nx >= 0 && ny >= 0 && nx < P.mb_w) ok = wait_flag(P.rflag + ny * P.mb_w + nx, P.epoch, P.wait_limit, P.error);
        }
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT);
            return;
        }
        bool nb[4];
#pragma unroll
        for (int n = 0; n < 4; n++) nb[n] = S.q.nb >> n & 1;
        intra_mb(S, P, lane, mbx, mby, nb, Y, U, V);
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(P.rflag + addr, P.epoch);
    }
}

// One MB row of a band.  w: row index inside the band; last: w is the band's
// last row (publishes to global memory for the next band).
__device__ void wave_band_row(const H264Launch &P, BandSmem &B, int w, int my, bool last, int lane) {
    RowTile &T = B.r[w].T;
    uint8_t *Y = P.dpb + (size_t)P.out_slot * P.slot_bytes;
    uint8_t *U = Y + P.u_off, *V = Y + P.v_off;
    const uint32_t tag = (P.epoch & 0xffffu) << 16;
    const bool luma = lane < 16;
    const int cc = (lane - 16) >> 3, li = luma ? lane : (lane - 16) & 7;
    const bool below = my + 1 < P.mb_h;
    const bool ring_out = !last && below;  // the next row of the band reads this row's ring
    uint4 pre_y = make_uint4(0, 0, 0, 0);
    uint2 pre_c = make_uint2(0, 0);
    uint32_t pre_db = 0;
    // intra reconstruction of MB column x in rows y, y+1 (lanes 0, 1)
    auto wait_intra = [&](int x) -> bool {
        bool ok = true;
        if (lane < 2 && x < P.mb_w) {
            const int ry = my + lane;
            if (ry < P.mb_h) {
                const int a = ry * P.mb_w + x;
                if (wave_intra(__ldg(&P.mbs[a].kind))) ok = wait_flag(P.rflag + a, P.epoch, P.wait_limit, P.error);
            }
        }
        return __all_sync(0xffffffffu, ok);
    };
    auto prefetch = [&](int x) {
        if (luma) pre_y = __ldcg((const uint4 *)(Y + (size_t)(my * 16 + lane) * P.pitch + x * 16));
        else pre_c = __ldcg((const uint2 *)((cc ? V : U) + (size_t)(my * 8 + li) * P.cpitch + x * 8));
        if (lane < 12) pre_db = __ldcg((const uint32_t *)(P.db + (size_t)my * P.mb_w + x) + lane);
    };
    // wait until a helper-published shared counter reaches `need`
    auto wait_shared = [&](volatile int *c, int need) -> bool {
        bool ok = true;
        if (lane == 0) {
            uint32_t it = 0;
            while (*c < need) {
                if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) { ok = false; break; }
                if (it > 1024) __nanosleep(32);
            }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        __threadfence_block();
        return ok;
    };
    (void)wait_intra;
    if (!wait_shared(&B.icol, min(1, P.mb_w))) { if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT); return; }
    prefetch(0);
    for (int x = 0; x < P.mb_w; x++) {
        // ---- stage MB x
        if (luma) {
            uint32_t q[4] = {pre_y.x, pre_y.y, pre_y.z, pre_y.w};
#pragma unroll
            for (int i = 0; i < 4; i++) *(uint32_t *)&T.y[lane + 4][4 + 4 * i] = q[i];
        } else {
            *(uint32_t *)&T.c[cc][li + 4][4] = pre_c.x;
            *(uint32_t *)&T.c[cc][li + 4][8] = pre_c.y;
        }
        if (lane < 12) ((uint32_t *)&T.db)[lane] = pre_db;
        // ---- intra MBs this MB's edges touch: (x+1, y) and (x+1, y+1) are new
        if (!wait_shared(&B.icol, min(x + 2, P.mb_w))) { if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT); return; }
        // ---- the MB above, rows 12..15 (final once row y-1 has finished MBs 0..x)
        if (my > 0) {
            const uint32_t need = (uint32_t)min(x + 1, P.mb_w);
            bool ok = true;
            if (w == 0) {
                if (!wait_shared(&B.above, (int)need)) { if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT); return; }
                if (lane < 4) {
                    uint4 v = __ldcg((const uint4 *)(Y + (size_t)(my * 16 - 4 + lane) * P.pitch + x * 16));
                    uint32_t q[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int i = 0; i < 4; i++) *(uint32_t *)&T.y[lane][4 + 4 * i] = q[i];
                } else if (lane < 12) {
                    int c = (lane - 4) >> 2, r = (lane - 4) & 3;
                    uint2 v = __ldcg((const uint2 *)((c ? V : U) + (size_t)(my * 8 - 4 + r) * P.cpitch + x * 8));
                    *(uint32_t *)&T.c[c][r][4] = v.x;
                    *(uint32_t *)&T.c[c][r][8] = v.y;
                }
            } else {
                if (lane == 0) {
                    uint32_t it = 0;
                    while (B.prog[w - 1] < (int)need) {
                        if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) { ok = false; break; }
                        if (it > 1024) __nanosleep(32);
                    }
                }
                if (!__shfl_sync(0xffffffffu, ok, 0)) { if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT); return; }
                __threadfence_block();
                const uint8_t *slot = B.r[w - 1].ring[x % RING];
                if (lane < 16) {  // luma rows 12..15: 4 rows x 16 bytes as 16 words
                    *(uint32_t *)&T.y[lane >> 2][4 + 4 * (lane & 3)] = *(const uint32_t *)(slot + 4 * lane);
                } else {          // chroma: 2 planes x 4 rows x 8 bytes as 16 words
                    int k = lane - 16, c = k >> 3, r = (k >> 1) & 3, h = k & 1;
                    *(uint32_t *)&T.c[c][r][4 + 4 * h] = *(const uint32_t *)(slot + 64 + 4 * k);
                }
            }
        }
        __syncwarp();
        if (x + 1 < P.mb_w) prefetch(x + 1);
        const DbMb &db = T.db;
        if (db.flags) {
            const int aoff = db.aoff, boff = db.boff;
            {  // vertical edges, one row per lane
                int sv[20];
                uint8_t *row = luma ? T.y[lane + 4] : T.c[cc][li + 4];
                const int n = luma ? 20 : 12;
#pragma unroll
                for (int i = 0; i < 20; i++) sv[i] = i < n ? row[i] : 0;
                const int k = luma ? li >> 2 : li >> 1;
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int bsv = db.bs[(e << 2) | k];
                    const bool strong = db.bs[e << 2] >= 4;
                    int alpha, beta, tc0;
                    if (luma) {
                        edge_consts(e == 0 ? db.qp[1] : db.qp[0], db.qp[0], bsv, aoff, boff, alpha, beta, tc0);
                        filt_luma(sv + 4 * e, bsv, strong, alpha, beta, tc0);
                    } else if ((e & 1) == 0) {
                        edge_consts(e == 0 ? db.qpc[1][cc] : db.qpc[0][cc], db.qpc[0][cc], bsv, aoff, boff, alpha,
                                    beta, tc0);
                        filt_chroma(sv + 2 * e, bsv, strong, alpha, beta, tc0);
                    }
                }
#pragma unroll
                for (int i = 0; i < 20; i++)
                    if (i < n) row[i] = (uint8_t)sv[i];
            }
            __syncwarp();
            {  // horizontal edges, one column per lane
                int sv[20];
                const int n = luma ? 20 : 12;
#pragma unroll
                for (int i = 0; i < 20; i++) sv[i] = i < n ? (luma ? T.y[i][lane + 4] : T.c[cc][i][li + 4]) : 0;
                const int k = luma ? li >> 2 : li >> 1;
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int bsv = db.bs[16 | (e << 2) | k];
                    const bool strong = db.bs[16 | (e << 2)] >= 4;
                    int alpha, beta, tc0;
                    if (luma) {
                        edge_consts(e == 0 ? db.qp[2] : db.qp[0], db.qp[0], bsv, aoff, boff, alpha, beta, tc0);
                        filt_luma(sv + 4 * e, bsv, strong, alpha, beta, tc0);
                    } else if ((e & 1) == 0) {
                        edge_consts(e == 0 ? db.qpc[2][cc] : db.qpc[0][cc], db.qpc[0][cc], bsv, aoff, boff, alpha,
                                    beta, tc0);
                        filt_chroma(sv + 2 * e, bsv, strong, alpha, beta, tc0);
                    }
                }
#pragma unroll
                for (int i = 0; i < 20; i++)
                    if (i < n) {
                        if (luma) T.y[i][lane + 4] = (uint8_t)sv[i];
                        else T.c[cc][i][li + 4] = (uint8_t)sv[i];
                    }
            }
            __syncwarp();
        }
        // ---- final samples to the picture (as h264_deblock_kernel)
        if (luma) {
            uint8_t *dst = Y + (size_t)(my * 16 + lane) * P.pitch + x * 16;
            const uint8_t *r = T.y[lane + 4];
            *(uint32_t *)(dst + 0) = *(const uint32_t *)(r + 4);
            *(uint32_t *)(dst + 4) = *(const uint32_t *)(r + 8);
            *(uint32_t *)(dst + 8) = *(const uint32_t *)(r + 12);
            if (x > 0) *(uint32_t *)(dst - 4) = *(const uint32_t *)(r + 0);
            if (x == P.mb_w - 1) *(uint32_t *)(dst + 12) = *(const uint32_t *)(r + 16);
        } else {
            uint8_t *dst = (cc ? V : U) + (size_t)(my * 8 + li) * P.cpitch + x * 8;
            const uint8_t *r = T.c[cc][li + 4];
            *(uint32_t *)(dst + 0) = *(const uint32_t *)(r + 4);
            if (x > 0) *(uint32_t *)(dst - 4) = *(const uint32_t *)(r + 0);
            if (x == P.mb_w - 1) *(uint32_t *)(dst + 4) = *(const uint32_t *)(r + 8);
        }
        if (my > 0 && db.flags) {
            if (lane < 3) {
                uint8_t *dst = Y + (size_t)(my * 16 - 3 + lane) * P.pitch + x * 16;
                const uint8_t *r = T.y[lane + 1] + 4;
                *(uint4 *)dst = make_uint4(*(const uint32_t *)(r), *(const uint32_t *)(r + 4),
                                           *(const uint32_t *)(r + 8), *(const uint32_t *)(r + 12));
            } else if (lane < 5) {
                int c = lane - 3;
                uint8_t *dst = (c ? V : U) + (size_t)(my * 8 - 1) * P.cpitch + x * 8;
                const uint8_t *r = T.c[c][3] + 4;
                *(uint2 *)dst = make_uint2(*(const uint32_t *)(r), *(const uint32_t *)(r + 4));
            }
        }
        // ---- bottom rows for the next row of the band: MB x columns 0..11
        // now, MB x-1 columns 12..15 (final after this MB's left edge)
        if (ring_out) {
            bool ok = true;
            if (lane == 0) {
                uint32_t it = 0;
                while (B.prog[w + 1] < x - RING + 1) {
                    if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) { ok = false; break; }
                    if (it > 1024) __nanosleep(32);
                }
            }
            if (!__shfl_sync(0xffffffffu, ok, 0)) { if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT); return; }
            uint8_t *cur = B.r[w].ring[x % RING], *prev = B.r[w].ring[(x + RING - 1) % RING];
            if (lane < 16) {
                const int r = lane >> 2, q = lane & 3;  // luma row 12 + r, word q (columns 4q..4q+3)
                if (q < 3) *(uint32_t *)(cur + 4 * lane) = *(const uint32_t *)&T.y[16 + r][4 + 4 * q];
                else {
                    if (x > 0) *(uint32_t *)(prev + 4 * lane) = *(const uint32_t *)&T.y[16 + r][0];
                    if (x == P.mb_w - 1) *(uint32_t *)(cur + 4 * lane) = *(const uint32_t *)&T.y[16 + r][16];
                }
            } else {
                const int k = lane - 16, c = k >> 3, r = (k >> 1) & 3, h = k & 1;  // chroma row 4 + r, half h
                if (h == 0) *(uint32_t *)(cur + 64 + 4 * k) = *(const uint32_t *)&T.c[c][8 + r][4];
                else {
                    if (x > 0) *(uint32_t *)(prev + 64 + 4 * k) = *(const uint32_t *)&T.c[c][8 + r][0];
                    if (x == P.mb_w - 1) *(uint32_t *)(cur + 64 + 4 * k) = *(const uint32_t *)&T.c[c][8 + r][8];
                }
            }
        }
        __syncwarp();
        const int done = x == P.mb_w - 1 ? P.mb_w : x;
        // progress: in shared memory for the rows of this band (the row below
        // reads it, the row above throttles its ring on it), and in global
        // memory for the band's last row (read by the next band; every 4 MBs)
        if (last && ((x & 3) == 3 || done == P.mb_w)) {
            __threadfence();
            __syncwarp();
            if (lane == 0) {
                st_release(P.rowprog + my, tag | (uint32_t)done);
                B.prog[w] = done;
            }
        } else {
            __threadfence_block();
            __syncwarp();
            if (lane == 0) B.prog[w] = done;
        }
        // ---- shift: this MB's columns 12..15 become the next MB's left columns
        if (luma) *(uint32_t *)&T.y[lane + 4][0] = *(const uint32_t *)&T.y[lane + 4][16];
        else *(uint32_t *)&T.c[cc][li + 4][0] = *(const uint32_t *)&T.c[cc][li + 4][8];
        __syncwarp();
    }
}

// Helper warp 0 of a band: confirms, column by column, that the intra MBs of
// the band's rows and of the row below are reconstructed (acquire loads of
// their flags) and publishes the count of ready columns in shared memory.
__device__ void wave_band_intra_helper(const H264Launch &P, BandSmem &B, int y0, int rows, int lane) {
    const int ry = y0 + lane;
    const bool mine = lane <= rows && ry < P.mb_h;
    for (int x = 0; x < P.mb_w; x++) {
        bool ok = true;
        if (mine) {
            const int a = ry * P.mb_w + x;
            if (wave_intra(__ldg(&P.mbs[a].kind))) ok = wait_flag(P.rflag + a, P.epoch, P.wait_limit, P.error);
        }
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT);
            return;
        }
        __threadfence_block();
        __syncwarp();
        if (lane == 0) B.icol = x + 1;
    }
}

// Helper warp 1 of a band: mirrors the global progress word of the row above
// the band into shared memory.
__device__ void wave_band_above_helper(const H264Launch &P, BandSmem &B, int y0, int lane) {
    if (lane != 0) return;
    if (y0 == 0) { B.above = P.mb_w; return; }
    const uint32_t tag = (P.epoch & 0xffffu) << 16;
    const uint32_t *f = P.rowprog + y0 - 1;
    uint32_t it = 0;
    int seen = 0;
    while (seen < P.mb_w) {
        const uint32_t v = ld_acquire(f);
        if ((v & 0xffff0000u) == tag && (int)(v & 0xffffu) > seen) {
            seen = v & 0xffffu;
            __threadfence_block();
            B.above = seen;
            it = 0;
            continue;
        }
        if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) {
            set_error(P.error, RC_DEV_ERR_TIMEOUT);
            return;
        }
        if (it > 256) __nanosleep(64);
    }
}

__global__ void __launch_bounds__((WAVE_WARPS + 2) * 32) h264_wave_kernel(H264Launch P) {
    __shared__ WaveSmem sm;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if ((int)blockIdx.x < P.intra_blocks) {
        if (warp < WAVE_WARPS) wave_intra_worker(P, sm.iw[warp], lane);
        return;
    }
    const int band = blockIdx.x - P.intra_blocks;
    const int y0 = band * WAVE_WARPS, rows = min(WAVE_WARPS, P.mb_h - y0);
    if (threadIdx.x < WAVE_WARPS) sm.band.prog[threadIdx.x] = 0;
    if (threadIdx.x == 0) { sm.band.icol = 0; sm.band.above = 0; }
    __syncthreads();
    if (warp == WAVE_WARPS) { wave_band_intra_helper(P, sm.band, y0, rows, lane); return; }
    if (warp == WAVE_WARPS + 1) { wave_band_above_helper(P, sm.band, y0, lane); return; }
    const int my = y0 + warp;
    if (my >= P.mb_h) return;
    const bool last = warp == WAVE_WARPS - 1 || my == P.mb_h - 1;
    wave_band_row(P, sm.band, warp, my, last, lane);
}

}  // namespace

void rc_launch_h264_mb(const H264Launch &p, cudaStream_t st) {
    h264_mb_kernel<<<p.mb_w * p.mb_h, 256, 0, st>>>(p);
}

int rc_h264_wave_capacity() {
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, h264_wave_kernel, (WAVE_WARPS + 2) * 32, 0) != cudaSuccess)
        return 0;
    return per * sms;
}

int rc_launch_h264_wave(const H264Launch &p, cudaStream_t st) {
    cudaMemsetAsync(p.counter, 0, sizeof(uint32_t), st);
    const int bands = (p.mb_h + WAVE_WARPS - 1) / WAVE_WARPS;
    H264Launch q = p;
    void *args[] = {&q};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)h264_wave_kernel, dim3(p.intra_blocks + bands),
                                                dim3((WAVE_WARPS + 2) * 32), args, 0, st);
    return e == cudaSuccess ? 0 : -1;
}

// ===========================================================================
// Allocation-free deblocking: rc_h264_deblock_noalloc
// ===========================================================================
// Callers that own every byte of device memory (a decoder embedded in a
// process whose allocator is fixed at start-up, a real-time pipeline that
// must not stall in cudaMalloc, code running while a stream is captured) can
// deblock an already reconstructed picture without the library allocating.
// The scratch the loop filter needs -- per-MB filter parameters (48 bytes per
// MB) and per-row progress words -- lives in this one static device array,
// sized for RC_NOALLOC_MAX_MBS macroblocks and RC_NOALLOC_MAX_ROWS rows; every
// device that loads the library holds it until the process exits.
#define RC_NOALLOC_DB_WORDS (RC_NOALLOC_MAX_MBS * (int)(sizeof(DbMb) / 4))
static __device__ __align__(256) uint32_t g_noalloc_scratch[RC_NOALLOC_DB_WORDS + RC_NOALLOC_MAX_ROWS];

#include <mutex>

namespace {
std::mutex g_noalloc_mu;
uint32_t *g_noalloc_addr[64];
bool g_noalloc_ready[64];

// Device address of the static scratch for the current device; looked up once
// per device (the host-side name is not a device address).
int noalloc_scratch(uint32_t **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return RC_ENODEV;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ready[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return RC_ECUDA;
        }
        g_noalloc_addr[dev] = (uint32_t *)p;
        g_noalloc_ready[dev] = true;
    }
    *out = g_noalloc_addr[dev];
    return RC_OK;
}
}  // namespace

extern "C" int rc_h264_deblock_noalloc(const rc_h264_picture *pic, int mb_w, int mb_h, void *y, void *u, void *v,
                                       int luma_pitch, int chroma_pitch, uint32_t *status, void *cuda_stream) {
    if (!pic || pic->mem != RC_MEM_DEVICE || !pic->mbs || !pic->slices || pic->num_slices <= 0) return RC_EINVAL;
    if (mb_w <= 0 || mb_h <= 0 || !y || !u || !v || !status) return RC_EINVAL;
    if ((long long)mb_w * mb_h > RC_NOALLOC_MAX_MBS || mb_h > RC_NOALLOC_MAX_ROWS) return RC_EINVAL;
    if (luma_pitch < mb_w * 16 || chroma_pitch < mb_w * 8 || (luma_pitch & 15) || (chroma_pitch & 7)) return RC_EINVAL;
    if (((uintptr_t)y & 15) || ((uintptr_t)u & 7) || ((uintptr_t)v & 7)) return RC_EINVAL;
    uint32_t *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc != RC_OK) return rc;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    uint32_t *rows = scratch + RC_NOALLOC_DB_WORDS;
    // row progress must start at zero; the parameters are rewritten each call
    if (cudaMemsetAsync(rows, 0, (size_t)mb_h * sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemsetAsync(status, 0, sizeof(uint32_t), st) != cudaSuccess)
        return RC_ECUDA;
    H264Launch L;
    memset(&L, 0, sizeof L);
    L.mbs = pic->mbs;
    L.slices = pic->slices;
    L.num_slices = pic->num_slices;
    L.mb_w = mb_w;
    L.mb_h = mb_h;
    L.W = mb_w * 16;
    L.H = mb_h * 16;
    L.CW = mb_w * 8;
    L.CH = mb_h * 8;
    L.pitch = luma_pitch;
    L.cpitch = chroma_pitch;
    L.dpb = (uint8_t *)y;
    L.slot_bytes = 0;
    L.out_slot = 0;
    L.u_off = (unsigned long long)((uintptr_t)u - (uintptr_t)y);
    L.v_off = (unsigned long long)((uintptr_t)v - (uintptr_t)y);
    L.dpb_slots = 1;
    L.db = (DbMb *)scratch;
    L.rowprog = rows;
    L.error = status;
    L.epoch = 1;
    L.wait_limit = RC_WAIT_LIMIT;
    h264_db_params_kernel<<<(mb_w * mb_h + 3) / 4, 128, 0, st>>>(L);
    h264_deblock_kernel<<<mb_h, 32, 0, st>>>(L);
    return cudaGetLastError() == cudaSuccess ? RC_OK : RC_ECUDA;
}
