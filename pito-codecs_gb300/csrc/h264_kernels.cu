// h264_kernels.cu — H.264 block reconstruction on sm_103a.
//
// Per picture:
//
//  h264_edge_kernel     one warp per macroblock: boundary strengths and QPs
//                       of the MB's edges (deblock.rs) as 64 ready-to-use
//                       filter words; reads only syntax, so it runs on a side
//                       stream beside the previous picture's band kernel.
//  h264_mb_kernel       one CTA (256 threads) per macroblock, all in parallel.
//                       Inter MBs: dequantisation (scale4/scale8, chroma DC
//                       Hadamard), 4x4/8x8 inverse transforms, 6-tap luma and
//                       bilinear chroma motion compensation with edge
//                       extension by coordinate clamp, default / explicit
//                       weighted prediction, residual add and clip, fused.
//                       I_PCM MBs are copied.  Intra MBs are dequantised and
//                       transformed; their residuals wait for the band kernel.
//  h264_band_kernel     one cooperative launch, a CTA per band of MB rows:
//                       per row an intra warp (prediction block by block in
//                       decode order on a shared-memory canvas) and two
//                       loop-filter warps (luma, chroma) walking the row in
//                       the reference's MB-raster filter order
//                       (src/h264/dec/slicedec.rs:184-208) behind the intra
//                       warps; rows hand over through shared memory, bands
//                       through progress words in global memory.  An intra
//                       MB waits only for its intra neighbours in the row
//                       above; the luma filter reports MB x-1 to the row
//                       below as soon as MB x's left edge is filtered.
//
// Or, for a group of up to RC_H264_GROUP_MAX consecutive pictures:
//
//  h264_group_kernel    one cooperative launch: the band CTAs of every
//                       picture of the group, and CTAs that run the MB phase
//                       (edge words included) of all of them in picture
//                       order; an inter MB waits only for the reference rows
//                       its motion vectors reach, an intra warp only for the
//                       MBs of its row.  The wavefronts of consecutive
//                       pictures then run side by side.
//
// rc_h264_deblock_noalloc filters a reconstructed picture without allocating
// (h264_db_params_kernel, then h264_deblock_kernel: one warp per MB row).
//
// Arithmetic follows src/h264/dec/{transform,intra,inter,deblock}.rs and the
// reconstruction half of slicedec.rs; citations at each function.
#include <cuda.h>  // CUcontext and CUresult: driver calls reached through cudaGetDriverEntryPointByVersion
#include <stdint.h>
#include <string.h>

#include <cstddef>
#include <mutex>

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
// Polls read with relaxed loads and order what follows with one acquire
// fence once the value is seen: an acquire load invalidates the SM's L1 on
// every poll, and warps that poll while their neighbours read cached
// reference samples would keep emptying it.
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Asynchronous global -> shared copies (tracked per thread by commit groups,
// not by the warp's register scoreboards, so that a filter warp can keep two
// MBs in flight without stalling on them).
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all_but_1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all_but_4() { asm volatile("cp.async.wait_group 4;" ::: "memory"); }

__device__ __forceinline__ bool aborted(const uint32_t *err) {
    return (*(const volatile uint32_t *)err & RC_DEV_ERR_TIMEOUT) != 0;
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
// src/h264/dec/picture.rs:723-735).  CA: a coherent load (ld.global.ca), for
// references written during the same launch (a group launch); otherwise the
// read-only path.
template <bool CA = false>
__device__ __forceinline__ int rs(const Ref &r, int x, int y) {
    const uint8_t *q = r.p + clampi(y, 0, r.h - 1) * r.pitch + clampi(x, 0, r.w - 1);
    return CA ? __ldca(q) : __ldg(q);
}
__device__ __forceinline__ int tap6(int a, int b, int c, int d, int e, int f) { return a - 5 * b + 20 * c + 20 * d - 5 * e + f; }
__device__ __forceinline__ int avg2(int a, int b) { return (a + b + 1) >> 1; }
template <bool CA = false>
__device__ __forceinline__ int htap(const Ref &r, int x, int y) {
    return tap6(rs<CA>(r, x - 2, y), rs<CA>(r, x - 1, y), rs<CA>(r, x, y), rs<CA>(r, x + 1, y), rs<CA>(r, x + 2, y),
                rs<CA>(r, x + 3, y));
}
template <bool CA = false>
__device__ __forceinline__ int vtap(const Ref &r, int x, int y) {
    return tap6(rs<CA>(r, x, y - 2), rs<CA>(r, x, y - 1), rs<CA>(r, x, y), rs<CA>(r, x, y + 1), rs<CA>(r, x, y + 2),
                rs<CA>(r, x, y + 3));
}
// mc_luma_win_scalar, inter.rs:73-213, for the sample at integer position (x, y)
template <bool CA = false>
__device__ int luma_sample(const Ref &r, int x, int y, int fx, int fy) {
    if (fx == 0 && fy == 0) return rs<CA>(r, x, y);
    if (fy == 0) {
        int b = clip255((htap<CA>(r, x, y) + 16) >> 5);
        return fx == 1 ? avg2(rs<CA>(r, x, y), b) : fx == 2 ? b : avg2(rs<CA>(r, x + 1, y), b);
    }
    if (fx == 0) {
        int h = clip255((vtap<CA>(r, x, y) + 16) >> 5);
        return fy == 2 ? h : avg2(fy == 1 ? rs<CA>(r, x, y) : rs<CA>(r, x, y + 1), h);
    }
    if (fx == 2 || fy == 2) {
        int b1[6];
#pragma unroll
        for (int j = 0; j < 6; j++) b1[j] = htap<CA>(r, x, y + j - 2);
        int j = clip255((tap6(b1[0], b1[1], b1[2], b1[3], b1[4], b1[5]) + 512) >> 10);
        if (fx == 2 && fy == 2) return j;
        if (fx == 2) return avg2(clip255(((fy == 1 ? b1[2] : b1[3]) + 16) >> 5), j);
        return avg2(clip255((vtap<CA>(r, x + (fx == 1 ? 0 : 1), y) + 16) >> 5), j);
    }
    int t = htap<CA>(r, x, y + (fy == 1 ? 0 : 1));
    int v = vtap<CA>(r, x + (fx == 1 ? 0 : 1), y);
    return avg2(clip255((t + 16) >> 5), clip255((v + 16) >> 5));
}
// mc_chroma_win_scalar, inter.rs:217-247, one sample at integer position (x, y)
template <bool CA = false>
__device__ __forceinline__ int chroma_sample(const Ref &r, int x, int y, int fx, int fy) {
    if ((fx | fy) == 0) return rs<CA>(r, x, y);
    int v = (8 - fx) * (8 - fy) * rs<CA>(r, x, y) + fx * (8 - fy) * rs<CA>(r, x + 1, y) + (8 - fx) * fy * rs<CA>(r, x, y + 1) +
            fx * fy * rs<CA>(r, x + 1, y + 1);
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
__device__ void edge_words(const DbMb &d, int lane, uint32_t *out);

// ===========================================================================
// Kernel 0: the loop filter's parameters of every MB -- boundary strengths,
// QPs, alpha / beta / tc0 -- as the 64 edge words the band kernel's filter
// warps read (deblock.rs:7-124, 302-371).  One warp per MB: the derivation
// is a short serial chain per MB, so all MBs of a picture are in flight at
// once instead of holding up the CTA of h264_mb_kernel.
// ===========================================================================
constexpr int EDGE_MBS = 8;  // MBs (warps) per CTA
__global__ void __launch_bounds__(32 * EDGE_MBS) h264_edge_kernel(H264Launch P) {
    __shared__ __align__(16) rc_h264_mb rec[EDGE_MBS][3];  // the MB, its left and top neighbours
    __shared__ DbMb dbm[EDGE_MBS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int addr = blockIdx.x * EDGE_MBS + w;
    if (addr >= P.mb_w * P.mb_h) return;  // whole warps only
    const int mbx = addr % P.mb_w, mby = addr / P.mb_w;
    constexpr int RW = (int)(sizeof(rc_h264_mb) / 4);
    for (int i = lane; i < 3 * RW; i += 32) {
        const int which = i / RW, j = i - which * RW;
        const int src = which == 0 ? addr : which == 1 ? (mbx > 0 ? addr - 1 : -1) : (mby > 0 ? addr - P.mb_w : -1);
        if (src >= 0) ((uint32_t *)&rec[w][which])[j] = __ldg((const uint32_t *)(P.mbs + src) + j);
    }
    __syncwarp();
    compute_db(P, rec[w][0], rec[w][1], rec[w][2], addr, lane, &dbm[w]);
    __syncwarp();
    edge_words(dbm[w], lane, P.edges + (size_t)addr * RC_EDGE_WORDS);
}

// ===========================================================================
// Kernel 0: motion derived from syntax (rc_h264_motion), one thread per MB row
// ===========================================================================
// The reference derives an MB's vectors as its slice decoder parses it
// (src/h264/dec/slicedec.rs): nb_motion :581-621, mvp :635-662, median_pred
// :664-681, set_motion :683-716, colocated :718-731, spatial_direct_base
// :733-752, derive_direct :754-852, derive_p_skip :854-866,
// derive_inter_motion :868-935.  An MB reads the derived motion of its
// left, top, top-right and top-left neighbours, so the rows run as a
// wavefront: thread y derives row y left to right, MB x once row y-1 has
// derived MBs 0..x+1.  The rows hand over through shared-memory progress;
// the motion itself is written to the engine's records (global memory, read
// back by the same CTA) and the picture's co-located motion to its slot.
struct ColMb {  // co-located motion of one MB (Frame::publish, picture.rs:492)
    uint8_t intra;
    uint8_t pad[3];
    int8_t ref_idx[2][4];
    uint32_t ref_id[2][4];
    int16_t mv[2][16][2];
};
static_assert(sizeof(ColMb) == RC_COLMB_BYTES, "co-located motion layout");

struct MvNb {
    int avail, ref, mvx, mvy;
};

// An MB's derived motion, as the records hold it (ref_idx, then after the
// 4-byte wp field, mv: byte offsets 36 and 48 of rc_h264_mb).
struct MbMv {
    int8_t ref[2][4];
    int16_t mv[2][16][2];
};

// One warp's derivation state, in shared memory: the MB being derived (ref,
// mv, done) and copies of its neighbours' motion (nbm: A, B, C, D; nb[i] < 0
// where neighbour i is unavailable).
struct MvState {
    int nb[4];
    uint32_t done;
    int8_t ref[2][4];
    int16_t mv[2][16][2];
    const rc_h264_slice *sl;
    const rc_h264_slice_motion *sm;
    const ColMb *col;
    MbMv nbm[4];
};

__device__ MvNb mv_nb(const MvState &S, int l, int x, int y) {
    const MvNb na = {0, -1, 0, 0};
    int which, bx, by;
    if (x < 0) {
        if (y < 0) { which = 3; bx = 3; by = 3; }
        else if (y > 3) return na;
        else { which = 0; bx = 3; by = y; }
    } else if (x > 3) {
        if (y < 0) { which = 2; bx = 0; by = 3; }
        else return na;
    } else if (y < 0) {
        which = 1; bx = x; by = 3;
    } else {
        if (!(S.done >> (y * 4 + x) & 1)) return na;
        const int r = S.ref[l][(y >> 1) * 2 + (x >> 1)];
        if (r < 0) return {1, -1, 0, 0};
        return {1, r, S.mv[l][y * 4 + x][0], S.mv[l][y * 4 + x][1]};
    }
    if (S.nb[which] < 0) return na;
    const MbMv &m = S.nbm[which];
    const int r = m.ref[l][(by >> 1) * 2 + (bx >> 1)];
    if (r < 0) return {1, -1, 0, 0};
    return {1, r, m.mv[l][by * 4 + bx][0], m.mv[l][by * 4 + bx][1]};
}

__device__ void mv_abc(const MvState &S, int l, int x, int y, int w, MvNb &a, MvNb &b, MvNb &c) {
    a = mv_nb(S, l, x - 1, y);
    b = mv_nb(S, l, x, y - 1);
    c = mv_nb(S, l, x + w, y - 1);
    if (!c.avail) c = mv_nb(S, l, x - 1, y - 1);
}

__device__ __forceinline__ int med3(int a, int b, int c) { return max(min(a, b), min(max(a, b), c)); }

__device__ void mv_median(MvNb a, MvNb b, MvNb c, int ref, int &ox, int &oy) {
    if (!b.avail && !c.avail && a.avail) {
        b = a;
        c = a;
    }
    const bool ma = a.ref == ref, mb = b.ref == ref, mc = c.ref == ref;
    if (ma && !mb && !mc) { ox = a.mvx; oy = a.mvy; return; }
    if (!ma && mb && !mc) { ox = b.mvx; oy = b.mvy; return; }
    if (!ma && !mb && mc) { ox = c.mvx; oy = c.mvy; return; }
    ox = med3(a.mvx, b.mvx, c.mvx);
    oy = med3(a.mvy, b.mvy, c.mvy);
}

// shape 1: 16x8, 2: 8x16 (directional predictors); x, y, w in 4x4 blocks
__device__ void mv_pred(const MvState &S, int l, int x, int y, int w, int ref, int shape, int part, int &ox, int &oy) {
    MvNb a, b, c;
    mv_abc(S, l, x, y, w, a, b, c);
    if (shape == 1) {
        if (part == 0 && b.ref == ref) { ox = b.mvx; oy = b.mvy; return; }
        if (part == 1 && a.ref == ref) { ox = a.mvx; oy = a.mvy; return; }
    } else if (shape == 2) {
        if (part == 0 && a.ref == ref) { ox = a.mvx; oy = a.mvy; return; }
        if (part == 1 && c.ref == ref) { ox = c.mvx; oy = c.mvy; return; }
    }
    mv_median(a, b, c, ref, ox, oy);
}

__device__ void mv_set(MvState &S, int x, int y, int w, int h, const int refs[2], const int mvs[2][2]) {
    for (int l = 0; l < 2; l++) {
        // (x, y) of a block as one word: one shared-memory store per block
        const uint32_t v = refs[l] >= 0 ? ((uint32_t)(uint16_t)mvs[l][0] | (uint32_t)(uint16_t)mvs[l][1] << 16) : 0u;
        uint32_t *dst = (uint32_t *)S.mv[l];
        for (int yy = y; yy < y + h; yy++)
            for (int xx = x; xx < x + w; xx++) dst[yy * 4 + xx] = v;
        for (int by = y >> 1; by <= (y + h - 1) >> 1; by++)
            for (int bx = x >> 1; bx <= (x + w - 1) >> 1; bx++) S.ref[l][by * 2 + bx] = (int8_t)refs[l];
    }
    for (int yy = y; yy < y + h; yy++)
        for (int xx = x; xx < x + w; xx++) S.done |= 1u << (yy * 4 + xx);
}

__device__ void mv_colocated(const MvState &S, int raster, int &mvx, int &mvy, int &ref, uint32_t &id) {
    if (S.sm->direct_8x8_inference) raster = ((raster >> 2) >= 2 ? 12 : 0) + ((raster & 3) >= 2 ? 3 : 0);
    const ColMb *m = S.col;
    if (!m || m->intra) {
        mvx = mvy = 0;
        ref = -1;
        id = 0xffffffffu;
        return;
    }
    const int b8 = (raster >> 3) * 2 + ((raster & 3) >> 1);
    const int l = m->ref_idx[0][b8] >= 0 ? 0 : 1;
    mvx = m->mv[l][raster][0];
    mvy = m->mv[l][raster][1];
    ref = m->ref_idx[l][b8];
    id = m->ref_id[l][b8];
}

__device__ __forceinline__ int min_pos(int x, int y) { return (x >= 0 && y >= 0) ? min(x, y) : max(x, y); }
__device__ __forceinline__ bool small_mv(int x, int y) { return x >= -1 && x <= 1 && y >= -1 && y <= 1; }
__device__ __forceinline__ int wrap16(int v) { return (int)(int16_t)(uint16_t)(v & 0xffff); }

__device__ void mv_direct(MvState &S, int b8_mask) {
    const int spatial = S.sm->direct_spatial, d8i = S.sm->direct_8x8_inference;
    int base_refs[2] = {0, 0}, base_mvs[2][2] = {{0, 0}, {0, 0}};
    bool direct_zero = false;
    if (spatial) {
        MvNb nbs[2][3];
        for (int l = 0; l < 2; l++) {
            mv_abc(S, l, 0, 0, 4, nbs[l][0], nbs[l][1], nbs[l][2]);
            base_refs[l] = min_pos(nbs[l][0].ref, min_pos(nbs[l][1].ref, nbs[l][2].ref));
        }
        if (base_refs[0] < 0 && base_refs[1] < 0) {
            base_refs[0] = base_refs[1] = 0;
            direct_zero = true;
        } else {
            for (int l = 0; l < 2; l++)
                if (base_refs[l] >= 0) mv_median(nbs[l][0], nbs[l][1], nbs[l][2], base_refs[l], base_mvs[l][0], base_mvs[l][1]);
        }
    }
    const bool cst = S.sm->col_short_term != 0;
    const bool need_col = !direct_zero && cst && (base_refs[0] == 0 || base_refs[1] == 0);
    if (spatial && (!need_col || d8i)) {
        for (int b8 = 0; b8 < 4; b8++) {
            if (!(b8_mask >> b8 & 1)) continue;
            bool zero = false;
            if (need_col) {
                int cx, cy, r;
                uint32_t id;
                mv_colocated(S, (b8 >> 1) * 8 + (b8 & 1) * 2, cx, cy, r, id);
                zero = r == 0 && small_mv(cx, cy);
            }
            int mvs[2][2];
            for (int l = 0; l < 2; l++) {
                const bool z = direct_zero || base_refs[l] < 0 || (base_refs[l] == 0 && zero);
                mvs[l][0] = z ? 0 : base_mvs[l][0];
                mvs[l][1] = z ? 0 : base_mvs[l][1];
            }
            mv_set(S, (b8 & 1) * 2, (b8 >> 1) * 2, 2, 2, base_refs, mvs);
        }
        return;
    }
    for (int b8 = 0; b8 < 4; b8++) {
        if (!(b8_mask >> b8 & 1)) continue;
        const int x8 = (b8 & 1) * 2, y8 = (b8 >> 1) * 2, unit = d8i ? 2 : 1;
        for (int sub = 0; sub < (unit == 1 ? 4 : 1); sub++) {
            const int x = x8 + (sub & 1), y = y8 + (sub >> 1);
            int cx, cy, rc;
            uint32_t idc;
            mv_colocated(S, y * 4 + x, cx, cy, rc, idc);
            int refs[2], mvs[2][2];
            if (spatial) {
                const bool col_zero = cst && rc == 0 && small_mv(cx, cy);
                for (int l = 0; l < 2; l++) {
                    const bool z = direct_zero || base_refs[l] < 0 || (base_refs[l] == 0 && col_zero);
                    mvs[l][0] = z ? 0 : base_mvs[l][0];
                    mvs[l][1] = z ? 0 : base_mvs[l][1];
                    refs[l] = base_refs[l];
                }
            } else {
                const int n0 = min(__ldg(&S.sl->num_ref[0]), RC_H264_MAX_REFS);
                int ref0 = 0;
                if (rc >= 0)
                    for (int i = 0; i < n0; i++)
                        if (__ldg(&S.sl->ref_id[0][i]) == idc) { ref0 = i; break; }
                const bool copy = ref0 < n0 ? S.sm->direct_copy[ref0] != 0 : true;
                const int dsf = ref0 < n0 ? S.sm->dist_scale[ref0] : 256;
                if (copy) {
                    mvs[0][0] = cx; mvs[0][1] = cy;
                    mvs[1][0] = mvs[1][1] = 0;
                } else {
                    mvs[0][0] = (int16_t)((dsf * cx + 128) >> 8);
                    mvs[0][1] = (int16_t)((dsf * cy + 128) >> 8);
                    mvs[1][0] = wrap16(mvs[0][0] - cx);
                    mvs[1][1] = wrap16(mvs[0][1] - cy);
                }
                refs[0] = ref0;
                refs[1] = 0;
            }
            mv_set(S, x, y, unit, unit, refs, mvs);
        }
    }
}

// One inter MB's motion; false for a record the reference rejects (ref_idx
// past its list, a direct sub-partition outside a B slice).
__device__ bool mv_derive(MvState &S, const rc_h264_motion &mo) {
    const int n[2] = {min(__ldg(&S.sl->num_ref[0]), RC_H264_MAX_REFS), min(__ldg(&S.sl->num_ref[1]), RC_H264_MAX_REFS)};
    if (mo.shape == RC_H264_MOTION_SKIP) {
        if (S.sm->b_slice) {
            mv_direct(S, 0xf);
            return true;
        }
        if (n[0] < 1) return false;
        const MvNb a = mv_nb(S, 0, -1, 0), b = mv_nb(S, 0, 0, -1);
        int mvs[2][2] = {{0, 0}, {0, 0}};
        if (!(S.nb[0] < 0 || S.nb[1] < 0 || (a.ref == 0 && a.mvx == 0 && a.mvy == 0) ||
              (b.ref == 0 && b.mvx == 0 && b.mvy == 0)))
            mv_pred(S, 0, 0, 0, 4, 0, 0, 0, mvs[0][0], mvs[0][1]);
        const int refs[2] = {0, -1};
        mv_set(S, 0, 0, 4, 4, refs, mvs);
        return true;
    }
    if (mo.shape != RC_H264_MOTION_8x8) {
        const int np = mo.shape == RC_H264_MOTION_16x16 ? 1 : 2;
        const int shape = mo.shape == RC_H264_MOTION_16x8 ? 1 : mo.shape == RC_H264_MOTION_8x16 ? 2 : 0;
        for (int p = 0; p < np; p++) {
            const int x = shape == 2 ? 2 * p : 0, y = shape == 1 ? 2 * p : 0;
            const int w = shape == 2 ? 2 : 4, h = shape == 1 ? 2 : 4, b8 = (y >> 1) * 2 + (x >> 1);
            int refs[2] = {-1, -1}, mvs[2][2] = {{0, 0}, {0, 0}};
            for (int l = 0; l < 2; l++) {
                if (!(mo.pred[p] >> l & 1)) continue;
                const int r = mo.ref_idx[l][b8];
                if (r < 0 || r >= n[l]) return false;
                int px, py;
                mv_pred(S, l, x, y, w, r, shape, p, px, py);
                refs[l] = r;
                mvs[l][0] = wrap16(px + mo.mvd[l][y * 4 + x][0]);
                mvs[l][1] = wrap16(py + mo.mvd[l][y * 4 + x][1]);
            }
            mv_set(S, x, y, w, h, refs, mvs);
        }
        return true;
    }
    for (int p = 0; p < 4; p++) {
        const int x8 = (p & 1) * 2, y8 = (p >> 1) * 2, sub = mo.sub[p];
        if (sub == RC_H264_SUB_DIRECT) {
            if (!S.sm->b_slice) return false;
            mv_direct(S, 1 << p);
            continue;
        }
        if (sub > RC_H264_SUB_4x4) return false;
        int refs[2] = {-1, -1};
        for (int l = 0; l < 2; l++) {
            if (!(mo.pred[p] >> l & 1)) continue;
            const int v = mo.ref_idx[l][p];
            if (v < 0 || v >= n[l]) return false;
            refs[l] = v;
        }
        const int sw = (sub == RC_H264_SUB_8x8 || sub == RC_H264_SUB_8x4) ? 2 : 1;
        const int sh = (sub == RC_H264_SUB_8x8 || sub == RC_H264_SUB_4x8) ? 2 : 1;
        for (int sy = 0; sy < 2; sy += sh)
            for (int sx = 0; sx < 2; sx += sw) {
                const int x = x8 + sx, y = y8 + sy;
                int mvs[2][2] = {{0, 0}, {0, 0}};
                for (int l = 0; l < 2; l++) {
                    if (refs[l] < 0) continue;
                    int px, py;
                    mv_pred(S, l, x, y, sw, refs[l], 0, 0, px, py);
                    mvs[l][0] = wrap16(px + mo.mvd[l][y * 4 + x][0]);
                    mvs[l][1] = wrap16(py + mo.mvd[l][y * 4 + x][1]);
                }
                mv_set(S, x, y, sw, sh, refs, mvs);
            }
    }
    return true;
}

// The rows as warps of a cooperative launch: CTA c derives rows
// [c * R, c * R + R), one warp per row.  Rows of a CTA hand over through
// shared memory: each row keeps its MBs' bottom-row motion (all the row
// below reads of it) and its progress there.  A CTA's first row reads the
// row above from the records in global memory, behind that row's progress
// word (P.mvprog), which the CTA's last row publishes.  The inputs of the
// next MB -- its syntax and the record headers (kind, slice) of it and its
// neighbours, which never change -- are staged one MB ahead with cp.async.
// Per MB, lane 0 derives from shared memory and the lanes store the motion
// into the records and the co-located store.
static_assert(sizeof(MbMv) == 136 && offsetof(rc_h264_mb, ref_idx) == 36 && offsetof(rc_h264_mb, wp) == 44 &&
                  offsetof(rc_h264_mb, mv) == 48 && sizeof(rc_h264_motion) == 148 && sizeof(rc_h264_mb) % 16 == 0,
              "record layout the warp copies rely on");
constexpr int MV_MAX_WARPS = 16;

// Bottom-row motion of one MB: the ref_idx of its two bottom 8x8 blocks and
// the vectors of its four bottom 4x4 blocks, per list (9 words).
struct MbBottom {
    int8_t ref[2][2];
    int16_t mv[2][4][2];
};
static_assert(sizeof(MbBottom) == 36, "bottom-row motion layout");

struct __align__(16) MvWarp {
    MvState S;
    uint4 hdr[2][5];          // record headers of MB x, A, B, C, D (slot x & 1)
    rc_h264_motion mo[2];     // syntax of MB x (slot x & 1)
    int ok;
};

size_t mv_smem(int rows, int mb_w) { return (size_t)rows * (sizeof(MvWarp) + (size_t)mb_w * sizeof(MbBottom)); }

__global__ void __launch_bounds__(MV_MAX_WARPS * 32, 1) h264_mv_kernel(const __grid_constant__ H264Launch P) {
    extern __shared__ __align__(16) uint8_t mv_dyn[];
    __shared__ volatile int rprog[MV_MAX_WARPS];
    const int R = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y = blockIdx.x * R + w;
    if (threadIdx.x < MV_MAX_WARPS) rprog[threadIdx.x] = 0;
    __syncthreads();
    if (y >= P.mb_h) return;
    MvWarp &W = ((MvWarp *)mv_dyn)[w];
    MbBottom *bottom = (MbBottom *)(mv_dyn + (size_t)R * sizeof(MvWarp));
    MbBottom *mine = bottom + (size_t)w * P.mb_w, *above = w > 0 ? bottom + (size_t)(w - 1) * P.mb_w : nullptr;
    MvState &S = W.S;
    const uint32_t tag = (P.epoch & 0xffffu) << 16;
    const bool last = w == R - 1 || y == P.mb_h - 1;  // publishes for the next CTA
    ColMb *out = (ColMb *)(P.col + (size_t)P.out_slot * P.col_stride);
    // stage MB x's inputs into slot x & 1 (every lane commits one group)
    auto stage = [&](int x) {
        if (x < P.mb_w) {
            const int sl = x & 1;
            if (lane < 5) {
                const int dx = lane == 1 ? -1 : lane == 3 ? 1 : lane == 4 ? -1 : 0, dy = lane >= 2 ? -1 : 0;
                const int nx = x + dx, ny = y + dy;
                if (nx >= 0 && ny >= 0 && nx < P.mb_w) cp_async16(&W.hdr[sl][lane], P.mbs_out + ny * P.mb_w + nx);
                else W.hdr[sl][lane] = make_uint4(0, 0, 0, 0);  // kind RC_H264_NONE
            }
            const uint32_t *src = (const uint32_t *)(P.motion + y * P.mb_w + x);
            uint32_t *dst = (uint32_t *)&W.mo[sl];
            cp_async4(dst + lane, src + lane);
            if (lane < 5) cp_async4(dst + 32 + lane, src + 32 + lane);
        }
        cp_commit();
    };
    stage(0);
    int seen = y > 0 ? 0 : P.mb_w;  // progress of row y-1 observed so far
    for (int x = 0; x < P.mb_w; x++) {
        const int addr = y * P.mb_w + x, sl = x & 1;
        stage(x + 1);
        cp_wait_all_but_1();  // MB x's inputs
        __syncwarp();
        const int kind = ((const uint8_t *)&W.hdr[sl][0])[0], slice = ((const uint16_t *)&W.hdr[sl][0])[4];
        const bool inter = kind == RC_H264_INTER && slice < P.num_slices;
        // row y-1 through MB x+1 (the top-right neighbour)
        const int need = min(x + 2, P.mb_w);
        if (seen < need) {
            bool ok = true;
            int v = 0;
            if (lane == 0) {
                uint32_t it = 0, ns = 16;
                for (;;) {
                    if (w == 0) {
                        const uint32_t f = ld_acquire(P.mvprog + y - 1);
                        v = (f & 0xffff0000u) == tag ? (int)(f & 0xffffu) : 0;
                    } else {
                        v = rprog[w - 1];
                    }
                    if (v >= need) break;
                    if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) { ok = false; break; }
                    __nanosleep(ns);
                    ns = min(ns * 2, 128u);
                }
            }
            if (!__shfl_sync(0xffffffffu, ok, 0)) {
                if (lane == 0) {
                    set_error(P.error, RC_DEV_ERR_TIMEOUT);
                    rprog[w] = P.mb_w;  // the rows below give up too
                    if (last) st_release(P.mvprog + y, tag | (uint32_t)P.mb_w);
                }
                cp_wait_all();
                return;
            }
            seen = __shfl_sync(0xffffffffu, v, 0);
            __syncwarp();
            __threadfence_block();
        }
        if (inter) {
            // neighbour availability (A, B, C, D): decoded and in this slice
            if (lane < 4) {
                const uint4 h = W.hdr[sl][1 + lane];
                const int nk = ((const uint8_t *)&h)[0], ns = ((const uint16_t *)&h)[4];
                const int dx = lane == 0 ? -1 : lane == 2 ? 1 : lane == 3 ? -1 : 0, dy = lane == 0 ? 0 : -1;
                S.nb[lane] = (nk != RC_H264_NONE && ns == slice && x + dx >= 0 && x + dx < P.mb_w && y + dy >= 0)
                                 ? (y + dy) * P.mb_w + x + dx
                                 : -1;
            }
            __syncwarp();
            // B, C, D: the bottom-row motion of MBs x, x+1, x-1 of row y-1
            if (w > 0) {
                for (int k = lane; k < 27; k += 32) {
                    const int which = 1 + k / 9, j = k % 9;
                    if (S.nb[which] < 0) continue;
                    const int nx = x + (which == 2 ? 1 : which == 3 ? -1 : 0);
                    const uint32_t v = ((const uint32_t *)(above + nx))[j];
                    if (j == 0) {
                        ((uint16_t *)S.nbm[which].ref)[1] = (uint16_t)v;          // list 0, 8x8 blocks 2, 3
                        ((uint16_t *)S.nbm[which].ref)[3] = (uint16_t)(v >> 16);  // list 1
                    } else {
                        const int l = (j - 1) >> 2, b = (j - 1) & 3;
                        ((uint32_t *)S.nbm[which].mv)[l * 16 + 12 + b] = v;
                    }
                }
            } else {
                for (int k = lane; k < 3 * 34; k += 32) {
                    const int which = 1 + k / 34, j = k % 34, na = S.nb[which];
                    if (na < 0) continue;
                    // through L2: an L1 line loaded earlier may predate the row above's stores
                    const uint32_t *src = (const uint32_t *)(P.mbs_out + na);
                    ((uint32_t *)&S.nbm[which])[j] = __ldcg(src + (j < 2 ? 9 + j : 10 + j));
                }
            }
        }
        // the MB's motion starts empty (all lanes clear it, then lane 0 derives)
        ((uint32_t *)S.mv)[lane] = 0;
        if (lane < 2) ((uint32_t *)S.ref)[lane] = 0xffffffffu;
        __syncwarp();
        if (lane == 0) {
            W.ok = 1;
            if (inter) {
                S.done = 0;
                S.sl = P.slices + slice;
                S.sm = P.smotion + slice;
                S.col = nullptr;
                const int cs = S.sm->col_slot;
                if (S.sm->b_slice) {
                    if (cs >= 0 && cs < P.dpb_slots) S.col = (const ColMb *)(P.col + (size_t)cs * P.col_stride) + addr;
                    else W.ok = 0;
                }
                if (W.ok && !mv_derive(S, W.mo[sl])) W.ok = 0;
                if (!W.ok) {
                    set_error(P.error, RC_DEV_ERR_RECORD);
                    for (int l = 0; l < 2; l++)
                        for (int b8 = 0; b8 < 4; b8++) S.ref[l][b8] = -1;
                }
            } else if (kind == RC_H264_INTER) {
                set_error(P.error, RC_DEV_ERR_RECORD);
            }
        }
        __syncwarp();
        // the motion: bottom row for the row below, the records (ref_idx, wp,
        // mv: words 9..43), the co-located store (43 words), and MB x+1's
        // left neighbour
        const uint32_t *cur_ref = (const uint32_t *)S.ref, *cur_mv = (const uint32_t *)S.mv;
        if (lane < 9)
            ((uint32_t *)(mine + x))[lane] =
                lane == 0 ? ((cur_ref[0] >> 16) | (cur_ref[1] & 0xffff0000u)) : cur_mv[((lane - 1) >> 2) * 16 + 12 + ((lane - 1) & 3)];
        {
            uint32_t *rec = (uint32_t *)(P.mbs_out + addr);
            uint32_t *col = (uint32_t *)(out + addr);
            for (int i = lane; i < 35; i += 32) {
                uint32_t v;
                if (i < 2) v = cur_ref[i];
                else if (i == 2) {
                    v = 0;
                    for (int b8 = 0; b8 < 4; b8++) {
                        const uint32_t wv = inter ? P.smotion[slice].wp_map[(S.ref[0][b8] + 1) * (RC_H264_MAX_REFS + 1) +
                                                                             (S.ref[1][b8] + 1)]
                                                  : 0xffu;
                        v |= wv << (8 * b8);
                    }
                } else v = cur_mv[i - 3];
                rec[9 + i] = v;
            }
            for (int i = lane; i < 43; i += 32) {
                uint32_t v;
                if (i == 0) v = inter ? 0u : 1u;
                else if (i < 3) v = cur_ref[i - 1];
                else if (i < 11) {
                    const int l = (i - 3) >> 2, b8 = (i - 3) & 3, r = S.ref[l][b8];
                    v = r >= 0 ? __ldg(&P.slices[slice].ref_id[l][r]) : 0xffffffffu;
                } else v = cur_mv[i - 11];
                col[i] = v;
            }
            for (int i = lane; i < 34; i += 32) ((uint32_t *)&S.nbm[0])[i] = i < 2 ? cur_ref[i] : cur_mv[i - 2];
        }
        __syncwarp();
        if (lane == 0) {
            if (last && y + 1 < P.mb_h) {
                __threadfence();
                st_relaxed(P.mvprog + y, tag | (uint32_t)(x + 1));
            }
            __threadfence_block();
            rprog[w] = x + 1;
        }
    }
    cp_wait_all();
}

// ===========================================================================
// Kernel 1: inter MBs (prediction + residual) and I_PCM, one CTA per MB.
// ===========================================================================
// Group launches: before an inter MB is predicted, the rows of the in-flight
// pictures it references that its motion vectors reach (6-tap windows
// included) must be final.  Row r of a picture is final through MB column c
// once row r + 1 has loop-filtered and stored MBs 0..c+1 (the top edge of
// row r + 1 is the last change to row r's bottom lines, and MB c+1's left
// edge the last change to MB c), so the MB waits for the reference's filter
// progress on row min(R + 1, last) to reach column C + 2, R and C being the
// furthest MB row and column any of its blocks reads.  Chroma reads reach no
// further than luma.  Warp 0; false after a timeout.
__device__ bool mb_wait_refs(const H264Launch &P, const rc_h264_mb &m, const rc_h264_slice *sl, int mbx, int mby,
                             int t) {
    if (t >= 32) return true;
    const int k = t & 15, l = t >> 4, b8 = ((k >> 2) >> 1) * 2 + ((k & 3) >> 1);
    const int ri = m.ref_idx[l][b8];
    int slot = -1, r = -1, c = -1;
    if (ri >= 0 && ri < min(__ldg(&sl->num_ref[l]), RC_H264_MAX_REFS)) {
        slot = __ldg(&sl->ref_slot[l][ri]);
        const int bottom = mby * 16 + (k >> 2) * 4 + 3 + (m.mv[l][k][1] >> 2) + 3;
        const int right = mbx * 16 + (k & 3) * 4 + 3 + (m.mv[l][k][0] >> 2) + 3;
        r = clampi(bottom >> 4, 0, P.mb_h - 1);
        c = clampi(right >> 4, 0, P.mb_w - 1);
    }
    bool ok = true;
    for (int i = 0; i < P.nwait; i++) {
        const int rr = __reduce_max_sync(0xffffffffu, slot == P.wait_slot[i] ? r : -1);
        const int cc = __reduce_max_sync(0xffffffffu, slot == P.wait_slot[i] ? c : -1);
        if (rr < 0) continue;
        if (t == 0) {
            const uint32_t *f = P.wait_refprog[i] + (size_t)min(rr + 1, P.mb_h - 1) * RC_REFPROG_STRIDE;
            const uint32_t tag = (P.wait_epoch[i] & 0xffffu) << 16, need = (uint32_t)min(cc + 2, P.mb_w);
            // back off to 4 us between polls: many warps wait here at once,
            // and their polls would load the L2 that the band CTAs' hand-overs
            // go through
            uint32_t it = 0, v, ns = 64;
            while (((v = ld_relaxed(f)) & 0xffff0000u) != tag || (v & 0xffffu) < need) {
                if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) { ok = false; break; }
                __nanosleep(ns);
                ns = min(ns * 2, 4096u);
            }
            fence_acquire();
        }
    }
    return __shfl_sync(0xffffffffu, ok, 0);
}

// Shared state of one MB-phase worker (256 threads).
struct __align__(16) MbSmem {
    rc_h264_mb m;
    int32_t coef[256];
    int32_t coefc[128];
    uint8_t predy[256];
    uint8_t predc[128];
    uint32_t nzl, nzc, ibits;  // ibits, intra: neighbour availability (bits 0..3: left, top, top-right, top-left)
};

// Barrier `id` over the `n` threads of one MB worker (id 0 with n = the
// CTA's threads is __syncthreads).
__device__ __forceinline__ void bar_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

// One macroblock of the MB phase, 256 threads (t = 0..255, barrier `bar`):
// inter prediction with the residual, I_PCM copy, or an intra MB's residual
// and prediction parameters.
__device__ void mb_body(const H264Launch &P, MbSmem &M, const int addr, const int t, const int bar) {
    rc_h264_mb &m = M.m;
    int32_t *coef = M.coef, *coefc = M.coefc;
    uint8_t *predy = M.predy, *predc = M.predc;
    uint32_t &nzl = M.nzl, &nzc = M.nzc, &ibits = M.ibits;
    const int mbx = addr % P.mb_w, mby = addr / P.mb_w;
    constexpr int RW = (int)(sizeof(rc_h264_mb) / 4);
    if (t < RW) ((uint32_t *)&m)[t] = __ldg((const uint32_t *)(P.mbs + addr) + t);
    if (t == 0) { nzl = 0; nzc = 0; }
    coef[t] = 0;
    if (t < 128) coefc[t] = 0;
    bar_sync(bar, 256);
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
        if (P.bottom) {  // before a group launch: the unfiltered bottom rows
            uint8_t *b = P.bottom + (size_t)mby * P.mb_w * 32;
            if (t < 16) b[mbx * 16 + t] = (uint8_t)s[240 + t];
            else if (t < 32) b[P.mb_w * (16 + 8 * ((t - 16) >> 3)) + mbx * 8 + (t & 7)] = (uint8_t)s[256 + ((t - 16) >> 3) * 64 + 56 + (t & 7)];
        }
        return;
    }
    if (m.slice >= P.num_slices) { if (t == 0) set_error(P.error, RC_DEV_ERR_RECORD); return; }
    const rc_h264_slice *sl = P.slices + m.slice;
    const bool intra = kind != RC_H264_INTER;
    // residual-only pass (before a group launch): inter MBs store their
    // residual like intra MBs; the group kernel predicts and adds it
    const bool resid = intra || P.residual_only;
    const int t8 = m.transform_8x8, i16 = kind == RC_H264_I16x16;
    const int nl = __popc(m.luma_coded & (t8 ? 0xf : 0xffff)), ndc = __popc(m.dc_coded & 6);
    const int nlum = (i16 && (m.dc_coded & 1)) ? 16 : 0;
    const unsigned long long need =
        nlum + (unsigned long long)nl * (t8 ? 64 : 16) + ndc * 4 + __popc(m.chroma_coded) * 16;
    if (m.coef_off + need > P.num_levels) { if (t == 0) set_error(P.error, RC_DEV_ERR_RECORD); return; }
    if (intra) {
        if (t == 0) ibits = 0;
        bar_sync(bar, 256);
        if (t < 4) {
            // start_mb neighbour availability + intra_nb, slicedec.rs:489-508, 525-530
            const int dx = t == 0 ? -1 : t == 2 ? 1 : t == 3 ? -1 : 0, dy = t == 0 ? 0 : -1;
            const int nx = mbx + dx, ny = mby + dy;
            if (nx >= 0 && ny >= 0 && nx < P.mb_w) {
                const rc_h264_mb *pm = P.mbs + ny * P.mb_w + nx;
                const int nk = __ldg(&pm->kind);
                const bool a = nk != RC_H264_NONE && __ldg(&pm->slice) == m.slice && (!P.constrained_intra || is_intra(nk));
                if (a) atomicOr(&ibits, 1u << t);
            }
        }
    }
    if (!resid) {
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
    bar_sync(bar, 256);
    // ---- inverse transforms: rows, then columns
    if (t8) {
        if (t < 32 && (nzl >> (t >> 3) & 1)) idct8_1d(coef + (t >> 3) * 64 + (t & 7) * 8, 1);
    } else if (t < 64 && (nzl >> (t >> 2) & 1)) idct4_1d(coef + (t >> 2) * 16 + (t & 3) * 4, 1);
    if (t >= 64 && t < 96 && (nzc >> ((t - 64) >> 2) & 1)) idct4_1d(coefc + ((t - 64) >> 2) * 16 + (t & 3) * 4, 1);
    bar_sync(bar, 256);
    if (t8) {
        if (t < 32 && (nzl >> (t >> 3) & 1)) idct8_1d(coef + (t >> 3) * 64 + (t & 7), 8);
    } else if (t < 64 && (nzl >> (t >> 2) & 1)) idct4_1d(coef + (t >> 2) * 16 + (t & 3), 4);
    if (t >= 64 && t < 96 && (nzc >> ((t - 64) >> 2) & 1)) idct4_1d(coefc + ((t - 64) >> 2) * 16 + (t & 3), 4);
    bar_sync(bar, 256);
    if (resid) {
        // residual samples ((v + 32) >> 6, idct4_add / idct8_add) and, for
        // intra MBs, the prediction parameters for the intra wavefront
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
        if (intra && t == 0) {
            IntraInfo in;
            in.kind = (uint8_t)kind;
            in.t8 = (uint8_t)t8;
            in.i16_mode = m.i16_mode;
            in.chroma_mode = m.chroma_mode;
            in.nb = (uint8_t)(ibits & 15);
            in.pad0 = in.pad1 = in.pad2 = 0;
            for (int i = 0; i < 16; i++) in.modes[i] = m.intra_modes[i];
            in.pad3[0] = in.pad3[1] = 0;
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

// Six CTAs per SM (40 registers): the CTA's phases meet at barriers, and
// more resident CTAs hide them (1080p P+I sequence, MB kernel per picture:
// 4 CTAs per SM 60.9 us, 5 55.0, 6 52.3, 8 50.8 with 168 bytes of spills).
__global__ void __launch_bounds__(256, 6) h264_mb_kernel(const __grid_constant__ H264Launch P) {
    __shared__ MbSmem M;
    mb_body(P, M, blockIdx.x, threadIdx.x, 0);
}

// ===========================================================================
// Kernel 2: intra + deblocking wavefront, one warp per task.
// ===========================================================================
struct __align__(16) WarpSmem {
    IntraInfo q;          // the task's MB (modes, availability)
    int16_t res[384];     // residual samples: 16x16 luma, then 8x8 Cb, 8x8 Cr
    uint8_t cy[17 * 32];  // luma canvas: rows -1..15, cols -1..30 -> [(r+1)*32 + c+1]
    uint8_t cc[2][9 * 12];  // chroma canvas: rows -1..7, cols -1..10
    int32_t f[32];       // reference arrays: an 8x8 block's smoothed samples, or two 4x4 blocks'
};

__device__ __forceinline__ int cvy(const WarpSmem &S, int r, int c) { return S.cy[(r + 1) * 32 + c + 1]; }

// pred_nxn (src/h264/dec/intra.rs:64-192) and pred8x8 (intra.rs:194-238) as
// data.  For every mode and sample position of an n x n block (n = 4, 8) the
// table holds the three reference samples the prediction reads and the
// weights it combines them with, (w0 r0 + w1 r1 + w2 r2 + rnd) >> 2:
//   copy                        (4, 0, 0, 0)
//   (r0 + r1 + 1) >> 1          (2, 2, 0, 2)
//   (r0 + 2 r1 + r2 + 2) >> 2   (1, 2, 1, 2)
//   (r0 + 3 r1 + 2) >> 2        (1, 3, 0, 2)
// and DC copies the DC entry of the reference array.  A warp then predicts
// samples of any mix of modes and positions with one instruction sequence:
// no lane takes a branch of its own (divergent selects over the mode cost
// several times the arithmetic).  Reference arrays: 4x4 -- 0 corner, 1..8
// top 0..7, 9..12 left 0..3, 13 DC (4-bit indices); 8x8 -- the smoothed
// samples top 0..15, left 16..23, corner 24, DC 25 (5-bit indices).
template <int N>
struct PredTab {
    uint32_t e[9][N * N];
};
template <int N>
__host__ __device__ constexpr uint32_t ptS() { return N == 4 ? 4 : 5; }
template <int N>
__host__ __device__ constexpr int ptT(int i) { return N == 4 ? (i < 0 ? 0 : 1 + i) : (i < 0 ? 24 : i); }
template <int N>
__host__ __device__ constexpr int ptL(int j) { return N == 4 ? (j < 0 ? 0 : 9 + j) : (j < 0 ? 24 : 16 + j); }
template <int N>
__host__ __device__ constexpr int ptDC() { return N == 4 ? 13 : 25; }
// k: 0 copy, 1 (r0 + r1 + 1) >> 1, 2 (r0 + 2 r1 + r2 + 2) >> 2, 3 (r0 + 3 r1 + 2) >> 2
template <int N>
__host__ __device__ constexpr uint32_t ptE(int k, int a, int b = 0, int c = 0) {
    const uint32_t s = ptS<N>();
    const uint32_t w0 = k == 0 ? 4 : k == 1 ? 2 : 1, w1 = k == 0 ? 0 : k == 3 ? 3 : 2, w2 = k == 2 ? 1 : 0,
                   rnd = k == 0 ? 0 : 2;
    return (uint32_t)a | (uint32_t)b << s | (uint32_t)c << (2 * s) | w0 << (3 * s) | w1 << (3 * s + 3) |
           w2 << (3 * s + 5) | rnd << (3 * s + 6);
}
template <int N>
__host__ __device__ constexpr uint32_t pt_entry(int mode, int x, int y) {
    constexpr int n = N;
    switch (mode) {
    case 0: return ptE<N>(0, ptT<N>(x));
    case 1: return ptE<N>(0, ptL<N>(y));
    case 2: return ptE<N>(0, ptDC<N>());
    case 3:
        if (x == n - 1 && y == n - 1) return ptE<N>(3, ptT<N>(2 * n - 2), ptT<N>(2 * n - 1));
        return ptE<N>(2, ptT<N>(x + y), ptT<N>(x + y + 1), ptT<N>(x + y + 2));
    case 4:
        if (x > y) return ptE<N>(2, ptT<N>(x - y - 2), ptT<N>(x - y - 1), ptT<N>(x - y));
        if (x < y) return ptE<N>(2, ptL<N>(y - x - 2), ptL<N>(y - x - 1), ptL<N>(y - x));
        return ptE<N>(2, ptT<N>(0), ptT<N>(-1), ptL<N>(0));
    case 5: {
        const int z = 2 * x - y, i = x - (y >> 1);
        if (z >= 0 && (z & 1) == 0) return ptE<N>(1, ptT<N>(i - 1), ptT<N>(i));
        if (z > 0) return ptE<N>(2, ptT<N>(i - 2), ptT<N>(i - 1), ptT<N>(i));
        if (z == -1) return ptE<N>(2, ptL<N>(0), ptT<N>(-1), ptT<N>(0));
        return ptE<N>(2, ptL<N>(y - 2 * x - 1), ptL<N>(y - 2 * x - 2), ptL<N>(y - 2 * x - 3));
    }
    case 6: {
        const int z = 2 * y - x, i = y - (x >> 1);
        if (z >= 0 && (z & 1) == 0) return ptE<N>(1, ptL<N>(i - 1), ptL<N>(i));
        if (z > 0) return ptE<N>(2, ptL<N>(i - 2), ptL<N>(i - 1), ptL<N>(i));
        if (z == -1) return ptE<N>(2, ptL<N>(0), ptT<N>(-1), ptT<N>(0));
        return ptE<N>(2, ptT<N>(x - 2 * y - 1), ptT<N>(x - 2 * y - 2), ptT<N>(x - 2 * y - 3));
    }
    case 7: {
        const int i = x + (y >> 1);
        if ((y & 1) == 0) return ptE<N>(1, ptT<N>(i), ptT<N>(i + 1));
        return ptE<N>(2, ptT<N>(i), ptT<N>(i + 1), ptT<N>(i + 2));
    }
    default: {
        const int zmax = 2 * n - 3, z = x + 2 * y, i = y + (x >> 1);
        if (z < zmax && (z & 1) == 0) return ptE<N>(1, ptL<N>(i), ptL<N>(i + 1));
        if (z < zmax) return ptE<N>(2, ptL<N>(i), ptL<N>(i + 1), ptL<N>(i + 2));
        if (z == zmax) return ptE<N>(3, ptL<N>(n - 2), ptL<N>(n - 1));
        return ptE<N>(0, ptL<N>(n - 1));
    }
    }
}
template <int N>
__host__ __device__ constexpr PredTab<N> make_predtab() {
    PredTab<N> t{};
    for (int m = 0; m < 9; m++)
        for (int i = 0; i < N * N; i++) t.e[m][i] = pt_entry<N>(m, i % N, i / N);
    return t;
}
__constant__ PredTab<4> cPRED4 = make_predtab<4>();
__constant__ PredTab<8> cPRED8 = make_predtab<8>();

// Blocks of an Intra4x4 MB (raster index) whose top-right 4x4 block lies in
// the MB and precedes them in decode (8x8 zig-zag) order.
__host__ __device__ constexpr uint32_t tr_inside_mask() {
    constexpr int dec[16] = {0, 1, 4, 5, 2, 3, 6, 7, 8, 9, 12, 13, 10, 11, 14, 15};
    uint32_t m = 0;
    for (int b = 4; b < 16; b++)
        if ((b & 3) < 3 && dec[b - 3] < dec[b]) m |= 1u << b;
    return m;
}
constexpr uint32_t kTR_INSIDE = tr_inside_mask();
static_assert(kTR_INSIDE == 0x5750u, "top-right availability inside an Intra4x4 MB");

// One predicted sample from its table entry and the block's reference array.
template <int N>
__device__ __forceinline__ int pt_apply(uint32_t e, const int *ref) {
    constexpr uint32_t s = ptS<N>(), m = (1u << s) - 1;
    const int r0 = ref[e & m], r1 = ref[(e >> s) & m], r2 = ref[(e >> (2 * s)) & m];
    const int w0 = (e >> (3 * s)) & 7, w1 = (e >> (3 * s + 3)) & 3, w2 = (e >> (3 * s + 5)) & 1,
              rnd = (e >> (3 * s + 6)) & 3;
    return (w0 * r0 + w1 * r1 + w2 * r2 + rnd) >> 2;
}

// reconstruct_intra, src/h264/dec/slicedec.rs:1325-1388, one warp, on the
// canvas (neighbour samples already in row -1 and column -1).
// nb: availability of neighbours L, T, TR, TL for intra prediction.
__device__ void intra_mb(WarpSmem &S, int lane, const bool nb[4], const uint32_t *tab4, const uint32_t *tab8) {
    const IntraInfo &m = S.q;
    // ---- luma
    if (m.kind == RC_H264_I4x4) {
        // the 16 blocks in wavefront order bx + 2 by (each after its left, top,
        // top-left and top-right blocks), two blocks per step, 16 lanes each
        constexpr int8_t kA[10] = {0, 1, 2, 3, 6, 7, 10, 11, 14, 15};
        constexpr int8_t kB[10] = {-1, -1, 4, 5, 8, 9, 12, 13, -1, -1};
        const int g = lane >> 4, l = lane & 15, px = lane & 3, py = (lane >> 2) & 3;
        int *E = S.f + 16 * g;  // the reference array of this half-warp's block
        // this lane's table entry and residual sample of every step (a half-warp
        // without a block in a step shadows the other half's block, unstored)
        uint32_t ent[10];
        int rs[10];
#pragma unroll
        for (int st = 0; st < 10; st++) {
            const int b = (g && kB[st] >= 0) ? kB[st] : kA[st];
            ent[st] = tab4[m.modes[b] * 16 + py * 4 + px];
            rs[st] = S.res[((b >> 2) * 4 + py) * 16 + (b & 3) * 4 + px];
        }
#pragma unroll
        for (int st = 0; st < 10; st++) {
            const bool act = !g || kB[st] >= 0;
            const int b = (g && kB[st] >= 0) ? kB[st] : kA[st];
            const int bx = b & 3, by = b >> 2, bx0 = bx * 4, by0 = by * 4;
            // luma_avail4, slicedec.rs:1297-1323
            const bool aL = bx > 0 || nb[0], aT = by > 0 || nb[1];
            const bool aTL = (bx > 0 && by > 0) || (by > 0 ? nb[0] : bx > 0 ? nb[1] : nb[3]);
            const bool aTR = by == 0 ? (bx < 3 ? nb[1] : nb[2]) : (kTR_INSIDE >> b & 1);
            // reference array (load_edge, intra.rs:31-62: 128 where unavailable,
            // the last top sample for an unavailable top-right) and the DC
            {
                const bool isT = (unsigned)(l - 1) < 8u, isL = (unsigned)(l - 9) < 4u;
                const int ti = (l - 1 < 4 || aTR) ? l - 1 : 3;
                const int row = isL ? by0 + l - 9 : by0 - 1;
                const int col = isT ? bx0 + ti : bx0 - 1;
                const bool ok = isT ? aT : isL ? aL : aTL;
                const int raw = S.cy[(row + 1) * 32 + col + 1];
                const uint8_t *tp = S.cy + by0 * 32 + bx0 + 1;  // row -1 of the block
                const uint8_t *lp = S.cy + (by0 + 1) * 32 + bx0;  // column -1, row 0
                const int st4 = tp[0] + tp[1] + tp[2] + tp[3], sl4 = lp[0] + lp[32] + lp[64] + lp[96];
                const int dc = (aT && aL) ? (st4 + sl4 + 4) >> 3 : aL ? (sl4 + 2) >> 2 : aT ? (st4 + 2) >> 2 : 128;
                E[l] = l == 13 ? dc : ok ? raw : 128;
            }
            __syncwarp();
            {
                const int v = clip255(pt_apply<4>(ent[st], E) + rs[st]);
                if (act) S.cy[(by0 + py + 1) * 32 + bx0 + px + 1] = (uint8_t)v;
            }
            __syncwarp();
        }
    } else if (m.kind == RC_H264_I8x8) {
        uint32_t ent[4][2];
        int rs[4][2];
#pragma unroll
        for (int b8 = 0; b8 < 4; b8++) {
            const int bx = (b8 & 1) * 2, by = (b8 >> 1) * 2;
            const int mode = m.modes[by * 4 + bx];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int idx = lane + 32 * h, x = idx & 7, y = idx >> 3;
                ent[b8][h] = tab8[mode * 64 + idx];
                rs[b8][h] = S.res[(by * 4 + y) * 16 + bx * 4 + x];
            }
        }
#pragma unroll
        for (int b8 = 0; b8 < 4; b8++) {
            const int bx = (b8 & 1) * 2, by = (b8 >> 1) * 2, bx0 = bx * 4, by0 = by * 4;
            const bool aL = bx > 0 || nb[0], aT = by > 0 || nb[1];
            const bool aTL = (bx > 0 && by > 0) || (by > 0 ? nb[0] : bx > 0 ? nb[1] : nb[3]);
            const bool aTR = b8 == 0 ? nb[1] : b8 == 1 ? nb[2] : b8 == 2;
            // reference samples (load_edge, intra.rs:31-62) smoothed by
            // pred8x8's [1 2 1] filter (intra.rs:199-231).  On the line
            // L7..L0, corner, T0..T15 (u = 0..24) a sample takes a neighbour
            // only when both are available, else itself; lanes 25..31 the DC.
            {
                const int u = lane < 16 ? 9 + lane : lane < 24 ? 23 - lane : 8;
                auto at = [&](int w, bool &av) -> int {
                    av = w < 8 ? aL : w == 8 ? aTL : aT;
                    const int i = w - 9, ti = (i < 8 || aTR) ? i : 7;
                    const int row = w < 8 ? by0 + 7 - w : by0 - 1;
                    const int col = w <= 8 ? bx0 - 1 : bx0 + ti;
                    return S.cy[(row + 1) * 32 + col + 1];
                };
                bool ac, a1, a2;
                const int rc = at(u, ac), r1 = at(u > 0 ? u - 1 : 0, a1), r2 = at(u < 24 ? u + 1 : 24, a2);
                const int c = ac ? rc : 128;
                const int n1 = (u > 0 && ac && a1) ? r1 : c, n2 = (u < 24 && ac && a2) ? r2 : c;
                const int v = (n1 + 2 * c + n2 + 2) >> 2;
                const int st = (int)__reduce_add_sync(0xffffffffu, (unsigned)(lane < 8 ? v : 0));
                const int sl = (int)__reduce_add_sync(0xffffffffu, (unsigned)(lane >= 16 && lane < 24 ? v : 0));
                const int dc =
                    (aT && aL) ? (st + sl + 8) >> 4 : aL ? (sl + 4) >> 3 : aT ? (st + 4) >> 3 : 128;
                S.f[lane] = lane < 25 ? v : dc;
            }
            __syncwarp();
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int idx = lane + 32 * h, x = idx & 7, y = idx >> 3;
                const int v = clip255(pt_apply<8>(ent[b8][h], S.f) + rs[b8][h]);
                S.cy[(by0 + y + 1) * 32 + bx0 + x + 1] = (uint8_t)v;
            }
            __syncwarp();
        }
    } else {
        // pred16x16, src/h264/dec/intra.rs:240-305 (the DC sums and plane
        // gradients only for their modes; the mode is uniform over the warp)
        const bool al = nb[0], at = nb[1], atl = nb[3];
        const int mode = m.i16_mode;
        int dc = 128, aa = 0, bb = 0, cc = 0;
        if (mode == 2) {
            const int topv = at ? cvy(S, -1, lane & 15) : 0, leftv = al ? cvy(S, lane & 15, -1) : 0;
            const int st = (int)__reduce_add_sync(0xffffffffu, (unsigned)(lane < 16 ? topv : 0));
            const int sl = (int)__reduce_add_sync(0xffffffffu, (unsigned)(lane < 16 ? leftv : 0));
            dc = (at && al) ? (st + sl + 16) >> 5 : al ? (sl + 8) >> 4 : at ? (st + 8) >> 4 : 128;
        } else if (mode == 3) {
            const int tl = atl ? cvy(S, -1, -1) : 128;
            int hterm = 0, vterm = 0;
            if (lane < 8) {
                const int kk = lane;
                const int t8k = at ? cvy(S, -1, 8 + kk) : 0;
                const int t6k = (6 - kk) < 0 ? tl : (at ? cvy(S, -1, 6 - kk) : 0);
                const int l8k = al ? cvy(S, 8 + kk, -1) : 0;
                const int l6k = (6 - kk) < 0 ? tl : (al ? cvy(S, 6 - kk, -1) : 0);
                hterm = (kk + 1) * (t8k - t6k);
                vterm = (kk + 1) * (l8k - l6k);
            }
            const int H = (int)__reduce_add_sync(0xffffffffu, (unsigned)hterm);
            const int Vv = (int)__reduce_add_sync(0xffffffffu, (unsigned)vterm);
            aa = 16 * ((al ? cvy(S, 15, -1) : 0) + (at ? cvy(S, -1, 15) : 0));
            bb = (5 * H + 32) >> 6;
            cc = (5 * Vv + 32) >> 6;
        }
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
    // ---- chroma, pred_chroma, src/h264/dec/intra.rs:307-395.  The per-block
    // DC values (mode 0) or the per-component plane parameters (mode 3)
    // first, into S.f, then every sample with one sequence.
    {
        const bool al = nb[0], at = nb[1], atl = nb[3];
        const int mode = m.chroma_mode;
        if (mode == 0) {
            // lane & 7: component (bit 2) and 4x4 block (bx bit 0, by bit 1)
            const int c = (lane >> 2) & 1, bx = lane & 1, by = (lane >> 1) & 1;
            const uint8_t *cv = S.cc[c];
            int st = 0, sl = 0;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                st += at ? (int)cv[bx * 4 + i + 1] : 0;
                sl += al ? (int)cv[(by * 4 + i + 1) * 12] : 0;
            }
            const int both = (at && al) ? (st + sl + 4) >> 3 : al ? (sl + 2) >> 2 : at ? (st + 2) >> 2 : 128;
            const int topf = at ? (st + 2) >> 2 : al ? (sl + 2) >> 2 : 128;
            const int leftf = al ? (sl + 2) >> 2 : at ? (st + 2) >> 2 : 128;
            if (lane < 8) S.f[lane] = bx == by ? both : bx ? topf : leftf;
        } else if (mode == 3) {
            const int c = lane & 1;
            const uint8_t *cv = S.cc[c];
            const int tl = atl ? cv[0] : 128;
            int hh = 0, vv = 0;
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
                const int tm = kk == 3 ? tl : (at ? (int)cv[2 - kk + 1] : 0);
                const int lm = kk == 3 ? tl : (al ? (int)cv[(2 - kk + 1) * 12] : 0);
                hh += (kk + 1) * ((at ? (int)cv[4 + kk + 1] : 0) - tm);
                vv += (kk + 1) * ((al ? (int)cv[(4 + kk + 1) * 12] : 0) - lm);
            }
            if (lane < 2) {
                S.f[8 + 3 * c] = 16 * ((al ? (int)cv[8 * 12] : 0) + (at ? (int)cv[8] : 0));
                S.f[9 + 3 * c] = (34 * hh + 32) >> 6;
                S.f[10 + 3 * c] = (34 * vv + 32) >> 6;
            }
        }
        __syncwarp();
        int outv[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int idx = lane + 32 * h, c = idx >> 6, x = idx & 7, y = (idx >> 3) & 7;
            const uint8_t *cv = S.cc[c];
            int v;
            if (mode == 0) v = S.f[c * 4 + (y >> 2) * 2 + (x >> 2)];
            else if (mode == 1) v = al ? (int)cv[(y + 1) * 12] : 0;
            else if (mode == 2) v = at ? (int)cv[x + 1] : 0;
            else v = clip255((S.f[8 + 3 * c] + S.f[9 + 3 * c] * (x - 3) + S.f[10 + 3 * c] * (y - 3) + 16) >> 5);
            outv[h] = clip255(v + S.res[256 + c * 64 + y * 8 + x]);
        }
        __syncwarp();
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int idx = lane + 32 * h, c = idx >> 6, x = idx & 7, y = (idx >> 3) & 7;
            S.cc[c][(y + 1) * 12 + x + 1] = (uint8_t)outv[h];
        }
    }
    __syncwarp();
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

// The RC_EDGE_WORDS loop-filter words of one MB from its DbMb (edge
// parameters of deblock_mb, deblock.rs:386-403), two words per lane.
__device__ void edge_words(const DbMb &d, int lane, uint32_t *out) {
    const bool f = d.flags != 0;
    {  // luma word `lane`: dir, 4-line segment k, edge e
        const int dir = lane >> 4, k = (lane >> 2) & 3, e = lane & 3;
        const int bsv = f ? d.bs[(dir << 4) | (e << 2) | k] : 0;
        uint32_t w = 0;
        if (bsv) {
            int alpha, beta, tc0;
            edge_consts(e == 0 ? d.qp[1 + dir] : d.qp[0], d.qp[0], bsv, d.aoff, d.boff, alpha, beta, tc0);
            w = (uint32_t)alpha | (uint32_t)beta << 8 | (uint32_t)tc0 << 16 | (uint32_t)bsv << 24;
        }
        out[lane] = w;
    }
    {  // chroma word 32 + lane: dir, component c, 2-line segment k, chroma edge e (luma edge 2e)
        const int dir = lane >> 4, c = (lane >> 3) & 1, k = (lane >> 1) & 3, e = lane & 1;
        const int bsv = f ? d.bs[(dir << 4) | (e << 3) | k] : 0;
        uint32_t w = 0;
        if (bsv) {
            int alpha, beta, tc0;
            edge_consts(e == 0 ? d.qpc[1 + dir][c] : d.qpc[0][c], d.qpc[0][c], bsv, d.aoff, d.boff, alpha, beta,
                        tc0);
            w = (uint32_t)alpha | (uint32_t)beta << 8 | (uint32_t)tc0 << 16 | (uint32_t)bsv << 24;
        }
        out[32 + lane] = w;
    }
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
// Band kernel: intra reconstruction and the loop filter of one picture in one
// cooperative launch.  Band b owns MB rows [b*BR, b*BR + BR).  For each of
// its rows it runs three warps that walk the row left to right: an intra
// warp (reconstruct_intra of the row's intra MBs), a luma and a chroma
// loop-filter warp (deblock_mb: an MB's vertical edges, then its horizontal
// edges).  Rows of a band hand over through shared memory, bands through
// per-row progress words in global memory that the band's two helper warps
// mirror and publish.  When the device holds three (or two) CTAs per band at
// once, the band's roles run on CTAs of their own (H264Launch::band_split):
// each CTA keeps the warps of its roles, and the progress one role hands
// another crosses between them through the same global words (every row's
// intra progress, published by a warp of the intra CTA); a mirrored value
// never exceeds its source, so the waits below only become stricter.
//
// Order (every wait is capped, see wait_seen):
//   intra MB (x, y)    after intra row y-1 has reconstructed MBs 0..x+1;
//   filter MB (x, y)   after row y has reconstructed MBs 0..x+2 (every intra
//                      MB whose samples the step reads or changes, and MB
//                      x+2, which the step prefetches) and, for a band's last
//                      row, row y+1 MBs 0..x+1 (the next band's intra warps
//                      read row y's unfiltered samples from the picture;
//                      inside a band they read the intra warp's line copy);
//                      its horizontal edges, which read MB (x, y-1), also
//                      after row y-1 has filtered MB x+1's vertical edges
//                      (the last change to MB (x, y-1)) and stored MBs 0..x.
// A filter row stores MB x-1 once MB x's left edge is filtered (its last
// change in the row) and publishes its progress there, before MB x's
// horizontal edges, and stores the three rows above MB x after MB x's top
// edge.
// ===========================================================================
constexpr int BR = RC_H264_BAND_ROWS;
constexpr int DRING = 8;  // ring slots between filter rows of a band
constexpr int BAND_THREADS = (3 * BR + 2) * 32;  // intra, luma, chroma per row; mirror and publish warps
// an intra warp's staging: parameters (32 B) and residual (768 B), then one
// 4-byte word per lane holding the next MB's column -1 sample (luma rows
// 0..15, Cb rows 0..7, Cr rows 0..7)
constexpr int RC_BAND_STG_LEFT = 800;
constexpr int RC_BAND_STG = RC_BAND_STG_LEFT + 32 * 4;
static_assert(RC_BAND_STG % 16 == 0, "staging areas stay 16-byte aligned");

struct __align__(16) LumaRow {
    uint8_t t[20][16];        // rows -4..15 of the MB being filtered (horizontal edges)
    uint8_t ring[DRING][64];  // final rows 12..15 of this row's MBs, for the row below
    uint4 st[3][3][16];       // staged MBs x..x+2 (slot x % 3): sample rows, vertical and horizontal edge words
    uint8_t tn[2][4][16];     // a band's first row: the next MB's rows -4..-1 (slot x & 1), copied ahead
};
struct __align__(16) ChromaRow {
    uint8_t t[2][10][8];      // per component, rows -2..7
    uint8_t ring[DRING][32];  // final rows 6..7 per component, for the row below
    uint2 st[3][3][16];       // staged MBs, as LumaRow::st
    uint8_t tn[2][4][16];     // a band's first row: the 16-byte chunks holding the next MB's rows -2..-1
};
struct __align__(16) BandSmem {
    uint32_t tab4[9 * 16];  // copies of cPRED4 / cPRED8
    uint32_t tab8[9 * 64];
    WarpSmem iw[BR];
    LumaRow l[BR];
    ChromaRow c[BR];
    // progress: index 0 = the row above the band (mirrored), 1..BR = the band's
    // rows, BR + 1 = the row below the band (intra, mirrored)
    volatile int iprog[BR + 2];  // MBs 0..v-1 reconstructed
    volatile int lprog[BR + 1];  // MBs 0..v-1 luma-filtered and stored, ring slots 0..v-1 written
    volatile int cprog[BR + 1];  // same for chroma
};


// Polls of a band wait taken back to back before it starts to sleep.
#ifndef RC_SPIN_POLLS
#define RC_SPIN_POLLS 16384u
#endif

// Warp-wide wait until *c >= need.  Lane 0 polls shared memory, the first
// RC_SPIN_POLLS polls back to back: the waits on the wavefront's path end
// within a few microseconds, and a sleep, however short, delays seeing the
// progress by more than a poll costs (1080p P+I sequence: 1955 frames/s
// sleeping from the first poll, 1996 polling).  A longer wait then sleeps
// between polls (16 ns doubling to 128 ns), leaving the issue slots to the
// CTA's working warps.  False after the iteration cap or once another warp
// has reported an error.  The largest progress observed is remembered:
// progress only grows, so a value seen (and ordered by the fence) at an
// earlier wait answers later ones without another round through shared
// memory.
__device__ __forceinline__ bool wait_seen(volatile int *c, int &seen, int need, const H264Launch &P, int lane) {
    if (seen >= need) return true;
    bool ok = true;
    int v = 0;
    if (lane == 0) {
        v = *c;
        if (v < need) {
            uint32_t it = 0, ns = 16;
            do {
                if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) { ok = false; break; }
                if (it > RC_SPIN_POLLS) {
                    __nanosleep(ns);
                    ns = min(ns * 2, 128u);
                }
                v = *c;
            } while (v < need);
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    v = __shfl_sync(0xffffffffu, v, 0);
    __syncwarp();
    __threadfence_block();
    if (ok) seen = v;
    return ok;
}

// filter_lanes (deblock.rs:146-229) for one luma line s[0..7] = p3..q3 and
// one edge word (alpha | beta << 8 | tc0 << 16 | bS << 24), without
// branches: every candidate is computed and the results selected, so that a
// warp's lanes never diverge.  STRONG: the edge may carry bS 4 (MB edges);
// internal edges never do.
template <bool STRONG>
__device__ __forceinline__ void lf_luma(int *s, uint32_t wd) {
    const int alpha = wd & 255, beta = (wd >> 8) & 255, tc0 = (wd >> 16) & 255, bS = wd >> 24;
    const int p3 = s[0], p2 = s[1], p1 = s[2], p0 = s[3], q0 = s[4], q1 = s[5], q2 = s[6], q3 = s[7];
    const int d0 = abs(p0 - q0);
    const bool on = (bS != 0) & (d0 < alpha) & (abs(p1 - p0) < beta) & (abs(q1 - q0) < beta);
    const bool ap = abs(p2 - p0) < beta, aq = abs(q2 - q0) < beta;
    // bS 1..3
    const int tc = tc0 + ap + aq;
    const int delta = clampi((((q0 - p0) << 2) + (p1 - q1) + 4) >> 3, -tc, tc);
    const int avg = (p0 + q0 + 1) >> 1;
    int np0 = clip255(p0 + delta), nq0 = clip255(q0 - delta);
    int np1 = ap ? p1 + clampi((p2 + avg - (p1 << 1)) >> 1, -tc0, tc0) : p1;
    int nq1 = aq ? q1 + clampi((q2 + avg - (q1 << 1)) >> 1, -tc0, tc0) : q1;
    int np2 = p2, nq2 = q2;
    if (STRONG) {  // bS 4
        const bool big = bS >= 4, sm = d0 < ((alpha >> 2) + 2), sp = ap & sm, sq = aq & sm;
        const int sp0 = sp ? (p2 + 2 * p1 + 2 * p0 + 2 * q0 + q1 + 4) >> 3 : (2 * p1 + p0 + q1 + 2) >> 2;
        const int sp1 = sp ? (p2 + p1 + p0 + q0 + 2) >> 2 : p1;
        const int sp2 = sp ? (2 * p3 + 3 * p2 + p1 + p0 + q0 + 4) >> 3 : p2;
        const int sq0 = sq ? (p1 + 2 * p0 + 2 * q0 + 2 * q1 + q2 + 4) >> 3 : (2 * q1 + q0 + p1 + 2) >> 2;
        const int sq1 = sq ? (p0 + q0 + q1 + q2 + 2) >> 2 : q1;
        const int sq2 = sq ? (2 * q3 + 3 * q2 + q1 + q0 + p0 + 4) >> 3 : q2;
        np0 = big ? sp0 : np0;
        np1 = big ? sp1 : np1;
        np2 = big ? sp2 : np2;
        nq0 = big ? sq0 : nq0;
        nq1 = big ? sq1 : nq1;
        nq2 = big ? sq2 : nq2;
    }
    s[1] = on ? np2 : p2;
    s[2] = on ? np1 : p1;
    s[3] = on ? np0 : p0;
    s[4] = on ? nq0 : q0;
    s[5] = on ? nq1 : q1;
    s[6] = on ? nq2 : q2;
}

// the chroma filter (deblock.rs:146-229, chroma lanes) for s[0..3] = p1, p0,
// q0, q1, without branches
__device__ __forceinline__ void lf_chroma(int *s, uint32_t wd) {
    const int alpha = wd & 255, beta = (wd >> 8) & 255, tc0 = (wd >> 16) & 255, bS = wd >> 24;
    const int p1 = s[0], p0 = s[1], q0 = s[2], q1 = s[3];
    const bool on = (bS != 0) & (abs(p0 - q0) < alpha) & (abs(p1 - p0) < beta) & (abs(q1 - q0) < beta);
    const int tc = tc0 + 1;
    const int delta = clampi((((q0 - p0) << 2) + (p1 - q1) + 4) >> 3, -tc, tc);
    const bool big = bS >= 4;
    const int np0 = big ? (2 * p1 + p0 + q1 + 2) >> 2 : clip255(p0 + delta);
    const int nq0 = big ? (2 * q1 + q0 + p1 + 2) >> 2 : clip255(q0 - delta);
    s[1] = on ? np0 : p0;
    s[2] = on ? nq0 : q0;
}

__device__ __forceinline__ void band_fail(const H264Launch &P, int lane) {
    if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT);
}


// Intra warp of band row w (picture row my).  `lines` holds, per band row,
// the row's unfiltered bottom samples (luma row 15, then Cb and Cr row 7):
// filled from the picture at the start (inter MBs are final already) and
// updated as the row's intra MBs are reconstructed, so that the row below
// reads its top neighbours from shared memory.  `stg` stages the next intra
// MB's parameters, residual and (when its left neighbour is an inter MB) the
// words holding its column -1, loaded with cp.async while the current MB is
// reconstructed.  All of these are final before the kernel starts and stay
// unchanged until this warp reports the MB after them reconstructed (the
// filter warps wait for that), so they may be read early.
//
// In a group launch (P.mbdone set) inter MBs are predicted beside the band
// CTAs: inter MB x of the row is ready once mbdone[x] holds the picture's
// epoch (the other kinds are ready when the launch starts).  The warp
// reports an MB only once it and every inter MB before it are ready, so
// that the filter warps wait on inter MBs through the same progress word.
// The row below reads the unfiltered bottom rows of MBs that are not intra
// from P.bottom (written with the MB: by the pre-pass for I_PCM, by the
// group kernel for inter MBs, once per MB), after their mbdone: its intra
// MBs keep waiting on this row only where an intra neighbour is.
// GROUPED: a group launch (P.mbdone set), compiled apart so that the one-
// picture kernel carries none of its waits.
template <bool GROUPED>
__device__ __forceinline__ void band_intra_row(const H264Launch &P, BandSmem &B, uint8_t *lines, uint8_t *stg, int w, int my,
                               int lane) {
    WarpSmem &S = B.iw[w];
    constexpr bool grouped = GROUPED;
    const uint32_t *done = grouped ? P.mbdone + (size_t)my * P.mb_w : nullptr;
    uint8_t *Y = P.dpb + (size_t)P.out_slot * P.slot_bytes;
    uint8_t *U = Y + P.u_off, *V = Y + P.v_off;
    const int LW = P.mb_w * 32;
    uint8_t *ly = lines + (size_t)w * LW, *lu = ly + P.mb_w * 16, *lv = lu + P.mb_w * 8;
    const uint8_t *ay = ly - LW, *au = lu - LW, *av = lv - LW;  // the row above (w > 0)
    volatile int *above = &B.iprog[w], *mine = &B.iprog[w + 1];
    // the intra MBs of this row (word) and of the row above (aword): lane j
    // holds the bits of MBs 32 j .. 32 j + 31 (rows of up to 1024 MBs, see
    // rc_h264_band_capacity)
    const int nwords = (P.mb_w + 31) >> 5;
    uint32_t word = 0, aword = 0, iword = 0, aiword = 0;  // iword / aiword: the inter MBs of this row / the row above
    for (int j0 = 0; j0 < nwords; j0 += 4) {
        int kinds[4], akinds[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int xl = (j0 + u) * 32 + lane;
            kinds[u] = xl < P.mb_w ? __ldg(&P.mbs[my * P.mb_w + xl].kind) : RC_H264_NONE;
            akinds[u] = xl < P.mb_w && my > 0 ? __ldg(&P.mbs[(my - 1) * P.mb_w + xl].kind) : RC_H264_NONE;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint32_t b = __ballot_sync(0xffffffffu, wave_intra(kinds[u]));
            const uint32_t a = __ballot_sync(0xffffffffu, wave_intra(akinds[u]));
            const uint32_t e = __ballot_sync(0xffffffffu, kinds[u] == RC_H264_INTER);
            const uint32_t ae = __ballot_sync(0xffffffffu, akinds[u] == RC_H264_INTER);
            if (lane == j0 + u) {
                word = b;
                aword = a;
                iword = e;
                aiword = ae;
            }
        }
    }
    auto above_intra = [&](int x) -> bool {  // MB (x, my - 1) is intra
        const uint32_t b = __shfl_sync(0xffffffffu, aword, (x >> 5) & 31);
        return x >= 0 && x < P.mb_w && (b >> (x & 31) & 1);
    };
    // the progress of the row above that MB x's prediction needs: its intra
    // neighbours among MBs x-1, x, x+1 of that row reconstructed (inter ones
    // are final from the start: in the line copy, which the row above fills
    // before its first report, or in the picture for a band's first row)
    auto above_need = [&](int x) -> int {
        // (a group launch has no initial line copy: the row above's inter
        // MBs come from P.bottom once predicted, see above_inter_ready)
        const int base = w > 0 && !grouped ? 1 : 0;
        if (above_intra(x + 1)) return min(x + 2, P.mb_w);
        if (above_intra(x)) return x + 1;
        if (above_intra(x - 1)) return max(x, base);
        return base;
    };
    auto next_intra = [&](int from) -> int {  // the first intra MB at or after `from`, else mb_w
        for (int j = from >> 5; j < nwords; j++) {
            uint32_t b = __shfl_sync(0xffffffffu, word, j);
            if (j == (from >> 5)) b &= ~0u << (from & 31);
            if (b) return j * 32 + __ffs(b) - 1;
        }
        return P.mb_w;
    };
    auto is_inter = [&](int x) -> bool {  // MB (x, my) is predicted in the launch; any lane's x
        return (__shfl_sync(0xffffffffu, iword, (x >> 5) & 31) >> (x & 31)) & 1;
    };
    // grouped: the inter MBs of this row before `filled`, and of the row
    // above before `afilled`, are predicted.  ready(...) makes the prefix
    // reach `need`: a round looks at the next 32 MBs at once (a lane each),
    // so that the prefix usually runs ahead of what is asked and later calls
    // cost nothing; while nothing moves, only the first missing flag is
    // polled, backing off to 1 us (the band CTAs of later pictures of a
    // group wait here, and their polls would slow the L2 round trips of the
    // wavefront that runs)
    int filled = 0, afilled = 0;
    auto ready = [&](int &pre, const uint32_t *flags, uint32_t bits_word, int need) -> bool {
        if (pre >= need) return true;
        uint32_t it = 0, ns = 32;
        bool all = true;  // probe 32 flags (else only the first missing one)
        while (pre < need) {
            const int x = pre + lane;
            const int xc = min(x, P.mb_w - 1);
            const bool inter_x = (__shfl_sync(0xffffffffu, bits_word, (xc >> 5) & 31) >> (xc & 31)) & 1;
            // lanes that do not look count as not ready, so the prefix stops at them
            bool rdy = false;
            if (all || lane == 0) rdy = !(x < P.mb_w && inter_x) || ld_relaxed(flags + x) == P.epoch;
            const uint32_t m = __ballot_sync(0xffffffffu, rdy);
            const int adv = m == 0xffffffffu ? 32 : __ffs(~m) - 1;
            pre = min(pre + adv, P.mb_w);
            if (pre >= need) break;
            if (adv > 0) {
                all = true;
                it = 0;
                ns = 32;
                continue;
            }
            bool give_up = false;
            if (lane == 0) give_up = ++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error));
            if (__shfl_sync(0xffffffffu, give_up, 0)) return false;
            all = false;
            __nanosleep(ns);
            ns = min(ns * 2, 1024u);
        }
        fence_acquire();  // the flags seen order the MBs' samples after them
        __syncwarp();
        return true;
    };
    auto advance = [&](int v) -> bool { return ready(filled, done, iword, v); };
    // the inter MBs among mx-1..mx+1 of the row above (their unfiltered
    // bottom rows are then in P.bottom)
    auto above_inter_ready = [&](int x) -> bool {
        return ready(afilled, P.mbdone + (size_t)(my - 1) * P.mb_w, aiword, min(x + 2, P.mb_w));
    };
    auto prefetch = [&](int nx) -> bool {
        // grouped: the left neighbour, when it is an inter MB, is predicted
        // in the launch (the MB's own parameters and residual, and every
        // other kind of MB, come from the pre-pass)
        if (grouped && nx < P.mb_w && nx > 0 && is_inter(nx - 1) && !ready(filled, done, iword, nx)) return false;
        if (nx < P.mb_w) {
            const int addr = my * P.mb_w + nx;
            const uint8_t *q = (const uint8_t *)(P.iinfo + addr), *res = (const uint8_t *)(P.ires + (size_t)addr * 384);
            // 16-byte chunks 0..1 parameters, 2..49 residual
            cp_async16(stg + lane * 16, lane < 2 ? q + lane * 16 : res + (lane - 2) * 16);
            if (lane < 18) cp_async16(stg + (32 + lane) * 16, res + (30 + lane) * 16);
            if (nx > 0) {
                const uint8_t *src = lane < 16 ? Y + (size_t)(my * 16 + lane) * P.pitch + nx * 16 - 4
                                               : ((lane >> 3) & 1 ? V : U) + (size_t)(my * 8 + (lane & 7)) * P.cpitch +
                                                     nx * 8 - 4;
                cp_async4(stg + RC_BAND_STG_LEFT + lane * 4, src);
            }
        }
        cp_commit();
        return true;
    };
    int mx = next_intra(0);
    if (!prefetch(mx)) {
        cp_wait_all();
        band_fail(P, lane);
        return;
    }
    if (!grouped) {
        const uint32_t *gy = (const uint32_t *)(Y + (size_t)(my * 16 + 15) * P.pitch);
        const uint32_t *gu = (const uint32_t *)(U + (size_t)(my * 8 + 7) * P.cpitch);
        const uint32_t *gv = (const uint32_t *)(V + (size_t)(my * 8 + 7) * P.cpitch);
        for (int i = lane; i < P.mb_w * 4; i += 32) ((uint32_t *)ly)[i] = __ldcg(gy + i);
        for (int i = lane; i < P.mb_w * 2; i += 32) {
            ((uint32_t *)lu)[i] = __ldcg(gu + i);
            ((uint32_t *)lv)[i] = __ldcg(gv + i);
        }
        __syncwarp();
        __threadfence_block();
    }
    int last = -2;  // the MB reconstructed last (its right column is still in the canvas)
    int above_seen = 0;  // the row above's intra progress observed so far
    while (mx < P.mb_w) {
        const int nx = next_intra(mx + 1);
        // the MBs before mx are reconstructed (inter ones by the MB phase)
        if (grouped && !advance(mx)) {
            cp_wait_all();
            band_fail(P, lane);
            return;
        }
        if (lane == 0 && *mine < mx) *mine = mx;
        // the staged parameters and residual; canvas column -1: MB mx-1's right
        // column, from the canvas when this warp reconstructed it, else staged
        cp_wait_all();
        __syncwarp();
        {
            const uint4 *sg = (const uint4 *)stg;
            uint4 *dq = (uint4 *)&S.q, *dr = (uint4 *)S.res;
            if (lane < 2) dq[lane] = sg[lane];
            else dr[lane - 2] = sg[lane];
            if (lane < 18) dr[30 + lane] = sg[32 + lane];
            if (mx > 0) {
                const int c = (lane >> 3) & 1, rr = lane & 7;
                const uint8_t v = last == mx - 1 ? (lane < 16 ? S.cy[(lane + 1) * 32 + 16] : S.cc[c][(rr + 1) * 12 + 8])
                                                 : stg[RC_BAND_STG_LEFT + lane * 4 + 3];
                if (lane < 16) S.cy[(lane + 1) * 32] = v;
                else S.cc[c][(rr + 1) * 12] = v;
            }
        }
        __syncwarp();
        if (!prefetch(nx)) {
            cp_wait_all();
            band_fail(P, lane);
            return;
        }
        if (my > 0 && !wait_seen(above, above_seen, above_need(mx), P, lane)) {
            cp_wait_all();
            band_fail(P, lane);
            return;
        }
        // canvas row -1: the row above's bottom samples, columns -1..30 (chroma
        // -1..8): the line (or, for a band's first row, the picture), and in a
        // group launch the bottom-row buffer for MBs that are not intra
        if (my > 0 && grouped && !above_inter_ready(mx)) {
            cp_wait_all();
            band_fail(P, lane);
            return;
        }
        if (my > 0) {
            const int gx = mx * 16 + lane - 1;
            const int c = lane / 10, gxc = mx * 8 + lane % 10 - 1;
            // (group launches only: all lanes shuffle)
            const bool ya = grouped ? above_intra(max(gx, 0) >> 4) : true;
            const bool ca = grouped ? above_intra(max(gxc, 0) >> 3) : true;
            const uint8_t *brow = grouped ? P.bottom + (size_t)(my - 1) * LW : nullptr;
            uint8_t v = 0;
            if (gx >= 0 && gx < P.W)
                v = grouped && !ya ? __ldcg(brow + gx)
                    : w > 0       ? ay[gx]
                                  : __ldcg(Y + (size_t)(my * 16 - 1) * P.pitch + gx);
            S.cy[lane] = v;
            if (lane < 20) {
                uint8_t u = 0;
                if (gxc >= 0 && gxc < P.CW)
                    u = grouped && !ca ? __ldcg(brow + P.mb_w * (16 + 8 * c) + gxc)
                        : w > 0       ? (c ? av : au)[gxc]
                                      : __ldcg((c ? V : U) + (size_t)(my * 8 - 1) * P.cpitch + gxc);
                S.cc[c][lane % 10] = u;
            }
        }
        __syncwarp();
        bool nb[4];
#pragma unroll
        for (int n = 0; n < 4; n++) nb[n] = S.q.nb >> n & 1;
        intra_mb(S, lane, nb, B.tab4, B.tab8);
        // store the MB; its bottom samples into this row's line
        {
            const int r = lane >> 1, half = lane & 1;
            const uint8_t *q = S.cy + (r + 1) * 32 + 1 + half * 8;
            const uint32_t lo = q[0] | q[1] << 8 | q[2] << 16 | (uint32_t)q[3] << 24;
            const uint32_t hi = q[4] | q[5] << 8 | q[6] << 16 | (uint32_t)q[7] << 24;
            *(uint2 *)(Y + (size_t)(my * 16 + r) * P.pitch + mx * 16 + half * 8) = make_uint2(lo, hi);
            if (lane < 16) {
                const int c = lane >> 3, rr = lane & 7;
                const uint8_t *t = S.cc[c] + (rr + 1) * 12 + 1;
                const uint32_t a0 = t[0] | t[1] << 8 | t[2] << 16 | (uint32_t)t[3] << 24;
                const uint32_t a1 = t[4] | t[5] << 8 | t[6] << 16 | (uint32_t)t[7] << 24;
                *(uint2 *)((c ? V : U) + (size_t)(my * 8 + rr) * P.cpitch + mx * 8) = make_uint2(a0, a1);
                ly[mx * 16 + lane] = S.cy[16 * 32 + lane + 1];
            } else {
                const int c = (lane >> 3) & 1, i = lane & 7;
                (c ? lv : lu)[mx * 8 + i] = S.cc[c][8 * 12 + i + 1];
            }
        }
        last = mx;
        filled = mx + 1;
        __syncwarp();
        __threadfence_block();
        if (lane == 0) *mine = mx + 1;
        mx = nx;
    }
    cp_wait_all();
    __syncwarp();
    if (grouped && !advance(P.mb_w)) {
        band_fail(P, lane);
        return;
    }
    if (lane == 0) *mine = P.mb_w;
}

// Luma loop-filter warp of band row w (picture row my); lanes 0..15 hold one
// sample row (vertical edges) or one column (horizontal edges) of the MB.
__device__ __forceinline__ void band_luma_row(const H264Launch &P, BandSmem &B, int w, int my, int rows, int lane) {
    LumaRow &R = B.l[w];
    uint8_t *Y = P.dpb + (size_t)P.out_slot * P.slot_bytes;
    const bool act = lane < 16;
    const int r = lane & 15, k = r >> 2;
    // the row below reads this row's unfiltered samples from the picture
    // only when it starts the next band (inside a band it reads the intra
    // warp's line copy), so only then must the filter wait for its intra
    const bool below = w + 1 == rows && my + 1 < P.mb_h, ring_out = w + 1 < rows;
    volatile int *iown = &B.iprog[w + 1], *ibelow = &B.iprog[w + 2];
    volatile int *dup = &B.lprog[w], *dmine = &B.lprog[w + 1], *ddown = &B.lprog[min(w + 2, BR)];
    const uint4 *E = (const uint4 *)(P.edges + (size_t)my * P.mb_w * RC_EDGE_WORDS);
    const uint4 z4 = make_uint4(0, 0, 0, 0);
    uint4 prev = z4;
    // MB x's sample rows and edge words into slot x % 3; every lane commits a
    // group per MB so that the group counts stay uniform
    auto stage = [&](int x) {
        if (act && x < P.mb_w) {
            const int sl = x % 3;
            cp_async16(&R.st[sl][0][r], Y + (size_t)(my * 16 + r) * P.pitch + x * 16);
            cp_async16(&R.st[sl][1][r], E + (size_t)x * (RC_EDGE_WORDS / 4) + k);
            cp_async16(&R.st[sl][2][r], E + (size_t)x * (RC_EDGE_WORDS / 4) + 4 + k);
        }
        cp_commit();
    };
    // rows -4..-1 of MB x: the row above's ring, or (first row of a band) the
    // picture; for the latter the next MB's rows are loaded one step early
    // when the row above is already far enough
    bool have_next = false;
    int iown_seen = 0, ibelow_seen = 0, dup_seen = 0, ddown_seen = 0;  // progress observed so far
    auto top_rows = [&](int x) -> uint4 {
        if (my == 0 || lane >= 4) return z4;
        if (w > 0) return *(const uint4 *)(B.l[w - 1].ring[x % DRING] + lane * 16);
        return __ldcg((const uint4 *)(Y + (size_t)(my * 16 - 4 + lane) * P.pitch + x * 16));
    };
    // a band's first row: copy MB x+1's top rows into shared memory as soon
    // as the row above has stored MB x+1, with cp.async (a register load here
    // stalled the warp until it returned).  Commits a group in every case.
    auto try_next = [&](int x) {
        if (w == 0 && my > 0 && !have_next && x + 1 < P.mb_w &&
            __shfl_sync(0xffffffffu, *dup >= x + 2 ? 1 : 0, 0)) {
            __threadfence_block();
            if (lane < 4)
                cp_async16(&R.tn[(x + 1) & 1][lane][0], Y + (size_t)(my * 16 - 4 + lane) * P.pitch + (x + 1) * 16);
            have_next = true;
        }
        cp_commit();
    };
    auto fail = [&]() {
        cp_wait_all();
        band_fail(P, lane);
    };
    // Groups: step x commits try_next(x-1) and stage(x+2) right after it
    // reports MB x-1 (off the path that the row below waits on), then
    // try_next(x) at its horizontal edges.  Before the loop, the same pattern
    // for steps -2 and -1 (empty try_next groups).  So at the top of step x
    // four groups are younger than stage(x)'s, and at step x's horizontal
    // edges one is younger than the last group that can hold MB x's top rows.
    if (!wait_seen(iown, iown_seen, min(2, P.mb_w), P, lane)) { fail(); return; }
    cp_commit();
    stage(0);
    cp_commit();
    cp_commit();
    stage(1);
    cp_commit();
    for (int x = 0; x < P.mb_w; x++) {
        if (below && !wait_seen(ibelow, ibelow_seen, min(x + 2, P.mb_w), P, lane)) { fail(); return; }
        cp_wait_all_but_4();
        __syncwarp();
        const int sl = x % 3;
        const uint4 cur = act ? R.st[sl][0][r] : z4, pv = act ? R.st[sl][1][r] : z4,
                    ph = act ? R.st[sl][2][r] : z4;
        // ---- vertical edges: lane r holds columns -4..15 of sample row r
        uint32_t wd[5] = {prev.w, cur.x, cur.y, cur.z, cur.w};
        const uint32_t ev[4] = {pv.x, pv.y, pv.z, pv.w};
        const bool vfilt = __any_sync(0xffffffffu, (ev[0] | ev[1] | ev[2] | ev[3]) != 0);
        int sv[20];
        if (vfilt) {
#pragma unroll
            for (int i = 0; i < 20; i++) sv[i] = (wd[i >> 2] >> (8 * (i & 3))) & 255;
            // the MB edge; the bS-4 form equals the other below bS 4, and an
            // edge with bS 0 leaves its samples unchanged
            lf_luma<true>(sv, ev[0]);
            wd[0] = (uint32_t)sv[0] | (uint32_t)sv[1] << 8 | (uint32_t)sv[2] << 16 | (uint32_t)sv[3] << 24;
        }
        // ---- MB x-1 is final once this MB's left edge is filtered (the inner
        // edges start at column 1): store it, and its rows 12..15 for the row below
        if (x > 0) {
            prev.w = wd[0];
            if (act) *(uint4 *)(Y + (size_t)(my * 16 + r) * P.pitch + (x - 1) * 16) = prev;
            if (ring_out) {
                if (x - DRING > 0 && !wait_seen(ddown, ddown_seen, x - DRING, P, lane)) { fail(); return; }
                if (act && r >= 12) *(uint4 *)(R.ring[(x - 1) % DRING] + (r - 12) * 16) = prev;
            }
        }
        // MBs 0..x-1 are final and stored: the row below may take MB x-1's
        // rows (its horizontal edges need nothing later of this row)
        __syncwarp();
        __threadfence_block();
        if (lane == 0) *dmine = x;
        // MB x+2 reconstructed (also orders this step's horizontal edges after
        // this row's intra prediction, which reads the row above): stage it
        if (!wait_seen(iown, iown_seen, min(x + 3, P.mb_w), P, lane)) { fail(); return; }
        try_next(x - 1);
        stage(x + 2);
        // the inner vertical edges, without a vote per edge
        if (vfilt) {
#pragma unroll
            for (int e = 1; e < 4; e++) lf_luma<false>(sv + 4 * e, ev[e]);
#pragma unroll
            for (int j = 1; j < 5; j++)
                wd[j] = (uint32_t)sv[4 * j] | (uint32_t)sv[4 * j + 1] << 8 | (uint32_t)sv[4 * j + 2] << 16 |
                        (uint32_t)sv[4 * j + 3] << 24;
        }
        if (act) *(uint4 *)R.t[4 + r] = make_uint4(wd[1], wd[2], wd[3], wd[4]);
        __syncwarp();
        // ---- horizontal edges: need MB (x, y-1) final, i.e. the row above past
        // MB x+1's vertical edges
        uint4 t4 = z4;
        if (my > 0) {
            if (!wait_seen(dup, dup_seen, x + 1, P, lane)) { fail(); return; }
            if (w == 0 && have_next) {
                cp_wait_all_but_1();  // the top rows' group, whichever try_next committed it
                t4 = *(const uint4 *)&R.tn[x & 1][lane & 3][0];
            } else {
                t4 = top_rows(x);
            }
            have_next = false;
        }
        try_next(x);
        if (my > 0 && lane < 4) *(uint4 *)R.t[lane] = t4;
        __syncwarp();
        const uint32_t eh[4] = {ph.x, ph.y, ph.z, ph.w};
        const bool top = my > 0 && __any_sync(0xffffffffu, eh[0] != 0);
        if (__any_sync(0xffffffffu, (eh[0] | eh[1] | eh[2] | eh[3]) != 0)) {
            int sv[20];
#pragma unroll
            for (int i = 0; i < 20; i++) sv[i] = R.t[i][r];
            lf_luma<true>(sv, eh[0]);
#pragma unroll
            for (int e = 1; e < 4; e++) lf_luma<false>(sv + 4 * e, eh[e]);
            __syncwarp();
            if (act) {
#pragma unroll
                for (int i = 1; i < 19; i++) R.t[i][r] = (uint8_t)sv[i];
            }
            __syncwarp();
        }
        prev = act ? *(const uint4 *)R.t[4 + r] : z4;
        // rows 13..15 of the MB above are final after this MB's top edge
        if (top && lane < 3)
            *(uint4 *)(Y + (size_t)(my * 16 - 3 + lane) * P.pitch + x * 16) = *(const uint4 *)R.t[1 + lane];
        __syncwarp();
    }
    cp_wait_all();
    // the row's last MB
    if (act) *(uint4 *)(Y + (size_t)(my * 16 + r) * P.pitch + (P.mb_w - 1) * 16) = prev;
    if (ring_out) {
        if (P.mb_w - DRING > 0 && !wait_seen(ddown, ddown_seen, P.mb_w - DRING, P, lane)) { band_fail(P, lane); return; }
        if (act && r >= 12) *(uint4 *)(R.ring[(P.mb_w - 1) % DRING] + (r - 12) * 16) = prev;
    }
    __syncwarp();
    __threadfence_block();
    if (lane == 0) *dmine = P.mb_w;
}

// Chroma loop-filter warp of band row w: lanes 0..7 Cb, 8..15 Cr, each one
// sample row (vertical edges) or column (horizontal edges) of the MB.
__device__ __forceinline__ void band_chroma_row(const H264Launch &P, BandSmem &B, int w, int my, int rows, int lane) {
    ChromaRow &R = B.c[w];
    uint8_t *Y = P.dpb + (size_t)P.out_slot * P.slot_bytes;
    const bool act = lane < 16;
    const int c = (lane >> 3) & 1, r = lane & 7, k = r >> 1;
    uint8_t *Cp = Y + (c ? P.v_off : P.u_off);
    // the row below reads this row's unfiltered samples from the picture
    // only when it starts the next band (inside a band it reads the intra
    // warp's line copy), so only then must the filter wait for its intra
    const bool below = w + 1 == rows && my + 1 < P.mb_h, ring_out = w + 1 < rows;
    volatile int *iown = &B.iprog[w + 1], *ibelow = &B.iprog[w + 2];
    volatile int *dup = &B.cprog[w], *dmine = &B.cprog[w + 1], *ddown = &B.cprog[min(w + 2, BR)];
    const uint2 *E = (const uint2 *)(P.edges + (size_t)my * P.mb_w * RC_EDGE_WORDS);
    const uint2 z2 = make_uint2(0, 0);
    uint2 prev = z2;
    auto stage = [&](int x) {
        if (act && x < P.mb_w) {
            const int sl = x % 3;
            cp_async8(&R.st[sl][0][lane], Cp + (size_t)(my * 8 + r) * P.cpitch + x * 8);
            cp_async8(&R.st[sl][1][lane], E + (size_t)x * (RC_EDGE_WORDS / 2) + 16 + c * 4 + k);
            cp_async8(&R.st[sl][2][lane], E + (size_t)x * (RC_EDGE_WORDS / 2) + 24 + c * 4 + k);
        }
        cp_commit();
    };
    // rows -2..-1 of MB x per component (lanes 0..3: component lane >> 1, row
    // lane & 1): the row above's ring, or (first row of a band) the picture,
    // the next MB's one step early when the row above is far enough
    bool have_next = false;
    int iown_seen = 0, ibelow_seen = 0, dup_seen = 0, ddown_seen = 0;  // progress observed so far
    auto top_rows = [&](int x) -> uint2 {
        if (my == 0 || lane >= 4) return z2;
        const int cc = lane >> 1, rr = lane & 1;
        if (w > 0) return *(const uint2 *)(B.c[w - 1].ring[x % DRING] + cc * 16 + rr * 8);
        return __ldcg((const uint2 *)(Y + (cc ? P.v_off : P.u_off) + (size_t)(my * 8 - 2 + rr) * P.cpitch + x * 8));
    };
    // a band's first row: MB x+1's top rows copied ahead, as for luma (the
    // 16-byte aligned chunk holding the MB's 8 bytes: cp.async from L2)
    auto try_next = [&](int x) {
        if (w == 0 && my > 0 && !have_next && x + 1 < P.mb_w &&
            __shfl_sync(0xffffffffu, *dup >= x + 2 ? 1 : 0, 0)) {
            __threadfence_block();
            if (lane < 4)
                cp_async16(&R.tn[(x + 1) & 1][lane][0], Y + ((lane >> 1) ? P.v_off : P.u_off) +
                                                            (size_t)(my * 8 - 2 + (lane & 1)) * P.cpitch +
                                                            ((x + 1) & ~1) * 8);
            cp_commit();
            have_next = true;
        }
    };
    if (!wait_seen(iown, iown_seen, min(2, P.mb_w), P, lane)) { band_fail(P, lane); return; }
    stage(0);
    stage(1);
    for (int x = 0; x < P.mb_w; x++) {
        if (!wait_seen(iown, iown_seen, min(x + 3, P.mb_w), P, lane)) { band_fail(P, lane); return; }
        if (below && !wait_seen(ibelow, ibelow_seen, min(x + 2, P.mb_w), P, lane)) { band_fail(P, lane); return; }
        try_next(x - 1);
        stage(x + 2);
        cp_wait_all_but_1();
        const int sl = x % 3;
        const uint2 cur = act ? R.st[sl][0][lane] : z2, pv = act ? R.st[sl][1][lane] : z2,
                    ph = act ? R.st[sl][2][lane] : z2;
        // ---- vertical edges: lane holds columns -4..7 of its row
        uint32_t wd[3] = {prev.y, cur.x, cur.y};
        if (__any_sync(0xffffffffu, (pv.x | pv.y) != 0)) {
            int sv[12];
#pragma unroll
            for (int i = 0; i < 12; i++) sv[i] = (wd[i >> 2] >> (8 * (i & 3))) & 255;
            lf_chroma(sv + 2, pv.x);  // bS 0: unchanged
            lf_chroma(sv + 6, pv.y);
#pragma unroll
            for (int j = 0; j < 3; j++)
                wd[j] = (uint32_t)sv[4 * j] | (uint32_t)sv[4 * j + 1] << 8 | (uint32_t)sv[4 * j + 2] << 16 |
                        (uint32_t)sv[4 * j + 3] << 24;
        }
        if (x > 0) {
            prev.y = wd[0];
            if (act) *(uint2 *)(Cp + (size_t)(my * 8 + r) * P.cpitch + (x - 1) * 8) = prev;
            if (ring_out) {
                if (x - DRING > 0 && !wait_seen(ddown, ddown_seen, x - DRING, P, lane)) { band_fail(P, lane); return; }
                if (act && r >= 6) *(uint2 *)(R.ring[(x - 1) % DRING] + c * 16 + (r - 6) * 8) = prev;
            }
        }
        if (act) *(uint2 *)R.t[c][2 + r] = make_uint2(wd[1], wd[2]);
        // MBs 0..x-1 final and stored
        __syncwarp();
        __threadfence_block();
        if (lane == 0) *dmine = x;
        // ---- horizontal edges: lane holds rows -2..7 of its column; need the
        // row above past MB x+1's vertical edges
        if (my > 0) {
            if (!wait_seen(dup, dup_seen, x + 1, P, lane)) { band_fail(P, lane); return; }
            const uint2 t2 = (w == 0 && have_next) ? *(const uint2 *)&R.tn[x & 1][lane & 3][(x & 1) * 8] : top_rows(x);
            have_next = false;
            try_next(x);
            if (lane < 4) *(uint2 *)R.t[lane >> 1][lane & 1] = t2;
        }
        __syncwarp();
        const bool top = my > 0 && __any_sync(0xffffffffu, ph.x != 0);
        if (__any_sync(0xffffffffu, (ph.x | ph.y) != 0)) {
            int sv[10];
#pragma unroll
            for (int i = 0; i < 10; i++) sv[i] = R.t[c][i][r];
            lf_chroma(sv + 0, ph.x);
            lf_chroma(sv + 4, ph.y);
            __syncwarp();
            if (act) {
#pragma unroll
                for (int i = 1; i < 9; i++) R.t[c][i][r] = (uint8_t)sv[i];
            }
            __syncwarp();
        }
        prev = act ? *(const uint2 *)R.t[c][2 + r] : z2;
        // row 7 of the MB above is final after this MB's top edge
        if (top && lane < 2)
            *(uint2 *)(Y + (lane ? P.v_off : P.u_off) + (size_t)(my * 8 - 1) * P.cpitch + x * 8) =
                *(const uint2 *)R.t[lane][1];
        __syncwarp();
    }
    if (act) *(uint2 *)(Cp + (size_t)(my * 8 + r) * P.cpitch + (P.mb_w - 1) * 8) = prev;
    if (ring_out) {
        if (P.mb_w - DRING > 0 && !wait_seen(ddown, ddown_seen, P.mb_w - DRING, P, lane)) { band_fail(P, lane); return; }
        if (act && r >= 6) *(uint2 *)(R.ring[(P.mb_w - 1) % DRING] + c * 16 + (r - 6) * 8) = prev;
    }
    __syncwarp();
    __threadfence_block();
    if (lane == 0) *dmine = P.mb_w;
}

// The hand-over to the neighbouring bands runs on two helper warps whose
// lanes poll together, so that one lane's fence or global load never holds
// up another's turn (lanes of one warp with loops of their own take turns).
//
// The roles of a band CTA (role r: bit r): all three, or in a split launch
// the ones its part of the band runs.
enum { BAND_INTRA = 1, BAND_LUMA = 2, BAND_CHROMA = 4, BAND_ALL = 7 };

// Mirror warp: copies progress published in global memory (acquire) into
// shared memory for the CTA's roles.  Lane 0: the row above's luma filter
// progress (with chroma in the CTA too, the row above's filter progress
// also stands for chroma's); lane 1: the row above's intra progress; lane 2:
// the row below's intra progress; lane 3, a chroma CTA of a split launch:
// the row above's chroma filter progress; lanes 4..4+rows-1, a CTA without
// intra: its rows' intra progress.
template <bool GROUPED>
__device__ __forceinline__ void band_mirror(const H264Launch &P, BandSmem &B, int y0, int rows, int lane, int part) {
    const uint32_t tag = (P.epoch & 0xffffu) << 16;
    const bool above = y0 > 0, below = y0 + rows < P.mb_h;
    const bool intra = part & BAND_INTRA, luma = part & BAND_LUMA, chroma = part & BAND_CHROMA;
    const uint32_t *src = nullptr;
    volatile int *d0 = nullptr, *d1 = nullptr;  // where a lane's progress goes
    if (lane == 0 && luma) {
        src = above ? P.rowprog + y0 - 1 : nullptr;
        d0 = &B.lprog[0];
        d1 = chroma ? &B.cprog[0] : nullptr;
    } else if (lane == 1 && intra) {
        src = above ? P.irowprog + y0 - 1 : nullptr;
        d0 = &B.iprog[0];
    } else if (lane == 2 && (luma || chroma)) {
        src = below ? P.irowprog + y0 + rows : nullptr;
        d0 = &B.iprog[rows + 1];
    } else if (lane == 3 && chroma && !luma) {
        src = above ? P.crowprog + y0 - 1 : nullptr;
        d0 = &B.cprog[0];
    } else if (lane >= 4 && lane < 4 + rows && !intra) {
        src = P.irowprog + y0 + lane - 4;
        d0 = &B.iprog[lane - 3];
    }
    if (d0 && !src) {
        *d0 = P.mb_w;
        if (d1) *d1 = P.mb_w;
    }
    int seen = src ? 0 : P.mb_w;
    uint32_t it = 0, ns = 32;
    while (!__all_sync(0xffffffffu, seen >= P.mb_w)) {
        bool moved = false;
        if (src && seen < P.mb_w) {
            const uint32_t v = ld_acquire(src);
            const int n = (v & 0xffff0000u) == tag ? (int)(v & 0xffffu) : 0;
            if (n > seen) {
                seen = n;
                moved = true;
                __threadfence_block();
                *d0 = seen;
                if (d1) *d1 = seen;
                it = 0;
            } else if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) {
                set_error(P.error, RC_DEV_ERR_TIMEOUT);
                seen = P.mb_w;  // give up; the waiting warps see the error
            }
        }
        // a group launch backs off (to 512 ns) while nothing moves: the
        // bands of its later pictures wait here a long time; one picture's
        // bands poll at the shortest step, the hand-over's latency being on
        // the wavefront's path
        if (GROUPED) ns = __any_sync(0xffffffffu, moved) ? 32 : min(ns * 2, 512u);
        __nanosleep(ns);
    }
}

// Publish warp: lane 0 publishes this band's last row's filter progress,
// lane 1 its intra progress (for the band below), lane 2 its first row's
// intra progress (for the band above).  One fence per round orders every
// store the band's warps made before the progress the lanes read (they
// fenced before publishing it in shared memory) ahead of the flags, which
// can then be relaxed stores (a release store costs about a fence more).
// In a split launch lane 0 publishes the luma filter's progress alone (a
// CTA with luma) or the chroma filter's (a chroma CTA, in crowprog), and the
// intra CTA's progress, every row's for the CTAs that filter them, goes out
// through a second warp (intra_rows, lanes 0..rows-1), so that its rounds
// never hold up the filter hand-over's.
template <bool GROUPED>
__device__ __forceinline__ void band_publish(const H264Launch &P, BandSmem &B, int y0, int rows, int lane, int part,
                                             bool intra_rows) {
    const uint32_t tag = (P.epoch & 0xffffu) << 16;
    const bool above = y0 > 0, below = y0 + rows < P.mb_h;
    // in a group launch, lanes 3.. also publish every row's filter progress
    // for the MB work of later pictures of the group that read this one, in
    // refprog: a word per 128-byte line, apart from the hand-over words, so
    // that the polls of the many waiting MB warps do not queue on the lines
    // that the bands hand over through
    constexpr bool grouped = GROUPED;
    const int prow = lane - 3;
    uint32_t *dst = nullptr;
    volatile int *a = nullptr, *b = nullptr;  // the lane publishes min(*a, *b), or *a
    if (intra_rows) {
        if (lane < rows) { dst = P.irowprog + y0 + lane; a = &B.iprog[lane + 1]; }
    } else if (part == BAND_CHROMA) {
        if (lane == 0 && below) { dst = P.crowprog + y0 + rows - 1; a = &B.cprog[rows]; }
    } else if (lane == 0) {
        if (below && (part & BAND_LUMA)) {
            dst = P.rowprog + y0 + rows - 1;
            a = &B.lprog[rows];
            b = part == BAND_ALL ? &B.cprog[rows] : nullptr;
        }
    } else if (part == BAND_ALL) {
        if (lane == 1 && below) { dst = P.irowprog + y0 + rows - 1; a = &B.iprog[rows]; }
        else if (lane == 2 && above) { dst = P.irowprog + y0; a = &B.iprog[1]; }
        else if (grouped && lane >= 3 && prow < rows) {
            dst = P.refprog + (size_t)(y0 + prow) * RC_REFPROG_STRIDE;
            a = &B.lprog[prow + 1];
            b = &B.cprog[prow + 1];
        }
    }
    int seen = dst ? 0 : P.mb_w;
    uint32_t it = 0;
    while (!__all_sync(0xffffffffu, seen >= P.mb_w)) {
        const int n = !dst ? seen : b ? min(*a, *b) : *a;
        const bool moved = n > seen;
        if (__any_sync(0xffffffffu, moved)) {
            __threadfence();
            if (moved) {
                st_relaxed(dst, tag | (uint32_t)n);
                seen = n;
            }
            it = 0;
        } else if (++it > P.wait_limit || ((it & 63) == 0 && aborted(P.error))) {
            if (lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT);
            break;
        }
        __nanosleep(32);
    }
}

// One band CTA: every thread of the CTA calls it; warps past the band's
// (3 BR + 2) roles leave after the shared state is set up, and so do the
// warps of the roles that `part` leaves to the other CTAs of a split launch
// (in the CTA with intra, the first chroma warp publishes every row's intra
// progress instead).
template <bool GROUPED>
__device__ __forceinline__ void band_body(const H264Launch &P, BandSmem &B, uint8_t *band_dyn, int band, int part) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y0 = band * BR, rows = min(BR, P.mb_h - y0);
    for (int i = threadIdx.x; i < 9 * 16; i += blockDim.x) B.tab4[i] = (&cPRED4.e[0][0])[i];
    for (int i = threadIdx.x; i < 9 * 64; i += blockDim.x) B.tab8[i] = (&cPRED8.e[0][0])[i];
    if (threadIdx.x < BR + 2) B.iprog[threadIdx.x] = 0;
    if (threadIdx.x < BR + 1) {
        B.lprog[threadIdx.x] = 0;
        B.cprog[threadIdx.x] = 0;
    }
    __syncthreads();
    if (warp == 3 * BR) { band_mirror<GROUPED>(P, B, y0, rows, lane, part); return; }
    if (warp == 3 * BR + 1) { band_publish<GROUPED>(P, B, y0, rows, lane, part, false); return; }
    if (warp >= 3 * BR + 2) return;
    const int role = warp / BR, w = warp % BR;
    if (part != BAND_ALL && (part & BAND_INTRA) && warp == 2 * BR) {
        band_publish<GROUPED>(P, B, y0, rows, lane, part, true);
        return;
    }
    if (w >= rows || !(part & (1 << role))) return;
    if (role == 0)
        band_intra_row<GROUPED>(P, B, band_dyn + BR * RC_BAND_STG, band_dyn + w * RC_BAND_STG, w, y0 + w, lane);
    else if (role == 1) band_luma_row(P, B, w, y0 + w, rows, lane);
    else band_chroma_row(P, B, w, y0 + w, rows, lane);
}

__global__ void __launch_bounds__(BAND_THREADS, 1) h264_band_kernel(const __grid_constant__ H264Launch P) {
    __shared__ BandSmem B;
    // dynamic: per band row the intra warp's staging (RC_BAND_STG bytes), then
    // per band row its line of bottom samples (mb_w x 32 bytes)
    extern __shared__ __align__(16) uint8_t band_dyn[];
    // split launch, CTAs bands wide per part: two parts intra + luma, then
    // chroma; three parts luma, intra, chroma.  Where the roles sit in the
    // grid decides which SMs they get (1080p band launch: luma, intra,
    // chroma 331 us; intra, chroma, luma 334; chroma, intra, luma 335;
    // intra, luma, chroma 337; luma, chroma, intra 337.5; chroma, luma,
    // intra 339; the three roles of a band side by side 351)
    const int bands = (P.mb_h + BR - 1) / BR, k = blockIdx.x / bands;
    const int part = P.band_split == 3   ? (k == 0 ? BAND_LUMA : k == 1 ? BAND_INTRA : BAND_CHROMA)
                     : P.band_split == 2 ? (k == 0 ? BAND_INTRA | BAND_LUMA : BAND_CHROMA)
                                         : BAND_ALL;
    band_body<false>(P, B, band_dyn, blockIdx.x % bands, part);
}

// ===========================================================================
// Kernel 3: a group of pictures in one cooperative launch.
// ===========================================================================
// Before the launch, per picture, h264_edge_kernel writes the edge words and
// h264_mb_kernel (residual_only) the residuals of every MB, the intra MBs'
// parameters and the I_PCM samples: all of it depends on the records alone.
// In the launch, n*bands CTAs spread over the grid are the band CTAs of the
// group's pictures (band CTA b: picture b % n, band b / n); every
// warp of the other CTAs takes (picture, MB) items in order from one counter
// -- every item of a picture before any item of the next, and a picture's
// MBs in the order of G.order, anti-diagonals that follow the wavefronts --
// predicts the item's MB if it is an inter MB, adds its residual, stores it
// and publishes mbdone[addr] = epoch.  (In raster order the few hundred
// items in flight would cover a row or two of a picture, released only as
// fast as one row of the picture it references is filtered, while that
// picture's wavefront finishes its rows side by side.)
// An item of picture j waits (mb_wait_refs) only for rows of earlier
// pictures of the group, whose items were all taken before it by warps that
// are running and whose band CTAs are resident (cooperative launch): every
// wait ends.  The MB work and the wavefronts wait on one another, so they
// share one launch: separate launches are not guaranteed to run at the same
// time.  The launch ends when every picture is filtered, so the next launch
// on the stream reads finished references.
constexpr int GROUP_THREADS = 512;
static_assert(GROUP_THREADS >= BAND_THREADS, "a group CTA holds a band CTA's warps");

// One inter MB of a group launch, one warp: the prediction of h264_mb_kernel
// plus the stored residual, clipped.  Lane l takes luma column l % 16, rows
// l / 16, +2, .., +14, and chroma column l % 8 of component (l / 8) % 2,
// rows l / 16, +2, +4, +6: each load and store of the warp covers two rows
// of consecutive samples, as in h264_mb_kernel.  Reads the references with
// coherent loads after waiting for the rows of the in-flight ones that its
// vectors reach.  False after a timeout.
__device__ bool mb_predict_warp(const H264Launch &P, int addr, int lane) {
    const rc_h264_mb &m = P.mbs[addr];
    const int mbx = addr % P.mb_w, mby = addr / P.mb_w;
    const int si = m.slice;
    if (si >= P.num_slices) {
        if (lane == 0) set_error(P.error, RC_DEV_ERR_RECORD);
        return true;
    }
    const rc_h264_slice *sl = P.slices + si;
    if (P.nwait > 0 && !mb_wait_refs(P, m, sl, mbx, mby, lane)) return false;
    __syncwarp();
    uint8_t *Y = P.dpb + (size_t)P.out_slot * P.slot_bytes;
    const int16_t *res = P.ires + (size_t)addr * 384;
    const int nref0 = min(__ldg(&sl->num_ref[0]), RC_H264_MAX_REFS), nref1 = min(__ldg(&sl->num_ref[1]), RC_H264_MAX_REFS);
    // the reference slot of list l for 8x8 block b8 (-1: unused); bad slots
    // are record errors, as in h264_mb_kernel
    auto ref_slot = [&](int l, int b8, bool report) -> int {
        const int ri = m.ref_idx[l][b8];
        if (ri < 0) return -1;
        const int slot = ri < (l ? nref1 : nref0) ? __ldg(&sl->ref_slot[l][ri]) : -1;
        if (slot < 0 || slot >= P.dpb_slots) {
            if (report) set_error(P.error, RC_DEV_ERR_RECORD);
            return -1;
        }
        return slot;
    };
    struct Wt {
        bool ex;
        int lw, w0, w1, o0, o1;
    };
    auto weight = [&](int b8, int cc) -> Wt {
        const int wi = m.wp[b8];
        const rc_h264_weight *w = (wi != 0xff && wi < P.num_weights) ? P.weights + wi : nullptr;
        const bool ex = w && (w->explicit_mask >> cc & 1);
        return {ex, ex ? w->log_wd[cc] : 0, ex ? w->w0[cc] : 0, ex ? w->w1[cc] : 0, ex ? w->o0[cc] : 0,
                ex ? w->o1[cc] : 0};
    };
    uint8_t *brow = P.bottom + (size_t)mby * P.mb_w * 32;
    {  // luma
        const int x = lane & 15, y0 = lane >> 4;
#pragma unroll 1
        for (int half = 0; half < 2; half++) {  // rows 0..7, then 8..15: one 8x8 block's list slots
            const int b8 = half * 2 + (x >> 3);
            int slot[2];
#pragma unroll
            for (int l = 0; l < 2; l++) slot[l] = ref_slot(l, b8, true);
            const Wt w = weight(b8, 0);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int y = half * 8 + y0 + 2 * i, k = (y >> 2) * 4 + (x >> 2);
                int v[2] = {0, 0};
#pragma unroll
                for (int l = 0; l < 2; l++) {
                    if (slot[l] < 0) continue;
                    const Ref r{P.dpb + (size_t)slot[l] * P.slot_bytes, P.pitch, P.W, P.H};
                    const int mvx = m.mv[l][k][0], mvy = m.mv[l][k][1];
                    v[l] = luma_sample<true>(r, mbx * 16 + x + (mvx >> 2), mby * 16 + y + (mvy >> 2), mvx & 3, mvy & 3);
                }
                const int pred = weigh(v[0], v[1], slot[0] >= 0, slot[1] >= 0, w.ex, w.lw, w.w0, w.w1, w.o0, w.o1);
                const uint8_t o = (uint8_t)clip255(pred + res[y * 16 + x]);
                Y[(size_t)(mby * 16 + y) * P.pitch + mbx * 16 + x] = o;
                if (y == 15) brow[mbx * 16 + x] = o;
            }
        }
    }
    {  // chroma
        const int x = lane & 7, c = (lane >> 3) & 1, y0 = lane >> 4, cc = 1 + c;
        uint8_t *C = c ? Y + P.v_off : Y + P.u_off;
#pragma unroll 1
        for (int half = 0; half < 2; half++) {  // rows 0..3, then 4..7
            const int b8 = half * 2 + (x >> 2);
            int slot[2];
#pragma unroll
            for (int l = 0; l < 2; l++) slot[l] = ref_slot(l, b8, false);
            const Wt w = weight(b8, cc);
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int y = half * 4 + y0 + 2 * i, k = (y >> 1) * 4 + (x >> 1);
                int v[2] = {0, 0};
#pragma unroll
                for (int l = 0; l < 2; l++) {
                    if (slot[l] < 0) continue;
                    const Ref r{P.dpb + (size_t)slot[l] * P.slot_bytes + (c ? P.v_off : P.u_off), P.cpitch, P.CW, P.CH};
                    const int mvx = m.mv[l][k][0], mvy = m.mv[l][k][1];
                    v[l] = chroma_sample<true>(r, mbx * 8 + x + (mvx >> 3), mby * 8 + y + (mvy >> 3), mvx & 7, mvy & 7);
                }
                const int pred = weigh(v[0], v[1], slot[0] >= 0, slot[1] >= 0, w.ex, w.lw, w.w0, w.w1, w.o0, w.o1);
                const uint8_t o = (uint8_t)clip255(pred + res[256 + c * 64 + y * 8 + x]);
                C[(size_t)(mby * 8 + y) * P.cpitch + mbx * 8 + x] = o;
                if (y == 7) brow[P.mb_w * (16 + 8 * c) + mbx * 8 + x] = o;
            }
        }
    }
    return true;
}

__global__ void __launch_bounds__(GROUP_THREADS, 1) h264_group_kernel(const __grid_constant__ H264Group G) {
    __shared__ BandSmem B;
    extern __shared__ __align__(16) uint8_t band_dyn[];
    // band CTAs are every stride-th CTA of the grid: spread over the GPU
    // instead of packed into neighbouring SMs, the band wavefront runs much
    // faster (1080p picture alone in a 152-CTA launch on GB300: 951 us with
    // the band CTAs first in the grid, 498 us spread); G.workers of the other
    // CTAs, spread the same way, predict inter MBs, and the rest leave
    const int nb = G.n * G.bands, stride = (int)gridDim.x / nb;
    const int bid = (int)blockIdx.x % stride == 0 && (int)blockIdx.x / stride < nb ? (int)blockIdx.x / stride : -1;
    if (bid >= 0) {
        // one inlined copy per picture index, so that the picture's
        // parameters stay immediate constant-bank operands
        // pictures interleaved, so that each picture's bands spread over
        // the whole GPU too
        const int j = bid % G.n, band = bid / G.n;
        static_assert(RC_H264_GROUP_MAX == 4, "one case per group position");
        switch (j) {
        case 0: band_body<true>(G.pic[0], B, band_dyn, band, BAND_ALL); break;
        case 1: band_body<true>(G.pic[1], B, band_dyn, band, BAND_ALL); break;
        case 2: band_body<true>(G.pic[2], B, band_dyn, band, BAND_ALL); break;
        default: band_body<true>(G.pic[3], B, band_dyn, band, BAND_ALL); break;
        }
        return;
    }
    {
        // rank among the CTAs that are not band CTAs
        const int rank = (int)blockIdx.x - min(nb, (int)blockIdx.x / stride + 1);
        const int others = (int)gridDim.x - nb, wstride = max(1, others / max(G.workers, 1));
        if (rank % wstride != 0 || rank / wstride >= G.workers) return;
    }
    const int lane = threadIdx.x & 31;
    const int n_mb = G.pic[0].mb_w * G.pic[0].mb_h, total = G.n * n_mb;
    for (;;) {
        int w = 0;
        if (lane == 0) w = (int)atomicAdd(G.counter, 1u);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= total) return;
        const int j = w / n_mb, addr = (int)__ldg(G.order + (w - j * n_mb));
        const H264Launch &P = G.pic[j];
        if (__ldg(&P.mbs[addr].kind) != RC_H264_INTER) continue;  // done by the pre-pass
        if (!mb_predict_warp(P, addr, lane) && lane == 0) set_error(P.error, RC_DEV_ERR_TIMEOUT);
        __syncwarp();
        if (lane == 0) {
            __threadfence();
            st_release(P.mbdone + addr, P.epoch);  // published even after an error: nothing waits forever
        }
    }
}

}  // namespace

void rc_launch_h264_edge(const H264Launch &p, cudaStream_t st) {
    const int n = p.mb_w * p.mb_h;
    h264_edge_kernel<<<(n + EDGE_MBS - 1) / EDGE_MBS, 32 * EDGE_MBS, 0, st>>>(p);
}

int rc_launch_h264_mv(const H264Launch &p, cudaStream_t st) {
    // rows per CTA: up to 16, as many as the rows' bottom-row buffers allow
    int rows = MV_MAX_WARPS;
    while (rows > 1 && mv_smem(rows, p.mb_w) > 160 * 1024) rows--;
    const size_t smem = mv_smem(rows, p.mb_w);
    const int ctas = (p.mb_h + rows - 1) / rows;
    int dev = 0, sms = 0, per = 0;
    if (smem > 200 * 1024 || cudaGetDevice(&dev) != cudaSuccess) return -1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaFuncSetAttribute(h264_mv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, h264_mv_kernel, rows * 32, smem) != cudaSuccess ||
        ctas > per * sms) {
        cudaGetLastError();
        return -1;
    }
    H264Launch q = p;
    void *args[] = {&q};
    return cudaLaunchCooperativeKernel((const void *)h264_mv_kernel, dim3(ctas), dim3(rows * 32), args, smem, st) ==
                   cudaSuccess
               ? 0
               : -1;
}

void rc_launch_h264_mb(const H264Launch &p, cudaStream_t st) {
    h264_mb_kernel<<<p.mb_w * p.mb_h, 256, 0, st>>>(p);
}

size_t rc_h264_band_smem(int mb_w) { return (size_t)BR * (RC_BAND_STG + (size_t)mb_w * 32); }

// The kernel's dynamic shared-memory limit is one attribute for every stream
// of the process: raise it to the widest picture any stream needs (never
// lower it, so a narrower stream created later cannot break a wider one).
// Kernel k: 0 the band kernel, 1 the group kernel.
static std::mutex g_band_attr_mu;
static int g_band_attr[2][64];

static bool band_smem_attr(int k, size_t dyn) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    std::lock_guard<std::mutex> lock(g_band_attr_mu);
    if ((int)dyn <= g_band_attr[k][dev]) return true;
    const void *fn = k ? (const void *)h264_group_kernel : (const void *)h264_band_kernel;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    g_band_attr[k][dev] = (int)dyn;
    return true;
}

int rc_h264_band_capacity(int mb_w) {
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (mb_w <= 0 || mb_w > 1024) return 0;  // the intra warps' row bitmaps
    const size_t dyn = rc_h264_band_smem(mb_w);
    if (!band_smem_attr(0, dyn)) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, h264_band_kernel, BAND_THREADS, dyn) != cudaSuccess)
        return 0;
    return per * sms;
}

int rc_launch_h264_band(const H264Launch &p, cudaStream_t st) {
    const int bands = (p.mb_h + BR - 1) / BR;
    if (!band_smem_attr(0, rc_h264_band_smem(p.mb_w))) return -1;
    H264Launch q = p;
    q.mbdone = nullptr;
    q.nwait = 0;
    void *args[] = {&q};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)h264_band_kernel, dim3(p.band_split > 1 ? p.band_split * bands : bands),
                                                dim3(BAND_THREADS), args, rc_h264_band_smem(p.mb_w), st);
    return e == cudaSuccess ? 0 : -1;
}

int rc_h264_group_capacity(int mb_w) {
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (mb_w <= 0 || mb_w > 1024) return 0;
    const size_t dyn = rc_h264_band_smem(mb_w);
    if (!band_smem_attr(1, dyn)) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, h264_group_kernel, GROUP_THREADS, dyn) != cudaSuccess)
        return 0;
    return per * sms;
}

int rc_launch_h264_group(const H264Group &g, int ctas, cudaStream_t st) {
    const int mb_w = g.pic[0].mb_w;
    if (g.n < 1 || g.n > RC_H264_GROUP_MAX || ctas <= g.n * g.bands || g.workers < 1 ||
        g.workers > ctas - g.n * g.bands)
        return -1;
    if (!band_smem_attr(1, rc_h264_band_smem(mb_w))) return -1;
    if (cudaMemsetAsync(g.counter, 0, sizeof(uint32_t), st) != cudaSuccess) return -1;
    H264Group q = g;
    void *args[] = {&q};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)h264_group_kernel, dim3(ctas), dim3(GROUP_THREADS), args,
                                                rc_h264_band_smem(mb_w), st);
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


namespace {
// The array's device address belongs to the CUDA context the module was
// loaded into, not to the device number: after cudaDeviceReset (or after the
// primary context is released and created again) the module loads into a new
// context and the array moves.  Addresses are therefore remembered per
// context, keyed by the context's id (cuCtxGetId), which the driver never
// gives to two contexts of one process, so a recreated context -- even one
// whose handle value repeats -- is looked up afresh.  The two driver calls
// are reached through the runtime's entry-point query, so the library does
// not link the driver library itself.
typedef CUresult (*CtxCurrentFn)(CUcontext *);
typedef CUresult (*CtxIdFn)(CUcontext, unsigned long long *);
std::mutex g_noalloc_mu;
CtxCurrentFn g_ctx_current = nullptr;
CtxIdFn g_ctx_id = nullptr;
bool g_ctx_fns_looked_up = false;
struct NoallocEntry {
    unsigned long long ctx_id;
    uint32_t *addr;
};
NoallocEntry g_noalloc_seen[64];
int g_noalloc_count = 0, g_noalloc_next = 0;

// Id of the context current on this thread, or 0 if there is none yet.
bool current_ctx_id(unsigned long long *id) {
    *id = 0;
    if (!g_ctx_fns_looked_up) {
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void **)&g_ctx_current, 4000, cudaEnableDefault,
                                             &q1) != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", (void **)&g_ctx_id, 12000, cudaEnableDefault, &q2) !=
                cudaSuccess || q2 != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            g_ctx_current = nullptr;
            g_ctx_id = nullptr;
            return false;
        }
        g_ctx_fns_looked_up = true;
    }
    CUcontext c = nullptr;
    if (g_ctx_current(&c) != CUDA_SUCCESS) return false;
    if (!c) return true;
    return g_ctx_id(c, id) == CUDA_SUCCESS;
}

// Device address of the static scratch in the current context.  The first
// call in a context looks it up with cudaGetSymbolAddress (the host-side name
// of a __device__ array is not a device address); later calls in the same
// context reuse it.
int noalloc_scratch(uint32_t **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    unsigned long long id = 0;
    if (!current_ctx_id(&id)) return RC_ECUDA;
    if (id)
        for (int i = 0; i < g_noalloc_count; i++)
            if (g_noalloc_seen[i].ctx_id == id) {
                *out = g_noalloc_seen[i].addr;
                return RC_OK;
            }
    // not seen in this context (or no context yet: the lookup creates the
    // device's primary context and makes it current)
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return RC_ECUDA;
    }
    if (!id && (!current_ctx_id(&id) || !id)) return RC_ECUDA;
    NoallocEntry &e = g_noalloc_seen[g_noalloc_count < 64 ? g_noalloc_count++ : (g_noalloc_next++ & 63)];
    e.ctx_id = id;
    e.addr = (uint32_t *)p;
    *out = e.addr;
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
    // each launch checked on its own return code: an error the caller left
    // pending from earlier work is neither reported here nor cleared
    void *args[] = {&L};
    if (cudaLaunchKernel((const void *)h264_db_params_kernel, dim3((mb_w * mb_h + 3) / 4), dim3(128), args, 0, st) !=
            cudaSuccess ||
        cudaLaunchKernel((const void *)h264_deblock_kernel, dim3(mb_h), dim3(32), args, 0, st) != cudaSuccess)
        return RC_ECUDA;
    return RC_OK;
}
