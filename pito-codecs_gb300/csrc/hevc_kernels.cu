// hevc_kernels.cu — HEVC block reconstruction on sm_103a.
//
// Per picture (samples are uint8_t for 8-bit, uint16_t for 10-bit streams):
//
//  hevc_residual_kernel  one warp per transform block, all in parallel:
//                        dequantisation (flat or scaling lists), 4..32
//                        inverse DCT / 4x4 DST as two matrix passes through
//                        shared memory (clamp between), transform skip, the
//                        DC-only shortcut, transquant bypass -> int16 residual
//                        planes.
//  hevc_inter_kernel     one 64-thread CTA per 16x16 luma area; a thread
//                        takes four adjacent luma samples (two chroma) of one
//                        motion field and reads each reference row once for
//                        them: 8-tap / 4-tap interpolation with i16
//                        intermediates, default or explicit weighted
//                        prediction, residual add, clip.
//  hevc_intra_kernel     persistent CTAs of 16 warps take CTBs in anti-diagonal
//                        order and reconstruct a CTB's intra blocks in shared
//                        memory, one warp per block in decode order: one lane
//                        per reference unit decides availability and waits
//                        (capped) only for intra neighbour blocks --
//                        shared-memory flags inside the CTB, global ready
//                        flags across CTBs -- a ballot gives the available
//                        units, the reference samples are gathered with
//                        substitution in one pass, smoothed, and predicted
//                        (planar, DC, 33 angles read straight from the
//                        references + edge filters) into the CTB copy; the
//                        block reaches the picture after its ready flags.
//  hevc_loopfilter_kernel one CTA per 64x64 tile: the tile and a 4-sample
//                        halo of the reconstructed picture into shared
//                        memory, vertical edges, then horizontal edges (one
//                        thread per 4-sample edge segment: edges 8 samples
//                        apart never interact within a direction), then SAO
//                        band / edge offsets, four samples per thread, into
//                        the DPB slot: the picture is read once and written
//                        once.
//
// Arithmetic follows src/hevc/{transform,intra,inter,filter}.rs and the
// reconstruction half of src/hevc/slicedec.rs; citations at each function.
#include <stdint.h>

#include <type_traits>

#include <algorithm>

#include "recon_internal.h"

namespace {

// The 32x32 inverse-transform matrix (TRANS_MATRIX, src/hevc/spec_tables.rs:107),
// built at compile time from the standard's integer cosine sets: entry (k, n)
// stands for 64 sqrt(2) cos((2n+1) k pi / 64); with k = 2^e o (o odd) the
// angle is (2n+1) o pi / (64 >> e), folded into the first quadrant, where the
// set of the (64 >> e)-point transform gives its value.
struct TransMatrix {
    int8_t m[32][32];
};
__host__ __device__ constexpr int trans_cos(int den, int j) {
    // integer cos(j pi / den), j odd, 0 < j < den / 2 (per transform size)
    constexpr int c4[1] = {64}, c8[2] = {83, 36}, c16[4] = {89, 75, 50, 18};
    constexpr int c32[8] = {90, 87, 80, 70, 57, 43, 25, 9};
    constexpr int c64[16] = {90, 90, 88, 85, 82, 78, 73, 67, 61, 54, 46, 38, 31, 22, 13, 4};
    const int i = (j - 1) / 2;
    return den == 4 ? c4[i] : den == 8 ? c8[i] : den == 16 ? c16[i] : den == 32 ? c32[i] : c64[i];
}
__host__ __device__ constexpr int trans_entry(int k, int n) {
    if (k == 0) return 64;
    int e = 0;
    while (!((k >> e) & 1)) e++;
    const int o = k >> e, den = 64 >> e;
    int j = ((2 * n + 1) * o) % (2 * den), sign = 1;
    if (j > den) j = 2 * den - j;  // cos(2 pi - a) = cos(a)
    if (j > den / 2) {             // cos(pi - a) = -cos(a)
        j = den - j;
        sign = -1;
    }
    return sign * trans_cos(den, j);
}
__host__ __device__ constexpr TransMatrix make_trans_matrix() {
    TransMatrix t{};
    for (int k = 0; k < 32; k++)
        for (int n = 0; n < 32; n++) t.m[k][n] = (int8_t)trans_entry(k, n);
    return t;
}
__constant__ TransMatrix cTRANSM = make_trans_matrix();
#define cTRANS (cTRANSM.m)
__constant__ int8_t cDST[4][4] = {{29, 55, 74, 84}, {74, 74, 0, -74}, {84, -29, -74, 55}, {55, -84, 74, -29}};
__constant__ int cLEVEL_SCALE[6] = {40, 45, 51, 57, 64, 72};
__constant__ int8_t cANGLE[35] = {0,  0,  32, 26, 21, 17, 13, 9,  5,  2,   0,   -2,  -5,  -9,  -13, -17, -21, -26,
                                  -32, -26, -21, -17, -13, -9, -5, -2, 0, 2, 5, 9, 13, 17, 21, 26, 32};
__constant__ int16_t cINV_ANGLE[15] = {-4096, -1638, -910, -630, -482, -390, -315, -256,
                                       -315,  -390,  -482, -630, -910, -1638, -4096};
__constant__ uint8_t cQPC_30_43[14] = {29, 30, 31, 32, 33, 33, 34, 34, 35, 35, 36, 36, 37, 37};
__constant__ uint8_t cBETA[52] = {0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  0,  6,  7,
                                  8,  9,  10, 11, 12, 13, 14, 15, 16, 17, 18, 20, 22, 24, 26, 28, 30, 32,
                                  34, 36, 38, 40, 42, 44, 46, 48, 50, 52, 54, 56, 58, 60, 62, 64};
__constant__ uint8_t cTC[54] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 5, 5, 6, 6, 7, 8, 9, 10, 11, 13, 14, 16, 18, 20, 22, 24};
__constant__ int8_t cLUMA_F[4][8] = {
    {0, 0, 0, 64, 0, 0, 0, 0}, {-1, 4, -10, 58, 17, -5, 1, 0}, {-1, 4, -11, 40, 40, -11, 4, -1}, {0, 1, -5, 17, 58, -10, 4, -1}};
__constant__ int8_t cCHROMA_F[8][4] = {{0, 64, 0, 0},    {-2, 58, 10, -2}, {-4, 54, 16, -2}, {-6, 46, 28, -4},
                                       {-4, 36, 36, -4}, {-4, 28, 46, -6}, {-2, 16, 54, -4}, {-2, 10, 58, -2}};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }
__device__ __forceinline__ int qpc_420(int q) { return q < 30 ? q : q > 43 ? q - 6 : cQPC_30_43[q - 30]; }

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ bool aborted(const uint32_t *err) {
    return (*(const volatile uint32_t *)err & RC_DEV_ERR_TIMEOUT) != 0;
}
__device__ bool wait_flag(const uint32_t *f, uint32_t epoch, uint32_t limit, const uint32_t *err) {
    uint32_t it = 0;
    while (ld_acquire(f) != epoch) {
        if (++it > limit) return false;
        if ((it & 63) == 0 && aborted(err)) return false;
        if (it > 16) __nanosleep(32);
    }
    return true;
}

// Plane access in the DPB / work layout (pitch in bytes).
template <class T>
__device__ __forceinline__ T *plane_ptr(uint8_t *base, const HevcLaunch &P, int c) {
    return (T *)(base + (c == 0 ? 0 : c == 1 ? P.u_off : P.v_off));
}
__device__ __forceinline__ int pitch_el(const HevcLaunch &P, int c, int size) { return (c ? P.cpitch : P.pitch) / size; }
__device__ __forceinline__ int16_t *res_plane(const HevcLaunch &P, int c) {
    return P.res + (c == 0 ? 0 : (size_t)P.W * P.H + (size_t)(c - 1) * P.CW * P.CH);
}
__device__ __forceinline__ const rc_hevc_slice *slice_of_ctb(const HevcLaunch &P, int ctb) {
    int s = P.ctbs[ctb].slice;
    return P.slices + (s < P.num_slices ? s : 0);
}
__device__ __forceinline__ int ctb_of(const HevcLaunch &P, int x, int y) {
    return (y >> P.log2ctb) * P.wctb + (x >> P.log2ctb);
}
__device__ __forceinline__ uint32_t slice_addr(const HevcLaunch &P, int ctb) { return slice_of_ctb(P, ctb)->slice_addr; }
// CTB of a transform block (records outside the picture map to CTB 0; the
// kernels that use the block reject it)
__device__ __forceinline__ int tu_ctb(const HevcLaunch &P, const rc_hevc_tu &t) {
    const int sc = t.c ? 2 : 1, x = t.x0 * sc, y = t.y0 * sc;
    if (x < 0 || y < 0 || x >= P.W || y >= P.H) return 0;
    return (y >> P.log2ctb) * P.wctb + (x >> P.log2ctb);
}

// ===========================================================================
// Residuals: reconstruct, src/hevc/slicedec.rs:2004-2049 with dequant /
// inverse / inverse_dc / transform_skip of src/hevc/transform.rs.
// ===========================================================================
__global__ void __launch_bounds__(128) hevc_residual_kernel(HevcLaunch P) {
    __shared__ int8_t mat[32][32];
    __shared__ int32_t buf[4][2][1024];
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) mat[i >> 5][i & 31] = cTRANS[i >> 5][i & 31];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t *co = buf[w][0], *col = buf[w][1];
    for (int ti = blockIdx.x * 4 + w; ti < P.num_tus; ti += gridDim.x * 4) {
        const rc_hevc_tu t = P.tus[ti];
        if (lane == 0) {  // the range of transform blocks of each CTB (contiguous in decode order)
            const int c = tu_ctb(P, t);
            if (ti == 0 || tu_ctb(P, P.tus[ti - 1]) != c) P.ctb_first[c] = ti;
            if (ti == P.num_tus - 1 || tu_ctb(P, P.tus[ti + 1]) != c) P.ctb_end[c] = ti + 1;
            if (t.flags & RC_HEVC_TU_INTRA) atomicAdd(&P.ctb_nintra[c], 1u);  // CTBs without any skip the intra kernel
        }
        if (!(t.flags & RC_HEVC_TU_CBF) || (t.flags & RC_HEVC_TU_PCM)) continue;
        const int log2 = t.log2, n = 1 << log2, c = t.c, mx = t.max_x, my = t.max_y;
        const unsigned long long cnt = (unsigned long long)(mx + 1) * (my + 1);
        const int pw = c ? P.CW : P.W, ph = c ? P.CH : P.H;
        if (log2 < 2 || log2 > 5 || c > 2 || mx >= n || my >= n || t.coef_off + cnt > P.num_levels ||
            t.x0 + n > pw || t.y0 + n > ph || (!(t.flags & RC_HEVC_TU_BYPASS) && t.qp < 0)) {
            if (lane == 0) atomicOr(P.error, RC_DEV_ERR_RECORD);
            continue;
        }
        for (int i = lane; i < n * n; i += 32) co[i] = 0;
        __syncwarp();
        const int16_t *lv = P.levels + t.coef_off;
        for (int i = lane; i < (int)cnt; i += 32) co[(i / (mx + 1)) * n + i % (mx + 1)] = lv[i];
        __syncwarp();
        const int bd = P.bd, intra = t.flags & RC_HEVC_TU_INTRA;
        int16_t *rp = res_plane(P, c) + (size_t)t.y0 * (c ? P.CW : P.W) + t.x0;
        const int rpitch = c ? P.CW : P.W;
        if (!(t.flags & RC_HEVC_TU_BYPASS)) {
            const bool ts = t.flags & RC_HEVC_TU_SKIP;
            const int qp = t.qp, bd_shift = bd + log2 - 5;
            const long long round = 1ll << (bd_shift - 1);
            const long long scale = (long long)cLEVEL_SCALE[qp % 6] << (qp / 6);
            const uint8_t *m = nullptr;
            if (P.scaling && !(ts && n > 4)) {
                const int off[4] = {0, 6 * 16, 6 * (16 + 64), 6 * (16 + 64 + 256)};
                m = P.scaling + off[log2 - 2] + (intra ? c : 3 + c) * (n * n);
            }
            // dequant, transform.rs:84-108
            for (int i = lane; i < (int)cnt; i += 32) {
                int y = i / (mx + 1), x = i % (mx + 1);
                int v = co[y * n + x];
                if (v) {
                    long long f = m ? m[y * n + x] : 16;
                    long long r = ((long long)v * f * scale + round) >> bd_shift;
                    co[y * n + x] = (int32_t)(r < -32768 ? -32768 : r > 32767 ? 32767 : r);
                }
            }
            __syncwarp();
            const int bs2 = 20 - bd, round2 = 1 << (bs2 - 1);
            if (ts) {  // transform_skip, transform.rs:73-81
                for (int i = lane; i < n * n; i += 32)
                    co[i] = clampi(((co[i] << (5 + log2)) + round2) >> bs2, -32768, 32767);
            } else if (mx == 0 && my == 0 && !(intra && c == 0 && n == 4)) {  // inverse_dc, transform.rs:68-71
                int e = clampi((64 * co[0] + 64) >> 7, -32768, 32767);
                int v = clampi((64 * e + round2) >> bs2, -32768, 32767);
                __syncwarp();
                for (int i = lane; i < n * n; i += 32) co[i] = v;
            } else {  // inverse::<N>, transform.rs:26-66
                const bool dst = intra && c == 0 && n == 4;
                const int step = 32 / n;
                for (int pr = lane; pr < (mx + 1) * n; pr += 32) {
                    int x = pr / n, i = pr % n, acc = 0;
                    for (int j = 0; j <= my; j++) acc += (dst ? cDST[j][i] : mat[j * step][i]) * co[j * n + x];
                    col[x * n + i] = clampi((acc + 64) >> 7, -32768, 32767);
                }
                __syncwarp();
                for (int pr = lane; pr < n * n; pr += 32) {
                    int y = pr / n, i = pr % n, out = round2;
                    for (int j = 0; j <= mx; j++) out += (dst ? cDST[j][i] : mat[j * step][i]) * col[j * n + y];
                    co[y * n + i] = clampi(out >> bs2, -32768, 32767);
                }
            }
            __syncwarp();
        }
        for (int i = lane; i < n * n; i += 32) rp[(i >> log2) * rpitch + (i & (n - 1))] = (int16_t)co[i];
        __syncwarp();
    }
}

// ===========================================================================
// Inter prediction (src/hevc/inter.rs, motion_compensate of slicedec.rs)
// ===========================================================================
template <class T>
__device__ __forceinline__ int rsamp(const T *p, int pitch, int w, int h, int x, int y) {
    return __ldg(p + (size_t)clampi(y, 0, h - 1) * pitch + clampi(x, 0, w - 1));
}

// Four horizontally adjacent samples of a plane row (x a multiple of 4: the
// planes' widths and pitches keep such groups aligned)
template <class T> struct Quad;
template <> struct Quad<uint8_t> {
    __device__ static void load(const uint8_t *p, int v[4]) {
        const uint32_t w = *(const uint32_t *)p;
        for (int i = 0; i < 4; i++) v[i] = (w >> (8 * i)) & 255;
    }
    __device__ static void store(uint8_t *p, const int v[4]) {
        *(uint32_t *)p = (uint32_t)v[0] | (uint32_t)v[1] << 8 | (uint32_t)v[2] << 16 | (uint32_t)v[3] << 24;
    }
};
template <> struct Quad<uint16_t> {
    __device__ static void load(const uint16_t *p, int v[4]) {
        const uint2 w = *(const uint2 *)p;
        v[0] = w.x & 0xffff; v[1] = w.x >> 16; v[2] = w.y & 0xffff; v[3] = w.y >> 16;
    }
    __device__ static void store(uint16_t *p, const int v[4]) {
        *(uint2 *)p = make_uint2((uint32_t)v[0] | (uint32_t)v[1] << 16, (uint32_t)v[2] | (uint32_t)v[3] << 16);
    }
};

// interpolate, inter.rs:86-133, for N horizontally adjacent samples from
// integer position (xi, yi) with one motion vector: each reference row's
// N + TAPS - 1 samples are read once for the N outputs
template <class T, int TAPS, int N>
__device__ void interp_n(const T *p, int pitch, int w, int h, int xi, int yi, int fx, int fy, int bd, int out[N]) {
    constexpr int m = TAPS / 2 - 1, W = N + TAPS - 1;
    const int shift1 = min(bd, 12) - 8, shift3 = 14 - bd;
    if (fx == 0 && fy == 0) {
#pragma unroll
        for (int i = 0; i < N; i++) out[i] = (int16_t)(rsamp(p, pitch, w, h, xi + i, yi) << shift3);
        return;
    }
    const int8_t *hf = TAPS == 8 ? cLUMA_F[fx] : cCHROMA_F[fx];
    const int8_t *vf = TAPS == 8 ? cLUMA_F[fy] : cCHROMA_F[fy];
    if (fy == 0) {
        int s[W];
#pragma unroll
        for (int j = 0; j < W; j++) s[j] = rsamp(p, pitch, w, h, xi - m + j, yi);
#pragma unroll
        for (int i = 0; i < N; i++) {
            int a = 0;
#pragma unroll
            for (int k = 0; k < TAPS; k++) a += hf[k] * s[i + k];
            out[i] = (int16_t)(a >> shift1);
        }
        return;
    }
    if (fx == 0) {
        int a[N];
#pragma unroll
        for (int i = 0; i < N; i++) a[i] = 0;
#pragma unroll
        for (int k = 0; k < TAPS; k++)
#pragma unroll
            for (int i = 0; i < N; i++) a[i] += vf[k] * rsamp(p, pitch, w, h, xi + i, yi - m + k);
#pragma unroll
        for (int i = 0; i < N; i++) out[i] = (int16_t)(a[i] >> shift1);
        return;
    }
    int v[N];
#pragma unroll
    for (int i = 0; i < N; i++) v[i] = 0;
#pragma unroll
    for (int r = 0; r < TAPS; r++) {
        int s[W];
#pragma unroll
        for (int j = 0; j < W; j++) s[j] = rsamp(p, pitch, w, h, xi - m + j, yi - m + r);
#pragma unroll
        for (int i = 0; i < N; i++) {
            int a = 0;
#pragma unroll
            for (int k = 0; k < TAPS; k++) a += hf[k] * s[i + k];
            v[i] += vf[r] * (int16_t)(a >> shift1);
        }
    }
#pragma unroll
    for (int i = 0; i < N; i++) out[i] = (int16_t)(v[i] >> 6);
}

// motion_compensate + put_uni / put_bi / put_weighted_*, for N horizontally
// adjacent samples of one motion field
template <class T, int N>
__device__ void mc_n(const HevcLaunch &P, int c, int x, int y, const rc_hevc_mvf &f, const rc_hevc_slice *sl, int out[N]) {
    const int bd = P.bd, max = (1 << bd) - 1;
    int pv[2][N];
    bool use[2] = {false, false};
    const int pw = c ? P.CW : P.W, ph = c ? P.CH : P.H, pitch = pitch_el(P, c, sizeof(T));
#pragma unroll
    for (int l = 0; l < 2; l++) {
#pragma unroll
        for (int i = 0; i < N; i++) pv[l][i] = 0;
        int ri = f.ref_idx[l];
        if (ri < 0) continue;
        int slot = ri < min(sl->num_ref[l], RC_HEVC_MAX_REFS) ? sl->ref_slot[l][ri] : -1;
        if (slot < 0 || slot >= P.dpb_slots) { atomicOr(P.error, RC_DEV_ERR_RECORD); continue; }
        use[l] = true;
        const T *p = plane_ptr<T>(P.dpb + (size_t)slot * P.slot_bytes, P, c);
        int mvx = f.mv[l][0], mvy = f.mv[l][1];
        if (c == 0) interp_n<T, 8, N>(p, pitch, pw, ph, x + (mvx >> 2), y + (mvy >> 2), mvx & 3, mvy & 3, bd, pv[l]);
        else interp_n<T, 4, N>(p, pitch, pw, ph, x + (mvx >> 3), y + (mvy >> 3), mvx & 7, mvy & 7, bd, pv[l]);
    }
    const bool bi = use[0] && use[1];
    if (!sl->weighted) {
        if (bi) {
            const int shift = 15 - bd;
#pragma unroll
            for (int i = 0; i < N; i++) out[i] = clampi((pv[0][i] + pv[1][i] + (1 << (shift - 1))) >> shift, 0, max);
            return;
        }
        const int shift = 14 - bd, off = shift > 0 ? 1 << (shift - 1) : 0;
#pragma unroll
        for (int i = 0; i < N; i++) out[i] = clampi(((use[0] ? pv[0][i] : pv[1][i]) + off) >> shift, 0, max);
        return;
    }
    const int log2wd = (c ? sl->chroma_log2_denom : sl->luma_log2_denom) + 14 - bd;
    int w[2] = {0, 0}, o[2] = {0, 0};
#pragma unroll
    for (int l = 0; l < 2; l++) {
        if (!use[l]) continue;
        int ri = f.ref_idx[l];
        w[l] = c ? sl->chroma_w[l][ri][c - 1] : sl->luma_w[l][ri];
        o[l] = (c ? sl->chroma_o[l][ri][c - 1] : sl->luma_o[l][ri]) * (1 << (bd - 8));
    }
    if (bi) {
#pragma unroll
        for (int i = 0; i < N; i++)
            out[i] = clampi((pv[0][i] * w[0] + pv[1][i] * w[1] + ((o[0] + o[1] + 1) << log2wd)) >> (log2wd + 1), 0, max);
        return;
    }
    const int l = use[0] ? 0 : 1;
#pragma unroll
    for (int i = 0; i < N; i++) {
        int v = (l ? pv[1][i] : pv[0][i]) * w[l];
        v = log2wd >= 1 ? ((v + (1 << (log2wd - 1))) >> log2wd) + o[l] : v + o[l];
        out[i] = clampi(v, 0, max);
    }
}

// A unit is late when one of the references it reads lies in slot
// P.late_slot, the previous picture (HevcLaunch::inter_pass).  References
// that do not resolve to a slot count as early; the early pass reports them.
__device__ __forceinline__ bool unit_is_late(const HevcLaunch &P, const rc_hevc_mvf &f, const rc_hevc_slice *sl) {
    bool late = false;
#pragma unroll
    for (int l = 0; l < 2; l++) {
        const int ri = f.ref_idx[l];
        late = late || (ri >= 0 && ri < min(sl->num_ref[l], RC_HEVC_MAX_REFS) && sl->ref_slot[l][ri] == P.late_slot);
    }
    return late;
}

// Four adjacent luma samples (x a multiple of 4) of an inter unit with
// motion f: prediction, residual, clip into the work picture.
template <class T>
__device__ __forceinline__ void inter_luma_quad(const HevcLaunch &P, int x, int y, const rc_hevc_mvf &f,
                                                const rc_hevc_slice *sl) {
    int v[4];
    mc_n<T, 4>(P, 0, x, y, f, sl, v);
    const int16_t *r = res_plane(P, 0) + (size_t)y * P.W + x;
    const int max = (1 << P.bd) - 1;
#pragma unroll
    for (int i = 0; i < 4; i++) v[i] = clampi(v[i] + r[i], 0, max);
    Quad<T>::store(plane_ptr<T>(P.work, P, 0) + (size_t)y * pitch_el(P, 0, sizeof(T)) + x, v);
}
// Two adjacent samples (x even) of chroma plane c.
template <class T>
__device__ __forceinline__ void inter_chroma_pair(const HevcLaunch &P, int c, int x, int y, const rc_hevc_mvf &f,
                                                  const rc_hevc_slice *sl) {
    int v[2];
    mc_n<T, 2>(P, c, x, y, f, sl, v);
    const int16_t *r = res_plane(P, c) + (size_t)y * P.CW + x;
    T *o = plane_ptr<T>(P.work, P, c) + (size_t)y * pitch_el(P, c, sizeof(T)) + x;
    const int max = (1 << P.bd) - 1;
#pragma unroll
    for (int i = 0; i < 2; i++) o[i] = (T)clampi(v[i] + r[i], 0, max);
}

// Appends the items of the lanes that push to the late list: one atomic per
// warp (all 32 lanes of the warp call it).
__device__ __forceinline__ void late_push(const HevcLaunch &P, bool push, uint32_t item) {
    const unsigned m = __ballot_sync(0xffffffffu, push);
    if (!m) return;
    const int lane = threadIdx.x & 31, lead = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == lead) base = atomicAdd(P.late_count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, lead);
    if (push) P.late_items[base + __popc(m & ((1u << lane) - 1))] = item;
}

// One CTA per 16x16 luma area: a thread reconstructs four adjacent luma
// samples of one 4x4 unit, then two adjacent chroma samples (of one unit
// too), each group with its motion field read once.  In the early pass
// (inter_pass 1) a late unit's groups go to the late list instead, as items
// c << 30 | y << 16 | x, for hevc_inter_late_kernel.
template <class T>
__global__ void __launch_bounds__(64) hevc_inter_kernel(HevcLaunch P) {
    const int t = threadIdx.x;
    const bool early = P.inter_pass == 1;
    {
        const int x = blockIdx.x * 16 + (t & 3) * 4, y = blockIdx.y * 16 + (t >> 2);
        bool push = false;
        if (x < P.W && y < P.H) {  // W is a multiple of 8: the group lies inside
            const int bi = (y >> 2) * P.w4 + (x >> 2);
            const rc_hevc_blk b = P.blk[bi];
            if ((b.flags & RC_HEVC_F_CODED) && !(b.flags & RC_HEVC_F_INTRA)) {
                const rc_hevc_mvf f = P.mvf[bi];
                const rc_hevc_slice *sl = slice_of_ctb(P, ctb_of(P, x, y));
                push = early && unit_is_late(P, f, sl);
                if (!push) inter_luma_quad<T>(P, x, y, f, sl);
            }
        }
        if (early) late_push(P, push, (uint32_t)y << 16 | (uint32_t)x);
    }
    {
        const int c = 1 + (t >> 5), x = blockIdx.x * 8 + (t & 3) * 2, y = blockIdx.y * 8 + ((t >> 2) & 7);
        bool push = false;
        if (x < P.CW && y < P.CH) {  // CW is a multiple of 4
            const int bi = ((2 * y) >> 2) * P.w4 + ((2 * x) >> 2);
            const rc_hevc_blk b = P.blk[bi];
            if ((b.flags & RC_HEVC_F_CODED) && !(b.flags & RC_HEVC_F_INTRA)) {
                const rc_hevc_mvf f = P.mvf[bi];
                const rc_hevc_slice *sl = slice_of_ctb(P, ctb_of(P, 2 * x, 2 * y));
                push = early && unit_is_late(P, f, sl);
                if (!push) inter_chroma_pair<T>(P, c, x, y, f, sl);
            }
        }
        if (early) late_push(P, push, (uint32_t)c << 30 | (uint32_t)y << 16 | (uint32_t)x);
    }
}

// The late pass: the groups the early pass listed, one per thread (a fixed
// grid strides over the list, whose length the early pass left on the device).
template <class T>
__global__ void __launch_bounds__(256) hevc_inter_late_kernel(HevcLaunch P) {
    const uint32_t n = min(*P.late_count, P.late_cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t it = P.late_items[i];
        const int c = it >> 30, y = (it >> 16) & 0x3fff, x = it & 0xffff;
        const int lx = c ? 2 * x : x, ly = c ? 2 * y : y;
        const int bi = (ly >> 2) * P.w4 + (lx >> 2);
        const rc_hevc_mvf f = P.mvf[bi];
        const rc_hevc_slice *sl = slice_of_ctb(P, ctb_of(P, lx, ly));
        if (c == 0) inter_luma_quad<T>(P, x, y, f, sl);
        else inter_chroma_pair<T>(P, c, x, y, f, sl);
    }
}

// ===========================================================================
// Intra task order: CTBs by anti-diagonal cx + 2 cy (then by cy).  CTBs on one
// anti-diagonal depend on none of each other, and every neighbour an intra
// block reads lies in its own CTB or in a CTB of an earlier anti-diagonal, so
// persistent CTAs that take CTBs in this order only ever wait for CTBs
// already taken.  One thread per CTB counts the CTBs before it.
// ===========================================================================
__global__ void __launch_bounds__(256) hevc_ctb_order_kernel(HevcLaunch P) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.wctb * P.hctb) return;
    const int cx = c % P.wctb, cy = c / P.wctb, key = cx + 2 * cy;
    int pos = 0;
    for (int y = 0; y < P.hctb; y++) {
        const int lim = key - 2 * y;  // CTBs (x, y) with x < lim come earlier
        pos += max(0, min(P.wctb, lim));
        if (y < cy && lim >= 0 && lim < P.wctb) pos++;  // same anti-diagonal, higher row
    }
    P.ctb_base[pos] = c;
}

// ===========================================================================
// Intra prediction in decode order (src/hevc/intra.rs, intra_predict of
// src/hevc/slicedec.rs:1673-1738)
// ===========================================================================
__device__ __forceinline__ uint32_t morton4(uint32_t x, uint32_t y) {
    uint32_t r = 0;
#pragma unroll
    for (int i = 0; i < 5; i++) r |= ((x >> i) & 1u) << (2 * i) | ((y >> i) & 1u) << (2 * i + 1);
    return r;
}
// zavail, src/hevc/slicedec.rs:625-643 (luma coordinates)
__device__ bool zavail(const HevcLaunch &P, int xc, int yc, int xn, int yn) {
    if (xn < 0 || yn < 0 || xn >= P.W || yn >= P.H) return false;
    const int s = P.log2ctb;
    const int cn = (yn >> s) * P.wctb + (xn >> s), cc = (yc >> s) * P.wctb + (xc >> s);
    if (cn != cc) {
        const rc_hevc_ctb &n = P.ctbs[cn], &q = P.ctbs[cc];
        return n.ts < q.ts && slice_addr(P, cn) == slice_addr(P, cc) && n.tile == q.tile;
    }
    const int m = (1 << s) - 1;
    return morton4((xn & m) >> 2, (yn & m) >> 2) <= morton4((xc & m) >> 2, (yc & m) >> 2);
}

struct __align__(16) IntraSmem {
    uint16_t left[136], top[136];   // reference samples (index 0 = corner)
    uint16_t fleft[136], ftop[136]; // smoothed copy
};

// The CTB a CTA reconstructs: its luma origin and size, a shared-memory copy
// of its samples (pre-deblock: inter blocks and residuals are already in
// place when the CTA starts, intra blocks land as they are reconstructed)
// and one flag per component and luma 4x4 unit: intra block reconstructed.
template <class T>
struct CtbCanvas {
    int x0, y0, s;       // luma origin, CTB size (<= 64)
    T *cv;               // luma s x s, then Cb and Cr (s/2) x (s/2)
    const int16_t *res;  // the CTB's residuals, same layout
    const uint8_t *blkf; // the CTB's 4x4 block flags (rc_hevc_blk::flags), 16 x 16
    volatile uint8_t *rdy;  // [3][16 x 16]: component, unit row, unit column
    __device__ __forceinline__ bool inside(int xl, int yl) const {
        return xl >= x0 && yl >= y0 && xl < x0 + s && yl < y0 + s;
    }
    // component c sample at plane coordinates (x, y), which must be inside
    __device__ __forceinline__ T &at(int c, int x, int y) const {
        if (c == 0) return cv[(y - y0) * s + (x - x0)];
        const int h = s >> 1;
        return cv[s * s + (c - 1) * h * h + (y - (y0 >> 1)) * h + (x - (x0 >> 1))];
    }
    __device__ __forceinline__ volatile uint8_t &flag(int c, int xl, int yl) const {
        return rdy[c * 256 + ((yl - y0) >> 2) * 16 + ((xl - x0) >> 2)];
    }
    __device__ __forceinline__ int resid(int c, int x, int y) const {
        if (c == 0) return res[(y - y0) * s + (x - x0)];
        const int h = s >> 1;
        return res[s * s + (c - 1) * h * h + (y - (y0 >> 1)) * h + (x - (x0 >> 1))];
    }
};

// Capped wait on a shared-memory flag of the CTB (another warp of this CTA).
__device__ bool wait_local(volatile uint8_t &f, uint32_t limit, const uint32_t *err) {
    uint32_t it = 0;
    while (!f) {
        if (++it > limit) return false;
        if ((it & 63) == 0 && aborted(err)) return false;
        if (it > 256) __nanosleep(32);  // a neighbour block is usually done within a few hundred polls
    }
    return true;
}

// One intra transform block, src/hevc/intra.rs and intra_predict of
// src/hevc/slicedec.rs:1673-1738, with its CTB in shared memory: neighbours
// inside the CTB are read (and waited for) there, neighbours outside it in
// the picture, after their global ready flags.
template <class T>
__device__ void intra_tu(const HevcLaunch &P, IntraSmem &S, const CtbCanvas<T> &C, const rc_hevc_tu &t, int lane) {
    // reference units: 4 luma samples, 2 chroma samples (shifts by lu, not
    // divisions by a run-time unit size)
    const int log2 = t.log2, n = 1 << log2, c = t.c, sc = c ? 2 : 1, lu = c ? 1 : 2, unit = 1 << lu;
    const int x0 = t.x0, y0 = t.y0, xl = x0 * sc, yl = y0 * sc, bd = P.bd, max = (1 << bd) - 1;
    T *pl = plane_ptr<T>(P.work, P, c);
    const int pitch = pitch_el(P, c, sizeof(T));
    const int n2 = 2 * n;
    // Reference units in the substitution scan order of src/hevc/intra.rs:
    // 19-65 (k: 0..NL-1 the left column's units bottom-up, NL the corner,
    // NL+1..2 NL the top row's units left to right).  Lane k decides unit k's
    // availability (and waits for it when it is an intra block); a ballot
    // gives the mask of available units.
    const int NL = n2 >> lu, nk = 2 * NL + 1;
    auto unit_xy = [&](int k, int &xn, int &yn) {  // the unit's first luma sample
        if (k < NL) { xn = xl - 1; yn = (y0 + ((NL - 1 - k) << lu)) * sc; }
        else if (k == NL) { xn = xl - 1; yn = yl - 1; }
        else { xn = (x0 + ((k - NL - 1) << lu)) * sc; yn = yl - 1; }
    };
    auto unit_avail = [&](int k, bool &ok) -> bool {
        int xn, yn;
        unit_xy(k, xn, yn);
        bool a = zavail(P, xl, yl, xn, yn);
        const bool in = C.inside(xn, yn);
        const uint8_t bf = !a ? 0 : in ? C.blkf[((yn - C.y0) >> 2) * 16 + ((xn - C.x0) >> 2)] : P.blk[(yn >> 2) * P.w4 + (xn >> 2)].flags;
        if (a && P.constrained_intra && !(bf & RC_HEVC_F_INTRA)) a = false;
        if (a && (bf & RC_HEVC_F_INTRA)) {
            if (in) ok = ok && wait_local(C.flag(c, xn, yn), P.wait_limit, P.error);
            else
                ok = ok && wait_flag(P.ready + (size_t)c * P.w4 * P.h4 + (yn >> 2) * P.w4 + (xn >> 2), P.epoch,
                                     P.wait_limit, P.error);
        }
        return a;
    };
    bool ok = true;
    const bool a0 = lane < nk && unit_avail(lane, ok);
    const bool a1 = lane + 32 < nk && unit_avail(lane + 32, ok);  // a 32x32 luma block's last top unit
    const unsigned long long mask =
        (unsigned long long)__ballot_sync(0xffffffffu, a1) << 32 | __ballot_sync(0xffffffffu, a0);
    if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) atomicOr(P.error, RC_DEV_ERR_TIMEOUT);
        return;
    }
    __threadfence_block();
    // ---- reference samples with substitution in one pass: scan-order
    // sample j (0..n2-1 left bottom-up, n2 the corner, n2+1.. top) reads
    // itself when its unit is available, else the last sample of the nearest
    // available unit before it, else (a leading run) the first available
    // sample; none available: 1 << (bd - 1)
    {
        const int first = __ffsll((long long)mask) - 1;
        auto unit_first = [&](int k) -> int { return k < NL ? k << lu : k == NL ? n2 : n2 + 1 + ((k - NL - 1) << lu); };
        // a lane's samples j = lane + 32 m (2 n2 + 1 of them, 17 to 129):
        // every address first, then the CTB copy's samples, then -- when a
        // lane of the warp needs one -- the picture's samples, all loads
        // issued before any is waited for, then the writes
        auto gather = [&](auto m_count) {
            constexpr int M = decltype(m_count)::value;
            int off[M];
            bool in[M];
            const T *cvc = &C.at(c, c ? C.x0 >> 1 : C.x0, c ? C.y0 >> 1 : C.y0);
            const int cst = c ? C.s >> 1 : C.s;
            bool outside = false;
#pragma unroll
            for (int m = 0; m < M; m++) {
                if (!mask) {  // no reference available: nothing is read
                    in[m] = true;
                    off[m] = 0;
                    continue;
                }
                const int j = min(lane + 32 * m, 2 * n2);
                const int k = j < n2 ? j >> lu : j == n2 ? NL : NL + 1 + ((j - n2 - 1) >> lu);
                const unsigned long long below = mask & ((1ull << k) - 1);
                const int kb = below ? 63 - __clzll((long long)below) : 0;
                const int src =
                    (mask >> k & 1) ? j : below ? unit_first(kb) + (kb == NL ? 0 : unit - 1) : unit_first(first);
                const int x = src <= n2 ? x0 - 1 : x0 + src - n2 - 1;
                const int y = src < n2 ? y0 + n2 - 1 - src : y0 - 1;
                in[m] = C.inside(x * sc, y * sc);
                // the CTB copy's offset, or the picture's
                off[m] = in[m] ? (y - (c ? C.y0 >> 1 : C.y0)) * cst + (x - (c ? C.x0 >> 1 : C.x0)) : y * pitch + x;
                outside = outside || !in[m];
            }
            uint16_t v[M];
#pragma unroll
            for (int m = 0; m < M; m++) v[m] = (uint16_t)cvc[in[m] ? off[m] : 0];
            if (__any_sync(0xffffffffu, outside)) {
                uint16_t g[M];
#pragma unroll
                for (int m = 0; m < M; m++) g[m] = (uint16_t)__ldcg(pl + (in[m] ? 0 : off[m]));
#pragma unroll
                for (int m = 0; m < M; m++) v[m] = in[m] ? v[m] : g[m];
            }
#pragma unroll
            for (int m = 0; m < M; m++) {
                const int j = lane + 32 * m;
                const uint16_t w = mask ? v[m] : (uint16_t)(1 << (bd - 1));
                if (j <= n2) S.left[n2 - j] = w;
                if (j >= n2 && j <= 2 * n2) S.top[j - n2] = w;
            }
        };
        if (n2 < 16) gather(std::integral_constant<int, 1>());
        else if (n2 < 32) gather(std::integral_constant<int, 2>());
        else if (n2 < 48) gather(std::integral_constant<int, 3>());
        else gather(std::integral_constant<int, 5>());
    }
    __syncwarp();
    const int mode = t.mode;
    // ---- filter, src/hevc/intra.rs:67-111 (luma only)
    const uint16_t *L = S.left, *Tp = S.top;
    if (c == 0 && mode != 1 && n != 4) {
        int md = min(abs(mode - 26), abs(mode - 10));
        int thres = n == 8 ? 7 : n == 16 ? 1 : 0;
        if (md > thres) {
            const int cc = S.left[0];
            bool strong = false;
            if (P.strong_intra && n == 32) {
                int bl = S.left[n2], tr = S.top[n2], thr = 1 << (bd - 5);
                strong = abs(cc + tr - 2 * S.top[n]) < thr && abs(cc + bl - 2 * S.left[n]) < thr;
                if (strong) {
                    for (int i = lane; i < 63; i += 32) {
                        S.fleft[1 + i] = (uint16_t)(((63 - i) * cc + (i + 1) * bl + 32) >> 6);
                        S.ftop[1 + i] = (uint16_t)(((63 - i) * cc + (i + 1) * tr + 32) >> 6);
                    }
                    if (lane == 0) {
                        S.fleft[0] = S.left[0]; S.ftop[0] = S.top[0];
                        S.fleft[64] = S.left[64]; S.ftop[64] = S.top[64];
                    }
                }
            }
            if (!strong) {
                for (int i = lane; i <= n2; i += 32) {
                    if (i == 0) S.fleft[0] = S.ftop[0] = (uint16_t)((S.left[1] + 2 * cc + S.top[1] + 2) >> 2);
                    else if (i == n2) { S.fleft[i] = S.left[i]; S.ftop[i] = S.top[i]; }
                    else {
                        S.fleft[i] = (uint16_t)((S.left[i - 1] + 2 * S.left[i] + S.left[i + 1] + 2) >> 2);
                        S.ftop[i] = (uint16_t)((S.top[i - 1] + 2 * S.top[i] + S.top[i + 1] + 2) >> 2);
                    }
                }
            }
            L = S.fleft;
            Tp = S.ftop;
        }
    }
    __syncwarp();
    // ---- predict, src/hevc/intra.rs:113-222
    const bool edge = c == 0 && n < 32;
    int dc = 0;
    if (mode == 1) {
        int s = 0;
        for (int i = lane; i < n; i += 32) s += Tp[1 + i] + L[1 + i];
        s = __reduce_add_sync(0xffffffffu, (unsigned)s);
        dc = (s + n) >> (log2 + 1);
    }
    // angular: ref[r] of src/hevc/intra.rs is read where it is needed, the
    // main side's sample r for r >= 0, else (a negative angle) the side
    // reference projected onto it, p[-1][-1 + ((r * invAngle + 128) >> 8)];
    // r < 0 only occurs when (n * angle) >> 5 < -1, as the standard has it
    const int angle = mode >= 2 ? cANGLE[mode] : 0, inv = angle < 0 ? cINV_ANGLE[mode - 11] : 0;
    const uint16_t *mn = mode >= 18 ? Tp : L, *sd = mode >= 18 ? L : Tp;
    // the block's place in the CTB copy and its residuals (the picture gets
    // the block after its ready flags, copy_out); predictions lie in
    // [0, max], so a block without residual adds 0 and clamps to itself
    const int cs = c ? C.s >> 1 : C.s;
    const int base = (c ? C.s * C.s + (c - 1) * cs * cs : 0) + (y0 - (c ? C.y0 >> 1 : C.y0)) * cs +
                     (x0 - (c ? C.x0 >> 1 : C.x0));
    T *out = C.cv + base;
    const int16_t *res = C.res + base;
    const bool cbf = t.flags & RC_HEVC_TU_CBF;
    auto put = [&](int x, int y, int v) {
        const int r = cbf ? res[y * cs + x] : 0;
        out[y * cs + x] = (T)clampi(v + r, 0, max);
    };
    // one loop per prediction kind, without branches in its body, four
    // samples per step: their reads (references, residuals) before their
    // writes, which could alias them
    auto run4 = [&](auto pred) {
        int i = lane;
        for (; i + 96 < n * n; i += 128) {
            int v[4], r[4], o[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int k = i + 32 * q, y = k >> log2, x = k & (n - 1);
                o[q] = y * cs + x;
                v[q] = pred(x, y);
                r[q] = cbf ? res[o[q]] : 0;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) out[o[q]] = (T)clampi(v[q] + r[q], 0, max);
        }
        for (; i < n * n; i += 32) {
            const int y = i >> log2, x = i & (n - 1);
            put(x, y, pred(x, y));
        }
    };
    if (mode == 0) {
        const int tr = Tp[1 + n], bl = L[1 + n];
        run4([&](int x, int y) {
            return ((n - 1 - x) * L[1 + y] + (x + 1) * tr + (n - 1 - y) * Tp[1 + x] + (y + 1) * bl + n) >> (log2 + 1);
        });
    } else if (mode == 1) {
        if (!edge) {
            run4([&](int, int) { return dc; });
        } else {
            const int corner = (L[1] + 2 * dc + Tp[1] + 2) >> 2;
            run4([&](int x, int y) {
                const int top = (Tp[1 + x] + 3 * dc + 2) >> 2, left = (L[1 + y] + 3 * dc + 2) >> 2;
                return (x == 0 && y == 0) ? corner : y == 0 ? top : x == 0 ? left : dc;
            });
        }
    } else {
        // output (x, y): horizontal modes (< 18) run j along x, vertical
        // along y; the reference index r of src/hevc/intra.rs, read from the
        // main side (r >= 0) or the side reference projected onto it
        const bool horizontal = mode < 18;
        run4([&](int x, int y) {
            const int j = horizontal ? x : y, ii = horizontal ? y : x;
            const int pos = (j + 1) * angle, idx = pos >> 5, fact = pos & 31;
            const int r = ii + idx + 1;
            const uint16_t *a0 = r >= 0 ? mn + r : sd + ((r * inv + 128) >> 8);
            const uint16_t *a1 = r + 1 >= 0 ? mn + r + 1 : sd + (((r + 1) * inv + 128) >> 8);
            return ((32 - fact) * (int)*a0 + fact * (int)*a1 + 16) >> 5;
        });
        // the edge filter of the pure directions: mode 26 rewrites column 0
        // from the left reference, mode 10 row 0 from the top one
        if (edge && (mode == 26 || mode == 10)) {
            __syncwarp();
            for (int k = lane; k < n; k += 32) {
                const int fv = horizontal ? L[1] + ((Tp[1 + k] - Tp[0]) >> 1) : Tp[1] + ((L[1 + k] - L[0]) >> 1);
                put(horizontal ? k : 0, horizontal ? 0 : k, clampi(fv, 0, max));
            }
        }
    }
}

// A reconstructed block's rows from the CTB copy to the picture, in 16-,
// 8- or 4-byte pieces (a block's rows are whole pieces: n * sizeof(T) is
// 4..64 bytes, and its x is a multiple of n)
template <class T>
__device__ void copy_out(const HevcLaunch &P, const CtbCanvas<T> &C, int c, int x0, int y0, int n, int lane) {
    T *pl = plane_ptr<T>(P.work, P, c);
    const int pitch = pitch_el(P, c, sizeof(T)), bytes = n * (int)sizeof(T);
    if (bytes >= 16) {
        const int q = bytes / 16;
        for (int i = lane; i < n * q; i += 32) {
            const int y = i / q, j = i % q;
            *((uint4 *)(pl + (size_t)(y0 + y) * pitch + x0) + j) = *((const uint4 *)&C.at(c, x0, y0 + y) + j);
        }
    } else if (bytes == 8) {
        if (lane < n) *(uint2 *)(pl + (size_t)(y0 + lane) * pitch + x0) = *(const uint2 *)&C.at(c, x0, y0 + lane);
    } else if (lane < n) {
        *(uint32_t *)(pl + (size_t)(y0 + lane) * pitch + x0) = *(const uint32_t *)&C.at(c, x0, y0 + lane);
    }
}


template <class T>
__device__ void pcm_tu(const HevcLaunch &P, const CtbCanvas<T> &C, const rc_hevc_tu &t, int lane) {
    const int n = 1 << t.log2;
    T *pl = plane_ptr<T>(P.work, P, t.c);
    const int pitch = pitch_el(P, t.c, sizeof(T));
    if (t.coef_off + (unsigned long long)n * n > P.num_levels) {
        if (lane == 0) atomicOr(P.error, RC_DEV_ERR_RECORD);
        return;
    }
    const int16_t *s = P.levels + t.coef_off;
    for (int i = lane; i < n * n; i += 32) {
        const int x = t.x0 + (i & (n - 1)), y = t.y0 + (i >> t.log2);
        pl[(size_t)y * pitch + x] = (T)s[i];
        C.at(t.c, x, y) = (T)s[i];
    }
}

// Persistent CTAs (INTRA_WARPS warps) take CTBs in the anti-diagonal task order.
// A CTA copies its CTB into shared memory; its warps then take the CTB's
// transform blocks in decode order and reconstruct the intra ones, each
// waiting only for the intra neighbour blocks it reads: in the CTB on the
// shared-memory flags (blocks earlier in decode order, taken by running
// warps), outside it on the global ready flags of CTBs taken earlier.  The
// CTB's residuals, 4x4 block flags and transform-block records are copied
// to shared memory first, so a block inside the CTB reads nothing global on
// its way; only blocks on the CTB's right column or bottom row, which later
// CTBs read, publish global flags (after a fence).
constexpr int INTRA_WARPS = 16;  // measured on 1080p Main: 4 warps 1325, 8 1518, 16 1650, 32 1600 frames/s
constexpr int INTRA_TU_CACHE = 256;  // a CTB's transform-block records copied to shared memory
template <class T>
__global__ void __launch_bounds__(32 * INTRA_WARPS) hevc_intra_kernel(HevcLaunch P) {
    extern __shared__ __align__(16) IntraSmem sm[];  // one per warp (dynamic: INTRA_WARPS of them)
    __shared__ __align__(16) T canvas[64 * 64 * 3 / 2];
    __shared__ __align__(16) int16_t resid[64 * 64 * 3 / 2];
    __shared__ __align__(16) rc_hevc_tu tuc[INTRA_TU_CACHE];
    __shared__ uint8_t rdy[3 * 256], blkf[256];
    __shared__ int task, next;
    const int tid = threadIdx.x, lane = tid & 31;
    IntraSmem &S = sm[tid >> 5];
    const int s = 1 << P.log2ctb, nctb = P.wctb * P.hctb;
    CtbCanvas<T> C;
    C.s = s;
    C.cv = canvas;
    C.res = resid;
    C.blkf = blkf;
    C.rdy = rdy;
    for (;;) {
        __syncthreads();  // the previous CTB is finished with the shared state
        if (tid == 0) {  // the error word and the next task, both requests in flight at once
            const uint32_t er = *(const volatile uint32_t *)P.error;
            const int tk = (int)atomicAdd(P.counter, 1u);
            task = (er & RC_DEV_ERR_TIMEOUT) ? nctb : tk;
        }
        __syncthreads();
        if (task >= nctb) return;
        const int cb = P.ctb_base[task];
        if (cb < 0 || cb >= nctb) {
            if (tid == 0) atomicOr(P.error, RC_DEV_ERR_RECORD);
            continue;
        }
        if (P.ctb_nintra[cb] == 0) continue;  // inter / residual work only: done by the earlier kernels
        const uint32_t f = P.ctb_first[cb], e = P.ctb_end[cb];
        C.x0 = (cb % P.wctb) << P.log2ctb;
        C.y0 = (cb / P.wctb) << P.log2ctb;
        // the CTB's samples: whole CTB-wide rows in 16-byte pieces (a row of a
        // CTB at the right edge still ends inside the plane's pitch, which is
        // a multiple of 128 bytes), the rows inside the picture
        {
            const int sh = min(s, P.H - C.y0);
            // 16-byte pieces per luma row, 8-byte pieces per chroma row (a
            // 16x16 CTB's 8-bit chroma rows are 8 bytes)
            const int lq = s * (int)sizeof(T) / 16, cq = (s >> 1) * (int)sizeof(T) / 8;
            const uint8_t *gy = P.work + (size_t)C.y0 * P.pitch + (size_t)C.x0 * sizeof(T);
            for (int i = tid; i < sh * lq; i += blockDim.x) {
                const int y = i / lq, q = i % lq;
                ((uint4 *)C.cv)[y * lq + q] = __ldcg((const uint4 *)(gy + (size_t)y * P.pitch) + q);
            }
            const int chh = sh >> 1, cs = (s >> 1) * (s >> 1);
            for (int i = tid; i < 2 * chh * cq; i += blockDim.x) {
                const int cc = i / (chh * cq), j = i % (chh * cq), y = j / cq, q = j % cq;
                const uint8_t *gc = P.work + (cc ? P.v_off : P.u_off) + (size_t)((C.y0 >> 1) + y) * P.cpitch +
                                    (size_t)(C.x0 >> 1) * sizeof(T);
                ((uint2 *)(C.cv + s * s + cc * cs))[y * cq + q] = __ldcg((const uint2 *)gc + q);
            }
            // its residuals (rows clipped to the plane: 16-byte pieces of luma,
            // 8-byte pieces of chroma; W and CW are multiples of 8 and 4)
            const int lw = min(s, P.W - C.x0), cwid = lw >> 1;
            for (int i = tid; i < sh * (lw >> 3); i += blockDim.x) {
                const int y = i / (lw >> 3), q = i % (lw >> 3);
                ((uint4 *)(resid + y * s))[q] = __ldcg((const uint4 *)(P.res + (size_t)(C.y0 + y) * P.W + C.x0) + q);
            }
            for (int i = tid; i < 2 * chh * (cwid >> 2); i += blockDim.x) {
                const int per = chh * (cwid >> 2), cc = i / per, j = i % per, y = j / (cwid >> 2), q = j % (cwid >> 2);
                const int16_t *rc = res_plane(P, 1 + cc) + (size_t)((C.y0 >> 1) + y) * P.CW + (C.x0 >> 1);
                ((uint2 *)(resid + s * s + cc * cs + y * (s >> 1)))[q] = __ldcg((const uint2 *)rc + q);
            }
            // its 4x4 block flags and transform-block records
            const int u = s >> 2;
            for (int i = tid; i < u * u; i += blockDim.x) {
                const int gx = (C.x0 >> 2) + i % u, gy = (C.y0 >> 2) + i / u;
                blkf[(i / u) * 16 + i % u] = (gx < P.w4 && gy < P.h4) ? P.blk[(size_t)gy * P.w4 + gx].flags : 0;
            }
            if (e - f <= (uint32_t)INTRA_TU_CACHE)
                for (int i = tid; i < (int)(e - f); i += blockDim.x) ((uint4 *)tuc)[i] = __ldg((const uint4 *)(P.tus + f) + i);
            for (int i = tid; i < 3 * 256; i += blockDim.x) rdy[i] = 0;
            if (tid == 0) next = (int)f;
        }
        __syncthreads();
        for (;;) {
            int ti = 0;
            if (lane == 0) ti = atomicAdd(&next, 1);
            ti = __shfl_sync(0xffffffffu, ti, 0);
            if (ti >= (int)e) break;
            const rc_hevc_tu t = e - f <= (uint32_t)INTRA_TU_CACHE ? tuc[ti - f] : P.tus[ti];
            if (!(t.flags & RC_HEVC_TU_INTRA)) continue;
            const int n = 1 << t.log2, sc = t.c ? 2 : 1;
            if (t.log2 < 2 || t.log2 > 5 || t.c > 2 || t.mode > 34 || (t.x0 + n) * sc > P.W || (t.y0 + n) * sc > P.H ||
                !C.inside(t.x0 * sc, t.y0 * sc) || !C.inside((t.x0 + n) * sc - 1, (t.y0 + n) * sc - 1)) {
                if (lane == 0) atomicOr(P.error, RC_DEV_ERR_RECORD);
                continue;
            }
            // the error word, read as the block starts and tested once its
            // flags are out (a global read there would delay every waiting
            // block by a round trip)
            const uint32_t err0 = *(const volatile uint32_t *)P.error;
            if (t.flags & RC_HEVC_TU_PCM) pcm_tu<T>(P, C, t, lane);
            else intra_tu<T>(P, S, C, t, lane);
            // the block's luma-grid 4x4 units, for the warps of this CTA
            __syncwarp();
            __threadfence_block();
            const int bw = (n * sc) >> 2;
            for (int i = lane; i < bw * bw; i += 32) C.flag(t.c, t.x0 * sc + (i % bw) * 4, t.y0 * sc + (i / bw) * 4) = 1;
            // then the picture's copy (blocks in this CTB read the CTB copy;
            // later CTBs read the picture after the global flags below)
            if (!(t.flags & RC_HEVC_TU_PCM)) copy_out<T>(P, C, t.c, t.x0, t.y0, n, lane);
            // a block on the CTB's right column or bottom row is read by later
            // CTBs: after a fence, its global ready flags (the shared ones are
            // set first, so this CTB's next blocks do not wait for the fence)
            if ((t.x0 + n) * sc >= C.x0 + s || (t.y0 + n) * sc >= C.y0 + s) {
                __threadfence();
                uint32_t *gr = P.ready + (size_t)t.c * P.w4 * P.h4;
                for (int i = lane; i < bw * bw; i += 32)
                    st_relaxed(gr + (size_t)(((t.y0 * sc) >> 2) + i / bw) * P.w4 + ((t.x0 * sc) >> 2) + i % bw, P.epoch);
            }
            if (err0 & RC_DEV_ERR_TIMEOUT) break;
        }
    }
}

// ===========================================================================
// Deblocking, src/hevc/filter.rs:75-519
// ===========================================================================
__device__ __forceinline__ uint32_t h_ref_id(const HevcLaunch &P, int ctb, const rc_hevc_mvf &f, int l) {
    const rc_hevc_slice *sl = slice_of_ctb(P, ctb);
    int r = f.ref_idx[l];
    return (r >= 0 && r < min(sl->num_ref[l], RC_HEVC_MAX_REFS)) ? sl->ref_id[l][r] : 0xfffffffeu;
}
__device__ __forceinline__ bool far_mv(const int16_t *a, const int16_t *b) {
    return abs(a[0] - b[0]) >= 4 || abs(a[1] - b[1]) >= 4;
}
// boundary_strength + motion_bs, filter.rs:84-144
__device__ int boundary_strength(const HevcLaunch &P, int pi, int qi, bool tu_edge, int pctb, int qctb) {
    const rc_hevc_blk p = P.blk[pi], q = P.blk[qi];
    if ((p.flags | q.flags) & RC_HEVC_F_INTRA) return 2;
    if (tu_edge && ((p.flags | q.flags) & RC_HEVC_F_CBF)) return 1;
    const rc_hevc_mvf mp = P.mvf[pi], mq = P.mvf[qi];
    const int np = (mp.ref_idx[0] >= 0) + (mp.ref_idx[1] >= 0), nq = (mq.ref_idx[0] >= 0) + (mq.ref_idx[1] >= 0);
    if (np != nq) return 1;
    if (np == 1) {
        int lp = mp.ref_idx[0] >= 0 ? 0 : 1, lq = mq.ref_idx[0] >= 0 ? 0 : 1;
        if (h_ref_id(P, pctb, mp, lp) != h_ref_id(P, qctb, mq, lq)) return 1;
        return far_mv(mp.mv[lp], mq.mv[lq]);
    }
    uint32_t p0 = h_ref_id(P, pctb, mp, 0), p1 = h_ref_id(P, pctb, mp, 1);
    uint32_t q0 = h_ref_id(P, qctb, mq, 0), q1 = h_ref_id(P, qctb, mq, 1);
    if (!((p0 == q0 && p1 == q1) || (p0 == q1 && p1 == q0))) return 1;
    if (p0 != p1) {
        if (p0 == q0) return far_mv(mp.mv[0], mq.mv[0]) || far_mv(mp.mv[1], mq.mv[1]);
        return far_mv(mp.mv[0], mq.mv[1]) || far_mv(mp.mv[1], mq.mv[0]);
    }
    return (far_mv(mp.mv[0], mq.mv[0]) || far_mv(mp.mv[1], mq.mv[1])) &&
           (far_mv(mp.mv[0], mq.mv[1]) || far_mv(mp.mv[1], mq.mv[0]));
}
// edge_params, filter.rs:146-176
__device__ bool edge_params(const HevcLaunch &P, int px, int py, int qx, int qy, int &tc_off, int &beta_off) {
    const int pc = ctb_of(P, px, py), qc = ctb_of(P, qx, qy);
    const rc_hevc_slice *sq = slice_of_ctb(P, qc);
    if (sq->deblock_disabled) return false;
    if (pc != qc) {
        if (slice_addr(P, pc) != slice_addr(P, qc) && !sq->lf_across) return false;
        if (!P.lf_across_tiles && P.ctbs[pc].tile != P.ctbs[qc].tile) return false;
    }
    tc_off = sq->tc_offset;
    beta_off = sq->beta_offset;
    return true;
}

// filter_luma, filter.rs:409-492; o = q0 of line 0
template <class T>
__device__ void filter_luma(T *s, long o, long step, long along, int tc, int beta, bool nfp, bool nfq, int bd) {
#define PX(k, i) ((int)s[o + (k) * along - ((i) + 1) * step])
#define QX(k, i) ((int)s[o + (k) * along + (i) * step])
    const int dp0 = abs(PX(0, 2) - 2 * PX(0, 1) + PX(0, 0)), dp3 = abs(PX(3, 2) - 2 * PX(3, 1) + PX(3, 0));
    const int dq0 = abs(QX(0, 2) - 2 * QX(0, 1) + QX(0, 0)), dq3 = abs(QX(3, 2) - 2 * QX(3, 1) + QX(3, 0));
    const int dpq0 = dp0 + dq0, dpq3 = dp3 + dq3, dp = dp0 + dp3, dq = dq0 + dq3, d = dpq0 + dpq3;
    if (d >= beta) return;
#define DSAM(k, dpq)                                                                                     \
    ((dpq) < (beta >> 2) && abs(PX(k, 3) - PX(k, 0)) + abs(QX(k, 0) - QX(k, 3)) < (beta >> 3) &&      \
     abs(PX(k, 0) - QX(k, 0)) < ((5 * tc + 1) >> 1))
    const bool strong = DSAM(0, 2 * dpq0) && DSAM(3, 2 * dpq3);
#undef DSAM
#undef PX
#undef QX
    const bool dep = dp < ((beta + (beta >> 1)) >> 3), deq = dq < ((beta + (beta >> 1)) >> 3);
    const int max = (1 << bd) - 1;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const long b = o + k * along;
        const int p0 = s[b - step], p1 = s[b - 2 * step], p2 = s[b - 3 * step], p3 = s[b - 4 * step];
        const int q0 = s[b], q1 = s[b + step], q2 = s[b + 2 * step], q3 = s[b + 3 * step];
        if (strong) {
            const int t2 = 2 * tc;
            if (!nfp) {
                s[b - step] = (T)clampi((p2 + 2 * p1 + 2 * p0 + 2 * q0 + q1 + 4) >> 3, p0 - t2, p0 + t2);
                s[b - 2 * step] = (T)clampi((p2 + p1 + p0 + q0 + 2) >> 2, p1 - t2, p1 + t2);
                s[b - 3 * step] = (T)clampi((2 * p3 + 3 * p2 + p1 + p0 + q0 + 4) >> 3, p2 - t2, p2 + t2);
            }
            if (!nfq) {
                s[b] = (T)clampi((p1 + 2 * p0 + 2 * q0 + 2 * q1 + q2 + 4) >> 3, q0 - t2, q0 + t2);
                s[b + step] = (T)clampi((p0 + q0 + q1 + q2 + 2) >> 2, q1 - t2, q1 + t2);
                s[b + 2 * step] = (T)clampi((p0 + q0 + q1 + 3 * q2 + 2 * q3 + 4) >> 3, q2 - t2, q2 + t2);
            }
        } else {
            int delta = (9 * (q0 - p0) - 3 * (q1 - p1) + 8) >> 4;
            if (abs(delta) >= tc * 10) continue;
            delta = clampi(delta, -tc, tc);
            if (!nfp) s[b - step] = (T)clampi(p0 + delta, 0, max);
            if (!nfq) s[b] = (T)clampi(q0 - delta, 0, max);
            if (dep && !nfp) s[b - 2 * step] = (T)clampi(p1 + clampi((((p2 + p0 + 1) >> 1) - p1 + delta) >> 1, -(tc >> 1), tc >> 1), 0, max);
            if (deq && !nfq) s[b + step] = (T)clampi(q1 + clampi((((q2 + q0 + 1) >> 1) - q1 - delta) >> 1, -(tc >> 1), tc >> 1), 0, max);
        }
    }
}
// filter_chroma, filter.rs:494-519
template <class T>
__device__ void filter_chroma(T *s, long o, long step, long along, int tc, bool nfp, bool nfq, int bd) {
    const int max = (1 << bd) - 1;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const long b = o + k * along;
        const int p0 = s[b - step], p1 = s[b - 2 * step], q0 = s[b], q1 = s[b + step];
        const int delta = clampi((((q0 - p0) << 2) + p1 - q1 + 4) >> 3, -tc, tc);
        if (!nfp) s[b - step] = (T)clampi(p0 + delta, 0, max);
        if (!nfq) s[b] = (T)clampi(q0 - delta, 0, max);
    }
}

// The loop filter works on one tile of the picture in shared memory: the
// tile's LF_TW x TH luma samples (half that per chroma plane) and a halo of
// LF_HALO samples on every side.  That halo holds every sample that the
// deblocking of the tile and of its one-sample SAO border reads: vertical
// edges lie 8 luma (8 chroma) samples apart and move at most 3 (1) samples
// beside them, reading 4 (2); horizontal edges do the same on the vertically
// filtered samples; so the edges at x0 .. x0 + LF_TW and y0 .. y0 + TH,
// filtered over the whole tile with its halo, leave every sample of the tile
// and its border as the picture-wide passes (all vertical edges, then all
// horizontal edges; filter.rs:178-407) leave it.  Edges on a tile boundary
// are filtered by both tiles, identically.
// Tiles are LF_TW wide and TH (64, 32 or 16: the stream's choice,
// rc_stream_set_lf_tile) rows high.
constexpr int LF_TW = 64, LF_HALO = 4, LF_THREADS = 256;
constexpr int LF_LW = LF_TW + 2 * LF_HALO, LF_CW = LF_TW / 2 + 2 * LF_HALO;
template <class T, int TH>
struct LfTile {
    static constexpr int LH = TH + 2 * LF_HALO, CH = TH / 2 + 2 * LF_HALO;
    T y[LH][LF_LW];
    T c[2][CH][LF_CW];
};
template <class T> struct Raw4;
template <> struct Raw4<uint8_t> { using type = uint32_t; };
template <> struct Raw4<uint16_t> { using type = uint2; };

// One edge segment (4 luma samples along the edge, or 4 chroma samples of
// both chroma planes) at 4x4 luma unit (bx, by): the decision from the
// records and the filter, on the tile (hevc_deblock's per-edge body,
// filter.rs:178-407).  x0, y0: luma picture position of the tile (its
// first sample inside the halo); dir 0 vertical edge (left of the unit), 1
// horizontal (top).
template <class T, int DIR, int TH>
__device__ void deblock_segment(const HevcLaunch &P, LfTile<T, TH> &S, int bx, int by, bool chroma, int x0, int y0) {
    const int qi = by * P.w4 + bx, pi = DIR == 0 ? qi - 1 : qi - P.w4;
    const int x = bx * 4, y = by * 4;
    const int px = DIR == 0 ? x - 1 : x, py = DIR == 0 ? y : y - 1;
    const rc_hevc_blk q = P.blk[qi], p = P.blk[pi];
    const int emask = DIR == 0 ? (RC_HEVC_E_TU_V | RC_HEVC_E_PU_V) : (RC_HEVC_E_TU_H | RC_HEVC_E_PU_H);
    if (!(q.edges & emask) || !(q.flags & RC_HEVC_F_CODED)) return;
    int tco, bo;
    if (!edge_params(P, px, py, x, y, tco, bo)) return;
    const int bs = boundary_strength(P, pi, qi, (q.edges & (DIR == 0 ? RC_HEVC_E_TU_V : RC_HEVC_E_TU_H)) != 0,
                                     ctb_of(P, px, py), ctb_of(P, x, y));
    const bool nfp = p.flags & RC_HEVC_F_NOFILTER, nfq = q.flags & RC_HEVC_F_NOFILTER;
    const int bd = P.bd;
    if (!chroma) {
        if (bs == 0) return;
        // tc_beta, filter.rs:74-82
        const int qpl = (p.qp + q.qp + 1) >> 1;
        const int qb = clampi(qpl + bo, 0, 51), qt = clampi(qpl + 2 * (bs - 1) + tco, 0, 53);
        const int tc = cTC[qt] << (bd - 8), beta = cBETA[qb] << (bd - 8);
        filter_luma<T>(&S.y[0][0], (long)(y - y0 + LF_HALO) * LF_LW + (x - x0 + LF_HALO), DIR == 0 ? 1 : LF_LW,
                       DIR == 0 ? LF_LW : 1,
                       tc, beta, nfp, nfq, bd);
    } else {
        if (bs != 2) return;
        for (int c = 1; c < 3; c++) {
            const int qpi = ((p.qp + q.qp + 1) >> 1) + (c == 1 ? P.cb_qp_offset : P.cr_qp_offset);
            const int qt = clampi(qpc_420(qpi) + 2 + tco, 0, 53), tc = cTC[qt] << (bd - 8);
            filter_chroma<T>(&S.c[c - 1][0][0], (long)(y / 2 - y0 / 2 + LF_HALO) * LF_CW + (x / 2 - x0 / 2 + LF_HALO),
                             DIR == 0 ? 1 : LF_CW, DIR == 0 ? LF_CW : 1, tc, nfp, nfq, bd);
        }
    }
}

// ===========================================================================
// SAO, src/hevc/filter.rs:521-894: four samples per thread, deblocked
// work picture -> DPB slot
// ===========================================================================
// cross_ok, filter.rs:605-632
__device__ bool cross_ok(const HevcLaunch &P, int rs, int nrs) {
    if (nrs == rs) return true;
    const rc_hevc_ctb &n = P.ctbs[nrs], &q = P.ctbs[rs];
    if (n.slice >= P.num_slices) return false;
    if (slice_addr(P, nrs) != slice_addr(P, rs)) {
        if (n.ts < q.ts && !slice_of_ctb(P, rs)->lf_across) return false;
        if (q.ts < n.ts && !P.slices[n.slice].lf_across) return false;
    }
    return P.lf_across_tiles || n.tile == q.tile;
}

// The loop filter of one tile (src/hevc/filter.rs:178-894): the
// reconstructed (pre-deblocking) samples of the tile and its halo into
// shared memory, vertical edges, horizontal edges, then SAO of the tile's
// samples from the deblocked tile (its neighbours pre-SAO, as the reference
// reads them) into the DPB slot.  The work picture is only read.
template <class T, int TH>
__global__ void __launch_bounds__(LF_THREADS) hevc_loopfilter_kernel(HevcLaunch P) {
    __shared__ __align__(16) LfTile<T, TH> S;
    constexpr int LF_LH = LfTile<T, TH>::LH, LF_CH = LfTile<T, TH>::CH;
    using R4 = typename Raw4<T>::type;
    const int x0 = blockIdx.x * LF_TW, y0 = blockIdx.y * TH;
    const int ox = x0 - LF_HALO, oy = y0 - LF_HALO;  // luma position of S.y[0][0]
    const int cx0 = x0 / 2, cy0 = y0 / 2, cox = cx0 - LF_HALO, coy = cy0 - LF_HALO;
    const int tid = threadIdx.x;
    // the intra kernel's task counter back to zero for the next picture: this
    // launch follows the picture's intra kernel on the same stream, and the
    // next intra kernel follows it
    if (blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) *P.counter = 0;
    // 1. load: four samples per step (W and H are multiples of 8, so a
    // 4-aligned group of four lies wholly inside or outside the picture;
    // outside ones, which no filter and no SAO class reads, are zero)
    {
        constexpr int LQ = LF_LH * (LF_LW / 4), CQ = LF_CH * (LF_CW / 4);
        const T *wy = plane_ptr<T>(P.work, P, 0);
        const long py = pitch_el(P, 0, sizeof(T)), pc = pitch_el(P, 1, sizeof(T));
        for (int i = tid; i < LQ + 2 * CQ; i += LF_THREADS) {
            const bool luma = i < LQ;
            const int c = luma ? 0 : 1 + (i - LQ) / CQ, j = luma ? i : (i - LQ) % CQ;
            const int rw = (luma ? LF_LW : LF_CW) / 4, r = j / rw, q = j % rw;
            const int x = (luma ? ox : cox) + 4 * q, y = (luma ? oy : coy) + r;
            const bool in = x >= 0 && y >= 0 && x < (luma ? P.W : P.CW) && y < (luma ? P.H : P.CH);
            R4 v{};
            if (in) v = __ldg((const R4 *)((luma ? wy : plane_ptr<T>(P.work, P, c)) + (size_t)y * (luma ? py : pc) + x));
            T *d = luma ? &S.y[r][4 * q] : &S.c[c - 1][r][4 * q];
            *(R4 *)d = v;
        }
    }
    __syncthreads();
    // 2. vertical edges: luma at x0 + 8e, every 4-row segment of the tile;
    // chroma at luma x0 + 16e, every 4-chroma-row segment
    {
        constexpr int LE = LF_TW / 8 + 1, LR = LF_LH / 4, CE = LF_TW / 16 + 1, CR = LF_CH / 4;
        for (int i = tid; i < LE * LR + CE * CR; i += LF_THREADS) {
            if (i < LE * LR) {
                const int bx = (x0 >> 2) + 2 * (i % LE), by = (oy >> 2) + i / LE;
                if (bx >= 2 && bx < P.w4 && by >= 0 && by < P.h4) deblock_segment<T, 0, TH>(P, S, bx, by, false, x0, y0);
            } else {
                const int k = i - LE * LR;
                const int bx = (x0 >> 2) + 4 * (k % CE), by = ((y0 - 2 * LF_HALO) >> 2) + 2 * (k / CE);
                if (bx >= 4 && bx < P.w4 && by >= 0 && by < P.h4) deblock_segment<T, 0, TH>(P, S, bx, by, true, x0, y0);
            }
        }
    }
    __syncthreads();
    // 3. horizontal edges: luma at y0 + 8e, every 4-column segment; chroma
    // at luma y0 + 16e, every 4-chroma-column segment
    {
        constexpr int LE = TH / 8 + 1, LR = LF_LW / 4, CE = TH / 16 + 1, CR = LF_CW / 4;
        for (int i = tid; i < LE * LR + CE * CR; i += LF_THREADS) {
            if (i < LE * LR) {
                const int by = (y0 >> 2) + 2 * (i / LR), bx = (ox >> 2) + i % LR;
                if (by >= 2 && by < P.h4 && bx >= 0 && bx < P.w4) deblock_segment<T, 1, TH>(P, S, bx, by, false, x0, y0);
            } else {
                const int k = i - LE * LR;
                const int by = (y0 >> 2) + 4 * (k / CR), bx = ((x0 - 2 * LF_HALO) >> 2) + 2 * (k % CR);
                if (by >= 4 && by < P.h4 && bx >= 0 && bx < P.w4) deblock_segment<T, 1, TH>(P, S, bx, by, true, x0, y0);
            }
        }
    }
    __syncthreads();
    // 4. SAO (filter.rs sao), four samples per thread, which share a CTB
    constexpr int LQ = TH * (LF_TW / 4), CQ = (TH / 2) * (LF_TW / 8);
    for (int i = tid; i < LQ + 2 * CQ; i += LF_THREADS) {
        const bool luma = i < LQ;
        const int c = luma ? 0 : 1 + (i - LQ) / CQ, j = luma ? i : (i - LQ) % CQ, sc = luma ? 0 : 1;
        const int rw = luma ? LF_TW / 4 : LF_TW / 8, tx = 4 * (j % rw), ty = j / rw;
        const int w = c ? P.CW : P.W, h = c ? P.CH : P.H;
        const int xq = (luma ? x0 : cx0) + tx, y = (luma ? y0 : cy0) + ty;
        if (xq >= w || y >= h) continue;
        // the tile's samples at tile position (sx, sy), halo included
        const T *tile = luma ? &S.y[0][0] : &S.c[c - 1][0][0];
        const int tw = luma ? LF_LW : LF_CW;
        auto at = [&](int sx, int sy) { return (int)tile[(sy + LF_HALO) * tw + sx + LF_HALO]; };
        int v[4], res[4];
#pragma unroll
        for (int k = 0; k < 4; k++) res[k] = v[k] = at(tx + k, ty);
        const int s = P.log2ctb - sc;
        const int rs = (y >> s) * P.wctb + (xq >> s);
        const rc_hevc_ctb &ct = P.ctbs[rs];
        const rc_hevc_slice *sl = slice_of_ctb(P, rs);
        const int type = ct.sao.type_idx[c];
        if ((c ? sl->sao_chroma : sl->sao_luma) && type != 0 && ct.slice < P.num_slices) {
            const int bd = P.bd, max = (1 << bd) - 1;
            if (type == 1) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int band = v[k] >> (bd - 5), e = (band - ct.sao.band_pos[c]) & 31;
                    if (e < 4) res[k] = clampi(v[k] + ct.sao.offsets[c][e], 0, max);
                }
            } else {
                const int cls = ct.sao.eo_class[c] & 3;
                const int hp0 = cls == 1 ? 0 : cls == 3 ? 1 : -1, hp1 = -hp0;
                const int vp0 = cls == 0 ? 0 : -1, vp1 = -vp0;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    bool good = true;
                    int nv[2];
#pragma unroll
                    for (int m = 0; m < 2; m++) {
                        const int xn = xq + k + (m ? hp1 : hp0), yn = y + (m ? vp1 : vp0);
                        good = good && xn >= 0 && yn >= 0 && xn < w && yn < h &&
                               cross_ok(P, rs, (yn >> s) * P.wctb + (xn >> s));
                        nv[m] = at(tx + k + (m ? hp1 : hp0), ty + (m ? vp1 : vp0));
                    }
                    if (!good) continue;
                    const int sum = (v[k] > nv[0]) - (v[k] < nv[0]) + (v[k] > nv[1]) - (v[k] < nv[1]);
                    // edge_map [1, 2, 0, 3, 4]: sum -2 -> offsets[0], -1 -> [1], 0 -> none, 1 -> [2], 2 -> [3]
                    const int e = sum == -2 ? 0 : sum == -1 ? 1 : sum == 1 ? 2 : sum == 2 ? 3 : -1;
                    if (e >= 0) res[k] = clampi(v[k] + ct.sao.offsets[c][e], 0, max);
                }
            }
        }
        // PCM with the loop filter off and transquant bypass keep the
        // deblocked sample (one 4x4 luma unit per luma sample, two per
        // group of four chroma samples)
        const rc_hevc_blk *brow = P.blk + (size_t)((y << sc) >> 2) * P.w4;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (brow[((xq + k) << sc) >> 2].flags & RC_HEVC_F_NOFILTER) res[k] = v[k];
        T *out = plane_ptr<T>(P.dpb + (size_t)P.out_slot * P.slot_bytes, P, c);
        Quad<T>::store(out + (size_t)y * pitch_el(P, c, sizeof(T)) + xq, res);
    }
}

}  // namespace

void rc_launch_hevc_residual(const HevcLaunch &p, cudaStream_t st) {
    cudaMemsetAsync(p.res, 0, ((size_t)p.W * p.H + 2 * (size_t)p.CW * p.CH) * sizeof(int16_t), st);
    // CTBs without transform blocks keep first = end = 0 and no intra blocks
    cudaMemsetAsync(p.ctb_first, 0, 2 * (size_t)p.wctb * p.hctb * sizeof(uint32_t), st);
    cudaMemsetAsync(p.ctb_nintra, 0, (size_t)p.wctb * p.hctb * sizeof(uint32_t), st);
    int blocks = (p.num_tus + 3) / 4;
    blocks = blocks < 1 ? 1 : blocks > 4096 ? 4096 : blocks;
    hevc_residual_kernel<<<blocks, 128, 0, st>>>(p);
}

void rc_launch_hevc_inter(const HevcLaunch &p, cudaStream_t st) {
    if (p.inter_pass == 2) {
        // one item per thread for lists up to a quarter of the groups (the
        // kernel strides over longer ones)
        const int grid = std::max<int>(152, (int)((p.late_cap / 4 + 255) / 256));
        if (p.bd > 8) hevc_inter_late_kernel<uint16_t><<<grid, 256, 0, st>>>(p);
        else hevc_inter_late_kernel<uint8_t><<<grid, 256, 0, st>>>(p);
        return;
    }
    if (p.inter_pass == 1) cudaMemsetAsync(p.late_count, 0, sizeof(uint32_t), st);
    dim3 grid((p.W + 15) / 16, (p.H + 15) / 16);
    if (p.bd > 8) hevc_inter_kernel<uint16_t><<<grid, 64, 0, st>>>(p);
    else hevc_inter_kernel<uint8_t><<<grid, 64, 0, st>>>(p);
}

void rc_launch_hevc_intra(const HevcLaunch &p, cudaStream_t st, int blocks, bool order) {
    const int nctb = p.wctb * p.hctb;
    if (order) hevc_ctb_order_kernel<<<(nctb + 255) / 256, 256, 0, st>>>(p);
    blocks = blocks < 1 ? 1 : blocks > nctb ? nctb : blocks;
    const size_t dyn = INTRA_WARPS * sizeof(IntraSmem);
    static bool attr_set = false;  // per process; the attribute is per kernel
    if (!attr_set) {
        cudaFuncSetAttribute(hevc_intra_kernel<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        cudaFuncSetAttribute(hevc_intra_kernel<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        attr_set = true;
    }
    if (p.bd > 8) hevc_intra_kernel<uint16_t><<<blocks, 32 * INTRA_WARPS, dyn, st>>>(p);
    else hevc_intra_kernel<uint8_t><<<blocks, 32 * INTRA_WARPS, dyn, st>>>(p);
}

template <int TH>
static void launch_loopfilter(const HevcLaunch &p, cudaStream_t st) {
    dim3 grid((p.W + LF_TW - 1) / LF_TW, (p.H + TH - 1) / TH);
    if (p.bd > 8) hevc_loopfilter_kernel<uint16_t, TH><<<grid, LF_THREADS, 0, st>>>(p);
    else hevc_loopfilter_kernel<uint8_t, TH><<<grid, LF_THREADS, 0, st>>>(p);
}
void rc_launch_hevc_loopfilter(const HevcLaunch &p, cudaStream_t st) {
    if (p.lf_rows == 16) launch_loopfilter<16>(p, st);
    else if (p.lf_rows == 32) launch_loopfilter<32>(p, st);
    else launch_loopfilter<64>(p, st);
}
