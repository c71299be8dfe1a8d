/*
 * oracle.h — CPU restatement of pito-codecs' block reconstruction.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it, as the checker.  Each function follows the reference's
 * scalar implementation (cited file:line, paths inside the pito-codecs
 * crate), driven by the same syntax records the GPU consumes
 * (include/pito_recon.h).
 *
 * Planes are tightly packed at the coded size, as the reference stores them:
 * luma stride = mb_w * 16, chroma stride = mb_w * 8 (H.264).
 */
#ifndef PITO_ORACLE_H
#define PITO_ORACLE_H

#include <stdint.h>
#include "../include/pito_recon.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Reconstruct one H.264 picture (pre-deblock recon of every MB in raster
 * order, then deblock_mb in raster order).  ref_*[slot] are the DPB planes
 * indexed by rc_h264_slice.ref_slot.  Returns 0 or RC_EINVAL. */
int oracle_h264_recon(int mb_w, int mb_h, const rc_h264_picture *pic,
                      const uint8_t *const *ref_y, const uint8_t *const *ref_u,
                      const uint8_t *const *ref_v, uint8_t *y, uint8_t *u,
                      uint8_t *v);

/* Same, but skipping the loop filter (for kernel-level tests). */
int oracle_h264_recon_nofilter(int mb_w, int mb_h, const rc_h264_picture *pic,
                               const uint8_t *const *ref_y,
                               const uint8_t *const *ref_u,
                               const uint8_t *const *ref_v, uint8_t *y,
                               uint8_t *u, uint8_t *v);

/* Co-located motion of one MB, as Frame::publish stores it
 * (src/h264/dec/picture.rs:492): no motion for intra, I_PCM and undecoded
 * MBs; else each 8x8 block's ref_idx and referenced picture identity and
 * each 4x4 block's vectors, per list. */
typedef struct {
    uint8_t intra;
    uint8_t pad[3];
    int8_t ref_idx[2][4];
    uint32_t ref_id[2][4];
    int16_t mv[2][16][2];
} oracle_h264_colmb;        /* 172 bytes */

/* Derive every inter MB's mv, ref_idx and wp from pic->motion and
 * pic->slice_motion (h264_motion.c) into `mbs`, a copy of pic->mbs that the
 * caller owns, reading co-located motion from col[slot] (NULL: the slot
 * holds none), and write the picture's co-located motion into out_col
 * (mb_w * mb_h entries).  Returns 0 or RC_EINVAL. */
int oracle_h264_derive_motion(int mb_w, int mb_h, const rc_h264_picture *pic,
                              const oracle_h264_colmb *const *col, int slots,
                              rc_h264_mb *mbs, oracle_h264_colmb *out_col);

/* oracle_h264_recon (filter != 0) or _nofilter, after deriving the motion
 * when pic->motion is set; out_col receives the picture's co-located motion
 * either way. */
int oracle_h264_recon_motion(int mb_w, int mb_h, const rc_h264_picture *pic,
                             const oracle_h264_colmb *const *col, int slots,
                             oracle_h264_colmb *out_col,
                             const uint8_t *const *ref_y,
                             const uint8_t *const *ref_u,
                             const uint8_t *const *ref_v, uint8_t *y,
                             uint8_t *u, uint8_t *v, int filter);

/* Deblock an already reconstructed picture in place. */
void oracle_h264_deblock(int mb_w, int mb_h, const rc_h264_picture *pic,
                         uint8_t *y, uint8_t *u, uint8_t *v);

/* Block-level entry points used by the known-answer tests. */
void oracle_h264_idct4_add(const int32_t d[16], uint8_t *dst, int stride);
void oracle_h264_idct8_add(const int32_t d[64], uint8_t *dst, int stride);
void oracle_h264_luma_dc_dequant(int32_t c[16], int qp, int32_t ls00);
void oracle_h264_chroma_dc_dequant(int32_t c[4], int qp, int32_t ls00);
void oracle_h264_level_scale(const uint8_t *m4, const uint8_t *m8,
                             int32_t ls4[6][6][16], int32_t ls8[6][6][64]);
void oracle_h264_mc_luma(const uint8_t *plane, int width, int height, int px,
                         int py, int mvx, int mvy, int bw, int bh,
                         uint8_t *out, int os);
void oracle_h264_mc_chroma(const uint8_t *plane, int cwidth, int cheight,
                           int cpx, int cpy, int mvx, int mvy, int bw, int bh,
                           uint8_t *out, int os);

/* Reconstruct one HEVC picture of width x height luma samples at
 * bit_depth 8 or 10.  Planes are uint16_t at every bit depth, tightly
 * packed.  stages: bit 0 deblocking, bit 1 SAO (3 = the full path).
 * Returns 0 or RC_EINVAL. */
int oracle_hevc_recon(int width, int height, int bit_depth, const rc_hevc_picture *pic,
                      const uint16_t *const *ref_y, const uint16_t *const *ref_u,
                      const uint16_t *const *ref_v, uint16_t *y, uint16_t *u, uint16_t *v,
                      int stages);
void oracle_hevc_inverse(int16_t *co, int log2, int dst, int max_x, int max_y, int bd_shift);
int oracle_hevc_inverse_dc(int dc, int bd_shift);
void oracle_hevc_intra_predict_refs(const uint16_t *left, const uint16_t *top, int mode, int log2,
                                    int is_luma, int strong, int bd, int *out);

#ifdef __cplusplus
}
#endif

#endif
