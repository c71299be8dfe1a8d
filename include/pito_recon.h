/*
 * pito_recon.h — C ABI of the GB300 block-reconstruction engine.
 *
 * The engine replaces the reconstruction half of pito-codecs' H.264 and HEVC
 * slice decoders.  In the reference, reconstruction is interleaved with the
 * entropy parse, one macroblock / transform unit at a time:
 *
 *   H.264  reconstruct_intra / predict_inter + reconstruct_inter_residual
 *          (src/h264/dec/slicedec.rs:1743-1749, src/h264/dec/cabac_mb.rs:712-717),
 *          then the row-lagged loop filter flush_rows -> deblock_mb
 *          (src/h264/dec/slicedec.rs:184-208).
 *   HEVC   intra_predict / reconstruct / motion_compensate
 *          (src/hevc/slicedec.rs:1642-1669, 2169), then filter::ctb_decoded /
 *          finish (src/hevc/filter.rs:13-72).
 *
 * Here the host parse fills syntax records for a whole picture and one call
 * reconstructs it on the GPU against a decoded-picture buffer (DPB) that stays
 * resident in device memory.  Every call is asynchronous on the stream's CUDA
 * stream; the syntax buffers must stay valid until rc_stream_sync returns (or
 * until the stream's next submit when they are host buffers, which are staged
 * through pinned memory before the call returns).
 *
 * All functions return 0 on success and a negative RC_E* code on failure.
 */
#ifndef PITO_RECON_H
#define PITO_RECON_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ------------------------------------------------------- */
#define RC_OK 0
#define RC_EINVAL (-1)       /* bad argument or syntax record rejected on the host */
#define RC_ENOMEM (-2)       /* device or pinned allocation failed / over budget   */
#define RC_ECUDA (-3)        /* a CUDA runtime call failed                         */
#define RC_ETIMEOUT (-4)     /* a device wavefront wait gave up (sticky)           */
#define RC_EDEVICE (-5)      /* the device reported a bad record (sticky)          */
#define RC_ENODEV (-6)       /* no CUDA device / kernels not loadable              */

/* ---- codecs ------------------------------------------------------------ */
#define RC_CODEC_H264 1
#define RC_CODEC_HEVC 2

/* where a submitted syntax buffer lives */
#define RC_MEM_HOST 0
#define RC_MEM_DEVICE 1

typedef struct rc_stream rc_stream;

/* ======================================================================== */
/*  H.264 syntax records                                                     */
/* ======================================================================== */

/* rc_h264_mb.kind — the MbKind values of src/h264/dec/picture.rs:42-53
 * folded to what reconstruction distinguishes (P_Skip, B_Skip, B_Direct and
 * ordinary inter macroblocks are all RC_H264_INTER). */
#define RC_H264_NONE 0 /* not decoded (missing slice): unusable neighbour */
#define RC_H264_I4x4 1
#define RC_H264_I8x8 2
#define RC_H264_I16x16 3
#define RC_H264_IPCM 4
#define RC_H264_INTER 5

/*
 * One macroblock.  Mirrors the reconstruction fields of MbState
 * (src/h264/dec/picture.rs:66-84) plus the coefficient levels that the parse
 * hands to put_luma4/put_luma8/put_luma_dc/put_chroma_dc/put_chroma_ac
 * (src/h264/dec/slicedec.rs:1462-1555), which the device dequantises.
 *
 * Level payload at levels[coef_off...] (int16, scan order as parsed):
 *   (dc_coded & 1)  16 levels  Intra16x16 luma DC, 4x4 zig-zag scan
 *   luma blocks     for each set bit of luma_coded, ascending:
 *                   transform_8x8 ? 64 levels (8x8 zig-zag, bit = 8x8 index)
 *                                 : 16 levels (4x4 zig-zag, bit = 4x4 raster
 *                                   index; level 0 ignored for Intra16x16)
 *   (dc_coded & 2)  4 levels Cb DC;  (dc_coded & 4)  4 levels Cr DC
 *   chroma AC       for each set bit of chroma_coded (0-3 Cb, 4-7 Cr):
 *                   16 levels, level 0 ignored
 *   kind == IPCM    384 samples instead: 256 Y, 64 Cb, 64 Cr (raster)
 *
 * mv[l][k] is the motion vector (quarter-pel) that motion-compensates 4x4
 * block k (raster) from list l; ref_idx is per 8x8 block.  Partition shapes
 * are not needed: every sample's prediction depends only on its block's
 * vector, reference and weights.
 */
typedef struct rc_h264_mb {
    uint8_t kind;          /* RC_H264_* */
    uint8_t transform_8x8; /* 0/1 */
    uint8_t qp;            /* luma QP 0..51 (0 for I_PCM)                     */
    uint8_t qpc[2];        /* chroma QP per component after the QPC table     */
    uint8_t i16_mode;      /* Intra16x16 prediction mode 0..3                 */
    uint8_t chroma_mode;   /* intra chroma prediction mode 0..3               */
    uint8_t dc_coded;      /* bit0 luma DC, bit1 Cb DC, bit2 Cr DC            */
    uint16_t slice;        /* index into rc_h264_picture.slices               */
    uint16_t nz_mask;      /* 4x4 blocks (raster) with non-zero coefficients  */
    uint16_t luma_coded;   /* blocks with a level payload (see above)         */
    uint8_t chroma_coded;  /* chroma AC blocks with a level payload           */
    uint8_t reserved0;
    uint32_t coef_off;     /* offset of this MB's payload, in int16 units     */
    uint8_t intra_modes[16]; /* Intra4x4/8x8 modes per 4x4 block (raster)     */
    int8_t ref_idx[2][4];  /* per 8x8 block and list, -1 = list unused        */
    uint8_t wp[4];         /* weight-table entry per 8x8 block, 0xff = default */
    int16_t mv[2][16][2];  /* per 4x4 block and list, quarter-pel (x, y)      */
} rc_h264_mb;              /* 176 bytes */

/* Per-slice state the loop filter and motion compensation read
 * (SliceInfo, src/h264/dec/slicedec.rs:116-121; ref lists of SliceDecoder). */
#define RC_H264_MAX_REFS 32
typedef struct rc_h264_slice {
    int32_t disable_deblocking_filter_idc; /* 0, 1 or 2                        */
    int32_t alpha_offset;  /* slice_alpha_c0_offset_div2 * 2                   */
    int32_t beta_offset;   /* slice_beta_offset_div2 * 2                       */
    int32_t num_ref[2];    /* active references per list                      */
    int32_t ref_slot[2][RC_H264_MAX_REFS]; /* DPB slot of each reference       */
    uint32_t ref_id[2][RC_H264_MAX_REFS];  /* picture identity (RefPic::id)    */
} rc_h264_slice;

/* One resolved weighting (Weight after Weight::simplify,
 * src/h264/dec/inter.rs:249-282) for Y, Cb, Cr.  Bit c of `explicit` set:
 * component c uses the weighted formula, else the default copy / average. */
typedef struct rc_h264_weight {
    uint8_t explicit_mask;
    uint8_t reserved[3];
    int32_t log_wd[3];
    int32_t w0[3], w1[3], o0[3], o1[3];
} rc_h264_weight;          /* 64 bytes */

/* Motion syntax of one MB, for motion derived on the GPU (no counterpart in
 * the reference, whose slice decoder derives each MB's vectors as it parses
 * it: mvp / median_pred / derive_p_skip / derive_direct,
 * src/h264/dec/slicedec.rs:581-935).  The parse only needs the parsed
 * syntax -- CABAC and CAVLC contexts read neighbouring mvd and ref_idx, never
 * derived vectors -- so a decoder can hand it over and let the engine derive
 * every vector: motion vector prediction plus mvd (8.4.1.3), P_Skip
 * (8.4.1.1), B direct spatial and temporal (8.4.1.2) from the co-located
 * picture's stored motion, and each 8x8 block's weight entry.  `shape`:
 * RC_H264_MOTION_*.  `pred`: prediction lists (bit 0 list 0, bit 1 list 1)
 * of partition i (16x16: 0; 16x8, 8x16: 0..1; 8x8: the four 8x8 blocks).
 * `sub` (8x8 only): sub-partition of each 8x8 block, RC_H264_SUB_*.
 * `ref_idx`: the parsed ref_idx of the partition covering each 8x8 block.
 * `mvd`: per 4x4 block (raster) and list, the mvd of the (sub-)partition
 * covering it. */
#define RC_H264_MOTION_NONE 0  /* intra, I_PCM or not decoded: no motion     */
#define RC_H264_MOTION_SKIP 1  /* P_Skip (P slice); B_Skip, B_Direct_16x16 (B) */
#define RC_H264_MOTION_16x16 2
#define RC_H264_MOTION_16x8 3
#define RC_H264_MOTION_8x16 4
#define RC_H264_MOTION_8x8 5
#define RC_H264_SUB_8x8 0
#define RC_H264_SUB_8x4 1
#define RC_H264_SUB_4x8 2
#define RC_H264_SUB_4x4 3
#define RC_H264_SUB_DIRECT 4   /* B_Direct_8x8 */
typedef struct rc_h264_motion {
    uint8_t shape;
    uint8_t pred[4];
    uint8_t sub[4];
    uint8_t reserved[3];
    int8_t ref_idx[2][4];
    int16_t mvd[2][16][2];
} rc_h264_motion;           /* 148 bytes */

/* Per slice, for motion derived on the GPU: what the reference's slice
 * decoder keeps for direct prediction and weighting (SliceDecoder::new,
 * slicedec.rs:360-406: tdirect; build_weights).  `col_slot`: the DPB slot of
 * RefPicList1[0] (B slices), which must hold a picture submitted with motion
 * syntax.  `dist_scale` / `direct_copy` per refIdxL0: temporal direct's
 * DistScaleFactor, or 1 where mvL0 = mvCol and mvL1 = 0 (long-term
 * reference or equal POC distances).  `wp_map[(r0 + 1) * 33 + (r1 + 1)]`:
 * the weight-table entry for refIdxL0 = r0 and refIdxL1 = r1 (-1: list
 * unused), 0xff for the default average. */
typedef struct rc_h264_slice_motion {
    int32_t b_slice;
    int32_t direct_spatial;        /* direct_spatial_mv_pred_flag             */
    int32_t direct_8x8_inference;  /* SPS direct_8x8_inference_flag           */
    int32_t col_slot;
    int32_t col_short_term;        /* RefPicList1[0] is a short-term reference */
    int16_t dist_scale[RC_H264_MAX_REFS];
    uint8_t direct_copy[RC_H264_MAX_REFS];
    uint8_t wp_map[(RC_H264_MAX_REFS + 1) * (RC_H264_MAX_REFS + 1)];
    uint8_t reserved[3];
} rc_h264_slice_motion;     /* 1208 bytes */

typedef struct rc_h264_picture {
    int32_t mem;                      /* RC_MEM_HOST or RC_MEM_DEVICE          */
    int32_t constrained_intra_pred;   /* PPS flag                              */
    uint32_t frame_id;                /* identity of this picture              */
    int32_t num_slices;
    int32_t num_weights;
    int32_t reserved;
    size_t num_levels;                /* int16 entries in levels               */
    const rc_h264_mb *mbs;            /* mb_w * mb_h records, raster order     */
    const rc_h264_slice *slices;
    const rc_h264_weight *weights;
    const int16_t *levels;
    /* Scaling matrices of the PPS (ScalingMatrices m4[6][16], m8[6][64]);
     * NULL = flat 16.  Always host memory. */
    const uint8_t *scaling4;          /* [6][16] */
    const uint8_t *scaling8;          /* [6][64] */
    /* Optional (host memory, with mem == RC_MEM_HOST): motion syntax per MB
     * and per slice.  When set, the engine derives every inter MB's mv,
     * ref_idx and wp on the GPU and ignores those fields of `mbs`; it also
     * stores the picture's motion in its DPB slot, for later pictures that
     * use it as their co-located picture. */
    const rc_h264_motion *motion;
    const rc_h264_slice_motion *slice_motion;
} rc_h264_picture;

/* ======================================================================== */
/*  HEVC syntax records                                                      */
/* ======================================================================== */

/* rc_hevc_blk.flags / .edges — the Blk flags of src/hevc/slicedec.rs:19-28 */
#define RC_HEVC_F_INTRA 1     /* the CU is intra                              */
#define RC_HEVC_F_SKIP 2      /* skipped CU                                   */
#define RC_HEVC_F_NOFILTER 4  /* PCM with loop filter off, or transquant bypass */
#define RC_HEVC_F_CBF 8       /* the luma TU covering it has coefficients     */
#define RC_HEVC_F_CODED 16    /* decoded                                      */
#define RC_HEVC_E_TU_V 1      /* transform-unit edge on the block's left      */
#define RC_HEVC_E_PU_V 2      /* prediction-unit edge on the left             */
#define RC_HEVC_E_TU_H 4      /* transform-unit edge on top                   */
#define RC_HEVC_E_PU_H 8      /* prediction-unit edge on top                  */

/* Per 4x4 luma block (Blk, src/hevc/slicedec.rs:30-37, without the CABAC
 * depth): what the loop filters and intra availability read. */
typedef struct rc_hevc_blk {
    uint8_t flags;  /* RC_HEVC_F_* */
    uint8_t edges;  /* RC_HEVC_E_* */
    int8_t qp;      /* QpY of the CU (loop-filter QP)                       */
    uint8_t ipm;    /* luma intra mode (informational)                      */
} rc_hevc_blk;      /* 4 bytes */

/* Per 4x4 luma block motion (MvField, src/hevc/slicedec.rs:40-44):
 * quarter-pel luma vectors, ref_idx -1 = list unused. */
typedef struct rc_hevc_mvf {
    int16_t mv[2][2];
    int8_t ref_idx[2];
    uint16_t reserved;
} rc_hevc_mvf;      /* 12 bytes */

/* SAO parameters of one CTB (SaoParams, src/hevc/slicedec.rs:62-67):
 * type 0 off, 1 band, 2 edge; offsets already signed and scaled. */
typedef struct rc_hevc_sao {
    uint8_t type_idx[3];
    uint8_t band_pos[3];
    uint8_t eo_class[3];
    uint8_t reserved;
    int16_t offsets[3][4];
} rc_hevc_sao;      /* 34 bytes */

/* One CTB, raster order: its slice (index into the slice table), tile and
 * tile-scan position (Layout::rs_to_ts / tile_id), and SAO parameters. */
typedef struct rc_hevc_ctb {
    uint16_t slice;
    uint16_t tile;
    uint32_t ts;
    rc_hevc_sao sao;
    uint16_t reserved;
} rc_hevc_ctb;      /* 44 bytes */

/* rc_hevc_tu.flags */
#define RC_HEVC_TU_INTRA 1    /* intra CU: predict (mode) before the residual */
#define RC_HEVC_TU_CBF 2      /* coefficient levels present                   */
#define RC_HEVC_TU_SKIP 4     /* transform_skip_flag                          */
#define RC_HEVC_TU_BYPASS 8   /* cu_transquant_bypass: levels are the residual */
#define RC_HEVC_TU_PCM 16     /* PCM: n x n samples instead of levels         */

/*
 * One transform block of one colour component, in decode order (the order
 * transform_unit visits them, src/hevc/slicedec.rs:1602-1671: luma, then Cb
 * and Cr of the same TU or, for 4x4 luma blocks, after the fourth one).
 * Levels at levels[coef_off...]: (max_y+1) x (max_x+1) int16, row-major, the
 * parsed coefficients before dequantisation (reconstruct,
 * src/hevc/slicedec.rs:2004-2049).  Inter CUs are predicted from the
 * rc_hevc_mvf grid; their TUs carry only residual.
 */
typedef struct rc_hevc_tu {
    uint16_t x0, y0;  /* top-left in the component's own sample grid        */
    uint8_t log2;     /* 2..5                                               */
    uint8_t c;        /* 0 Y, 1 Cb, 2 Cr                                    */
    uint8_t flags;    /* RC_HEVC_TU_*                                       */
    uint8_t mode;     /* intra mode 0..34 (chroma: after the mode-34 rule)  */
    int8_t qp;        /* dequantisation QP: luma qp_y + 6(bd-8); chroma qp_cb/qp_cr */
    uint8_t max_x, max_y; /* last significant column / row                  */
    uint8_t reserved;
    uint32_t coef_off;
} rc_hevc_tu;         /* 16 bytes */

#define RC_HEVC_MAX_REFS 16
/* Per-slice state (SliceInfo, src/hevc/slicedec.rs:69-80) plus the
 * reference lists and the explicit weighted-prediction table the motion
 * compensation uses (motion_compensate, src/hevc/slicedec.rs:2205-2280). */
typedef struct rc_hevc_slice {
    uint32_t slice_addr;      /* SliceAddrRs: slices compare by this          */
    int32_t deblock_disabled;
    int32_t beta_offset;      /* slice_beta_offset_div2 * 2                   */
    int32_t tc_offset;        /* slice_tc_offset_div2 * 2                     */
    int32_t lf_across;        /* slice_loop_filter_across_slices_enabled_flag */
    int32_t sao_luma, sao_chroma;
    int32_t weighted;         /* explicit weighted prediction in this slice   */
    int32_t luma_log2_denom, chroma_log2_denom;
    int32_t num_ref[2];
    int32_t ref_slot[2][RC_HEVC_MAX_REFS];
    uint32_t ref_id[2][RC_HEVC_MAX_REFS]; /* picture identity for the bS test */
    int16_t luma_w[2][RC_HEVC_MAX_REFS], luma_o[2][RC_HEVC_MAX_REFS];
    int16_t chroma_w[2][RC_HEVC_MAX_REFS][2], chroma_o[2][RC_HEVC_MAX_REFS][2];
} rc_hevc_slice;

typedef struct rc_hevc_picture {
    int32_t mem;                   /* RC_MEM_HOST or RC_MEM_DEVICE            */
    int32_t log2_ctb;              /* 4..6                                    */
    int32_t constrained_intra_pred;
    int32_t strong_intra_smoothing;
    int32_t loop_filter_across_tiles;
    int32_t cb_qp_offset, cr_qp_offset; /* PPS offsets (loop-filter chroma QP) */
    int32_t num_slices;
    int32_t num_tus;
    uint32_t frame_id;
    size_t num_levels;
    const rc_hevc_ctb *ctbs;       /* ceil(w/ctb) * ceil(h/ctb), raster       */
    const rc_hevc_blk *blk;        /* (w/4) * (h/4), raster                   */
    const rc_hevc_mvf *mvf;        /* (w/4) * (h/4), raster                   */
    const rc_hevc_tu *tus;         /* decode order                            */
    const rc_hevc_slice *slices;
    const int16_t *levels;
    /* Expanded scaling factors (the Scaling tables, src/hevc/slicedec.rs:17):
     * for size_id 0..3 (4..32) and matrix_id 0..5 (intra Y Cb Cr, inter Y Cb
     * Cr), n*n bytes each, size_id-major; NULL = flat 16.  Host memory. */
    const uint8_t *scaling;        /* 6*(16+64+256+1024) bytes                */
} rc_hevc_picture;

/* ======================================================================== */
/*  Stream / DPB lifetime                                                    */
/* ======================================================================== */

/* Make `device` the CUDA device that streams created afterwards on this
 * thread use (the library keeps its own CUDA runtime state). */
int rc_device_select(int device);

/*
 * Create a reconstruction stream: device DPB of `dpb_slots` pictures of the
 * coded size (width, height rounded up to the codec's block grid), a CUDA
 * stream and the scratch the kernels use.  `hbm_budget` bounds the device
 * bytes the stream may hold (0 = unbounded); RC_ENOMEM if it would exceed it.
 * Replaces Decoder::with_threads (src/h264/mod.rs:38, src/hevc/decoder.rs:87)
 * and the decoder-owned frame pool (src/h264/dec/picture.rs:196).
 * `codec` may carry RC_STREAM_SHARED_GPU: the stream shares the GPU with
 * many others (the batched and served forms).  A stream without it (one
 * decoder on the GPU) dispatches its HEVC kernels' CTAs ahead of its side
 * stream's (1080p: 2410 -> 2500 frames/s); among many streams that
 * preference slows the mix (64 streams: 5486 -> 5331 frames/s), so shared
 * streams keep the default priority.
 */
#define RC_STREAM_SHARED_GPU 0x100
int rc_stream_create(int codec, int width, int height, int bit_depth,
                     int dpb_slots, size_t hbm_budget, rc_stream **out);

/* Release everything the stream owns (Drop of the reference Decoder). */
void rc_stream_destroy(rc_stream *s);

/* Reconstruct one H.264 picture into DPB slot `out_slot`: inter prediction
 * with residual, intra prediction with residual, then the deblocking filter.
 * Records are validated on the host first (slice index, ref_idx < num_ref,
 * DPB slots, payload bounds) and rejected with RC_EINVAL before any launch,
 * as slicedec.rs:888-892 and 1442-1446 reject bad syntax. */
int rc_h264_submit(rc_stream *s, const rc_h264_picture *pic, int out_slot);

/* Host-side validation rc_h264_submit applies to host-memory records, for a
 * stream of mb_w x mb_h macroblocks and dpb_slots DPB slots; needs no GPU.
 * Returns 0 or RC_EINVAL. */
int rc_h264_validate(int mb_w, int mb_h, int dpb_slots, const rc_h264_picture *pic);

/* Reconstruct one HEVC picture into DPB slot `out_slot`: residual for every
 * TU, inter prediction, intra prediction in decode order, deblocking (all
 * vertical edges, then all horizontal edges) and SAO.  Host-side validation
 * as for H.264 (src/hevc/slicedec.rs:2153-2160 rejects bad ref_idx).
 * Planes of >8-bit streams are uint16 samples. */
int rc_hevc_submit(rc_stream *s, const rc_hevc_picture *pic, int out_slot);

/* Host-side validation of an HEVC picture for a stream of the given luma
 * size and DPB slots; needs no GPU.  Returns 0 or RC_EINVAL. */
int rc_hevc_validate(int width, int height, int bit_depth, int dpb_slots,
                     const rc_hevc_picture *pic);

/* Wait for all submitted work; returns the sticky error word (0 if none). */
int rc_stream_sync(rc_stream *s);

/* Sticky device/host error (RC_ETIMEOUT, RC_EDEVICE, ...) or 0; clears it.
 * Replaces Decoder::take_error (src/h264/dec/decoder.rs:222). */
int rc_stream_error(rc_stream *s);

/* Copy a DPB picture into caller memory, cropped to (x, y, w, h) in luma
 * samples (chroma: x/2, y/2, ceil(w/2), ceil(h/2)); planes tightly packed,
 * 8-bit samples as bytes, >8-bit as little-endian uint16.  Synchronous.
 * Replaces Frame::copy_cropped (src/h264/dec/picture.rs:596-642) and
 * hevc Frame::copy_cropped (src/hevc/picture.rs:374). */
int rc_picture_download(rc_stream *s, int slot, int x, int y, int w, int h,
                        void *out_y, void *out_u, void *out_v);

/* Asynchronous form of rc_picture_download, ordered on the stream's CUDA
 * stream after all submitted work; outputs must be pinned host memory (or
 * device memory) and are valid after rc_stream_sync. */
int rc_picture_download_async(rc_stream *s, int slot, int x, int y, int w,
                              int h, void *out_y, void *out_u, void *out_v);

/* Fill a DPB slot from caller planes of the full coded size (tightly packed),
 * e.g. to seed references.  Synchronous.  Counterpart of Frame::fill
 * (src/h264/dec/picture.rs:508-519). */
int rc_picture_upload(rc_stream *s, int slot, const void *y, const void *u,
                      const void *v);

/* Geometry of the stream's DPB planes: coded width/height in luma samples,
 * row pitch of the luma and chroma planes in bytes, and device pointers of
 * one slot's planes (for zero-copy consumers). */
int rc_stream_geometry(rc_stream *s, int *coded_w, int *coded_h,
                       int *luma_pitch, int *chroma_pitch);
int rc_picture_device_planes(rc_stream *s, int slot, void **y, void **u,
                             void **v);

/* Per-kernel timing with CUDA events on the stream (off by default).
 * rc_stream_profile_read syncs, then returns for each kernel id
 * (RC_KERNEL_*) the accumulated milliseconds and launch counts since
 * profiling was enabled; returns the number of kernel ids filled. */
#define RC_KERNEL_H264_MB 0
#define RC_KERNEL_H264_BAND 1
#define RC_KERNEL_H264_EDGE 2
#define RC_KERNEL_HEVC_RESIDUAL 3
#define RC_KERNEL_HEVC_INTER 4      /* inter units whose references are final
                                      (beside the previous picture)      */
#define RC_KERNEL_HEVC_INTRA 5
#define RC_KERNEL_HEVC_LOOPFILTER 6 /* deblocking and SAO, one launch     */
#define RC_KERNEL_HEVC_INTER_LATE 7 /* inter units reading the previous
                                      picture (after it)                 */
#define RC_KERNEL_H264_GROUP 8
#define RC_KERNEL_H264_MV 9
#define RC_KERNEL_COUNT 10
int rc_stream_profile(rc_stream *s, int enable);
/* Schedule knob for many streams sharing one GPU: the HEVC intra kernel's
 * persistent CTAs per launch (default: about one per two 64x64 CTBs, at
 * least 8, at most two per SM).  ctas <= 0 restores the default; more than
 * 4096 is RC_EINVAL.  Takes effect from the next submit.  The arithmetic,
 * and so the output, does not depend on it. */
int rc_stream_set_intra_ctas(rc_stream *s, int ctas);
/* The current value (0 for an H.264 stream, which has no such kernel). */
int rc_stream_intra_ctas(rc_stream *s);
/* Schedule knob (tile shape): the HEVC loop filter's tile height in luma
 * rows, 64 (default), 32 or 16; tiles are 64 samples wide.  Anything else,
 * or an H.264 stream, is RC_EINVAL.  Takes effect from the next submit; the
 * output does not depend on it.  rc_stream_lf_tile returns the height (0
 * for an H.264 stream). */
int rc_stream_set_lf_tile(rc_stream *s, int rows);
int rc_stream_lf_tile(rc_stream *s);
/* Iteration cap of every device-side wait in this stream's kernels (no
 * counterpart in the reference, whose rayon jobs block on condition
 * variables).  A wait that polls `limit` times without progress records
 * RC_ETIMEOUT in the sticky error word and its launch unwinds, leaving the
 * context usable.  For tests of that failure path and for callers that want
 * a shorter bound; 0 restores the default (about a second of polling).
 * Takes effect from the next submit. */
int rc_stream_set_wait_limit(rc_stream *s, unsigned int limit);
/* H.264 only: reconstruct up to `pictures` consecutive pictures in one
 * launch (no counterpart in the reference, which decodes one picture at a
 * time per thread and overlaps pictures only across its worker threads).
 * The launch runs every picture's intra + loop-filter wavefront side by side
 * with the MB phase of all of them, each inter MB waiting only for the rows
 * of the pictures in the launch that its motion vectors reach; the output is
 * the same as one launch per picture.  rc_h264_submit then queues a picture
 * and launches when the group is full, when the next picture writes a DPB
 * slot that a queued picture writes or reads, when the scaling lists change,
 * before a picture whose records are in device memory, and in every call
 * that waits for or orders after the submitted work (rc_stream_sync,
 * rc_stream_error, rc_picture_download*, rc_picture_upload,
 * rc_picture_device_planes, rc_stream_mark, rc_stream_cuda_stream,
 * rc_stream_profile*).  1 launches each picture at its submit (the default);
 * 0 picks the library's default group; at most 4.  The group is lowered
 * until the pictures' band CTAs fit in two thirds of one launch.  Returns
 * the pictures per launch now in effect, or RC_EINVAL (HEVC stream, out of
 * range) / RC_ENOMEM (the per-picture scratch: about 1.2 KB per MB). */
int rc_stream_set_h264_group(rc_stream *s, int pictures);
int rc_stream_profile_read(rc_stream *s, double *ms, long long *launches,
                           int max_kernels);

/* Allocation-free H.264 deblocking (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory once they are running:
 * processes whose device memory is carved up by their own allocator at
 * start-up, real-time pipelines that must not stall in cudaMalloc, or code
 * issuing work while a stream is being captured.  It runs the same loop
 * filter rc_h264_submit applies, in place on caller planes (device memory:
 * the picture's coded size, luma 16-byte aligned with a pitch multiple of
 * 16, chroma 8-byte aligned with a pitch multiple of 8), from the picture's
 * syntax records in device memory (pic->mem == RC_MEM_DEVICE).  It allocates
 * nothing: its scratch is a static device array the library holds on every
 * device that loads it, sized for RC_NOALLOC_MAX_MBS macroblocks (8704:
 * up to 2048x1088) and RC_NOALLOC_MAX_ROWS MB rows; larger pictures get
 * RC_EINVAL.  The first call on a device looks up that array's device
 * address in the current CUDA context, so make the first call before any
 * stream capture.  A device reset (cudaDeviceReset) or a new context moves
 * the array; the first call in the new context looks it up again, and it too
 * belongs before any capture.  Every call
 * shares the one array: calls whose work overlaps on the GPU (on different
 * streams, or on different host threads) race and must be serialised by the
 * caller.  *status (device memory, 4 bytes) receives 0 or RC_DEV_* error bits
 * (1 a wait timed out, 2 a record pointed outside its buffers) once the
 * queued work completes on cuda_stream (a cudaStream_t; NULL = the default
 * stream). */
#define RC_NOALLOC_MAX_MBS 8704
#define RC_NOALLOC_MAX_ROWS 128
int rc_h264_deblock_noalloc(const rc_h264_picture *pic, int mb_w, int mb_h,
                            void *y, void *u, void *v, int luma_pitch,
                            int chroma_pitch, uint32_t *status,
                            void *cuda_stream);

/* Number of kernel launches this stream has issued so far. */
long long rc_stream_launches(rc_stream *s);

/* The CUDA stream (cudaStream_t) the stream's work is ordered on.  HEVC
 * streams also read reference slots from a second CUDA stream (a picture's
 * inter units whose references are final are predicted there, beside the
 * previous picture): work the caller enqueues on this stream that writes a
 * DPB slot is seen by later submits when this function, or
 * rc_picture_device_planes, is called after that work is enqueued. */
void *rc_stream_cuda_stream(rc_stream *s);

/* Completion marks, for request loops that keep many streams busy without a
 * host thread per stream (no counterpart in the reference, whose decoders
 * return frames synchronously from Decoder::decode, src/h264/mod.rs:76).
 * rc_stream_mark records a mark after all work submitted so far and returns
 * its id (increasing from 1); rc_stream_mark_done returns 1 once the work
 * before that mark has completed, 0 if not yet, or a negative RC_E* code.
 * Not thread-safe per stream. */
int rc_stream_mark(rc_stream *s, unsigned long long *mark);
int rc_stream_mark_done(rc_stream *s, unsigned long long mark);
/* Device bytes the stream holds (DPB, scratch and record buffers), for
 * admission control across streams. */
size_t rc_stream_device_bytes(rc_stream *s);

/* ======================================================================== */
/*  Output order (DPB bumping)                                               */
/* ======================================================================== */
/*
 * The engine reconstructs pictures into the DPB slots it is given, in
 * decoding order.  These calls give the order in which a decoder hands them
 * to its caller: the picture output process of the reference's DPBs
 * (src/syntax/hevc/dpb.rs:76-160 bump / bump_before_decode / insert;
 * src/syntax/h264/dpb.rs:73-132, 391-478 bump / idr / store_picture), after
 * H.265 C.5.2.2-C.5.2.4 and H.264 C.4.5.3.  A bump outputs the waiting
 * picture with the smallest POC.  Pictures are named by caller ids (e.g. DPB
 * slot << 32 | frame number).  Host-only; needs no GPU.
 *
 * Every call that can output pictures writes their ids, in output order,
 * to out_ids (room for cap ids, which must be at least rc_output_count + 1;
 * RC_EINVAL before any change otherwise) and their number to *n_out.
 */
typedef struct rc_output_dpb rc_output_dpb;

/* capacity: DPB size in pictures (sps_max_dec_pic_buffering_minus1 + 1, or
 * H.264 max_dec_frame_buffering); max_num_reorder: pictures that may wait
 * for output (sps_max_num_reorder_pics / max_num_reorder_frames);
 * max_latency_pictures: SpsMaxLatencyPictures, 0 for none. */
int rc_output_create(int capacity, int max_num_reorder, int max_latency_pictures, rc_output_dpb **out);
void rc_output_destroy(rc_output_dpb *d);

/* Before a picture is decoded.  new_sequence (an HEVC IRAP picture with
 * NoRaslOutputFlag, an H.264 IDR): every waiting picture is output in POC
 * order (none if no_output_of_prior_pics) and the DPB empties.  Otherwise
 * pictures neither waiting nor used for reference leave, and the DPB bumps
 * while it is over the reorder or latency limit or at capacity. */
int rc_output_begin(rc_output_dpb *d, int new_sequence, int no_output_of_prior_pics, uint64_t *out_ids, int cap,
                    int *n_out);

/* A picture is no longer used for reference (reference marking). */
int rc_output_unref(rc_output_dpb *d, uint64_t id);

/* After a picture is decoded: it enters the DPB (waiting for output when
 * output_flag is set, kept as a reference when is_reference is set); the
 * DPB bumps while over the reorder or latency limit. */
int rc_output_insert(rc_output_dpb *d, uint64_t id, int32_t poc, int output_flag, int is_reference,
                     uint64_t *out_ids, int cap, int *n_out);

/* End of the stream: every waiting picture in POC order; the DPB empties. */
int rc_output_flush(rc_output_dpb *d, uint64_t *out_ids, int cap, int *n_out);

/* Pictures the DPB holds (waiting for output or used for reference). */
int rc_output_count(rc_output_dpb *d);

#ifdef __cplusplus
}
#endif

#endif /* PITO_RECON_H */
