/*
 * synth.h — seeded synthetic syntax-record generators.
 *
 * They stand in for the host entropy parse: they emit the same records a
 * parse would hand to the reconstruction engine, with the statistics of the
 * benchmark workloads (intra/inter mix, partition sizes, motion range,
 * weighted prediction, coefficient sparsity, QP range).  Integer-only and
 * platform-independent: a seed gives identical records on every machine.
 */
#ifndef PITO_SYNTH_H
#define PITO_SYNTH_H

#include <stddef.h>
#include <stdint.h>
#include "../../include/pito_recon.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Knobs of the H.264 generator.  Fractions are in 1/1000. */
typedef struct rc_synth_h264_opts {
    uint64_t seed;
    int32_t mb_w, mb_h;
    int32_t intra_only;        /* 1 = every MB intra (an I picture)            */
    int32_t intra_permille;    /* share of intra MBs in inter pictures         */
    int32_t pcm_permille;      /* share of I_PCM among intra MBs               */
    int32_t wp_permille;       /* share of inter MBs with explicit weights     */
    int32_t zero_permille;     /* share of all-zero (uncoded) blocks           */
    int32_t outside_permille;  /* share of partitions pointing off-picture     */
    int32_t mv_range;          /* max |mv| in full pels                        */
    int32_t t8_permille;       /* transform_8x8 share of eligible MBs          */
    int32_t bipred_permille;   /* share of inter partitions using both lists   */
    int32_t qp_min, qp_max;
    int32_t num_slices;        /* slices split in raster order                 */
    int32_t constrained_intra_pred;
    int32_t deblock_idc;       /* 0, 1, 2 for every slice                      */
    int32_t alpha_offset, beta_offset;
    int32_t custom_scaling;    /* 1 = random scaling matrices                  */
    int32_t chroma_qp_offset;  /* added to QP before the QPC table             */
    int32_t num_ref[2];        /* references available per list               */
    int32_t ref_slot[2][4];    /* DPB slots of refidx 0..3                     */
    uint32_t ref_id[2][4];     /* reference identities                         */
    uint32_t frame_id;
    int32_t motion_syntax;     /* 1 = also emit motion syntax (rc_h264_motion)
                                  for the inter MBs: their partitions and refs
                                  with small random mvd and 20% P_Skip; the
                                  vectors are then the derived ones          */
} rc_synth_h264_opts;

/* Fill opts with the 1080p-style defaults (30% intra, 20% WP, 80% zero
 * blocks, +-128 px motion, 5% off-picture, QP 20-40, deblocking on). */
void rc_synth_h264_defaults(rc_synth_h264_opts *o);

/* Generate one picture.  Returns an opaque handle owning the buffers, or
 * NULL.  rc_synth_h264_picture() gives the record view (host memory). */
void *rc_synth_h264_new(const rc_synth_h264_opts *o);
const rc_h264_picture *rc_synth_h264_picture(void *h);
/* Bytes of syntax (records + slices + weights + levels) the picture holds. */
size_t rc_synth_h264_bytes(void *h);
void rc_synth_h264_free(void *h);

/* Knobs of the HEVC generator (fractions in 1/1000). */
typedef struct rc_synth_hevc_opts {
    uint64_t seed;
    int32_t width, height;       /* multiples of 8                            */
    int32_t bit_depth;           /* 8 or 10                                   */
    int32_t log2_ctb;            /* 4..6                                      */
    int32_t intra_only;
    int32_t intra_permille;      /* share of intra CUs in inter pictures      */
    int32_t zero_tu_permille;    /* share of TUs without coefficients         */
    int32_t split_permille;      /* CU / TU quadtree split probability        */
    int32_t mv_range;            /* max |mv| in full pels                     */
    int32_t bipred_permille;
    int32_t qp_min, qp_max;
    int32_t cb_qp_offset, cr_qp_offset;
    int32_t transform_skip_permille; /* of 4x4 TUs                           */
    int32_t pcm_permille;        /* of intra 2Nx2N CUs (8..32)                */
    int32_t pcm_loop_filter_disabled;
    int32_t bypass_permille;     /* CUs with cu_transquant_bypass             */
    int32_t scaling_lists;       /* 1 = random scaling lists                  */
    int32_t constrained_intra_pred;
    int32_t strong_intra_smoothing;
    int32_t weighted;            /* explicit weighted prediction              */
    int32_t num_slices;          /* slices split in tile-scan order           */
    int32_t tile_cols, tile_rows;
    int32_t loop_filter_across_tiles;
    int32_t lf_across_slices;
    int32_t deblock_disabled;
    int32_t beta_offset, tc_offset;
    int32_t sao;                 /* 1 = SAO on (band/edge, offsets +-7)       */
    int32_t num_ref[2];
    int32_t ref_slot[2][4];
    uint32_t ref_id[2][4];
    uint32_t frame_id;
} rc_synth_hevc_opts;

/* 1080p-style defaults: 25% intra, 75% zero TUs, +-256 px, QP 22-37,
 * deblocking and SAO on, CTB 64, 8-bit. */
void rc_synth_hevc_defaults(rc_synth_hevc_opts *o);
void *rc_synth_hevc_new(const rc_synth_hevc_opts *o);
const rc_hevc_picture *rc_synth_hevc_picture(void *h);
size_t rc_synth_hevc_bytes(void *h);
void rc_synth_hevc_free(void *h);

#ifdef __cplusplus
}
#endif

#endif
