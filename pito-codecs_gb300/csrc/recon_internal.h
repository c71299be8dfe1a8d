// recon_internal.h — launch parameters shared by the C ABI layer and the
// CUDA kernels.  Not part of the public interface.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pito_recon.h"

// Device error word values (sticky per stream).
#define RC_DEV_ERR_TIMEOUT 1u  // a wavefront wait exceeded its iteration cap
#define RC_DEV_ERR_RECORD 2u   // a record pointed outside its buffers

// Spin iterations a wavefront wait may take before it gives up (each
// iteration backs off with __nanosleep, so the cap is about a second).
#define RC_WAIT_LIMIT (1u << 22)

// Per-MB loop-filter parameters, derived from the records by h264_mb_kernel
// (boundary strengths of deblock_mb, src/h264/dec/deblock.rs:327-371, and
// the QPs / offsets its edge parameters use).
struct DbMb {
    uint8_t bs[32];     // [dir][edge][segment]; dir 0 = vertical edges
    uint8_t qp[3];      // luma QP of q, of p across edge 0 for dir 0, dir 1
    uint8_t flags;      // bit 0: some edge filters
    uint8_t qpc[3][2];  // chroma QPs, same order
    int8_t aoff, boff;  // slice alpha / beta offsets
    uint8_t pad[4];
};
static_assert(sizeof(DbMb) == 48, "DbMb layout");

// What an intra MB's reconstruction needs besides its residual, prepared by
// h264_mb_kernel: neighbour availability for intra prediction (bits 0..3:
// left, top, top-right, top-left).
struct IntraInfo {
    uint8_t kind, t8, i16_mode, chroma_mode;
    uint8_t nb, pad0, pad1, pad2;
    uint8_t modes[16];
    uint32_t pad3[2];
};
static_assert(sizeof(IntraInfo) == 32, "IntraInfo layout");

// Loop-filter edge words: per MB, 64 words of (alpha | beta << 8 | tc0 << 16
// | bS << 24), bS 0 meaning the line segment is not filtered.  Order, so that
// each filtering lane loads its words with one vector load:
//   [ 0..15] luma vertical edges    k * 4 + e    (k: 4-line segment, e: edge)
//   [16..31] luma horizontal edges  16 + k * 4 + e
//   [32..47] chroma vertical edges  32 + c * 8 + k * 2 + e   (c: Cb/Cr, e: chroma edge 0 / 4)
//   [48..63] chroma horizontal      48 + c * 8 + k * 2 + e
#define RC_EDGE_WORDS 64

#define RC_H264_GROUP_MAX 4
#define RC_H264_GROUP_DEFAULT 3  // rc_stream_set_h264_group(s, 0)
#define RC_H264_GROUP_WORKERS 24 // CTAs of a group launch that predict inter MBs
#define RC_H264_GROUP_SKEW 3     // MB work order: anti-diagonals of row * SKEW + column
#define RC_REFPROG_STRIDE 32     // words between two rows' refprog words (one 128-byte line each)

struct H264Launch {
    const rc_h264_mb *mbs;
    const rc_h264_slice *slices;
    const rc_h264_weight *weights;
    const int16_t *levels;
    const int32_t *ls4;  // [6][6][16]
    const int32_t *ls8;  // [6][6][64]
    unsigned long long num_levels;
    int num_slices, num_weights;
    // DPB: slot s luma at dpb + s * slot_bytes, chroma at + u_off / + v_off
    uint8_t *dpb;
    unsigned long long slot_bytes, u_off, v_off;
    int dpb_slots, out_slot;
    int mb_w, mb_h, W, H, CW, CH, pitch, cpitch;
    int constrained_intra;
    uint32_t epoch;
    uint32_t *error;
    uint32_t wait_limit;
    DbMb *db;             // per-MB loop-filter parameters (allocation-free entry point)
    uint32_t *edges;      // per MB: RC_EDGE_WORDS loop-filter edge words (band kernel)
    uint32_t *rowprog;    // per MB row: (epoch & 0xffff) << 16 | MBs loop-filtered and stored
    uint32_t *irowprog;   // per MB row: (epoch & 0xffff) << 16 | MBs reconstructed (intra included)
    // CTAs per band of the band launch (band_split: 1, or 2 for intra + luma
    // and chroma, or 3 for intra, luma and chroma on CTAs of their own), and
    // for a split launch per MB row, (epoch & 0xffff) << 16 | MBs
    // chroma-filtered and stored, for a band's last row (other rows' words
    // are unused)
    uint32_t *crowprog;
    int band_split;
    IntraInfo *iinfo;     // per MB (intra MBs)
    int16_t *ires;        // per MB: 256 luma + 2 x 64 chroma residual samples (intra MBs)
    // Pictures reconstructed together (H264Group): the MB phase of this
    // picture publishes each MB's completion as mbdone[addr] = epoch (null:
    // the MB phase finished before the band kernel started), and waits for
    // the rows of the in-flight pictures it references: nwait DPB slots with
    // their pictures' epochs and per-row filter progress (refprog layout).
    // motion derived from syntax (h264_mv_kernel): the records it writes
    // (the engine's own copy of mbs), the syntax, and the co-located motion
    // store (slot s at col + s * col_stride bytes)
    rc_h264_mb *mbs_out;
    const rc_h264_motion *motion;
    const rc_h264_slice_motion *smotion;
    uint8_t *col;
    unsigned long long col_stride;
    uint32_t *mvprog;  // per MB row: (epoch & 0xffff) << 16 | MBs whose motion is derived
    uint32_t *mbdone;
    uint8_t *bottom;    // per MB row, mb_w x 32 bytes: unfiltered luma row 15, then Cb and Cr row 7 (not intra MBs)
    int residual_only;  // h264_mb_kernel before a group launch: inter MBs store residuals, unpredicted
    int nwait;
    int wait_slot[RC_H264_GROUP_MAX];
    uint32_t wait_epoch[RC_H264_GROUP_MAX];
    uint32_t *wait_refprog[RC_H264_GROUP_MAX];
    uint32_t *refprog;  // group launch: per MB row, every RC_REFPROG_STRIDE words, rowprog's value for the MB work
};

// Up to RC_H264_GROUP_MAX consecutive pictures of one stream reconstructed
// by one cooperative launch: n * bands CTAs spread over the grid are the
// pictures' band CTAs, the others predict the inter MBs of all the pictures,
// taking (picture, MB) work items in order from *counter (zeroed by the
// launcher).
struct H264Group {
    int n, bands, workers;  // workers: CTAs that predict inter MBs
    uint32_t *counter;
    const uint32_t *order;  // mb_w * mb_h MB addresses in the order the MB work is taken
    H264Launch pic[RC_H264_GROUP_MAX];
};

struct HevcLaunch {
    const rc_hevc_ctb *ctbs;
    const rc_hevc_blk *blk;
    const rc_hevc_mvf *mvf;
    const rc_hevc_tu *tus;
    const rc_hevc_slice *slices;
    const int16_t *levels;
    const uint8_t *scaling;       // device copy of the expanded scaling factors, or null
    unsigned long long num_levels;
    int num_tus, num_slices;
    int W, H, CW, CH, bd, w4, h4, log2ctb, wctb, hctb;
    int constrained_intra, strong_intra, lf_across_tiles, cb_qp_offset, cr_qp_offset;
    // DPB (references + output slot) and the picture being reconstructed
    uint8_t *dpb;
    unsigned long long slot_bytes, u_off, v_off;
    int dpb_slots, out_slot;
    int pitch, cpitch;            // bytes
    uint8_t *work;                // pre-SAO picture, same layout as a slot
    int16_t *res;                 // residual planes: luma W*H, then Cb, Cr CW*CH
    uint32_t *ready;              // 3 planes of w4*h4 flags: epoch when reconstructed
    // per CTB (wctb * hctb): its first transform block, one past its last
    // (0, 0 for a CTB without blocks), its number of intra blocks; ctb_base:
    // the CTBs in the intra task order (anti-diagonal cx + 2 cy, then cy)
    uint32_t *ctb_first, *ctb_end, *ctb_base, *ctb_nintra;
    uint32_t *counter;
    uint32_t *error;
    uint32_t epoch, wait_limit;
    // which inter units a launch predicts: 0 all; 1 those that read no
    // reference in DPB slot late_slot (the previous picture, possibly still
    // being reconstructed), listing the others (late_items, late_count, at
    // most late_cap items); 2 the listed ones
    int inter_pass, late_slot;
    int lf_rows;  // the loop filter's tile height (64, 32 or 16 luma rows)
    uint32_t *late_items, *late_count;
    uint32_t late_cap;
};

void rc_launch_hevc_residual(const HevcLaunch &p, cudaStream_t st);
// Inter prediction plus residual of the units p.inter_pass selects.
void rc_launch_hevc_inter(const HevcLaunch &p, cudaStream_t st);
// Runs the intra kernel, first building the intra task order (a small
// launch) when `order` says the CTB grid differs from the last one built.
// The kernel's task counter (p.counter) must be zero: the stream zeroes it
// once, and every loop-filter launch zeroes it for the next picture.
void rc_launch_hevc_intra(const HevcLaunch &p, cudaStream_t st, int blocks, bool order);
// Deblocking and SAO in one launch: the work picture (read only) -> the
// output DPB slot; it also zeroes the intra kernel's task counter.
void rc_launch_hevc_loopfilter(const HevcLaunch &p, cudaStream_t st);

// Launchers (h264_kernels.cu).
void rc_launch_h264_edge(const H264Launch &p, cudaStream_t st);
// Motion derived from syntax (p.motion): every MB's mv, ref_idx and wp into
// p.mbs_out, and the picture's co-located motion into its slot of p.col.
// Returns 0 or -1 (picture taller than the kernel's rows).
int rc_launch_h264_mv(const H264Launch &p, cudaStream_t st);
// Bytes of one MB's co-located motion.
#define RC_COLMB_BYTES 172
void rc_launch_h264_mb(const H264Launch &p, cudaStream_t st);
// Intra reconstruction and the loop filter in one cooperative launch, one
// CTA per band of RC_H264_BAND_ROWS MB rows, or p.band_split CTAs per band
// that share the band's roles (2: intra and luma, chroma; 3: intra, luma,
// chroma); returns 0 or -1 (launch failed).
// Four rows per band: more rows share one SM's issue slots among more busy
// warps, fewer put more hand-overs through global memory on the critical
// path (1080p P+I sequence on GB300: 7 rows 1237, 5 1350, 4 1395, 3 1396,
// 2 1340, 1 1033 frames/s).
#define RC_H264_BAND_ROWS 4
int rc_launch_h264_band(const H264Launch &p, cudaStream_t st);
// A group of pictures in one cooperative launch of `ctas` CTAs (more than
// g.n * g.bands; at most rc_h264_group_capacity); returns 0 or -1.
int rc_launch_h264_group(const H264Group &g, int ctas, cudaStream_t st);
// CTAs of the group kernel that can be resident at once for pictures mb_w
// MBs wide (0 if unknown).
int rc_h264_group_capacity(int mb_w);
// Band CTAs that can be resident at once for pictures mb_w MBs wide (0 if
// unknown); the band kernel's dynamic shared memory for that width.  A
// picture of `bands` bands takes the split launch with the most CTAs per
// band (3, 2 or 1) whose CTAs fit.
int rc_h264_band_capacity(int mb_w);
size_t rc_h264_band_smem(int mb_w);
