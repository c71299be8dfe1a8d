// recon_api.cu — the C ABI of include/pito_recon.h: stream and DPB lifetime,
// host-side validation of syntax records, staging of host buffers through
// pinned memory, kernel launches and the sticky error word.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "recon_internal.h"

namespace {

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// LevelScale::new, src/h264/dec/transform.rs:10-28 (normAdjust tables of
// src/h264/dec/tables.rs:14-60): per-PPS dequantisation tables.
void h264_level_scale(const uint8_t *m4, const uint8_t *m8, int32_t *ls4, int32_t *ls8) {
    static const uint16_t N4[6][3] = {{10, 16, 13}, {11, 18, 14}, {13, 20, 16},
                                      {14, 23, 18}, {16, 25, 20}, {18, 29, 23}};
    static const uint16_t N8[6][6] = {{20, 18, 32, 19, 25, 24}, {22, 19, 35, 21, 28, 26},
                                      {26, 23, 42, 24, 33, 31}, {28, 25, 45, 26, 35, 33},
                                      {32, 28, 51, 30, 40, 38}, {36, 32, 58, 34, 46, 43}};
    for (int l = 0; l < 6; l++)
        for (int q = 0; q < 6; q++) {
            for (int p = 0; p < 16; p++) {
                int i = p / 4, j = p % 4;
                int k = (i % 2 == 0 && j % 2 == 0) ? 0 : (i % 2 == 1 && j % 2 == 1) ? 1 : 2;
                ls4[(l * 6 + q) * 16 + p] = (int32_t)(m4 ? m4[l * 16 + p] : 16) * N4[q][k];
            }
            for (int p = 0; p < 64; p++) {
                int i = p / 8, j = p % 8, k;
                if (i % 4 == 0 && j % 4 == 0) k = 0;
                else if (i % 2 == 1 && j % 2 == 1) k = 1;
                else if (i % 4 == 2 && j % 4 == 2) k = 2;
                else if ((i % 4 == 0 && j % 2 == 1) || (i % 2 == 1 && j % 4 == 0)) k = 3;
                else if ((i % 4 == 0 && j % 4 == 2) || (i % 4 == 2 && j % 4 == 0)) k = 4;
                else k = 5;
                ls8[(l * 6 + q) * 64 + p] = (int32_t)(m8 ? m8[l * 64 + p] : 16) * N8[q][k];
            }
        }
}

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

// Record sets: two by submit parity, or two groups' worth when H.264
// pictures launch in groups (the next group uploads while one runs).
constexpr int REC_SETS = 2 * RC_H264_GROUP_MAX;

}  // namespace

struct rc_stream {
    int codec = 0, bit_depth = 8, slots = 0;
    int width = 0, height = 0;  // coded size
    int mb_w = 0, mb_h = 0;
    int pitch = 0, cpitch = 0, cw = 0, ch = 0;
    size_t slot_bytes = 0, u_off = 0, v_off = 0;
    size_t budget = 0, held = 0;
    cudaStream_t st = nullptr;   // kernels
    // host <-> device copies run beside the kernels, uploads and downloads on
    // streams of their own (a download waits for the kernels before it, and
    // an upload queued behind it would too): records upload into one of two
    // sets (by submit parity) while the kernels read the other, and a submit
    // that writes a slot waits for that slot's download
    cudaStream_t cst = nullptr;  // uploads
    cudaStream_t dst = nullptr;  // downloads
    cudaEvent_t set_used[REC_SETS] = {};  // kernels of the last submit that read record set i
    cudaEvent_t set_ready[REC_SETS] = {}; // record set i uploaded
    bool set_busy[REC_SETS] = {};
    int nsets = 2;                        // record sets in use
    cudaEvent_t kernels_done = nullptr;            // recorded before each download
    std::vector<cudaEvent_t> slot_dl;              // per DPB slot: its last download
    std::vector<char> slot_dl_pending;
    uint8_t *dpb = nullptr;
    uint32_t *counter = nullptr, *error = nullptr;
    uint32_t *rowprog = nullptr, *irowprog = nullptr;
    // H.264: CTAs per band of the band launch (intra, the luma and the chroma
    // filter on CTAs of their own when three times the bands fit on the
    // device at once), and the chroma filter's hand-over words
    uint32_t *crowprog = nullptr;
    int band_split = 1;
    // The first kernel of a picture reads only its records (H.264 edge
    // words, HEVC residuals and CTB ranges): it runs on a side stream as soon
    // as the records are in, beside the previous picture's wavefront kernels,
    // writing one of two sets of these buffers by submit parity.
    uint32_t *edges[2] = {nullptr, nullptr};
    cudaStream_t est = nullptr;
    cudaEvent_t aux_used[2] = {nullptr, nullptr};  // the kernels that last read set i
    cudaEvent_t aux_ready = nullptr;
    bool aux_busy[2] = {false, false};
    IntraInfo *iinfo = nullptr;
    int16_t *ires = nullptr;
    // HEVC
    DevBuf ctbs[2], blk[2], mvf[2], tus[2], hslices[2], scaling;
    // the picture being reconstructed (pre-loop-filter), two by submit
    // parity: a picture's inter prediction runs on the side stream beside
    // the previous picture's intra and loop-filter kernels, for the units
    // whose references are final; work_free[i]: the loop filter that last
    // read work[i]
    uint8_t *work[2] = {nullptr, nullptr};
    uint32_t *late_items[2] = {nullptr, nullptr};  // the late inter units' groups
    uint32_t *late_count = nullptr;                // two counters
    size_t late_cap = 0;
    cudaEvent_t work_free[2] = {nullptr, nullptr};
    bool work_busy[2] = {false, false};
    // the previous picture's output slot (its units are predicted on the
    // main stream after it), and whether the caller may have written a slot
    // on the main stream since (rc_stream_cuda_stream, device planes), which
    // orders the next early pass after the main stream
    int hevc_prev_slot = -1;
    bool hevc_ext = false;
    int lf_rows = 64;  // the loop filter's tile height (rc_stream_set_lf_tile)
    int16_t *res[2] = {nullptr, nullptr};  // residual planes (two sets by submit parity)
    uint32_t *ready = nullptr;   // per 4x4 block and component
    uint32_t *ctb_ord[2] = {nullptr, nullptr};  // ctb_first, ctb_end, ctb_base, ctb_nintra (smallest CTB size)
    size_t nctb_max = 0;
    int w4 = 0, h4 = 0, log2ctb_alloc = 0;
    int bps = 1;
    DevBuf mbs[REC_SETS], slices[REC_SETS], weights[REC_SETS], levels[REC_SETS];
    // motion derived from syntax: the syntax per record set, the co-located
    // motion store (one entry per MB and DPB slot, allocated on first use)
    // and which slots hold stored motion
    DevBuf motion[REC_SETS], smotion[REC_SETS];
    uint8_t *col = nullptr;
    uint32_t *mvprog = nullptr;  // per MB row, the motion kernel's progress
    std::vector<char> slot_col;
    cudaEvent_t mv_ready = nullptr;
    // H.264 picture groups (rc_stream_set_h264_group): pictures per launch,
    // the launch's CTAs, the submitted pictures not yet launched (with the
    // DPB slots they read and their record sets), and per group position the
    // scratch of one picture: progress words, MB completion flags, edge
    // words, intra parameters and residuals
    int group = 1, group_ctas = 0, group_workers = 0;
    std::vector<H264Launch> pending;
    std::vector<std::vector<int>> pending_refs;
    std::vector<int> pending_sets;
    uint32_t *g_rowprog = nullptr, *g_irowprog = nullptr, *g_mbdone = nullptr, *g_edges = nullptr;
    uint8_t *g_bottom = nullptr;
    uint32_t *g_order = nullptr, *g_refprog = nullptr;
    IntraInfo *g_iinfo = nullptr;
    int16_t *g_ires = nullptr;
    int g_alloc = 0;  // positions allocated
    // device-memory records in a group: their slices are read back (on a
    // stream of their own, into pinned memory) for the reference slots
    cudaStream_t rst = nullptr;
    void *rb = nullptr;
    size_t rb_cap = 0;
    // asynchronous downloads of slots that pending pictures write, issued
    // once their group has launched
    struct Dl {
        int slot, x, y, w, h;
        void *py, *pu, *pv;
    };
    std::vector<Dl> pending_dl;
    int32_t *ls = nullptr;            // device ls4 (2304 ints) + ls8 (2304*4 ints)
    std::vector<int32_t> ls_host;     // last uploaded tables
    uint8_t ls_key[2 + 96 + 384] = {0};  // the scaling lists they were made from (flat: flag 0)
    std::vector<uint8_t> scal_host;      // HEVC: the scaling factors last uploaded
    bool ls_valid = false;
    void *staging[2] = {nullptr, nullptr};
    size_t staging_cap[2] = {0, 0};
    cudaEvent_t staged[2] = {nullptr, nullptr};
    int submits = 0;
    uint32_t epoch = 0;
    long long launches = 0;
    int sticky = 0;
    int wave_blocks = 0, wave_default = 0;  // HEVC intra CTAs per launch, and its default
    int ord_wctb = 0, ord_hctb = 0;         // HEVC: the CTB grid whose intra task order is built
    int sms = 0;
    uint32_t wait_limit = RC_WAIT_LIMIT;
    // per-kernel CUDA-event timing
    bool profiling = false;
    std::vector<cudaEvent_t> ev_free;
    // completion marks (rc_stream_mark): pending (id, event) in order
    std::deque<std::pair<unsigned long long, cudaEvent_t>> marks;
    std::vector<cudaEvent_t> mark_free;
    unsigned long long next_mark = 0, marks_done = 0;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    double prof_ms[RC_KERNEL_COUNT] = {0};
    long long prof_n[RC_KERNEL_COUNT] = {0};
};

namespace {

cudaEvent_t take_event(rc_stream *s) {
    if (!s->ev_free.empty()) {
        cudaEvent_t e = s->ev_free.back();
        s->ev_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Launch one kernel through `fn`, bracketed by timing events when profiling.
template <class F>
void timed(rc_stream *s, int kernel, F fn, cudaStream_t on = nullptr) {
    if (!on) on = s->st;
    if (!s->profiling) {
        fn();
        s->launches++;
        return;
    }
    cudaEvent_t a = take_event(s), b = take_event(s);
    cudaEventRecord(a, on);
    fn();
    cudaEventRecord(b, on);
    s->ev_pending.push_back({kernel, {a, b}});
    s->launches++;
}

void drain_profile(rc_stream *s) {
    for (auto &p : s->ev_pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
            s->prof_ms[p.first] += ms;
            s->prof_n[p.first] += 1;
        }
        s->ev_free.push_back(p.second.first);
        s->ev_free.push_back(p.second.second);
    }
    s->ev_pending.clear();
}

int cuda_fail(rc_stream *s) {
    if (s && !s->sticky) s->sticky = RC_ECUDA;
    return RC_ECUDA;
}

bool dev_alloc(rc_stream *s, void **p, size_t n) {
    if (s->budget && s->held + n > s->budget) return false;
    if (cudaMalloc(p, n) != cudaSuccess) return false;
    s->held += n;
    return true;
}
void dev_free(rc_stream *s, void *p, size_t n) {
    if (!p) return;
    cudaFree(p);
    s->held -= std::min(s->held, n);
}

// Grow a device buffer (waits for in-flight work that may read it).
int ensure(rc_stream *s, DevBuf &b, size_t n) {
    if (n <= b.cap) return 0;
    if (cudaStreamSynchronize(s->st) != cudaSuccess || cudaStreamSynchronize(s->cst) != cudaSuccess ||
        cudaStreamSynchronize(s->dst) != cudaSuccess || (s->est && cudaStreamSynchronize(s->est) != cudaSuccess))
        return cuda_fail(s);
    size_t want = std::max(n, b.cap + b.cap / 2);
    want = align_up(std::max<size_t>(want, 4096), 4096);
    dev_free(s, b.p, b.cap);
    b.p = nullptr;
    b.cap = 0;
    if (!dev_alloc(s, &b.p, want)) return RC_ENOMEM;
    b.cap = want;
    return 0;
}

bool is_pinned(const void *p) {
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Host-side validation of an H.264 picture (the checks of
// src/h264/dec/slicedec.rs:888-892, 1442-1446 and the payload bounds).
struct Geo {
    int mb_w, mb_h, slots;
};
// Motion syntax (rc_h264_motion, rc_h264_slice_motion): what the kernel
// rejects as a record error, rejected before launch (ref_idx past its list,
// direct modes outside B slices, unknown shapes), and weight entries that
// exist.  Whether the co-located slot holds stored motion is checked by the
// submit, which knows the stream's slots.
int validate_h264_motion(const Geo *s, const rc_h264_picture *p) {
    if (!p->slice_motion) return RC_EINVAL;
    for (int i = 0; i < p->num_slices; i++) {
        const rc_h264_slice_motion &sm = p->slice_motion[i];
        const rc_h264_slice &sl = p->slices[i];
        if ((sm.b_slice != 0 && sm.b_slice != 1) || (sm.b_slice && (sm.col_slot < 0 || sm.col_slot >= s->slots)))
            return RC_EINVAL;
        for (int r0 = -1; r0 < sl.num_ref[0]; r0++)
            for (int r1 = -1; r1 < sl.num_ref[1]; r1++) {
                const int w = sm.wp_map[(r0 + 1) * (RC_H264_MAX_REFS + 1) + (r1 + 1)];
                if (w != 0xff && w >= p->num_weights) return RC_EINVAL;
            }
    }
    const int n = s->mb_w * s->mb_h;
    for (int a = 0; a < n; a++) {
        const rc_h264_mb &m = p->mbs[a];
        const rc_h264_motion &mo = p->motion[a];
        const bool inter = m.kind == RC_H264_INTER;
        if (inter != (mo.shape != RC_H264_MOTION_NONE) || mo.shape > RC_H264_MOTION_8x8) return RC_EINVAL;
        if (!inter) continue;
        const rc_h264_slice &sl = p->slices[m.slice];
        const bool b = p->slice_motion[m.slice].b_slice != 0;
        auto ref_ok = [&](int l, int r) { return r >= 0 && r < sl.num_ref[l]; };
        if (mo.shape == RC_H264_MOTION_SKIP) {
            if (!b && sl.num_ref[0] < 1) return RC_EINVAL;
            continue;
        }
        if (mo.shape != RC_H264_MOTION_8x8) {
            const int np = mo.shape == RC_H264_MOTION_16x16 ? 1 : 2;
            for (int q = 0; q < np; q++) {
                const int b8 = mo.shape == RC_H264_MOTION_16x8 ? 2 * q : q;
                if (mo.pred[q] < 1 || mo.pred[q] > 3 || (!b && mo.pred[q] != 1)) return RC_EINVAL;
                for (int l = 0; l < 2; l++)
                    if ((mo.pred[q] >> l & 1) && !ref_ok(l, mo.ref_idx[l][b8])) return RC_EINVAL;
            }
            continue;
        }
        for (int q = 0; q < 4; q++) {
            if (mo.sub[q] == RC_H264_SUB_DIRECT) {
                if (!b) return RC_EINVAL;
                continue;
            }
            if (mo.sub[q] > RC_H264_SUB_4x4 || mo.pred[q] < 1 || mo.pred[q] > 3 || (!b && mo.pred[q] != 1))
                return RC_EINVAL;
            for (int l = 0; l < 2; l++)
                if ((mo.pred[q] >> l & 1) && !ref_ok(l, mo.ref_idx[l][q])) return RC_EINVAL;
        }
    }
    return 0;
}

int validate_h264(const Geo *s, const rc_h264_picture *p) {
    if (!p->mbs || p->num_slices <= 0 || !p->slices) return RC_EINVAL;
    if (p->num_weights < 0 || (p->num_weights > 0 && !p->weights)) return RC_EINVAL;
    if (p->num_levels > 0 && !p->levels) return RC_EINVAL;
    for (int i = 0; i < p->num_slices; i++) {
        const rc_h264_slice &sl = p->slices[i];
        if (sl.disable_deblocking_filter_idc < 0 || sl.disable_deblocking_filter_idc > 2) return RC_EINVAL;
        for (int l = 0; l < 2; l++) {
            if (sl.num_ref[l] < 0 || sl.num_ref[l] > RC_H264_MAX_REFS) return RC_EINVAL;
            for (int r = 0; r < sl.num_ref[l]; r++)
                if (sl.ref_slot[l][r] < 0 || sl.ref_slot[l][r] >= s->slots) return RC_EINVAL;
        }
    }
    const int n = s->mb_w * s->mb_h;
    for (int a = 0; a < n; a++) {
        const rc_h264_mb &m = p->mbs[a];
        if (m.kind > RC_H264_INTER) return RC_EINVAL;
        if (m.kind == RC_H264_NONE) continue;
        if (m.slice >= p->num_slices) return RC_EINVAL;
        if (m.qp > 51 || m.qpc[0] > 51 || m.qpc[1] > 51) return RC_EINVAL;
        if (m.kind == RC_H264_IPCM) {
            if ((size_t)m.coef_off + 384 > p->num_levels) return RC_EINVAL;
            continue;
        }
        if ((m.kind == RC_H264_I8x8) != (m.transform_8x8 != 0) && m.kind != RC_H264_INTER) return RC_EINVAL;
        if (m.kind == RC_H264_INTER && !p->motion) {  // with motion syntax, the motion is derived (below)
            const rc_h264_slice &sl = p->slices[m.slice];
            for (int b = 0; b < 4; b++) {
                int r0 = m.ref_idx[0][b], r1 = m.ref_idx[1][b];
                if (r0 < -1 || r1 < -1 || (r0 < 0 && r1 < 0)) return RC_EINVAL;
                if (r0 >= sl.num_ref[0] || r1 >= sl.num_ref[1]) return RC_EINVAL;
                if (m.wp[b] != 0xff && m.wp[b] >= p->num_weights) return RC_EINVAL;
            }
        } else {
            if (m.i16_mode > 3 || m.chroma_mode > 3) return RC_EINVAL;
            for (int i = 0; i < 16; i++)
                if (m.intra_modes[i] > 8) return RC_EINVAL;
        }
        int t8 = m.transform_8x8;
        size_t need = ((m.kind == RC_H264_I16x16 && (m.dc_coded & 1)) ? 16 : 0) +
                      (size_t)__builtin_popcount(m.luma_coded & (t8 ? 0xf : 0xffff)) * (t8 ? 64 : 16) +
                      (size_t)__builtin_popcount(m.dc_coded & 6) * 4 + (size_t)__builtin_popcount(m.chroma_coded) * 16;
        if ((size_t)m.coef_off + need > p->num_levels) return RC_EINVAL;
    }
    return p->motion ? validate_h264_motion(s, p) : 0;
}

void group_free(rc_stream *s) {
    if (!s->g_alloc) return;
    const size_t mbs = (size_t)s->mb_w * s->mb_h, n = (size_t)s->g_alloc;
    dev_free(s, s->g_rowprog, n * s->mb_h * sizeof(uint32_t));
    dev_free(s, s->g_irowprog, n * s->mb_h * sizeof(uint32_t));
    dev_free(s, s->g_mbdone, n * mbs * sizeof(uint32_t));
    dev_free(s, s->g_edges, n * mbs * RC_EDGE_WORDS * sizeof(uint32_t));
    dev_free(s, s->g_iinfo, n * mbs * sizeof(IntraInfo));
    dev_free(s, s->g_ires, n * mbs * 384 * sizeof(int16_t));
    dev_free(s, s->g_bottom, n * mbs * 32);
    dev_free(s, s->g_order, mbs * sizeof(uint32_t));
    dev_free(s, s->g_refprog, n * s->mb_h * RC_REFPROG_STRIDE * sizeof(uint32_t));
    s->g_refprog = nullptr;
    s->g_rowprog = s->g_irowprog = s->g_mbdone = s->g_edges = s->g_order = nullptr;
    s->g_bottom = nullptr;
    s->g_iinfo = nullptr;
    s->g_ires = nullptr;
    s->g_alloc = 0;
}

// The per-position scratch of groups of n pictures (zeroed: no flag or
// progress word matches a picture before it is written).
int group_alloc(rc_stream *s, int n) {
    if (n <= s->g_alloc) return 0;
    if (cudaStreamSynchronize(s->st) != cudaSuccess) return cuda_fail(s);
    group_free(s);
    const size_t mbs = (size_t)s->mb_w * s->mb_h;
    bool ok = dev_alloc(s, (void **)&s->g_rowprog, n * s->mb_h * sizeof(uint32_t)) &&
              dev_alloc(s, (void **)&s->g_irowprog, n * s->mb_h * sizeof(uint32_t)) &&
              dev_alloc(s, (void **)&s->g_mbdone, n * mbs * sizeof(uint32_t)) &&
              dev_alloc(s, (void **)&s->g_edges, n * mbs * RC_EDGE_WORDS * sizeof(uint32_t)) &&
              dev_alloc(s, (void **)&s->g_iinfo, n * mbs * sizeof(IntraInfo)) &&
              dev_alloc(s, (void **)&s->g_ires, n * mbs * 384 * sizeof(int16_t)) &&
              dev_alloc(s, (void **)&s->g_bottom, n * mbs * 32) &&
              dev_alloc(s, (void **)&s->g_order, mbs * sizeof(uint32_t)) &&
              dev_alloc(s, (void **)&s->g_refprog, n * s->mb_h * RC_REFPROG_STRIDE * sizeof(uint32_t));
    s->g_alloc = n;  // group_free releases whatever was allocated
    if (!ok) {
        cudaGetLastError();
        group_free(s);
        return RC_ENOMEM;
    }
    // the order the MB work is taken in: anti-diagonals row * skew + column
    // (then by row), the shape of the band wavefronts
    std::vector<uint32_t> order(mbs);
    for (size_t a = 0; a < mbs; a++) order[a] = (uint32_t)a;
    const int w = s->mb_w;
    std::stable_sort(order.begin(), order.end(), [w](uint32_t p, uint32_t q) {
        const int kp = (int)(p / w) * RC_H264_GROUP_SKEW + (int)(p % w), kq = (int)(q / w) * RC_H264_GROUP_SKEW + (int)(q % w);
        return kp < kq;
    });
    ok = cudaMemsetAsync(s->g_rowprog, 0, n * s->mb_h * sizeof(uint32_t), s->st) == cudaSuccess &&
         cudaMemsetAsync(s->g_irowprog, 0, n * s->mb_h * sizeof(uint32_t), s->st) == cudaSuccess &&
         cudaMemsetAsync(s->g_mbdone, 0, n * mbs * sizeof(uint32_t), s->st) == cudaSuccess &&
         cudaMemsetAsync(s->g_refprog, 0, n * s->mb_h * RC_REFPROG_STRIDE * sizeof(uint32_t), s->st) == cudaSuccess &&
         cudaMemcpyAsync(s->g_order, order.data(), mbs * sizeof(uint32_t), cudaMemcpyHostToDevice, s->st) == cudaSuccess &&
         cudaStreamSynchronize(s->st) == cudaSuccess;  // `order` is pageable and leaves scope
    return ok ? 0 : cuda_fail(s);
}

void destroy(rc_stream *s) {
    if (!s) return;
    s->pending.clear();  // submitted pictures not yet launched are dropped
    s->pending_dl.clear();
    if (s->rst) {
        cudaStreamSynchronize(s->rst);
        cudaStreamDestroy(s->rst);
    }
    if (s->rb) cudaFreeHost(s->rb);
    if (s->st) cudaStreamSynchronize(s->st);
    if (s->cst) cudaStreamSynchronize(s->cst);
    if (s->dst) cudaStreamSynchronize(s->dst);
    drain_profile(s);
    for (cudaEvent_t e : s->ev_free) cudaEventDestroy(e);
    for (auto &m : s->marks) cudaEventDestroy(m.second);
    for (cudaEvent_t e : s->mark_free) cudaEventDestroy(e);
    dev_free(s, s->dpb, s->slot_bytes * s->slots);
    for (int i = 0; i < 2; i++)
        for (DevBuf *b : {&s->ctbs[i], &s->blk[i], &s->mvf[i], &s->tus[i], &s->hslices[i]}) dev_free(s, b->p, b->cap);
    for (int i = 0; i < REC_SETS; i++)
        for (DevBuf *b : {&s->mbs[i], &s->slices[i], &s->weights[i], &s->levels[i], &s->motion[i], &s->smotion[i]})
            dev_free(s, b->p, b->cap);
    dev_free(s, s->col, (size_t)s->slots * s->mb_w * s->mb_h * RC_COLMB_BYTES);
    dev_free(s, s->mvprog, (size_t)s->mb_h * sizeof(uint32_t));
    if (s->mv_ready) cudaEventDestroy(s->mv_ready);
    group_free(s);
    dev_free(s, s->scaling.p, s->scaling.cap);
    for (int i = 0; i < 2; i++) {
        cudaFree(s->work[i]);
        if (s->late_items[i]) dev_free(s, s->late_items[i], s->late_cap * sizeof(uint32_t));
        if (s->work_free[i]) cudaEventDestroy(s->work_free[i]);
    }
    cudaFree(s->late_count);
    for (int i = 0; i < 2; i++) cudaFree(s->res[i]);
    cudaFree(s->ready);
    for (int i = 0; i < 2; i++) dev_free(s, s->ctb_ord[i], 4 * s->nctb_max * sizeof(uint32_t));
    cudaFree(s->counter);
    cudaFree(s->error);
    cudaFree(s->ls);
    cudaFree(s->rowprog);
    cudaFree(s->irowprog);
    cudaFree(s->crowprog);
    for (int i = 0; i < 2; i++) {
        if (s->edges[i]) dev_free(s, s->edges[i], (size_t)s->mb_w * s->mb_h * RC_EDGE_WORDS * sizeof(uint32_t));
        if (s->aux_used[i]) cudaEventDestroy(s->aux_used[i]);
    }
    if (s->aux_ready) cudaEventDestroy(s->aux_ready);
    if (s->est) {
        cudaStreamSynchronize(s->est);
        cudaStreamDestroy(s->est);
    }
    dev_free(s, s->iinfo, (size_t)s->mb_w * s->mb_h * sizeof(IntraInfo));
    dev_free(s, s->ires, (size_t)s->mb_w * s->mb_h * 384 * sizeof(int16_t));
    for (int i = 0; i < 2; i++) {
        if (s->staging[i]) cudaFreeHost(s->staging[i]);
        if (s->staged[i]) cudaEventDestroy(s->staged[i]);
    }
    for (int i = 0; i < REC_SETS; i++) {
        if (s->set_used[i]) cudaEventDestroy(s->set_used[i]);
        if (s->set_ready[i]) cudaEventDestroy(s->set_ready[i]);
    }
    if (s->kernels_done) cudaEventDestroy(s->kernels_done);
    for (cudaEvent_t e : s->slot_dl)
        if (e) cudaEventDestroy(e);
    if (s->cst) cudaStreamDestroy(s->cst);
    if (s->dst) cudaStreamDestroy(s->dst);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
}

struct Part {
    DevBuf *dst;
    const void *src;
    size_t n;
};

// Copy host buffers to device buffers on stream `on`: directly when every
// source is pinned, else through the stream's double-buffered pinned staging.
int upload(rc_stream *s, Part *parts, int np, cudaStream_t on) {
    int rc;
    for (int i = 0; i < np; i++)
        if ((rc = ensure(s, *parts[i].dst, std::max<size_t>(parts[i].n, 64)))) return rc;
    bool pinned = true;
    for (int i = 0; i < np; i++) pinned = pinned && is_pinned(parts[i].src);
    if (pinned) {
        for (int i = 0; i < np; i++)
            if (parts[i].n &&
                cudaMemcpyAsync(parts[i].dst->p, parts[i].src, parts[i].n, cudaMemcpyHostToDevice, on) != cudaSuccess)
                return cuda_fail(s);
        return 0;
    }
    const int k = s->submits & 1;
    size_t total = 0;
    for (int i = 0; i < np; i++) total += align_up(parts[i].n, 256);
    if (cudaEventSynchronize(s->staged[k]) != cudaSuccess) return cuda_fail(s);
    if (total > s->staging_cap[k]) {
        if (s->staging[k]) cudaFreeHost(s->staging[k]);
        s->staging[k] = nullptr;
        s->staging_cap[k] = 0;
        size_t want = align_up(total + total / 4, 1 << 20);
        if (cudaMallocHost(&s->staging[k], want) != cudaSuccess) return RC_ENOMEM;
        s->staging_cap[k] = want;
    }
    uint8_t *stage = (uint8_t *)s->staging[k];
    size_t off = 0;
    for (int i = 0; i < np; i++) {
        if (!parts[i].n) continue;
        memcpy(stage + off, parts[i].src, parts[i].n);
        if (cudaMemcpyAsync(parts[i].dst->p, stage + off, parts[i].n, cudaMemcpyHostToDevice, on) != cudaSuccess)
            return cuda_fail(s);
        off += align_up(parts[i].n, 256);
    }
    if (cudaEventRecord(s->staged[k], on) != cudaSuccess) return cuda_fail(s);
    return 0;
}

// Before uploading record set k on the copy stream: the kernels that last
// read it are done.  After: the kernels wait for the upload.
int set_begin(rc_stream *s, int k) {
    if (s->set_busy[k] && cudaStreamWaitEvent(s->cst, s->set_used[k], 0) != cudaSuccess) return cuda_fail(s);
    return 0;
}
int set_end(rc_stream *s, int k) {
    if (cudaEventRecord(s->set_ready[k], s->cst) != cudaSuccess ||
        cudaStreamWaitEvent(s->st, s->set_ready[k], 0) != cudaSuccess)
        return cuda_fail(s);
    return 0;
}
// Before a picture's kernels write slot `slot`: its pending download is done.
int slot_begin(rc_stream *s, int slot) {
    if (s->slot_dl_pending[slot]) {
        if (cudaStreamWaitEvent(s->st, s->slot_dl[slot], 0) != cudaSuccess) return cuda_fail(s);
        s->slot_dl_pending[slot] = 0;
    }
    return 0;
}
// After the kernels of a submit that read record set k.
int set_release(rc_stream *s, int k) {
    if (cudaEventRecord(s->set_used[k], s->st) != cudaSuccess) return cuda_fail(s);
    s->set_busy[k] = true;
    return 0;
}

// Queue a cropped copy of a DPB slot on the download stream, after every
// kernel launched so far (bounds checked by the caller, copy_cropped's rule,
// src/h264/dec/picture.rs:601-615); later submits that write the slot wait
// for it.
// One plane's rows to the caller: a single contiguous copy when the rows are
// whole plane rows (the crop spans the pitch), else a 2-D copy.
static bool copy_rows(void *dst, const uint8_t *src, size_t pitch, size_t row_bytes, int rows, cudaStream_t c) {
    if (row_bytes == pitch)
        return cudaMemcpyAsync(dst, src, row_bytes * rows, cudaMemcpyDeviceToHost, c) == cudaSuccess;
    return cudaMemcpy2DAsync(dst, row_bytes, src, pitch, row_bytes, rows, cudaMemcpyDeviceToHost, c) == cudaSuccess;
}

int issue_download(rc_stream *s, int slot, int x, int y, int w, int h, void *out_y, void *out_u, void *out_v) {
    const int cx = x / 2, cy = y / 2, ccw = (w + 1) / 2, cch = (h + 1) / 2, bps = s->bps;
    const uint8_t *base = s->dpb + (size_t)slot * s->slot_bytes;
    cudaStream_t c = s->dst;
    bool ok = cudaEventRecord(s->kernels_done, s->st) == cudaSuccess &&
              cudaStreamWaitEvent(c, s->kernels_done, 0) == cudaSuccess &&
              copy_rows(out_y, base + (size_t)y * s->pitch + (size_t)x * bps, s->pitch, (size_t)w * bps, h, c) &&
              copy_rows(out_u, base + s->u_off + (size_t)cy * s->cpitch + (size_t)cx * bps, s->cpitch,
                        (size_t)ccw * bps, cch, c) &&
              copy_rows(out_v, base + s->v_off + (size_t)cy * s->cpitch + (size_t)cx * bps, s->cpitch,
                        (size_t)ccw * bps, cch, c) &&
              cudaEventRecord(s->slot_dl[slot], c) == cudaSuccess;
    if (ok) s->slot_dl_pending[slot] = 1;
    return ok ? 0 : cuda_fail(s);
}

// Launch the pending group of H.264 pictures, if any.
int h264_flush(rc_stream *s) {
    if (s->pending.empty()) return 0;
    H264Group g;
    memset(&g, 0, sizeof g);
    g.n = (int)s->pending.size();
    g.bands = (s->mb_h + RC_H264_BAND_ROWS - 1) / RC_H264_BAND_ROWS;
    g.counter = s->counter;
    g.order = s->g_order;
    g.workers = std::min(s->group_workers, s->group_ctas - g.n * g.bands);
    for (int i = 0; i < g.n; i++) g.pic[i] = s->pending[i];
    int lrc = 0;
    timed(s, RC_KERNEL_H264_GROUP, [&] { lrc = rc_launch_h264_group(g, s->group_ctas, s->st); });
    int rc = lrc ? cuda_fail(s) : 0;
    for (int k : s->pending_sets)
        if (!rc && k >= 0) rc = set_release(s, k);
    s->pending.clear();
    s->pending_refs.clear();
    s->pending_sets.clear();
    for (const auto &d : s->pending_dl)
        if (!rc) rc = issue_download(s, d.slot, d.x, d.y, d.w, d.h, d.py, d.pu, d.pv);
    s->pending_dl.clear();
    return rc;
}

// The reference slots of a picture whose records are in device memory: its
// slices are read back (a few hundred bytes each) and the slots taken from
// them; out-of-range entries are left to the kernels' record checks.
int h264_device_ref_slots(rc_stream *s, const rc_h264_picture *p, std::vector<int> &out) {
    const size_t n = sizeof(rc_h264_slice) * (size_t)p->num_slices;
    if (!s->rst && cudaStreamCreateWithFlags(&s->rst, cudaStreamNonBlocking) != cudaSuccess) return cuda_fail(s);
    if (n > s->rb_cap) {
        if (s->rb) cudaFreeHost(s->rb);
        s->rb = nullptr;
        s->rb_cap = 0;
        if (cudaMallocHost(&s->rb, align_up(n, 4096)) != cudaSuccess) return RC_ENOMEM;
        s->rb_cap = align_up(n, 4096);
    }
    if (cudaMemcpyAsync(s->rb, p->slices, n, cudaMemcpyDeviceToHost, s->rst) != cudaSuccess ||
        cudaStreamSynchronize(s->rst) != cudaSuccess) {
        cudaGetLastError();
        return RC_EINVAL;
    }
    const rc_h264_slice *sl = (const rc_h264_slice *)s->rb;
    out.clear();
    for (int i = 0; i < p->num_slices; i++)
        for (int l = 0; l < 2; l++)
            for (int j = 0; j < std::min(std::max(sl[i].num_ref[l], 0), RC_H264_MAX_REFS); j++) {
                const int slot = sl[i].ref_slot[l][j];
                if (slot >= 0 && slot < s->slots && std::find(out.begin(), out.end(), slot) == out.end())
                    out.push_back(slot);
            }
    return 0;
}

// The DPB slots an H.264 picture's slices reference (validated records).
std::vector<int> h264_ref_slots(const rc_h264_picture *p) {
    std::vector<int> r;
    for (int i = 0; i < p->num_slices; i++)
        for (int l = 0; l < 2; l++)
            for (int j = 0; j < p->slices[i].num_ref[l]; j++) {
                const int slot = p->slices[i].ref_slot[l][j];
                if (std::find(r.begin(), r.end(), slot) == r.end()) r.push_back(slot);
            }
    return r;
}

struct HGeo {
    int W, H, bd, slots;
};

// A few host threads for the validation of large pictures: a 2160p HEVC
// picture has 518400 4x4 blocks and tens of thousands of transform blocks,
// which take one host thread about as long as the GPU takes for the picture.
// One job at a time; a caller that finds the pool busy (another stream's
// thread validating) does its job alone.
class HostPool {
public:
    static HostPool &get() {
        static HostPool pool;
        return pool;
    }
    // f(0) .. f(n - 1), on the workers and the calling thread
    void run(int n, const std::function<void(int)> &f) {
        std::unique_lock<std::mutex> one(call_, std::try_to_lock);
        if (!one.owns_lock() || th_.empty()) {
            for (int i = 0; i < n; i++) f(i);
            return;
        }
        {
            std::unique_lock<std::mutex> lk(m_);
            // a worker still inside the previous job (woken after its items
            // were all taken) leaves it before the job changes
            done_.wait(lk, [&] { return active_ == 0; });
            job_ = &f;
            n_ = n;
            next_.store(0);
            gen_++;
        }
        go_.notify_all();
        for (int i; (i = next_.fetch_add(1)) < n;) f(i);
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [&] { return active_ == 0; });
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(m_);
            quit_ = true;
        }
        go_.notify_all();
        for (auto &t : th_) t.join();
    }

private:
    HostPool() {
        const unsigned hw = std::thread::hardware_concurrency();
        const int workers = std::min(7, (int)(hw > 1 ? hw - 1 : 0));
        for (int i = 0; i < workers; i++) th_.emplace_back([this] { loop(); });
    }
    void loop() {
        unsigned long long seen = 0;
        for (;;) {
            const std::function<void(int)> *f;
            int n;
            {
                std::unique_lock<std::mutex> lk(m_);
                go_.wait(lk, [&] { return quit_ || gen_ != seen; });
                if (quit_) return;
                seen = gen_;
                f = job_;
                n = n_;
                active_++;
            }
            for (int i; (i = next_.fetch_add(1)) < n;) (*f)(i);
            std::lock_guard<std::mutex> lk(m_);
            if (--active_ == 0) done_.notify_all();
        }
    }
    std::mutex call_, m_;
    std::condition_variable go_, done_;
    std::vector<std::thread> th_;
    const std::function<void(int)> *job_ = nullptr;
    int n_ = 0, active_ = 0;
    std::atomic<int> next_{0};
    unsigned long long gen_ = 0;
    bool quit_ = false;
};

// Host-side validation of an HEVC picture (ranges, reference indices,
// payload bounds; src/hevc/slicedec.rs:2153-2160 rejects bad ref_idx).
int validate_hevc(const HGeo *g, const rc_hevc_picture *p) {
    if (p->log2_ctb < 4 || p->log2_ctb > 6 || p->num_slices <= 0 || !p->slices || !p->ctbs || !p->blk || !p->mvf)
        return RC_EINVAL;
    if (p->num_tus < 0 || (p->num_tus > 0 && !p->tus) || (p->num_levels > 0 && !p->levels)) return RC_EINVAL;
    const int ctb = 1 << p->log2_ctb, wctb = (g->W + ctb - 1) / ctb, hctb = (g->H + ctb - 1) / ctb;
    const int w4 = g->W / 4, h4 = g->H / 4, CW = g->W / 2, CH = g->H / 2;
    for (int i = 0; i < p->num_slices; i++) {
        const rc_hevc_slice &sl = p->slices[i];
        for (int l = 0; l < 2; l++) {
            if (sl.num_ref[l] < 0 || sl.num_ref[l] > RC_HEVC_MAX_REFS) return RC_EINVAL;
            for (int r = 0; r < sl.num_ref[l]; r++)
                if (sl.ref_slot[l][r] < 0 || sl.ref_slot[l][r] >= g->slots) return RC_EINVAL;
        }
        if (sl.weighted && (sl.luma_log2_denom < 0 || sl.luma_log2_denom > 7 || sl.chroma_log2_denom < 0 ||
                            sl.chroma_log2_denom > 7))
            return RC_EINVAL;
    }
    for (int i = 0; i < wctb * hctb; i++)
        if (p->ctbs[i].slice >= p->num_slices) return RC_EINVAL;
    // per 4x4 block, rows [y0, y1): the QP range, and an inter block's
    // reference indices against its slice's lists (walked one CTB-wide run
    // at a time, so that the slice is looked up once per run).  The checks
    // are OR-ed without branches and tested once per row.
    const int qmin = -6 * (g->bd - 8), run = ctb / 4;
    auto blocks = [&](int y0, int y1) -> bool {
        for (int by = y0; by < y1; by++) {
            const rc_hevc_ctb *crow = p->ctbs + (size_t)((by * 4) >> p->log2_ctb) * wctb;
            const rc_hevc_blk *brow = p->blk + (size_t)by * w4;
            const rc_hevc_mvf *frow = p->mvf + (size_t)by * w4;
            unsigned bad = 0;
            for (int cx = 0; cx < wctb; cx++) {
                const rc_hevc_slice &sl = p->slices[crow[cx].slice];
                const int n0 = sl.num_ref[0], n1 = sl.num_ref[1];
                const int bx1 = std::min(w4, (cx + 1) * run);
                for (int bx = cx * run; bx < bx1; bx++) {
                    const int qp = brow[bx].qp, fl = brow[bx].flags;
                    const int r0 = frow[bx].ref_idx[0], r1 = frow[bx].ref_idx[1];
                    const unsigned inter = (fl & (RC_HEVC_F_CODED | RC_HEVC_F_INTRA)) == RC_HEVC_F_CODED;
                    const unsigned refs = ((r0 < 0) & (r1 < 0)) | (r0 < -1) | (r1 < -1) | (r0 >= n0) | (r1 >= n1);
                    bad |= (qp < qmin) | (qp > 51) | (inter & refs);
                }
            }
            if (bad) return false;
        }
        return true;
    };
    // per transform block, [i0, i1): its size, component, mode and position,
    // and the levels it reads; OR-ed the same way
    const size_t nlev = (size_t)p->num_levels;
    const int qmax = 51 + 6 * (g->bd - 8);
    auto tus = [&](int i0, int i1) -> bool {
        unsigned bad = 0;
        for (int i = i0; i < i1; i++) {
            const rc_hevc_tu &t = p->tus[i];
            const int l2 = t.log2, n = 1 << (l2 & 7), pw = t.c ? CW : g->W, ph = t.c ? CH : g->H;
            const unsigned shape = (l2 < 2) | (l2 > 5) | (t.c > 2) | (t.mode > 34) | (t.x0 + n > pw) | (t.y0 + n > ph);
            const unsigned pcm = (size_t)t.coef_off + (size_t)n * n > nlev;
            const unsigned cbf = (t.max_x >= n) | (t.max_y >= n) |
                                 (((t.flags & RC_HEVC_TU_BYPASS) == 0) & ((t.qp < 0) | (t.qp > qmax))) |
                                 ((size_t)t.coef_off + (size_t)(t.max_x + 1) * (t.max_y + 1) > nlev);
            bad |= shape | ((t.flags & RC_HEVC_TU_PCM) ? pcm : ((t.flags & RC_HEVC_TU_CBF) != 0) & cbf);
        }
        return bad == 0;
    };
    // pictures above 1080p in pieces of 32 block rows and 8192 transform
    // blocks on the host pool
    constexpr int kRows = 32, kTus = 8192;
    if ((size_t)w4 * h4 <= (size_t)480 * 272) return blocks(0, h4) && tus(0, p->num_tus) ? 0 : RC_EINVAL;
    const int nr = (h4 + kRows - 1) / kRows, nt = (p->num_tus + kTus - 1) / kTus;
    std::atomic<bool> ok{true};
    HostPool::get().run(nr + nt, [&](int i) {
        const bool good = i < nr ? blocks(i * kRows, std::min(h4, (i + 1) * kRows))
                                 : tus((i - nr) * kTus, std::min(p->num_tus, (i - nr + 1) * kTus));
        if (!good) ok.store(false, std::memory_order_relaxed);
    });
    return ok.load() ? 0 : RC_EINVAL;
}

}  // namespace

extern "C" {

int rc_device_select(int device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return RC_ENODEV;
    }
    if (device < 0 || device >= n) return RC_EINVAL;
    return cudaSetDevice(device) == cudaSuccess ? RC_OK : RC_ECUDA;
}

int rc_stream_create(int codec, int width, int height, int bit_depth, int dpb_slots, size_t hbm_budget,
                     rc_stream **out) {
    if (!out) return RC_EINVAL;
    *out = nullptr;
    const bool shared_gpu = (codec & RC_STREAM_SHARED_GPU) != 0;
    codec &= ~RC_STREAM_SHARED_GPU;
    if (codec != RC_CODEC_H264 && codec != RC_CODEC_HEVC) return RC_EINVAL;
    if (width <= 0 || height <= 0 || width > 8192 || height > 8192 || dpb_slots <= 0 || dpb_slots > 64)
        return RC_EINVAL;
    if (codec == RC_CODEC_H264 && bit_depth != 8) return RC_EINVAL;
    if (codec == RC_CODEC_HEVC && ((bit_depth != 8 && bit_depth != 10) || (width & 7) || (height & 7)))
        return RC_EINVAL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return RC_ENODEV;
    }
    rc_stream *s = new (std::nothrow) rc_stream();
    if (!s) return RC_ENOMEM;
    s->codec = codec;
    s->bit_depth = bit_depth;
    s->slots = dpb_slots;
    s->budget = hbm_budget;
    s->bps = bit_depth > 8 ? 2 : 1;
    if (codec == RC_CODEC_H264) {
        s->mb_w = (width + 15) / 16;
        s->mb_h = (height + 15) / 16;
        s->width = s->mb_w * 16;
        s->height = s->mb_h * 16;
    } else {
        s->width = width;
        s->height = height;
        s->mb_w = s->mb_h = 1;
        s->w4 = width / 4;
        s->h4 = height / 4;
    }
    s->cw = s->width / 2;
    s->ch = s->height / 2;
    s->pitch = (int)align_up((size_t)s->width * s->bps, 128);
    s->cpitch = (int)align_up((size_t)s->cw * s->bps, 128);
    s->u_off = (size_t)s->pitch * s->height;
    s->v_off = s->u_off + (size_t)s->cpitch * s->ch;
    s->slot_bytes = align_up(s->v_off + (size_t)s->cpitch * s->ch, 256);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
    // persistent HEVC intra CTAs: about one per two 64x64 CTBs (the intra
    // wavefront's useful parallelism), at most two per SM, so that a small
    // picture leaves the GPU to the other streams that run beside it
    {
        const int c64 = ((s->width + 63) / 64) * ((s->height + 63) / 64);
        s->wave_blocks = std::max(8, std::min(s->sms * 2, c64 / 2));
        s->wave_default = s->wave_blocks;
    }
    if (const char *e = getenv("PITO_RECON_WAVE_BLOCKS")) {
        int v = atoi(e);
        if (v > 0 && v <= 4096) s->wave_blocks = v;
    }
    const int n = s->mb_w * s->mb_h;
    // HEVC alone on the GPU: the kernels' stream first when CTAs of both
    // kernel streams wait for an SM (the side stream's inter pass runs beside
    // the intra chain)
    int prio_low = 0, prio_high = 0;
    if (codec == RC_CODEC_HEVC && !shared_gpu) cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    bool ok = cudaStreamCreateWithPriority(&s->st, cudaStreamNonBlocking, prio_high) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->cst, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->dst, cudaStreamNonBlocking) == cudaSuccess;
    for (int i = 0; i < REC_SETS && ok; i++)
        ok = cudaEventCreateWithFlags(&s->set_used[i], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&s->set_ready[i], cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&s->kernels_done, cudaEventDisableTiming) == cudaSuccess &&
         cudaStreamCreateWithPriority(&s->est, cudaStreamNonBlocking, prio_low) == cudaSuccess &&
         cudaEventCreateWithFlags(&s->aux_ready, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < 2 && ok; i++) ok = cudaEventCreateWithFlags(&s->aux_used[i], cudaEventDisableTiming) == cudaSuccess;
    s->slot_dl.assign(s->slots, nullptr);
    s->slot_dl_pending.assign(s->slots, 0);
    s->slot_col.assign(s->slots, 0);
    ok = ok && cudaEventCreateWithFlags(&s->mv_ready, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < s->slots && ok; i++)
        ok = cudaEventCreateWithFlags(&s->slot_dl[i], cudaEventDisableTiming) == cudaSuccess;
    ok = ok && dev_alloc(s, (void **)&s->dpb, s->slot_bytes * s->slots);
    ok = ok && cudaMalloc(&s->counter, 64) == cudaSuccess;
    ok = ok && cudaMemsetAsync(s->counter, 0, 64, s->st) == cudaSuccess;
    ok = ok && cudaMalloc(&s->error, 64) == cudaSuccess;
    ok = ok && cudaMalloc(&s->ls, (2304 + 2304 * 4) * sizeof(int32_t)) == cudaSuccess;
    ok = ok && cudaMalloc(&s->rowprog, (size_t)s->mb_h * sizeof(uint32_t)) == cudaSuccess;
    ok = ok && cudaMalloc(&s->irowprog, (size_t)s->mb_h * sizeof(uint32_t)) == cudaSuccess;
    ok = ok && cudaMalloc(&s->crowprog, (size_t)s->mb_h * sizeof(uint32_t)) == cudaSuccess;
    if (codec == RC_CODEC_H264) {
        for (int i = 0; i < 2; i++)
            ok = ok && dev_alloc(s, (void **)&s->edges[i], (size_t)n * RC_EDGE_WORDS * sizeof(uint32_t));
        ok = ok && dev_alloc(s, (void **)&s->iinfo, (size_t)n * sizeof(IntraInfo));
        ok = ok && dev_alloc(s, (void **)&s->ires, (size_t)n * 384 * sizeof(int16_t));
        // band kernel: per band of RC_H264_BAND_ROWS MB rows one CTA, or two or
        // three when the roles fit apart; all resident (cooperative launch)
        const int bands = (s->mb_h + RC_H264_BAND_ROWS - 1) / RC_H264_BAND_ROWS;
        const int cap = ok ? rc_h264_band_capacity(s->mb_w) : 0;
        ok = ok && bands <= cap;
        s->band_split = 3 * bands <= cap ? 3 : 2 * bands <= cap ? 2 : 1;
    }
    if (codec == RC_CODEC_HEVC) {
        const size_t nres = (size_t)s->width * s->height + 2 * (size_t)s->cw * s->ch;
        // a luma group per four samples and a chroma group per two
        s->late_cap = (size_t)s->width * s->height / 4 + (size_t)s->cw * s->ch;
        ok = ok && cudaMalloc(&s->late_count, 2 * sizeof(uint32_t)) == cudaSuccess;
        for (int i = 0; i < 2; i++) {
            ok = ok && dev_alloc(s, (void **)&s->late_items[i], s->late_cap * sizeof(uint32_t));
            ok = ok && dev_alloc(s, (void **)&s->work[i], s->slot_bytes);
            ok = ok && cudaEventCreateWithFlags(&s->work_free[i], cudaEventDisableTiming) == cudaSuccess;
            ok = ok && cudaMemsetAsync(s->work[i], 0, s->slot_bytes, s->st) == cudaSuccess;
        }
        for (int i = 0; i < 2; i++) ok = ok && dev_alloc(s, (void **)&s->res[i], nres * sizeof(int16_t));
        ok = ok && dev_alloc(s, (void **)&s->ready, 3 * (size_t)s->w4 * s->h4 * sizeof(uint32_t));
        s->nctb_max = (size_t)((s->width + 15) / 16) * ((s->height + 15) / 16);
        for (int i = 0; i < 2; i++) ok = ok && dev_alloc(s, (void **)&s->ctb_ord[i], 4 * s->nctb_max * sizeof(uint32_t));
        ok = ok && cudaMemsetAsync(s->ready, 0, 3 * (size_t)s->w4 * s->h4 * sizeof(uint32_t), s->st) == cudaSuccess;
    }
    for (int i = 0; i < 2 && ok; i++) ok = cudaEventCreateWithFlags(&s->staged[i], cudaEventDisableTiming) == cudaSuccess;
    if (ok) {
        ok = cudaMemsetAsync(s->dpb, 0, s->slot_bytes * s->slots, s->st) == cudaSuccess &&
             cudaMemsetAsync(s->rowprog, 0, (size_t)s->mb_h * sizeof(uint32_t), s->st) == cudaSuccess &&
             cudaMemsetAsync(s->irowprog, 0, (size_t)s->mb_h * sizeof(uint32_t), s->st) == cudaSuccess &&
             cudaMemsetAsync(s->crowprog, 0, (size_t)s->mb_h * sizeof(uint32_t), s->st) == cudaSuccess &&
             cudaMemsetAsync(s->error, 0, 64, s->st) == cudaSuccess &&
             cudaStreamSynchronize(s->st) == cudaSuccess;
    }
    if (!ok) {
        int rc = (s->budget && s->held + s->slot_bytes * s->slots > s->budget) ? RC_ENOMEM : RC_ECUDA;
        cudaGetLastError();
        destroy(s);
        return rc;
    }
    *out = s;
    return RC_OK;
}

void rc_stream_destroy(rc_stream *s) { destroy(s); }

int rc_h264_validate(int mb_w, int mb_h, int dpb_slots, const rc_h264_picture *pic) {
    if (mb_w <= 0 || mb_h <= 0 || dpb_slots <= 0 || !pic) return RC_EINVAL;
    Geo g{mb_w, mb_h, dpb_slots};
    return validate_h264(&g, pic);
}

int rc_h264_submit(rc_stream *s, const rc_h264_picture *pic, int out_slot) {
    if (!s || !pic || s->codec != RC_CODEC_H264) return RC_EINVAL;
    if (out_slot < 0 || out_slot >= s->slots) return RC_EINVAL;
    if (pic->mem != RC_MEM_HOST && pic->mem != RC_MEM_DEVICE) return RC_EINVAL;
    const int n = s->mb_w * s->mb_h;
    int rc;
    if (pic->mem == RC_MEM_HOST) {
        Geo g{s->mb_w, s->mb_h, s->slots};
        if ((rc = validate_h264(&g, pic)) != 0) return rc;
    } else if (!pic->mbs || !pic->slices || pic->num_slices <= 0) {
        return RC_EINVAL;
    }
    // motion syntax: host records only, and every B slice's co-located slot
    // must hold motion stored by an earlier picture with motion syntax
    const bool derive = pic->motion != nullptr;
    if (derive) {
        if (pic->mem != RC_MEM_HOST) return RC_EINVAL;
        for (int i = 0; i < pic->num_slices; i++)
            if (pic->slice_motion[i].b_slice && !s->slot_col[pic->slice_motion[i].col_slot]) return RC_EINVAL;
        if (!s->col && !dev_alloc(s, (void **)&s->col, (size_t)s->slots * n * RC_COLMB_BYTES)) return RC_ENOMEM;
        if (!s->mvprog) {
            if (!dev_alloc(s, (void **)&s->mvprog, (size_t)s->mb_h * sizeof(uint32_t))) return RC_ENOMEM;
            if (cudaMemsetAsync(s->mvprog, 0, (size_t)s->mb_h * sizeof(uint32_t), s->est) != cudaSuccess)
                return cuda_fail(s);
        }
    }
    // Groups: a picture joins the pending group unless it writes a slot that
    // a pending picture writes or reads.
    const bool grouped = s->group > 1;
    std::vector<int> refs;
    if (grouped) {
        if (pic->mem == RC_MEM_HOST) refs = h264_ref_slots(pic);
        else if ((rc = h264_device_ref_slots(s, pic, refs)) != 0) return rc;
        bool clash = false;
        for (size_t i = 0; i < s->pending.size(); i++) {
            const auto &r = s->pending_refs[i];
            clash = clash || s->pending[i].out_slot == out_slot || std::find(r.begin(), r.end(), out_slot) != r.end();
        }
        if (clash && (rc = h264_flush(s)) != 0) return rc;
    } else if ((rc = h264_flush(s)) != 0) {
        return rc;
    }
    // level-scale tables (per PPS), uploaded only when they change.  The copy
    // goes on the stream itself: the stream does not order with the legacy
    // default stream, and a pageable cudaMemcpy may return before its DMA has
    // landed.  Its source, ls_host, lives until the next change, which first
    // launches the pending group and waits for the stream.
    {
        // compare the scaling lists (480 bytes), not the tables made from them
        uint8_t key[sizeof s->ls_key] = {0};
        key[0] = pic->scaling4 != nullptr;
        key[1] = pic->scaling8 != nullptr;
        if (pic->scaling4) memcpy(key + 2, pic->scaling4, 96);
        if (pic->scaling8) memcpy(key + 2 + 96, pic->scaling8, 384);
        if (!s->ls_valid || memcmp(key, s->ls_key, sizeof key) != 0) {
            std::vector<int32_t> ls(2304 + 2304 * 4);
            h264_level_scale(pic->scaling4, pic->scaling8, ls.data(), ls.data() + 2304);
            if ((rc = h264_flush(s)) != 0) return rc;
            if (cudaStreamSynchronize(s->st) != cudaSuccess) return cuda_fail(s);
            memcpy(s->ls_key, key, sizeof key);
            s->ls_host.swap(ls);
            if (cudaMemcpyAsync(s->ls, s->ls_host.data(), s->ls_host.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                                s->st) != cudaSuccess) {
                s->ls_valid = false;
                return cuda_fail(s);
            }
            s->ls_valid = true;
        }
    }
    H264Launch L;
    memset(&L, 0, sizeof L);
    // record set: none of the pending pictures uses it (at most group - 1
    // pend while 2 x group sets rotate)
    const int k = s->submits % s->nsets;
    if (pic->mem == RC_MEM_HOST) {
        const size_t b_mbs = sizeof(rc_h264_mb) * n, b_sl = sizeof(rc_h264_slice) * pic->num_slices;
        const size_t b_w = sizeof(rc_h264_weight) * pic->num_weights, b_lv = sizeof(int16_t) * pic->num_levels;
        Part parts[6] = {{&s->mbs[k], pic->mbs, b_mbs}, {&s->slices[k], pic->slices, b_sl},
                         {&s->weights[k], pic->weights, b_w}, {&s->levels[k], pic->levels, b_lv},
                         {&s->motion[k], pic->motion, derive ? sizeof(rc_h264_motion) * n : 0},
                         {&s->smotion[k], pic->slice_motion, derive ? sizeof(rc_h264_slice_motion) * pic->num_slices : 0}};
        if ((rc = set_begin(s, k)) != 0 || (rc = upload(s, parts, derive ? 6 : 4, s->cst)) != 0 ||
            (rc = set_end(s, k)) != 0)
            return rc;
        L.mbs = (const rc_h264_mb *)s->mbs[k].p;
        L.slices = (const rc_h264_slice *)s->slices[k].p;
        L.weights = (const rc_h264_weight *)s->weights[k].p;
        L.levels = (const int16_t *)s->levels[k].p;
    } else {
        L.mbs = pic->mbs;
        L.slices = pic->slices;
        L.weights = pic->weights;
        L.levels = pic->levels;
    }
    L.num_levels = pic->num_levels;
    L.num_slices = pic->num_slices;
    L.num_weights = pic->num_weights;
    L.ls4 = s->ls;
    L.ls8 = s->ls + 2304;
    L.dpb = s->dpb;
    L.slot_bytes = s->slot_bytes;
    L.u_off = s->u_off;
    L.v_off = s->v_off;
    L.dpb_slots = s->slots;
    L.out_slot = out_slot;
    L.mb_w = s->mb_w;
    L.mb_h = s->mb_h;
    L.W = s->width;
    L.H = s->height;
    L.CW = s->cw;
    L.CH = s->ch;
    L.pitch = s->pitch;
    L.cpitch = s->cpitch;
    L.constrained_intra = pic->constrained_intra_pred;
    L.epoch = ++s->epoch;
    L.error = s->error;
    L.wait_limit = s->wait_limit;
    L.db = nullptr;
    if ((rc = slot_begin(s, out_slot)) != 0) return rc;
    // motion derived from syntax, on the side stream after the records'
    // upload (the edge kernel, behind it there, and the MB kernel, which
    // waits for mv_ready, read the vectors it writes); the slot's co-located
    // motion is then this picture's
    if (derive) {
        L.mbs_out = (rc_h264_mb *)s->mbs[k].p;
        L.motion = (const rc_h264_motion *)s->motion[k].p;
        L.smotion = (const rc_h264_slice_motion *)s->smotion[k].p;
        L.col = s->col;
        L.col_stride = (unsigned long long)n * RC_COLMB_BYTES;
        L.mvprog = s->mvprog;
        int mrc = 0;
        if (cudaStreamWaitEvent(s->est, s->set_ready[k], 0) != cudaSuccess) return cuda_fail(s);
        timed(s, RC_KERNEL_H264_MV, [&] { mrc = rc_launch_h264_mv(L, s->est); }, s->est);
        if (mrc != 0 || cudaEventRecord(s->mv_ready, s->est) != cudaSuccess ||
            cudaStreamWaitEvent(s->st, s->mv_ready, 0) != cudaSuccess)
            return cuda_fail(s);
    }
    s->slot_col[out_slot] = derive;
    if (grouped) {
        // group position j: its scratch, and the rows of the pending
        // pictures it references to wait for
        const int j = (int)s->pending.size();
        const size_t mbs = (size_t)n;
        L.rowprog = s->g_rowprog + (size_t)j * s->mb_h;
        L.irowprog = s->g_irowprog + (size_t)j * s->mb_h;
        L.mbdone = s->g_mbdone + (size_t)j * mbs;
        L.edges = s->g_edges + (size_t)j * mbs * RC_EDGE_WORDS;
        L.iinfo = s->g_iinfo + (size_t)j * mbs;
        L.ires = s->g_ires + (size_t)j * mbs * 384;
        L.bottom = s->g_bottom + (size_t)j * mbs * 32;
        L.refprog = s->g_refprog + (size_t)j * s->mb_h * RC_REFPROG_STRIDE;
        for (int i = 0; i < j; i++) {
            const H264Launch &q = s->pending[i];
            if (std::find(refs.begin(), refs.end(), q.out_slot) == refs.end()) continue;
            L.wait_slot[L.nwait] = q.out_slot;
            L.wait_epoch[L.nwait] = q.epoch;
            L.wait_refprog[L.nwait] = q.refprog;
            L.nwait++;
        }
        // the pre-pass, from the records alone: edge words, every MB's
        // residual, intra parameters and I_PCM samples (on the stream, so
        // after the previous group's launch, which read this position's
        // buffers, and before this group's)
        L.residual_only = 1;
        timed(s, RC_KERNEL_H264_EDGE, [&] { rc_launch_h264_edge(L, s->st); });
        timed(s, RC_KERNEL_H264_MB, [&] { rc_launch_h264_mb(L, s->st); });
        L.residual_only = 0;
        s->pending.push_back(L);
        s->pending_refs.push_back(std::move(refs));
        s->pending_sets.push_back(pic->mem == RC_MEM_HOST ? k : -1);
        s->submits++;
        if ((int)s->pending.size() >= s->group && (rc = h264_flush(s)) != 0) return rc;
        if (cudaGetLastError() != cudaSuccess) return cuda_fail(s);
        return RC_OK;
    }
    const int ek = s->submits & 1;
    L.edges = s->edges[ek];
    L.rowprog = s->rowprog;
    L.irowprog = s->irowprog;
    L.crowprog = s->crowprog;
    L.band_split = s->band_split;
    L.iinfo = s->iinfo;
    L.ires = s->ires;
    // the edge kernel: after the picture's records (host records: their
    // upload) and after the band kernel that last read this set of edge words
    {
        bool ok = true;
        if (pic->mem == RC_MEM_HOST) ok = cudaStreamWaitEvent(s->est, s->set_ready[k], 0) == cudaSuccess;
        if (s->aux_busy[ek]) ok = ok && cudaStreamWaitEvent(s->est, s->aux_used[ek], 0) == cudaSuccess;
        if (!ok) return cuda_fail(s);
    }
    timed(s, RC_KERNEL_H264_EDGE, [&] { rc_launch_h264_edge(L, s->est); }, s->est);
    if (cudaEventRecord(s->aux_ready, s->est) != cudaSuccess) return cuda_fail(s);
    timed(s, RC_KERNEL_H264_MB, [&] { rc_launch_h264_mb(L, s->st); });
    if (cudaStreamWaitEvent(s->st, s->aux_ready, 0) != cudaSuccess) return cuda_fail(s);
    int lrc = 0;
    timed(s, RC_KERNEL_H264_BAND, [&] { lrc = rc_launch_h264_band(L, s->st); });
    if (lrc != 0) return cuda_fail(s);
    if (cudaEventRecord(s->aux_used[ek], s->st) != cudaSuccess) return cuda_fail(s);
    s->aux_busy[ek] = true;
    if (pic->mem == RC_MEM_HOST && (rc = set_release(s, k)) != 0) return rc;
    s->submits++;
    if (cudaGetLastError() != cudaSuccess) return cuda_fail(s);
    return RC_OK;
}

int rc_stream_set_h264_group(rc_stream *s, int pictures) {
    if (!s || s->codec != RC_CODEC_H264 || pictures < 0 || pictures > RC_H264_GROUP_MAX) return RC_EINVAL;
    int rc;
    if ((rc = h264_flush(s)) != 0) return rc;
    if (pictures == 0) pictures = RC_H264_GROUP_DEFAULT;
    // the band CTAs of a group take at most two thirds of the launch's CTAs
    const int bands = (s->mb_h + RC_H264_BAND_ROWS - 1) / RC_H264_BAND_ROWS;
    const int cap = pictures > 1 ? rc_h264_group_capacity(s->mb_w) : 0;
    while (pictures > 1 && pictures * bands * 3 > cap * 2) pictures--;
    if (pictures > 1 && (rc = group_alloc(s, pictures)) != 0) return rc;
    s->group = pictures;
    s->group_ctas = pictures > 1 ? cap : 0;
    s->group_workers = RC_H264_GROUP_WORKERS;
    if (const char *e = getenv("PITO_RECON_GROUP_WORKERS")) {
        const int v = atoi(e);
        if (v > 0 && v <= 4096) s->group_workers = v;
    }
    s->nsets = pictures > 1 ? 2 * pictures : 2;
    return pictures;
}

int rc_hevc_validate(int width, int height, int bit_depth, int dpb_slots, const rc_hevc_picture *pic) {
    if (!pic || width <= 0 || height <= 0 || (width & 7) || (height & 7) || dpb_slots <= 0 ||
        (bit_depth != 8 && bit_depth != 10))
        return RC_EINVAL;
    HGeo g{width, height, bit_depth, dpb_slots};
    return validate_hevc(&g, pic);
}

int rc_hevc_submit(rc_stream *s, const rc_hevc_picture *pic, int out_slot) {
    if (!s || !pic || s->codec != RC_CODEC_HEVC) return RC_EINVAL;
    if (out_slot < 0 || out_slot >= s->slots) return RC_EINVAL;
    if (pic->mem != RC_MEM_HOST && pic->mem != RC_MEM_DEVICE) return RC_EINVAL;
    if (pic->log2_ctb < 4 || pic->log2_ctb > 6) return RC_EINVAL;
    int rc;
    const int ctb = 1 << pic->log2_ctb, wctb = (s->width + ctb - 1) / ctb, hctb = (s->height + ctb - 1) / ctb;
    const size_t nblk = (size_t)s->w4 * s->h4;
    const size_t b_scal = 6 * (16 + 64 + 256 + 1024);
    HevcLaunch L;
    memset(&L, 0, sizeof L);
    if (pic->scaling) {  // scaling factors are host memory in both modes; uploaded when they change
        const uint8_t *sf = (const uint8_t *)pic->scaling;
        if (s->scal_host.size() != b_scal || memcmp(s->scal_host.data(), sf, b_scal) != 0) {
            Part sp{&s->scaling, pic->scaling, b_scal};  // on the side stream, after the residual kernels before
            if ((rc = upload(s, &sp, 1, s->est)) != 0) {
                s->scal_host.clear();
                return rc;
            }
            s->scal_host.assign(sf, sf + b_scal);
        }
        L.scaling = (const uint8_t *)s->scaling.p;
    }
    if (pic->mem == RC_MEM_HOST) {
        HGeo g{s->width, s->height, s->bit_depth, s->slots};
        if ((rc = validate_hevc(&g, pic)) != 0) return rc;
        const int k = s->submits & 1;
        Part parts[6] = {{&s->ctbs[k], pic->ctbs, sizeof(rc_hevc_ctb) * wctb * hctb},
                         {&s->blk[k], pic->blk, sizeof(rc_hevc_blk) * nblk},
                         {&s->mvf[k], pic->mvf, sizeof(rc_hevc_mvf) * nblk},
                         {&s->tus[k], pic->tus, sizeof(rc_hevc_tu) * pic->num_tus},
                         {&s->hslices[k], pic->slices, sizeof(rc_hevc_slice) * pic->num_slices},
                         {&s->levels[k], pic->levels, sizeof(int16_t) * pic->num_levels}};
        if ((rc = set_begin(s, k)) != 0 || (rc = upload(s, parts, 6, s->cst)) != 0 || (rc = set_end(s, k)) != 0)
            return rc;
        L.ctbs = (const rc_hevc_ctb *)s->ctbs[k].p;
        L.blk = (const rc_hevc_blk *)s->blk[k].p;
        L.mvf = (const rc_hevc_mvf *)s->mvf[k].p;
        L.tus = (const rc_hevc_tu *)s->tus[k].p;
        L.slices = (const rc_hevc_slice *)s->hslices[k].p;
        L.levels = (const int16_t *)s->levels[k].p;
    } else {
        if (!pic->ctbs || !pic->blk || !pic->mvf || !pic->slices || pic->num_slices <= 0) return RC_EINVAL;
        L.ctbs = pic->ctbs;
        L.blk = pic->blk;
        L.mvf = pic->mvf;
        L.tus = pic->tus;
        L.slices = pic->slices;
        L.levels = pic->levels;
    }
    L.num_levels = pic->num_levels;
    L.num_tus = pic->num_tus;
    L.num_slices = pic->num_slices;
    L.W = s->width;
    L.H = s->height;
    L.CW = s->cw;
    L.CH = s->ch;
    L.bd = s->bit_depth;
    L.w4 = s->w4;
    L.h4 = s->h4;
    L.log2ctb = pic->log2_ctb;
    L.wctb = wctb;
    L.hctb = hctb;
    L.constrained_intra = pic->constrained_intra_pred;
    L.strong_intra = pic->strong_intra_smoothing;
    L.lf_across_tiles = pic->loop_filter_across_tiles;
    L.cb_qp_offset = pic->cb_qp_offset;
    L.cr_qp_offset = pic->cr_qp_offset;
    L.dpb = s->dpb;
    L.slot_bytes = s->slot_bytes;
    L.u_off = s->u_off;
    L.v_off = s->v_off;
    L.dpb_slots = s->slots;
    L.out_slot = out_slot;
    L.pitch = s->pitch;
    L.cpitch = s->cpitch;
    const int ak = s->submits & 1;
    L.work = s->work[ak];
    L.res = s->res[ak];
    L.ready = s->ready;
    if ((size_t)wctb * hctb > s->nctb_max || wctb + 2 * hctb > 2048) return RC_EINVAL;
    L.ctb_first = s->ctb_ord[ak];
    L.ctb_end = s->ctb_ord[ak] + (size_t)wctb * hctb;
    L.ctb_base = s->ctb_ord[0] + 2 * s->nctb_max;  // written and read on the kernels' stream
    L.ctb_nintra = s->ctb_ord[ak] + 3 * s->nctb_max;
    L.counter = s->counter;
    L.error = s->error;
    L.epoch = ++s->epoch;
    L.wait_limit = s->wait_limit;
    if ((rc = slot_begin(s, out_slot)) != 0) return rc;
    // the residual kernel: after the picture's records (host records: their
    // upload) and after the intra kernel that last read this set
    {
        bool ok = true;
        if (pic->mem == RC_MEM_HOST) ok = cudaStreamWaitEvent(s->est, s->set_ready[s->submits & 1], 0) == cudaSuccess;
        if (s->aux_busy[ak]) ok = ok && cudaStreamWaitEvent(s->est, s->aux_used[ak], 0) == cudaSuccess;
        if (!ok) return cuda_fail(s);
    }
    timed(s, RC_KERNEL_HEVC_RESIDUAL, [&] { rc_launch_hevc_residual(L, s->est); }, s->est);
    // inter prediction in two passes (the decoder's frame threading waits
    // the same way for the reference rows a block reads,
    // src/hevc/decoder.rs:508-528): on the side stream, once this work
    // picture's last loop filter is done (so every picture before the
    // previous one is final), the units that do not read the previous
    // picture; on the main stream, after the previous picture, the units that
    // read it.  A picture that does not reference the previous one (host
    // records show it) needs no second pass.
    int late = s->hevc_prev_slot;
    if (late >= 0 && pic->mem == RC_MEM_HOST) {
        bool reads = false;
        for (int i = 0; i < pic->num_slices && !reads; i++)
            for (int l = 0; l < 2 && !reads; l++)
                for (int r = 0; r < pic->slices[i].num_ref[l] && r < RC_HEVC_MAX_REFS; r++)
                    reads = reads || pic->slices[i].ref_slot[l][r] == late;
        if (!reads) late = -1;
    }
    {
        bool ok = true;
        if (s->work_busy[ak]) ok = cudaStreamWaitEvent(s->est, s->work_free[ak], 0) == cudaSuccess;
        if (s->hevc_ext) {  // a slot the caller wrote on the main stream: after it
            ok = ok && cudaEventRecord(s->aux_ready, s->st) == cudaSuccess &&
                 cudaStreamWaitEvent(s->est, s->aux_ready, 0) == cudaSuccess;
            s->hevc_ext = false;
        }
        if (!ok) return cuda_fail(s);
    }
    if (s->height >= 16384 || s->width >= 65536) late = -1;  // beyond the list items' fields: one pass
    L.late_slot = late;
    L.inter_pass = late >= 0 ? 1 : 0;
    L.late_items = s->late_items[ak];
    L.late_count = s->late_count + ak;
    L.late_cap = (uint32_t)s->late_cap;
    L.lf_rows = s->lf_rows;
    timed(s, RC_KERNEL_HEVC_INTER, [&] { rc_launch_hevc_inter(L, s->est); }, s->est);
    if (cudaEventRecord(s->aux_ready, s->est) != cudaSuccess || cudaStreamWaitEvent(s->st, s->aux_ready, 0) != cudaSuccess)
        return cuda_fail(s);
    if (late >= 0) {
        L.inter_pass = 2;
        timed(s, RC_KERNEL_HEVC_INTER_LATE, [&] { rc_launch_hevc_inter(L, s->st); });
    }
    // the intra task order depends on the CTB grid alone: built again only
    // when a picture's CTB size changes it
    const bool order = wctb != s->ord_wctb || hctb != s->ord_hctb;
    s->ord_wctb = wctb;
    s->ord_hctb = hctb;
    timed(s, RC_KERNEL_HEVC_INTRA, [&] { rc_launch_hevc_intra(L, s->st, s->wave_blocks, order); });
    if (cudaEventRecord(s->aux_used[ak], s->st) != cudaSuccess) return cuda_fail(s);
    s->aux_busy[ak] = true;
    timed(s, RC_KERNEL_HEVC_LOOPFILTER, [&] { rc_launch_hevc_loopfilter(L, s->st); });
    if (cudaEventRecord(s->work_free[ak], s->st) != cudaSuccess) return cuda_fail(s);
    s->work_busy[ak] = true;
    s->hevc_prev_slot = out_slot;
    if (order) s->launches += 1;  // the intra task order
    if (pic->mem == RC_MEM_HOST && (rc = set_release(s, s->submits & 1)) != 0) return rc;
    s->submits++;
    if (cudaGetLastError() != cudaSuccess) return cuda_fail(s);
    return RC_OK;
}

int rc_stream_sync(rc_stream *s) {
    if (!s) return RC_EINVAL;
    h264_flush(s);
    if (cudaStreamSynchronize(s->st) != cudaSuccess || cudaStreamSynchronize(s->cst) != cudaSuccess ||
        cudaStreamSynchronize(s->dst) != cudaSuccess || (s->est && cudaStreamSynchronize(s->est) != cudaSuccess))
        return cuda_fail(s);
    uint32_t e = 0;
    if (cudaMemcpyAsync(&e, s->error, sizeof e, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
        cudaStreamSynchronize(s->st) != cudaSuccess)
        return cuda_fail(s);
    if (e) {
        if (!s->sticky) s->sticky = (e & RC_DEV_ERR_TIMEOUT) ? RC_ETIMEOUT : RC_EDEVICE;
        // on the stream, so that the next launch cannot overtake the reset
        cudaMemsetAsync(s->error, 0, sizeof e, s->st);
    }
    return s->sticky;
}

int rc_stream_error(rc_stream *s) {
    if (!s) return RC_EINVAL;
    int e = rc_stream_sync(s);
    s->sticky = 0;
    return e;
}

static int download(rc_stream *s, int slot, int x, int y, int w, int h, void *out_y, void *out_u, void *out_v,
                    bool wait) {
    if (!s || slot < 0 || slot >= s->slots || !out_y || !out_u || !out_v) return RC_EINVAL;
    int cx = x / 2, cy = y / 2, ccw = (w + 1) / 2, cch = (h + 1) / 2;
    auto fits = [](long at, long n, long size) { return n > 0 && at >= 0 && at + n <= size; };
    if (!(fits(x, w, s->width) && fits(y, h, s->height) && fits(cx, ccw, s->cw) && fits(cy, cch, s->ch)))
        return RC_EINVAL;
    // copy_cropped's bounds rule above; an asynchronous download of a slot
    // that a queued picture writes waits for that picture's group to launch,
    // anything else goes now
    bool queued = false;
    for (const auto &q : s->pending) queued = queued || q.out_slot == slot;
    if (queued && !wait) {
        s->pending_dl.push_back({slot, x, y, w, h, out_y, out_u, out_v});
        return RC_OK;
    }
    int rc;
    if (queued && (rc = h264_flush(s)) != 0) return rc;
    if ((rc = issue_download(s, slot, x, y, w, h, out_y, out_u, out_v)) != 0) return rc;
    return !wait || cudaStreamSynchronize(s->dst) == cudaSuccess ? RC_OK : cuda_fail(s);
}

int rc_picture_download(rc_stream *s, int slot, int x, int y, int w, int h, void *out_y, void *out_u, void *out_v) {
    return download(s, slot, x, y, w, h, out_y, out_u, out_v, true);
}

int rc_picture_download_async(rc_stream *s, int slot, int x, int y, int w, int h, void *out_y, void *out_u,
                              void *out_v) {
    return download(s, slot, x, y, w, h, out_y, out_u, out_v, false);
}

int rc_stream_set_intra_ctas(rc_stream *s, int ctas) {
    if (!s || ctas > 4096) return RC_EINVAL;
    s->wave_blocks = ctas <= 0 ? s->wave_default : ctas;
    return RC_OK;
}

int rc_stream_intra_ctas(rc_stream *s) { return s && s->codec == RC_CODEC_HEVC ? s->wave_blocks : 0; }

int rc_stream_set_lf_tile(rc_stream *s, int rows) {
    if (!s || s->codec != RC_CODEC_HEVC || (rows != 16 && rows != 32 && rows != 64)) return RC_EINVAL;
    s->lf_rows = rows;
    return RC_OK;
}
int rc_stream_lf_tile(rc_stream *s) { return s && s->codec == RC_CODEC_HEVC ? s->lf_rows : 0; }

int rc_stream_set_wait_limit(rc_stream *s, unsigned int limit) {
    if (!s) return RC_EINVAL;
    s->wait_limit = limit ? limit : RC_WAIT_LIMIT;
    return RC_OK;
}

int rc_stream_profile(rc_stream *s, int enable) {
    if (!s) return RC_EINVAL;
    h264_flush(s);
    if (cudaStreamSynchronize(s->st) != cudaSuccess || (s->est && cudaStreamSynchronize(s->est) != cudaSuccess))
        return cuda_fail(s);
    drain_profile(s);
    for (int k = 0; k < RC_KERNEL_COUNT; k++) {
        s->prof_ms[k] = 0;
        s->prof_n[k] = 0;
    }
    s->profiling = enable != 0;
    return RC_OK;
}

int rc_stream_profile_read(rc_stream *s, double *ms, long long *launches, int max_kernels) {
    if (!s || max_kernels < 0) return RC_EINVAL;
    h264_flush(s);
    if (cudaStreamSynchronize(s->st) != cudaSuccess || (s->est && cudaStreamSynchronize(s->est) != cudaSuccess))
        return cuda_fail(s);
    drain_profile(s);
    int n = std::min(max_kernels, RC_KERNEL_COUNT);
    for (int k = 0; k < n; k++) {
        if (ms) ms[k] = s->prof_ms[k];
        if (launches) launches[k] = s->prof_n[k];
    }
    return n;
}

int rc_picture_upload(rc_stream *s, int slot, const void *py, const void *pu, const void *pv) {
    if (!s || slot < 0 || slot >= s->slots || !py || !pu || !pv) return RC_EINVAL;
    const int bps = s->bps;
    uint8_t *base = s->dpb + (size_t)slot * s->slot_bytes;
    if (h264_flush(s) != 0 || slot_begin(s, slot) != 0) return cuda_fail(s);
    // stream-ordered copies (the stream does not order with the legacy default
    // stream), complete before returning so that the caller may free its planes
    bool ok = cudaMemcpy2DAsync(base, s->pitch, py, (size_t)s->width * bps, (size_t)s->width * bps, s->height,
                                cudaMemcpyHostToDevice, s->st) == cudaSuccess &&
              cudaMemcpy2DAsync(base + s->u_off, s->cpitch, pu, (size_t)s->cw * bps, (size_t)s->cw * bps, s->ch,
                                cudaMemcpyHostToDevice, s->st) == cudaSuccess &&
              cudaMemcpy2DAsync(base + s->v_off, s->cpitch, pv, (size_t)s->cw * bps, (size_t)s->cw * bps, s->ch,
                                cudaMemcpyHostToDevice, s->st) == cudaSuccess &&
              cudaStreamSynchronize(s->st) == cudaSuccess;
    return ok ? RC_OK : cuda_fail(s);
}

int rc_stream_geometry(rc_stream *s, int *coded_w, int *coded_h, int *luma_pitch, int *chroma_pitch) {
    if (!s) return RC_EINVAL;
    if (coded_w) *coded_w = s->width;
    if (coded_h) *coded_h = s->height;
    if (luma_pitch) *luma_pitch = s->pitch;
    if (chroma_pitch) *chroma_pitch = s->cpitch;
    return RC_OK;
}

int rc_picture_device_planes(rc_stream *s, int slot, void **y, void **u, void **v) {
    if (!s || slot < 0 || slot >= s->slots) return RC_EINVAL;
    int rc;
    if ((rc = h264_flush(s)) != 0) return rc;
    uint8_t *base = s->dpb + (size_t)slot * s->slot_bytes;
    s->hevc_ext = true;
    if (y) *y = base;
    if (u) *u = base + s->u_off;
    if (v) *v = base + s->v_off;
    return RC_OK;
}

long long rc_stream_launches(rc_stream *s) { return s ? s->launches : 0; }

void *rc_stream_cuda_stream(rc_stream *s) {
    if (!s) return nullptr;
    h264_flush(s);  // a launch error stays in the sticky word
    s->hevc_ext = true;
    return (void *)s->st;
}

size_t rc_stream_device_bytes(rc_stream *s) { return s ? s->held : 0; }

int rc_stream_mark(rc_stream *s, unsigned long long *mark) {
    if (!s || !mark) return RC_EINVAL;
    int rc;
    if ((rc = h264_flush(s)) != 0) return rc;
    cudaEvent_t e = nullptr;
    if (!s->mark_free.empty()) {
        e = s->mark_free.back();
        s->mark_free.pop_back();
    } else if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        return cuda_fail(s);
    }
    if (cudaEventRecord(e, s->st) != cudaSuccess) {
        s->mark_free.push_back(e);
        return cuda_fail(s);
    }
    s->marks.push_back({++s->next_mark, e});
    *mark = s->next_mark;
    return RC_OK;
}

int rc_stream_mark_done(rc_stream *s, unsigned long long mark) {
    if (!s || mark == 0 || mark > s->next_mark) return RC_EINVAL;
    while (!s->marks.empty()) {
        cudaError_t q = cudaEventQuery(s->marks.front().second);
        if (q == cudaErrorNotReady) break;
        if (q != cudaSuccess) return cuda_fail(s);
        s->marks_done = s->marks.front().first;
        s->mark_free.push_back(s->marks.front().second);
        s->marks.pop_front();
    }
    return mark <= s->marks_done ? 1 : 0;
}

}  // extern "C"
