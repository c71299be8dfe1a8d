// output_order.cpp — output order of decoded pictures (DPB "bumping"), the
// host half of the C ABI's rc_output_* calls.
//
// The engine reconstructs each picture into the DPB slot it is given; a
// decoder built on it must still hand pictures to its caller in output
// order.  This is the picture output process of the reference's decoded
// picture buffers (src/syntax/hevc/dpb.rs:76-160: bump, bump_before_decode,
// insert; src/syntax/h264/dpb.rs:73-132, 391-478: bump, idr, store_picture),
// which follow H.265 C.5.2.2-C.5.2.4 and H.264 C.4.5.3:
//
//  * before a picture is decoded: a picture that starts a new coded video
//    sequence (HEVC IRAP with NoRaslOutputFlag, H.264 IDR) empties the DPB,
//    outputting every waiting picture in POC order unless
//    no_output_of_prior_pics is set; otherwise pictures neither waiting for
//    output nor used for reference leave, and the DPB bumps while more
//    pictures wait than the reorder limit allows, one has waited longer
//    than the latency limit, or the DPB is at capacity;
//  * after it is decoded, it enters (waiting for output if its output flag
//    is set), every waiting picture's latency count grows, and the DPB
//    bumps again while over the reorder or latency limit;
//  * a bump outputs the waiting picture with the smallest POC.
//
// Pictures are named by caller ids (e.g. a DPB slot and a frame number).
#include <stdint.h>

#include <algorithm>
#include <new>
#include <vector>

#include "../../include/pito_recon.h"

struct rc_output_dpb {
    struct Entry {
        uint64_t id;
        int32_t poc;
        uint32_t latency;
        bool waiting;    // needed for output
        bool reference;  // used for reference
    };
    int capacity = 16, max_reorder = 16;
    uint32_t max_latency = 0;  // 0: no latency limit
    std::vector<Entry> entries;
};

namespace {

struct Sink {
    uint64_t *ids;
    int n;
    void put(uint64_t id) { ids[n++] = id; }
};

int num_waiting(const rc_output_dpb *d) {
    int n = 0;
    for (const auto &e : d->entries) n += e.waiting;
    return n;
}

bool latency_exceeded(const rc_output_dpb *d) {
    if (!d->max_latency) return false;
    for (const auto &e : d->entries)
        if (e.waiting && e.latency >= d->max_latency) return true;
    return false;
}

void remove_unused(rc_output_dpb *d) {
    d->entries.erase(std::remove_if(d->entries.begin(), d->entries.end(),
                                    [](const rc_output_dpb::Entry &e) { return !e.waiting && !e.reference; }),
                     d->entries.end());
}

// Output the waiting picture with the smallest POC; false if none waits.
bool bump(rc_output_dpb *d, Sink &s) {
    rc_output_dpb::Entry *best = nullptr;
    for (auto &e : d->entries)
        if (e.waiting && (!best || e.poc < best->poc)) best = &e;
    if (!best) return false;
    best->waiting = false;
    s.put(best->id);
    remove_unused(d);
    return true;
}

int finish(const Sink &s, int *n_out) {
    if (n_out) *n_out = s.n;
    return RC_OK;
}

// A call outputs at most every picture the DPB holds plus the one entering:
// callers pass room for that many ids, checked before anything changes.
bool room(const rc_output_dpb *d, const uint64_t *ids, int cap) {
    return ids && cap >= (int)d->entries.size() + 1;
}

}  // namespace

extern "C" {

int rc_output_create(int capacity, int max_num_reorder, int max_latency_pictures, rc_output_dpb **out) {
    if (!out) return RC_EINVAL;
    *out = nullptr;
    if (capacity < 1 || capacity > 64 || max_num_reorder < 0 || max_num_reorder > 64 || max_latency_pictures < 0)
        return RC_EINVAL;
    rc_output_dpb *d = new (std::nothrow) rc_output_dpb();
    if (!d) return RC_ENOMEM;
    d->capacity = capacity;
    d->max_reorder = max_num_reorder;
    d->max_latency = (uint32_t)max_latency_pictures;
    *out = d;
    return RC_OK;
}

void rc_output_destroy(rc_output_dpb *d) { delete d; }

int rc_output_begin(rc_output_dpb *d, int new_sequence, int no_output_of_prior_pics, uint64_t *out_ids, int cap,
                    int *n_out) {
    if (!d || !room(d, out_ids, cap)) return RC_EINVAL;
    Sink s{out_ids, 0};
    if (new_sequence) {
        if (!no_output_of_prior_pics)
            while (bump(d, s)) {
            }
        d->entries.clear();
        return finish(s, n_out);
    }
    remove_unused(d);
    for (;;) {
        const bool full = (int)d->entries.size() >= d->capacity;
        if (!(num_waiting(d) > d->max_reorder || latency_exceeded(d) || full) || !bump(d, s)) break;
    }
    return finish(s, n_out);
}

int rc_output_unref(rc_output_dpb *d, uint64_t id) {
    if (!d) return RC_EINVAL;
    for (auto &e : d->entries)
        if (e.id == id) e.reference = false;
    remove_unused(d);
    return RC_OK;
}

int rc_output_insert(rc_output_dpb *d, uint64_t id, int32_t poc, int output_flag, int is_reference,
                     uint64_t *out_ids, int cap, int *n_out) {
    if (!d || !room(d, out_ids, cap)) return RC_EINVAL;
    Sink s{out_ids, 0};
    for (auto &e : d->entries)
        if (e.waiting) e.latency++;
    d->entries.push_back({id, poc, 0u, output_flag != 0, is_reference != 0});
    remove_unused(d);
    while ((num_waiting(d) > d->max_reorder || latency_exceeded(d)) && bump(d, s)) {
    }
    return finish(s, n_out);
}

int rc_output_flush(rc_output_dpb *d, uint64_t *out_ids, int cap, int *n_out) {
    if (!d || !room(d, out_ids, cap)) return RC_EINVAL;
    Sink s{out_ids, 0};
    while (bump(d, s)) {
    }
    d->entries.clear();
    return finish(s, n_out);
}

int rc_output_count(rc_output_dpb *d) { return d ? (int)d->entries.size() : RC_EINVAL; }

}  // extern "C"
