#!/usr/bin/env python3
"""Throughput of H.264 / HEVC block reconstruction on GB300.

Default workload (h264_1080p): Plain H.264 High 1920x1080 (coded 1920x1088,
8160 MBs/frame), 120 frames from seeded per-MB syntax records: frame 0 all
intra, then P frames with 2 references, 30% intra MBs (I4x4/I8x8/I16x16),
70% inter (16x16..4x4 partitions), quarter-pel motion within +-128 px with
5% off the picture, 20% of inter MBs with explicit weighted prediction, 80%
all-zero blocks with Laplacian(b=2) levels elsewhere, transform_8x8 on half
of the eligible MBs, QP 20..40, deblocking on.

--workload hevc_1080p_8 | hevc_1080p_10 | hevc_2160p_8 | hevc_2160p_10:
Plain HEVC Main / Main10, 60 frames from seeded per-CTB syntax records:
CTB 64, random quadtree (CU 8..64, TU 4..32), frame 0 all intra, then 25%
intra / 75% inter with 4 references, motion within +-256 px, 75% zero TUs
with Laplacian(b=3) levels, QP 22..37, deblocking and SAO on.

One step = reconstructing the whole sequence (every picture through the C
ABI submit call of its codec).

  value   frames/s with the syntax records resident in HBM (RC_MEM_DEVICE)
  e2e     frames/s through the same C ABI from pinned host records
          (host->device copies inside the timed region) with every output
          frame copied back to pinned host memory (cropped)

--impl reference times the oracle (the CPU restatement of the reference's
reconstruction) on the host's cores instead.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = pathlib.Path(__file__).resolve().parent
SEED = 20261203


def _load(name, path, pkgdir=None):
    import importlib.util
    if name in sys.modules:
        return sys.modules[name]
    kw = {"submodule_search_locations": [str(pkgdir)]} if pkgdir else {}
    spec = importlib.util.spec_from_file_location(name, path, **kw)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def engine():
    pkg = REPO / "pito-codecs_gb300"
    return _load("pito_codecs_gb300", pkg / "__init__.py", pkg)


def oracle():
    return _load("pyoracle", REPO / "oracle" / "pyoracle.py")


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------
class H264Workload:
    name = "h264_1080p"
    metric = "1080p H.264 recon frames/s"
    W, H, bd, frames = 1920, 1080, 8, 120
    MB_W, MB_H = 120, 68
    slots = 4
    # pictures per launch (rc_stream_set_h264_group): one.  The generator
    # sends 5% of inter partitions outside the picture, so every MB row has
    # MBs that read a reference's clamped last row and must wait until that
    # whole picture is filtered: groups cannot overlap these pictures.
    group = 1
    crop = (0, 0, 1920, 1080)
    description = ("h264_1080p_plain: 1920x1080 High 8-bit 4:2:0, 120 frames, I then P with 2 refs, 30% intra, "
                   "20% explicit WP, 80% zero blocks, QP 20-40, deblocking on")
    kernels = {2: ("h264_edge_kernel", "edge"), 0: ("h264_mb_kernel", "mb"), 1: ("h264_band_kernel", "band"),
               8: ("h264_group_kernel", "group")}
    buffer_keys = ("mbs", "slices", "weights", "levels")

    def __init__(self, E, frames=None):
        self.E = E
        if frames:
            self.frames = frames

    def codec(self):
        return self.E.RC_CODEC_H264

    def sequence(self, seed, frames=None):
        E, pics = self.E, []
        for n in range(frames or self.frames):
            refs = [(0, (n - k) % self.slots, n - k) for k in (1, 2) if n - k >= 0]
            pics.append(E.SynthH264(seed=seed + n, mb_w=self.MB_W, mb_h=self.MB_H, intra_only=int(n == 0),
                                    refs=refs, frame_id=n))
        return pics

    def picture_struct(self):
        return self.E.H264Picture()

    def copy_header(self, dst, p):
        for f in ("constrained_intra_pred", "frame_id", "num_slices", "num_weights", "num_levels"):
            setattr(dst, f, getattr(p.pic, f))

    def submit(self, st, ptr, slot):
        st.submit_h264(ptr, slot)

    def stats(self, p, n=0):
        """Algorithmic bytes of one picture per kernel and for the whole job."""
        E = self.E
        recs = p.mbs().reshape(-1, 176)
        kind = recs[:, E.H264Mb.kind.offset]
        off = recs[:, E.H264Mb.coef_off.offset:E.H264Mb.coef_off.offset + 4].copy().view(np.uint32)[:, 0]
        off = off.astype(np.int64)
        nxt = np.append(off[1:], p.pic.num_levels)
        lv_bytes = (nxt - off) * 2
        ref = recs[:, E.H264Mb.ref_idx.offset:E.H264Mb.ref_idx.offset + 8].view(np.int8).reshape(-1, 2, 4)
        inter = kind == E.RC_H264_INTER
        lists_b8 = (ref >= 0).sum(axis=1)
        ref_bytes = int((lists_b8[inter] * 96).sum())  # 64 luma + 2 x 16 chroma samples per 8x8 and list
        intra = np.isin(kind, [1, 2, 3])
        mbk = inter | (kind == E.RC_H264_IPCM)
        out_frame = self.MB_W * 16 * self.MB_H * 16 * 3 // 2
        n = len(kind)
        edges = 256  # loop-filter edge words per MB
        # h264_edge_kernel: every record (176 B; its left/top neighbours' come
        # from L2) in, the edge words out
        edge = int(n * (176 + edges))
        # h264_mb_kernel: every record and its levels in; inter/PCM samples out
        # with their reference samples in; intra MBs' residuals (768 B) and
        # parameters (32 B) out
        mb = int(n * 176 + lv_bytes.sum() + mbk.sum() * 384 + ref_bytes + intra.sum() * (768 + 32))
        # h264_band_kernel: intra MBs' parameters and residuals in; the picture
        # read and written once by the loop filter with the edge words in
        band = int(intra.sum() * (32 + 768) + 2 * out_frame + n * edges)
        # h264_group_kernel, per picture: the MB phase and the band work, with
        # the edge words written once (the records are read by the MB phase)
        group = mb + band + n * edges
        return {"edge": edge, "mb": mb, "band": band, "group": group, "job": out_frame + ref_bytes + p.nbytes,
                "syntax": p.nbytes}

    def oracle_dpb(self, O):
        return O.H264Dpb(self.MB_W, self.MB_H, self.slots)


class HevcWorkload:
    frames = 60
    slots = 5
    kernels = {3: ("hevc_residual_kernel", "residual"), 4: ("hevc_inter_kernel", "inter"),
               5: ("hevc_intra_kernel", "intra"), 6: ("hevc_loopfilter_kernel", "loopfilter"),
               7: ("hevc_inter_kernel_late", "inter_late")}
    buffer_keys = ("ctbs", "blk", "mvf", "tus", "slices", "levels", "scaling")

    def __init__(self, E, W, H, bd, frames=None):
        self.E, self.W, self.H, self.bd = E, W, H, bd
        if frames:
            self.frames = frames
        tag = "1080p" if H == 1080 else "2160p"
        self.name = f"hevc_{tag}_{bd}"
        self.metric = f"{tag} HEVC recon frames/s"
        self.crop = (0, 0, W, H)
        self.description = (f"hevc_{tag}_{'main10' if bd == 10 else 'main'}: {W}x{H} {bd}-bit 4:2:0, "
                            f"{self.frames} frames, I then P/B with 4 refs, CTB 64, 25% intra, 75% zero TUs, "
                            "QP 22-37, deblocking + SAO on")

    def codec(self):
        return self.E.RC_CODEC_HEVC

    def sequence(self, seed, frames=None):
        E, pics = self.E, []
        for n in range(frames or self.frames):
            refs = [(0, (n - k) % self.slots, n - k) for k in (1, 2, 3, 4) if n - k >= 0]
            pics.append(E.SynthHevc(seed=seed + n, width=self.W, height=self.H, bit_depth=self.bd,
                                    intra_only=int(n == 0), refs=refs, frame_id=n))
        return pics

    def picture_struct(self):
        return self.E.HevcPicture()

    def copy_header(self, dst, p):
        for f in ("log2_ctb", "constrained_intra_pred", "strong_intra_smoothing", "loop_filter_across_tiles",
                  "cb_qp_offset", "cr_qp_offset", "num_slices", "num_tus", "frame_id", "num_levels"):
            setattr(dst, f, getattr(p.pic, f))

    def submit(self, st, ptr, slot):
        st.submit_hevc(ptr, slot)

    def stats(self, p, n=0):
        """Coarse algorithmic bytes per kernel (whole planes) and for the job;
        picture n of the sequence (its inter units split between the pass
        beside the previous picture and the one after it)."""
        b = p.buffers()
        bps = 2 if self.bd > 8 else 1
        samples = self.W * self.H * 3 // 2
        plane = samples * bps
        res = samples * 2
        mvf = np.frombuffer(b["mvf"], np.uint8).reshape(-1, 12)
        ref_idx = mvf[:, 8:10].view(np.int8).astype(np.int64)
        lists = (ref_idx >= 0).sum(axis=1)
        inter_frac = float((lists > 0).mean()) if len(lists) else 0.0
        ref_bytes = int(lists.sum()) * 24 * bps  # 16 luma + 2 x 4 chroma samples per 4x4 and list
        # units that read the previous picture's slot (the second inter pass)
        late = np.zeros(len(lists), bool)
        if n > 0 and len(lists):
            E = self.E
            sl = (E.HevcSlice * p.pic.num_slices).from_buffer_copy(b["slices"])
            ref_slot = np.array([[list(s.ref_slot[l]) for l in range(2)] for s in sl])
            nref = np.array([list(s.num_ref) for s in sl])
            ctb_slice = np.frombuffer(b["ctbs"], np.uint8).reshape(-1, ctypes.sizeof(E.HevcCtb))[:, :2].copy()
            ctb_slice = np.minimum(ctb_slice.view(np.uint16)[:, 0], len(sl) - 1)
            w4, h4 = self.W // 4, self.H // 4
            lg, wctb = p.pic.log2_ctb, -(-self.W >> p.pic.log2_ctb)
            uy, ux = np.divmod(np.arange(w4 * h4), w4)
            us = ctb_slice[((uy * 4) >> lg) * wctb + ((ux * 4) >> lg)]
            prev = (n - 1) % self.slots
            for l in range(2):
                ri = ref_idx[:, l]
                ok = (ri >= 0) & (ri < np.minimum(nref[us, l], 16))
                late |= ok & (ref_slot[us, l, np.clip(ri, 0, 15)] == prev)
        late_frac = float(late.mean()) if len(lists) else 0.0
        late_ref = int(lists[late].sum()) * 24 * bps
        syn = p.nbytes
        return {
            "residual": len(b["tus"]) + len(b["levels"]) + res,
            "inter": ref_bytes - late_ref + int((inter_frac - late_frac) * (res + plane)),
            "inter_late": late_ref + int(late_frac * (res + plane)),
            "intra": int((1 - inter_frac) * (res + plane)),
            "loopfilter": 2 * plane + len(b["blk"]) + len(b["ctbs"]),
            "job": plane + ref_bytes + syn,
            "syntax": syn,
        }

    def oracle_dpb(self, O):
        return O.HevcDpb(self.W, self.H, self.bd, self.slots)


def workload(E, name, frames=None):
    if name == "h264_1080p":
        return H264Workload(E, frames)
    table = {"hevc_1080p_8": (1920, 1080, 8), "hevc_1080p_10": (1920, 1080, 10),
             "hevc_2160p_8": (3840, 2160, 8), "hevc_2160p_10": (3840, 2160, 10)}
    if name not in table:
        raise SystemExit(f"unknown workload {name}")
    return HevcWorkload(E, *table[name], frames=frames)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = str(device)
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(device).uuid)
            if uuid:
                self.device = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
        except Exception:
            pass
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.device, f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def oracle_pass(wl, O, pics):
    """The oracle (CPU restatement) on one host thread over the whole
    sequence: its rate is the cpu_baseline, and the per-plane MD5 of every
    frame is what the GPU's output is checked against."""
    import hashlib
    dpb = wl.oracle_dpb(O)
    md5s = []
    busy = 0.0
    for i, p in enumerate(pics):
        t0 = time.perf_counter()
        if dpb.recon(p.ptr, i % wl.slots) != 0:
            raise RuntimeError("oracle rejected a picture")
        busy += time.perf_counter() - t0
        md5s.append(tuple(hashlib.md5(np.ascontiguousarray(pl).tobytes()).hexdigest()
                          for pl in _planes_as_stream(wl, dpb.planes(i % wl.slots))))
    base = {"value": len(pics) / busy, "unit": "frames/s", "cores": 1, "kind": "port",
            "sample": f"all {len(pics)} frames of the same sequence, one host thread"}
    return base, md5s


def _planes_as_stream(wl, planes):
    """Oracle planes (uint16 samples) in the stream's sample type."""
    dt = np.uint8 if wl.bd == 8 else np.uint16
    return [np.asarray(pl).astype(dt) for pl in planes]


def gpu_md5s(wl, st, pics):
    """Per-plane MD5 of every frame as the engine reconstructs the sequence
    through the C ABI (host records), each frame read back before its slot
    is reused."""
    import hashlib
    out = []
    for i, p in enumerate(pics):
        wl.submit(st, p.ptr, i % wl.slots)
        rc = st.sync()
        if rc != 0:
            raise SystemExit(f"device error {rc} in the parity pass")
        out.append(tuple(hashlib.md5(np.ascontiguousarray(pl).tobytes()).hexdigest()
                         for pl in st.download(i % wl.slots)))
    return out


# What bounds each dominant kernel, from its measured critical path (ncu
# summaries in profiles/): the HBM roofline is the ceiling the fraction is
# quoted against, not the limiter.
LIMITER = {
    "h264_group_kernel": "wavefront dependency latency, several pictures deep: each picture's 17 band CTAs walk its "
                         "MB rows while the other CTAs run the MB phase; a picture's inter MBs wait for the "
                         "reference rows their vectors reach",
    "h264_band_kernel": "wavefront dependency latency: at 1080p 17 bands of 4 MB rows, each on three CTAs "
                        "(intra, luma filter, chroma filter) on SMs of their own, walk a picture's MB rows behind "
                        "each other (critical path = the intra chain and the luma filter's per-MB steps, each "
                        "about 300 us of the 337)",
    "hevc_intra_kernel": "intra dependency chain: blocks wait for their reconstructed neighbours in decode order "
                         "(critical path = chain of intra blocks + same-CTB hand-overs)",
}


def peaks():
    f = REPO / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def traffic_for(kernel: str, workload_name: str):
    f = REPO / "profiles" / "traffic.json"
    if f.exists():
        d = json.loads(f.read_text())
        v = d.get(workload_name, {}).get(kernel)
        if isinstance(v, dict):
            return v.get("bytes_per_launch")
    return None


def run_reference(args, rank):
    if rank != 0:
        return
    E, O = engine(), oracle()
    wl = workload(E, args.workload)
    frames = args.ref_frames
    pics = wl.sequence(SEED, frames)
    threads = os.cpu_count() or 1

    def one_step():
        def work():
            dpb = wl.oracle_dpb(O)
            for i, p in enumerate(pics):
                dpb.recon(p.ptr, i % wl.slots)
        ts = [threading.Thread(target=work) for _ in range(threads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()

    for _ in range(args.warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_step()
    dt = time.perf_counter() - t0
    value = threads * frames * args.steps / dt
    sample = (f"{threads} host threads, each reconstructing frames 0..{frames - 1} of the sequence "
              f"(independent replicas) per step")
    line = {"metric": wl.metric, "value": value, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1000,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u8" if wl.bd == 8 else "u16",
            "data": "synthetic (seeded syntax records)", "impl": "reference",
            "config": {"workload": wl.description + f"; sample of {frames} frames per replica",
                       "frames_per_step": threads * frames, "parallelism": f"{threads} CPU threads"},
            "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _job_roofline(specs, fps, frames):
    """Whole-mix output bytes (coded planes written once, the B_out term of
    the algorithmic bytes) per second against the measured HBM peak: a lower
    bound of the job's fraction, reference and syntax reads not counted."""
    peak, kind = peaks()
    out = sum(s.width * s.height * 3 // 2 * (2 if getattr(s, "bit_depth", 8) > 8 else 1) * s.frames for s in specs)
    gbs = out / frames * fps / 1e9
    return {"alg_bytes_per_frame": out / frames, "terms": "B_out only", "achieved": gbs, "peak": peak,
            "unit": "GB/s", "frac": gbs / peak, "peak_source": kind}


def run_multistream(args):
    """The batched (64 mixed streams in flight together, against the plain
    per-stream loop) and served (Poisson request traces through the request
    loop, against the plain path serving the same trace) forms."""
    import hashlib
    import importlib
    E = engine()
    M = importlib.import_module("pito_codecs_gb300.multistream")
    if E.lib().rc_device_select(0) != 0:
        raise SystemExit("rc_device_select failed")
    specs = M.mix_specs(args.streams, seed=SEED)
    t0 = time.perf_counter()
    tpl = {s.key: M.Templates(s) for s in specs}
    import torch

    def upload(raw):
        d = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
        return d.data_ptr(), d

    for t in tpl.values():  # records resident in HBM, as the plain line's value
        t.to_device(upload)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0

    def digest(st):
        h = hashlib.sha256()
        for slot in range(st.slots):
            for plane in st.download(slot):
                h.update(plane.tobytes())
        return h.hexdigest()

    def luma_samples(s, frames):
        return s.width * s.height * frames

    base = {"n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u16",
            "data": "synthetic (seeded syntax records; template pictures replayed per stream)"}
    mix = (f"{args.streams} streams: resolutions uniform over 426x240..3840x2160, half H.264 8-bit, half HEVC "
           "8/10-bit, 30-240 frames each")
    if args.workload == "batched":
        # warm-up: one frame per stream on separate streams
        warm = {s.key: M.open_stream(s) for s in specs}
        for s in specs:
            M.submit(warm[s.key], s, *tpl[s.key].picture(0))
        for st in warm.values():
            st.sync()
            st.close()
        alone = {s.key: M.open_stream(s) for s in specs}
        t_plain = M.run_plain(specs, tpl, alone)
        # the schedule: the autotuner's choice for this mix (each candidate
        # runs the first 16 pictures of every stream, so that predicted
        # pictures outweigh the intra one as in the full streams), unless given
        if args.depth > 0:
            schedule, rates = M.Schedule(args.depth, 1.0), {}
        else:
            schedule, rates = M.autotune(specs, tpl, frames=16)
        mixed = {s.key: M.open_stream(s) for s in specs}
        M.apply_schedule(mixed, specs, schedule)
        clocks = ClockSampler(0)
        clocks.start()
        t_batch = M.run_batched(specs, tpl, mixed, depth=schedule.depth)
        clk = clocks.stop()
        frames = sum(s.frames for s in specs)
        check = specs[: args.parity_streams]
        same = all(digest(alone[s.key]) == digest(mixed[s.key]) for s in check)
        launches = sum(st.launches() for st in mixed.values())
        for st in list(alone.values()) + list(mixed.values()):
            st.close()
        line = dict(base, metric="C4 batched recon frames/s", value=frames / t_batch, unit="frames/s",
                    steps=1, warmup=1, ms_per_step=t_batch * 1000,
                    config={"workload": "batched_c4: " + mix, "frames": frames, "depth": schedule.depth,
                            "schedule": schedule.describe(),
                            "autotune_fps": {k: round(v, 1) for k, v in rates.items()},
                            "plain_loop_fps": frames / t_plain, "speedup_vs_plain": t_plain / t_batch,
                            "luma_msamples_per_s": sum(luma_samples(s, s.frames) for s in specs) / t_batch / 1e6,
                            "parity": f"{'identical' if same else 'DIFFERENT'} DPBs in the mix and alone for the "
                                      f"first {len(check)} streams", "template_setup_s": setup_s},
                    e2e={"value": frames / t_batch, "unit": "frames/s", "h2d_bytes_per_step": None,
                         "d2h_bytes_per_step": 0},
                    gpu_launches=launches, clocks=clk,
                    roofline_job=_job_roofline(specs, frames / t_batch, frames))
        print(json.dumps(line), flush=True)
        return
    # served
    out = {}
    clk = None
    for rate in args.rates:
        count = max(20, int(rate * args.trace_seconds))
        trace = M.poisson_trace(rate, count, len(specs), seed=SEED + int(rate))
        srv = M.Server(specs, tpl, hbm_budget=args.hbm_budget_gb << 30, depth=args.depth or 2)
        clocks = ClockSampler(0)
        clocks.start()
        srv.run(trace)
        clk = clocks.stop()
        served = M.latency_stats(trace)
        served["evictions"] = srv.evictions
        srv.close()
        trace2 = M.poisson_trace(rate, count, len(specs), seed=SEED + int(rate))
        M.serve_plain(specs, tpl, trace2)
        out[str(rate)] = {"served": served, "plain": M.latency_stats(trace2)}
    top = out[str(args.rates[-1])]["served"]
    line = dict(base, metric="C5 served recon: p50/p99 latency and frames/s", value=top["frames_per_s"],
                unit="frames/s", steps=1, warmup=0, ms_per_step=None,
                config={"workload": "served_c5: Poisson arrivals, requests of 1..12 frames (half single-frame) "
                                    "on streams of the mix: " + mix,
                        "hbm_budget_gb": args.hbm_budget_gb, "trace_seconds": args.trace_seconds,
                        "rates": out},
                e2e={"value": top["frames_per_s"], "unit": "frames/s", "h2d_bytes_per_step": None,
                     "d2h_bytes_per_step": 0},
                clocks=clk)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--frames", type=int, default=0, help="pictures per step (default: the workload's)")
    ap.add_argument("--workload", default="h264_1080p",
                    choices=["h264_1080p", "hevc_1080p_8", "hevc_1080p_10", "hevc_2160p_8", "hevc_2160p_10",
                             "batched", "served"])
    ap.add_argument("--streams", type=int, default=64, help="batched / served: streams in the mix")
    ap.add_argument("--depth", type=int, default=0,
                    help="batched: pictures queued per stream (0: the autotuner's schedule); served: 0 means 2")
    ap.add_argument("--parity-streams", type=int, default=64, help="batched: streams whose DPBs are compared")
    ap.add_argument("--rates", type=float, nargs="+", default=[50.0, 200.0, 800.0], help="served: requests/s")
    ap.add_argument("--trace-seconds", type=float, default=3.0, help="served: trace length")
    ap.add_argument("--hbm-budget-gb", type=int, default=120, help="served: DPB budget")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-frames", type=int, default=6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--group", type=int, default=-1,
                    help="H.264: pictures per launch (rc_stream_set_h264_group; default: the workload's)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload in ("batched", "served"):
        run_multistream(args)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    E = engine()
    if E.lib().rc_device_select(local) != 0:
        raise SystemExit("rc_device_select failed")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    wl = workload(E, args.workload, args.frames or None)
    frames = wl.frames
    pics = wl.sequence(SEED + 7919 * rank)
    stats = [wl.stats(p, n) for n, p in enumerate(pics)]
    bps = 2 if wl.bd > 8 else 1

    # device-resident and pinned-host copies of every picture's records
    keep = []
    dev_pics, host_pics = [], []
    h2d_bytes = 0
    for p in pics:
        b = p.buffers()
        dp, hp = wl.picture_struct(), wl.picture_struct()
        for obj, mem in ((dp, E.RC_MEM_DEVICE), (hp, E.RC_MEM_HOST)):
            obj.mem = mem
            wl.copy_header(obj, p)
        for key in wl.buffer_keys:
            raw = b.get(key)
            if not raw:
                continue
            h = torch.frombuffer(bytearray(raw), dtype=torch.uint8).pin_memory()
            keep.append(h)
            setattr(hp, key, h.data_ptr())
            h2d_bytes += len(raw)
            if key == "scaling":  # the scaling factors stay in host memory (rc_hevc_picture)
                setattr(dp, key, h.data_ptr())
                continue
            d = h.to(dev)
            keep.append(d)
            setattr(dp, key, d.data_ptr())
        dev_pics.append(dp)
        host_pics.append(hp)
    torch.cuda.synchronize()

    st = E.ReconStream(wl.codec(), wl.W, wl.H, wl.bd, wl.slots)
    group = 1
    if wl.codec() == E.RC_CODEC_H264:
        group = st.set_h264_group(args.group if args.group >= 0 else wl.group)
    cs = torch.cuda.ExternalStream(st.cuda_stream(), device=dev)

    def step(src):
        for n, pic in enumerate(src):
            wl.submit(st, ctypes.addressof(pic), n % wl.slots)

    # ---- value: records resident in HBM
    for _ in range(args.warmup):
        step(dev_pics)
    if st.sync() != 0:
        raise SystemExit("device error during warm-up")
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = st.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # e0 is recorded on the idle stream and has executed before the first
    # submit, so no kernel of the timed region (the first picture's
    # record-only kernel runs on a side stream) can start before it; every
    # side-stream kernel is joined into the stream before e1
    e0.record(cs)
    e0.synchronize()
    for _ in range(args.steps):
        step(dev_pics)
    e1.record(cs)
    e1.synchronize()
    launches = st.launches() - launches0
    clk = clocks.stop()
    rc = st.sync()
    if rc != 0:
        raise SystemExit(f"device error {rc} in the timed region")
    t_ms = e0.elapsed_time(e1)
    # per-kernel times: one more pass with CUDA events around every kernel,
    # outside the timed region (the events themselves cost time)
    st.profile(True)
    step(dev_pics)
    prof = st.profile_read()
    st.profile(False)
    if st.sync() != 0:
        raise SystemExit("device error in the profiled pass")
    if dist:
        t = torch.tensor([t_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_ms = float(t.item())
        dist.barrier()
    value = frames * args.steps * world / (t_ms / 1000.0)

    # ---- e2e: pinned host records in, cropped frames out, through the C ABI
    cw, chh = wl.W, wl.H
    ring = []
    for _ in range(8):
        ring.append(tuple(torch.empty(n * bps, dtype=torch.uint8).pin_memory()
                          for n in (cw * chh, cw * chh // 4, cw * chh // 4)))
    d2h_bytes = frames * (cw * chh * 3 // 2) * bps

    def e2e_step():
        for n, pic in enumerate(host_pics):
            wl.submit(st, ctypes.addressof(pic), n % wl.slots)
            y, u, v = ring[n % 8]
            st.download_async(n % wl.slots, wl.crop, y.data_ptr(), u.data_ptr(), v.data_ptr())

    for _ in range(args.warmup):
        e2e_step()
    st.sync()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    rc = st.sync()
    e2e_s = time.perf_counter() - t0
    if rc != 0:
        raise SystemExit(f"device error {rc} in the e2e region")
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = frames * args.steps * world / e2e_s

    # ---- roofline of the dominant kernel
    per_kernel = {}
    for k, (ms, n) in prof.items():
        if k not in wl.kernels or n == 0:
            continue
        name, key = wl.kernels[k]
        # the profiled pass's pictures over its launches of the kernel (a
        # group launch covers several pictures; the second inter pass runs
        # for the pictures that reference the previous one)
        alg = sum(s[key] for s in stats) / n
        per_kernel[name] = {"launches": n, "ms_total": ms, "us_per_launch": ms / n * 1000,
                            "alg_bytes_per_launch": alg, "achieved_gbs": alg / (ms / n / 1000) / 1e9}
    dom = max(per_kernel, key=lambda k: per_kernel[k]["ms_total"])
    peak, peak_kind = peaks()
    ach = per_kernel[dom]["achieved_gbs"]
    job_bytes = statistics.mean(s["job"] for s in stats)
    result = {
        "metric": wl.metric, "value": value, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8" if wl.bd == 8 else "u16",
        "data": "synthetic (seeded syntax records; no public clip available)",
        "config": {"workload": wl.description, "frames_per_step": frames,
                   "parallelism": "replicas" if world > 1 else "single stream",
                   "pictures_per_launch": group, "dpb_slots": wl.slots,
                   "l2": f"inputs larger than L2 (syntax {sum(s['syntax'] for s in stats) / 1e6:.0f} MB per step)",
                   "luma_msamples_per_s": value * wl.W * wl.H / 1e6},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "peak_source": peak_kind, "traffic": traffic_for(dom, wl.name),
                     "limiter": LIMITER.get(dom, "unmeasured")},
        "roofline_job": {"alg_bytes_per_frame": job_bytes, "achieved": job_bytes * value / world / 1e9,
                         "peak": peak, "unit": "GB/s", "frac": job_bytes * value / world / 1e9 / peak},
        "kernels": per_kernel,
        "e2e": {"value": e2e, "unit": "frames/s", "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base, want = oracle_pass(wl, oracle(), pics)
        got = gpu_md5s(wl, st, pics)
        bad = [i for i, (g, w) in enumerate(zip(got, want)) if g != w]
        result["cpu_baseline"] = base
        result["parity"] = {"frames": len(pics), "mismatches": len(bad), "first_mismatch": bad[0] if bad else None,
                            "compared": "per-plane MD5 of every frame of the timed sequence: engine (C ABI, host "
                                        "records) against the oracle"}
    if rank == 0:
        print(json.dumps(result), flush=True)
    st.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
