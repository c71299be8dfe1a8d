#!/usr/bin/env python3
"""Throughput of H.264 1080p block reconstruction on GB300.

Workload: Plain H.264 High 1920x1080 (coded 1920x1088, 8160 MBs/frame),
120 frames from seeded per-MB syntax records: frame 0 all intra, then P
frames with 2 references, 30% intra MBs (I4x4/I8x8/I16x16), 70% inter
(16x16..4x4 partitions), quarter-pel motion within +-128 px with 5% off the
picture, 20% of inter MBs with explicit weighted prediction, 80% all-zero
blocks with Laplacian(b=2) levels elsewhere, transform_8x8 on half of the
eligible MBs, QP 20..40, deblocking on.

One step = reconstructing the whole 120-frame sequence (every picture
through rc_h264_submit: inter/residual kernel + intra/deblocking wavefront).

  value   frames/s with the syntax records resident in HBM (RC_MEM_DEVICE)
  e2e     frames/s through the same C ABI from pinned host records
          (host->device copies inside the timed region) with every output
          frame copied back to pinned host memory (cropped 1920x1080)

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
MB_W, MB_H = 120, 68
CROP = (0, 0, 1920, 1080)
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


def make_sequence(E, frames, seed):
    pics = []
    for n in range(frames):
        refs = [(0, (n - k) % 4, n - k) for k in (1, 2) if n - k >= 0]
        pics.append(E.SynthH264(seed=seed + n, mb_w=MB_W, mb_h=MB_H, intra_only=int(n == 0), refs=refs,
                                frame_id=n))
    return pics


def picture_stats(E, p):
    """Algorithmic bytes of one picture, per kernel and for the whole job."""
    recs = p.mbs().reshape(-1, 176)
    kind = recs[:, E.H264Mb.kind.offset]
    off = recs[:, E.H264Mb.coef_off.offset:E.H264Mb.coef_off.offset + 4].copy().view(np.uint32)[:, 0].astype(np.int64)
    nxt = np.append(off[1:], p.pic.num_levels)
    lv_bytes = (nxt - off) * 2
    ref = recs[:, E.H264Mb.ref_idx.offset:E.H264Mb.ref_idx.offset + 8].view(np.int8).reshape(-1, 2, 4)
    inter = kind == E.RC_H264_INTER
    lists_b8 = (ref >= 0).sum(axis=1)  # lists used per 8x8
    ref_bytes = int((lists_b8[inter] * 96).sum())  # 64 luma + 2*16 chroma samples per 8x8 per list
    wave_intra = np.isin(kind, [1, 2, 3])
    mbk = inter | (kind == E.RC_H264_IPCM)
    out_frame = MB_W * 16 * MB_H * 16 * 3 // 2
    syn = p.nbytes
    n = len(kind)
    # h264_mb_kernel: every record and its levels once, loop-filter parameters
    # for all MBs (48 B), inter/PCM samples out with their references, and the
    # intra MBs' residuals (768 B) and parameters (32 B) out
    mb_kernel = int(n * (176 + 48) + lv_bytes.sum() + mbk.sum() * 384 + ref_bytes + wave_intra.sum() * (768 + 32))
    # h264_wave_kernel: intra MBs' parameters (32 B) and residuals (768 B) in,
    # then the whole picture read and written once by the loop filter + its
    # per-MB parameters (48 B)
    wave_kernel = int(wave_intra.sum() * (32 + 768) + 2 * out_frame + n * 48)
    return {"mb": mb_kernel, "wave": wave_kernel, "job": out_frame + ref_bytes + syn, "syntax": syn}


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


def cpu_baseline(E, O, pics, budget_s=10.0):
    """Oracle (CPU restatement) on one host thread over the first frames of
    the same sequence, bounded to about budget_s seconds."""
    dpb = O.H264Dpb(MB_W, MB_H, 4)
    t0 = time.perf_counter()
    n = 0
    for i, p in enumerate(pics):
        if dpb.recon(p.ptr, i % 4) != 0:
            raise RuntimeError("oracle rejected a picture")
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "frames/s", "cores": 1, "kind": "port",
            "sample": f"first {n} of the 120 frames of the same sequence, one host thread"}


def peaks():
    f = REPO / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def traffic_for(kernel: str):
    f = REPO / "profiles" / "traffic.json"
    if f.exists():
        d = json.loads(f.read_text())
        v = d.get(kernel)
        if isinstance(v, dict):
            return v.get("bytes_per_launch")
    return None


def run_reference(args, rank):
    if rank != 0:
        return
    E, O = engine(), oracle()
    frames = args.ref_frames
    pics = make_sequence(E, frames, SEED)
    threads = os.cpu_count() or 1

    def one_step():
        def work():
            dpb = O.H264Dpb(MB_W, MB_H, 4)
            for i, p in enumerate(pics):
                dpb.recon(p.ptr, i % 4)
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
    line = {"metric": "1080p H.264 recon frames/s", "value": value, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1000,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded per-MB syntax records)", "impl": "reference",
            "config": {"workload": "h264_1080p_plain: 1920x1080 High 8-bit 4:2:0, P with 2 refs, sample of "
                                   f"{frames} frames per replica", "frames_per_step": threads * frames,
                       "parallelism": f"{threads} CPU threads"},
            "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--frames", type=int, default=120)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-frames", type=int, default=6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
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

    frames = args.frames
    pics = make_sequence(E, frames, SEED + 7919 * rank)
    stats = [picture_stats(E, p) for p in pics]

    # device-resident and pinned-host copies of every picture's records
    keep = []
    dev_pics, host_pics = [], []
    h2d_bytes = 0
    for p in pics:
        b = p.buffers()
        dp = E.H264Picture()
        hp = E.H264Picture()
        for obj, mem in ((dp, E.RC_MEM_DEVICE), (hp, E.RC_MEM_HOST)):
            obj.mem = mem
            obj.constrained_intra_pred = p.pic.constrained_intra_pred
            obj.frame_id = p.pic.frame_id
            obj.num_slices = p.pic.num_slices
            obj.num_weights = p.pic.num_weights
            obj.num_levels = p.pic.num_levels
        for key in ("mbs", "slices", "weights", "levels"):
            raw = b[key]
            if not raw:
                continue
            h = torch.frombuffer(bytearray(raw), dtype=torch.uint8).pin_memory()
            d = h.to(dev)
            keep += [h, d]
            setattr(hp, key, h.data_ptr())
            setattr(dp, key, d.data_ptr())
            h2d_bytes += len(raw)
        dev_pics.append(dp)
        host_pics.append(hp)
    torch.cuda.synchronize()

    st = E.ReconStream(E.RC_CODEC_H264, 1920, 1080, 8, 4)
    cs = torch.cuda.ExternalStream(st.cuda_stream(), device=dev)

    def step(src):
        for n, pic in enumerate(src):
            st.submit_h264(ctypes.addressof(pic), n % 4)

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
    st.profile(True)
    launches0 = st.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(cs)
    for _ in range(args.steps):
        step(dev_pics)
    e1.record(cs)
    e1.synchronize()
    launches = st.launches() - launches0
    prof = st.profile_read()
    st.profile(False)
    clk = clocks.stop()
    rc = st.sync()
    if rc != 0:
        raise SystemExit(f"device error {rc} in the timed region")
    t_ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([t_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_ms = float(t.item())
        dist.barrier()
    value = frames * args.steps * world / (t_ms / 1000.0)

    # ---- e2e: pinned host records in, cropped frames out, through the C ABI
    ring = []
    for _ in range(8):
        ring.append(tuple(torch.empty(n, dtype=torch.uint8).pin_memory() for n in (1920 * 1080, 960 * 540, 960 * 540)))
    d2h_bytes = frames * (1920 * 1080 + 2 * 960 * 540)

    def e2e_step():
        for n, pic in enumerate(host_pics):
            st.submit_h264(ctypes.addressof(pic), n % 4)
            y, u, v = ring[n % 8]
            st.download_async(n % 4, CROP, y.data_ptr(), u.data_ptr(), v.data_ptr())

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
    names = {0: ("h264_mb_kernel", "mb"), 1: ("h264_wave_kernel", "wave")}
    per_kernel = {}
    for k, (ms, n) in prof.items():
        name, key = names[k]
        alg = statistics.mean(s[key] for s in stats)
        per_kernel[name] = {"launches": n, "ms_total": ms, "us_per_launch": ms / n * 1000,
                            "alg_bytes_per_launch": alg, "achieved_gbs": alg / (ms / n / 1000) / 1e9}
    dom = max(per_kernel, key=lambda k: per_kernel[k]["ms_total"])
    peak, peak_kind = peaks()
    ach = per_kernel[dom]["achieved_gbs"]
    job_bytes = statistics.mean(s["job"] for s in stats)
    result = {
        "metric": "1080p H.264 recon frames/s", "value": value, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded per-MB syntax records; no public clip available)",
        "config": {"workload": "h264_1080p_plain: 1920x1080 High 8-bit 4:2:0, 120 frames, I then P with 2 refs, "
                               "30% intra, 20% explicit WP, 80% zero blocks, QP 20-40, deblocking on",
                   "frames_per_step": frames, "parallelism": "replicas" if world > 1 else "single stream",
                   "l2": f"inputs larger than L2 (syntax {sum(s['syntax'] for s in stats) / 1e6:.0f} MB per step)",
                   "luma_msamples_per_s": value * 1920 * 1080 / 1e6},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "peak_source": peak_kind, "traffic": traffic_for(dom)},
        "roofline_job": {"alg_bytes_per_frame": job_bytes, "achieved": job_bytes * value / world / 1e9,
                         "peak": peak, "unit": "GB/s", "frac": job_bytes * value / world / 1e9 / peak},
        "kernels": per_kernel,
        "e2e": {"value": e2e, "unit": "frames/s", "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(E, oracle(), pics)
    if rank == 0:
        print(json.dumps(result), flush=True)
    st.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
