"""Many streams at once on one GPU: the batched and the served forms.

Pictures of different streams do not depend on each other.  Each stream
(rc_stream) orders its pictures on its own CUDA stream, so the kernels of
different streams overlap on the GPU while every stream's pictures stay in
decode order; a picture's bytes do not depend on what else runs beside it.

* Batched form: a mix of streams of uneven resolution, codec and bit depth
  (``mix_specs``) kept in flight together -- ``run_batched`` submits the
  streams' pictures round-robin, ``run_plain`` one stream after the other;
  ``autotune`` picks its schedule for a mix by timing the candidates:
  pictures queued per stream, and per shape class (codec, coded size, bit
  depth) the HEVC intra kernel's CTAs per launch and loop-filter tile
  height, or the H.264 pictures per launch.
* Served form: ``Server`` admits decode requests (a stream and a number of
  frames) as they arrive, while the device bytes of the resident streams
  stay within an HBM budget; streams stay resident between requests and idle
  ones are evicted least-recently-used when a new stream needs the room.
  Admitted requests' frames are submitted as soon as their streams allow and
  overlap on the GPU; completion marks (rc_stream_mark) time every frame.

Synthetic pictures come from the package's seeded generators: a stream
replays a small set of template pictures (an intra picture, then one
predicted picture per DPB-slot phase, each referencing the slots before
it), which keeps the mix's set-up time small while every frame does full
work.
"""
from __future__ import annotations

import collections
import dataclasses
import hashlib
import json
import os
import random
import time

from . import (RC_CODEC_H264, RC_CODEC_HEVC, ReconStream, SynthH264, SynthHevc)

# Resolutions of the batched configuration (display sizes; the coded size is
# rounded up to the codec's block grid and cropped back on output).
MIX_SIZES = [(426, 240), (854, 480), (1280, 720), (1920, 1080), (3840, 2160)]


@dataclasses.dataclass
class StreamSpec:
    key: int
    codec: int
    width: int      # display size
    height: int
    bit_depth: int
    frames: int
    seed: int

    @property
    def coded(self):
        if self.codec == RC_CODEC_H264:
            return (self.width + 15) // 16 * 16, (self.height + 15) // 16 * 16
        return (self.width + 7) // 8 * 8, (self.height + 7) // 8 * 8

    @property
    def slots(self):
        return 4 if self.codec == RC_CODEC_H264 else 5

    @property
    def crop(self):
        return (0, 0, self.width, self.height)


def mix_specs(n: int = 64, seed: int = 20261203, min_frames: int = 30, max_frames: int = 240):
    """The batched configuration: resolutions drawn uniformly from MIX_SIZES,
    half H.264 (8-bit) and half HEVC (8- and 10-bit alternating), 30..240
    frames per stream."""
    rng = random.Random(seed)
    specs = []
    for i in range(n):
        w, h = rng.choice(MIX_SIZES)
        codec = RC_CODEC_H264 if i % 2 == 0 else RC_CODEC_HEVC
        bd = 8 if codec == RC_CODEC_H264 else (8 if (i // 2) % 2 == 0 else 10)
        specs.append(StreamSpec(i, codec, w, h, bd, rng.randint(min_frames, max_frames), seed * 1000 + i * 17))
    return specs


class Templates:
    """Template pictures of one stream: an intra picture for frame 0; for frame
    n >= 1 the predicted picture of phase n % slots, written to slot
    n % slots and referencing the slots of the frames before it."""

    def __init__(self, spec: StreamSpec):
        self.spec = spec
        W, H = spec.coded
        s = spec.slots

        def make(intra: bool, phase: int, seed: int):
            depth = (1, 2) if spec.codec == RC_CODEC_H264 else (1, 2, 3, 4)
            refs = None if intra else [(0, (phase - k) % s, (phase - k) % s + 1) for k in depth]
            if spec.codec == RC_CODEC_H264:
                return SynthH264(seed=seed, mb_w=W // 16, mb_h=H // 16, intra_only=int(intra), refs=refs,
                                 frame_id=phase + 1)
            return SynthHevc(seed=seed, width=W, height=H, bit_depth=spec.bit_depth, intra_only=int(intra),
                             refs=refs, frame_id=phase + 1)

        self.intra = make(True, 0, spec.seed)
        self.pred = [make(False, p, spec.seed + 1 + p) for p in range(s)]

        self._dev = None

    def to_device(self, upload):
        """Keep device-resident copies of the template records (RC_MEM_DEVICE
        pictures), so that submits move no record bytes.  `upload(raw)` puts
        the bytes on the device and returns (device address, keepalive)."""
        from . import RC_MEM_DEVICE, H264Picture, HevcPicture
        self._keep = []

        def dev(pic):
            h264 = self.spec.codec == RC_CODEC_H264
            d = H264Picture() if h264 else HevcPicture()
            for f, _ in d._fields_:
                if f not in ("mbs", "slices", "weights", "levels", "ctbs", "blk", "mvf", "tus", "scaling"):
                    setattr(d, f, getattr(pic.pic, f))
            d.mem = RC_MEM_DEVICE
            for key, raw in pic.buffers().items():
                if not raw or key in ("scaling4", "scaling8"):
                    continue
                if key == "scaling":  # expanded scaling factors stay in host memory
                    setattr(d, key, getattr(pic.pic, key))
                    continue
                addr, keep = upload(raw)
                self._keep.append(keep)
                setattr(d, key, addr)
            if h264:
                d.scaling4, d.scaling8 = pic.pic.scaling4, pic.pic.scaling8
            return d

        self._dev = (dev(self.intra), [dev(p) for p in self.pred])

    def picture(self, n: int):
        """(picture, out_slot) of frame n."""
        import ctypes
        intra, pred = (self.intra, self.pred) if self._dev is None else self._dev
        if n == 0:
            pic, slot = intra, 0
        else:
            slot = n % self.spec.slots
            pic = pred[slot]
        return (pic if self._dev is None else ctypes.addressof(pic)), slot


def open_stream(spec: StreamSpec, hbm_budget: int = 0) -> ReconStream:
    W, H = spec.coded
    return ReconStream(spec.codec, W, H, spec.bit_depth, spec.slots, hbm_budget, shared_gpu=True)


def submit(st: ReconStream, spec: StreamSpec, pic, slot: int):
    if spec.codec == RC_CODEC_H264:
        st.submit_h264(pic, slot)
    else:
        st.submit_hevc(pic, slot)


def run_plain(specs, templates, streams):
    """Every stream alone, one after the other (each fully finished before the
    next starts).  Returns wall seconds."""
    t0 = time.perf_counter()
    for spec in specs:
        st, tp = streams[spec.key], templates[spec.key]
        for n in range(spec.frames):
            submit(st, spec, *tp.picture(n))
        if st.sync() != 0:
            raise RuntimeError(f"stream {spec.key}: device error")
    return time.perf_counter() - t0


def run_batched(specs, templates, streams, depth: int = 2):
    """All streams in flight together: round-robin submission, at most `depth`
    pictures queued per stream ahead of its completed work.  An H.264 stream
    that reconstructs g pictures per launch (``h264_group``) takes one
    completion mark per g pictures (a mark launches the queued ones) and
    may hold g pictures.  Returns wall seconds."""
    t0 = time.perf_counter()
    nxt = {s.key: 0 for s in specs}
    inflight = {s.key: collections.deque() for s in specs}  # (mark, pictures)
    unmarked = {s.key: 0 for s in specs}
    live = [s for s in specs]
    while live:
        progressed = False
        for spec in list(live):
            st, q = streams[spec.key], inflight[spec.key]
            g = max(1, getattr(st, "h264_group", 1))
            while q and st.mark_done(q[0][0]):
                q.popleft()
            held = sum(n for _, n in q) + unmarked[spec.key]
            while held < max(depth, g) and nxt[spec.key] < spec.frames:
                submit(st, spec, *templates[spec.key].picture(nxt[spec.key]))
                nxt[spec.key] += 1
                unmarked[spec.key] += 1
                held += 1
                progressed = True
                if unmarked[spec.key] == g or nxt[spec.key] == spec.frames:
                    q.append((st.mark(), unmarked[spec.key]))
                    unmarked[spec.key] = 0
            if nxt[spec.key] >= spec.frames and not q:
                live.remove(spec)
        if not progressed:
            time.sleep(20e-6)
    for spec in specs:
        if streams[spec.key].sync() != 0:
            raise RuntimeError(f"stream {spec.key}: device error")
    return time.perf_counter() - t0


# ---------------------------------------------------------------------------
# Schedule autotuner for the batched form
# ---------------------------------------------------------------------------
@dataclasses.dataclass(frozen=True)
class ClassKnobs:
    """The schedule of one shape class of streams (codec, coded size, bit
    depth).  None of the knobs changes a byte of the output."""
    intra_scale: float = 1.0  # HEVC: intra kernel CTAs per launch, the CTB wavefront's width (x the default)
    lf_rows: int = 64         # HEVC: loop-filter tile height in luma rows, the tile shape (64, 32, 16)
    group: int = 1            # H.264: pictures per launch, their wavefronts side by side (1..4)

    def label(self, codec: int) -> str:
        if codec == RC_CODEC_H264:
            return f"group {self.group}"
        return f"intra x{self.intra_scale}, lf tile {self.lf_rows}"


@dataclasses.dataclass(frozen=True)
class Schedule:
    depth: int = 2            # pictures queued per stream ahead of its completed work
    intra_scale: float = 1.0  # HEVC intra CTAs per launch, times each stream's default (classes without knobs)
    classes: tuple = ()       # ((shape class, ClassKnobs), ...): per-class knobs, sorted by class

    def knobs(self, spec) -> ClassKnobs:
        return dict(self.classes).get(shape_class(spec), ClassKnobs(intra_scale=self.intra_scale))

    def describe(self) -> dict:
        return {"depth": self.depth, "intra_scale": self.intra_scale,
                "classes": {c: dataclasses.asdict(k) for c, k in self.classes}}


def shape_class(spec) -> str:
    """A stream's shape class: codec, coded size and bit depth."""
    W, H = spec.coded
    return f"{'h264' if spec.codec == RC_CODEC_H264 else 'hevc'}_{W}x{H}_{spec.bit_depth}"


def mix_signature(specs) -> str:
    """A key for a stream mix: the codec, coded size and bit depth of its streams."""
    items = sorted((s.codec, *s.coded, s.bit_depth) for s in specs)
    return hashlib.sha256(repr(items).encode()).hexdigest()[:16]


def apply_schedule(streams, specs, schedule: Schedule):
    """Set every stream's knobs for `schedule`: HEVC intra CTAs per launch
    (relative to the stream's default) and loop-filter tile height, H.264
    pictures per launch."""
    for s in specs:
        st, k = streams[s.key], schedule.knobs(s)
        if s.codec == RC_CODEC_HEVC:
            st.set_intra_ctas(0)
            st.set_intra_ctas(max(1, int(round(st.intra_ctas() * k.intra_scale))))
            st.set_lf_tile(k.lf_rows)
        else:
            st.set_h264_group(k.group)


def _load_cache(cache_path):
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            cache = json.load(f)
        if isinstance(cache, dict) and "mixes" in cache and "classes" in cache:
            return cache
    return {"mixes": {}, "classes": {}}


def autotune(specs, templates, depths=(1, 2, 3, 4), intra_scales=(0.5, 1.0, 2.0), lf_rows=(64, 32, 16),
             groups=(1, 2, 3), frames: int = 8, open_fn=open_stream, runner=None, cache_path=None,
             class_depth: int = 2):
    """Choose the batched form's schedule for a stream mix.

    Per shape class (codec, coded size, bit depth), the class's own streams
    run the first `frames` pictures of each, `class_depth` pictures queued per
    stream, once untimed and then once per candidate, knob by knob (HEVC: the
    intra CTAs per launch, then the loop-filter tile height with the best of
    those; H.264: pictures per launch); each knob keeps its fastest value.
    Then the whole mix, with every class's knobs, runs the same prefix on
    fresh streams for each number of pictures queued per stream, and the
    fastest wins.  No knob changes a picture's bytes.  With `cache_path`
    (JSON) the choice is kept per class and per mix signature and reused.
    Returns (schedule, {candidate label: frames/s}); the dict is empty when
    the whole schedule came from the cache."""
    runner = runner or run_batched
    key = mix_signature(specs)
    cache = _load_cache(cache_path)
    if key in cache["mixes"]:
        m = cache["mixes"][key]
        return Schedule(m["depth"], classes=tuple(sorted((c, ClassKnobs(**cache["classes"][c]))
                                                          for c in m["classes"]))), {}
    prefix = [dataclasses.replace(s, frames=min(s.frames, frames)) for s in specs]
    by_class = collections.defaultdict(list)
    for s in prefix:
        by_class[shape_class(s)].append(s)
    rates, classes = {}, {}
    for cls in sorted(by_class):
        members = by_class[cls]
        if cls in cache["classes"]:
            classes[cls] = ClassKnobs(**cache["classes"][cls])
            continue
        codec = members[0].codec
        streams = {s.key: open_fn(s) for s in members}
        try:
            timed = {}

            def fps(k: ClassKnobs) -> float:
                if k not in timed:
                    apply_schedule(streams, members, Schedule(class_depth, classes=((cls, k),)))
                    seconds = runner(members, templates, streams, depth=class_depth)
                    timed[k] = sum(s.frames for s in members) / seconds
                    rates[f"{cls}: {k.label(codec)}"] = timed[k]
                return timed[k]

            best = ClassKnobs()
            apply_schedule(streams, members, Schedule(class_depth, classes=((cls, best),)))
            runner(members, templates, streams, depth=class_depth)  # untimed: first use of the streams
            if codec == RC_CODEC_HEVC:
                best = max((dataclasses.replace(best, intra_scale=v) for v in intra_scales), key=fps)
                best = max((dataclasses.replace(best, lf_rows=v) for v in lf_rows), key=fps)
            else:
                best = max((dataclasses.replace(best, group=v) for v in groups), key=fps)
            classes[cls] = best
        finally:
            for st in streams.values():
                st.close()
    knobs = tuple(sorted(classes.items()))
    total = sum(s.frames for s in prefix)
    by_depth = {}
    for depth in depths:
        schedule = Schedule(depth, classes=knobs)
        streams = {s.key: open_fn(s) for s in prefix}
        try:
            apply_schedule(streams, prefix, schedule)
            seconds = runner(prefix, templates, streams, depth=depth)
        finally:
            for st in streams.values():
                st.close()
        by_depth[schedule] = total / seconds
        rates[f"mix: depth {depth}"] = by_depth[schedule]
    best = max(by_depth, key=by_depth.get)
    if cache_path:
        for c, k in knobs:
            cache["classes"][c] = dataclasses.asdict(k)
        cache["mixes"][key] = {"depth": best.depth, "classes": [c for c, _ in knobs],
                               "frames_per_s": by_depth[best]}
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    return best, rates


# ---------------------------------------------------------------------------
# Served form
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Request:
    rid: int
    arrival: float      # seconds from the start of the trace
    stream: int         # StreamSpec.key
    frames: int
    # filled while serving
    first: int = -1     # stream frame index of the request's first frame
    submitted: list = dataclasses.field(default_factory=list)
    done: list = dataclasses.field(default_factory=list)
    admitted: float = -1.0


def poisson_trace(rate: float, count: int, n_streams: int, seed: int = 7, max_frames: int = 12):
    """`count` requests with exponential inter-arrival times at `rate` per
    second; each picks a stream uniformly and asks for 1..max_frames frames
    (half single-frame, half filmstrips)."""
    rng = random.Random(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.expovariate(rate)
        frames = 1 if rng.random() < 0.5 else rng.randint(2, max_frames)
        out.append(Request(i, t, rng.randrange(n_streams), frames))
    return out


class Server:
    """Continuous-batching request loop (one host thread).

    A request is admitted once its stream is resident: if it is not, the
    stream is created, after evicting idle resident streams least-recently
    used while the device bytes would exceed `hbm_budget`; a request that
    cannot get room waits at the head of the queue.  Requests of one stream
    run one after the other (the stream's frames continue where the last
    request stopped; an evicted stream starts again from its intra picture).
    Admitted requests submit up to `depth` frames ahead of completion each,
    so requests that arrive while others are on the GPU overlap with them.
    """

    def __init__(self, specs, templates, hbm_budget: int, depth: int = 2, open_fn=open_stream):
        self.specs = {s.key: s for s in specs}
        self.templates = templates
        self.budget = hbm_budget
        self.depth = depth
        self.open_fn = open_fn
        self.resident = collections.OrderedDict()  # key -> ReconStream (LRU order)
        self.position = {}                          # key -> next frame index
        self.busy = {}                              # key -> active Request
        self.bytes = 0
        self.evictions = 0

    def _make_room(self, need: int) -> bool:
        while self.bytes + need > self.budget:
            victim = next((k for k in self.resident if k not in self.busy), None)
            if victim is None:
                return False
            st = self.resident.pop(victim)
            self.bytes -= st.device_bytes()
            st.close()
            self.position.pop(victim, None)
            self.evictions += 1
        return True

    def _admit(self, req: Request, now: float) -> bool:
        key = req.stream
        if key in self.busy:
            return False
        if key not in self.resident:
            spec = self.specs[key]
            # a stream's device bytes are known once it exists: estimate by
            # creating it, then undo if the budget cannot hold it
            st = self.open_fn(spec)
            need = st.device_bytes()
            if not self._make_room(need):
                st.close()
                return False
            self.resident[key] = st
            self.bytes += need
            self.position[key] = 0
        self.resident.move_to_end(key)
        self.busy[key] = req
        req.first = self.position[key]
        req.admitted = now
        return True

    def run(self, trace, clock=time.perf_counter):
        """Serve `trace` (requests sorted by arrival) in real time; returns the
        trace's requests with their submit / completion times filled in."""
        t0 = clock()
        pending = collections.deque(sorted(trace, key=lambda r: r.arrival))
        queue = collections.deque()
        inflight = {}  # key -> deque of (mark, frame_number_in_request)
        remaining = len(trace)
        while remaining:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            # admission in arrival order; a request whose stream is busy waits
            # for it, others may pass it (different streams are independent)
            waiting = collections.deque()
            blocked = False
            while queue:
                r = queue.popleft()
                if blocked or not self._admit(r, now):
                    waiting.append(r)
                    if r.stream not in self.busy:
                        blocked = True  # out of room: keep arrival order for the rest
            queue = waiting
            progressed = False
            for key, req in list(self.busy.items()):
                st = self.resident[key]
                q = inflight.setdefault(key, collections.deque())
                t = clock() - t0
                while q and st.mark_done(q[0][0]):
                    q.popleft()
                    req.done.append(t)
                    progressed = True
                while len(q) < self.depth and len(req.submitted) < req.frames:
                    n = self.position[key]
                    pic, slot = self.templates[key].picture(n)
                    submit(st, self.specs[key], pic, slot)
                    self.position[key] = n + 1
                    q.append((st.mark(), len(req.submitted)))
                    req.submitted.append(clock() - t0)
                    progressed = True
                if len(req.done) == req.frames:
                    del self.busy[key]
                    remaining -= 1
            if not progressed:
                nxt = pending[0].arrival - (clock() - t0) if pending else 0.0
                time.sleep(min(max(nxt, 20e-6), 1e-3) if not self.busy else 20e-6)
        return trace

    def close(self):
        for st in self.resident.values():
            st.close()
        self.resident.clear()
        self.bytes = 0


def serve_plain(specs, templates, trace, clock=time.perf_counter, open_fn=open_stream):
    """The plain path on the same trace: one request at a time in arrival
    order, each request's frames submitted and finished before the next
    request starts (streams stay open)."""
    specs = {s.key: s for s in specs}
    streams = {}
    position = {}
    t0 = clock()
    for req in sorted(trace, key=lambda r: r.arrival):
        while clock() - t0 < req.arrival:
            # the arrival may pass between the test and this read of the clock
            time.sleep(max(0.0, min(1e-3, req.arrival - (clock() - t0))))
        key = req.stream
        if key not in streams:
            streams[key] = open_fn(specs[key])
            position[key] = 0
        st = streams[key]
        req.admitted = clock() - t0
        req.first = position[key]
        marks = []
        for i in range(req.frames):
            pic, slot = templates[key].picture(position[key])
            submit(st, specs[key], pic, slot)
            position[key] += 1
            req.submitted.append(clock() - t0)
            marks.append(st.mark())
        for m in marks:
            while not st.mark_done(m):
                time.sleep(10e-6)
            req.done.append(clock() - t0)
    for st in streams.values():
        st.close()
    return trace


def latency_stats(trace):
    """p50 / p99 of time to first frame (arrival to first completion) and of
    per-frame latency (submission to completion), in milliseconds, and the
    trace's frames per second."""
    ttff = sorted((r.done[0] - r.arrival) * 1e3 for r in trace if r.done)
    per = sorted((d - s) * 1e3 for r in trace for s, d in zip(r.submitted, r.done))
    span = max(r.done[-1] for r in trace if r.done) - min(r.arrival for r in trace)
    frames = sum(len(r.done) for r in trace)

    def pct(v, p):
        return v[min(len(v) - 1, int(round(p / 100 * (len(v) - 1))))] if v else None

    return {"ttff_p50_ms": pct(ttff, 50), "ttff_p99_ms": pct(ttff, 99), "frame_p50_ms": pct(per, 50),
            "frame_p99_ms": pct(per, 99), "frames_per_s": frames / span if span > 0 else None, "frames": frames,
            "requests": len(trace)}
