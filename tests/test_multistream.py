"""The batched and served forms (pito-codecs_gb300/multistream.py).

CPU: the request loop's admission under an HBM budget, least-recently-used
eviction of idle streams, per-stream request order and frame positions,
with fake streams.  GPU: streams run together (batched) or served from a
request trace leave every stream's DPB exactly as running it alone does.
"""
from __future__ import annotations

import hashlib
import importlib

import pytest


def ms(engine):
    return importlib.import_module("pito_codecs_gb300.multistream")


class FakeStream:
    def __init__(self, spec, nbytes, log):
        self.spec, self.nbytes, self.log = spec, nbytes, log
        self.marks = 0
        self.open = True
        log.append(("open", spec.key))

    def device_bytes(self):
        return self.nbytes

    def submit_h264(self, pic, slot):
        self.log.append(("frame", self.spec.key, pic))

    submit_hevc = submit_h264

    def mark(self):
        self.marks += 1
        return self.marks

    def mark_done(self, m):
        return True

    def close(self):
        self.open = False
        self.log.append(("close", self.spec.key))


class FakeTemplates:
    def __init__(self, slots):
        self.slots = slots

    def picture(self, n):
        return n, n % self.slots


def test_server_admission_eviction_and_order(engine):
    M = ms(engine)
    specs = M.mix_specs(3, min_frames=5, max_frames=5)
    log = []
    tpl = {s.key: FakeTemplates(s.slots) for s in specs}
    srv = M.Server(specs, tpl, hbm_budget=250, depth=2, open_fn=lambda spec: FakeStream(spec, 100, log))
    trace = [M.Request(0, 0.0, 0, 3), M.Request(1, 0.0, 1, 2), M.Request(2, 0.0, 0, 2), M.Request(3, 0.0, 2, 1)]
    srv.run(trace)
    assert all(len(r.done) == r.frames for r in trace)
    # stream 0's two requests ran one after the other, frames continuing
    frames0 = [e[2] for e in log if e[0] == "frame" and e[1] == 0]
    assert frames0[:5] == [0, 1, 2, 3, 4]
    assert trace[0].first == 0 and trace[2].first == 3
    # the budget holds two streams: opening stream 2 evicted an idle one
    assert srv.evictions >= 1
    assert srv.bytes <= 250
    srv.close()


def test_trace_and_stats(engine):
    M = ms(engine)
    tr = M.poisson_trace(200.0, 2000, 64, seed=3)
    gaps = [b.arrival - a.arrival for a, b in zip(tr, tr[1:])]
    assert abs(sum(gaps) / len(gaps) - 1 / 200.0) < 0.2 / 200.0
    assert all(1 <= r.frames <= 12 for r in tr)
    for r in tr[:10]:
        r.submitted = [r.arrival + 0.001 * i for i in range(r.frames)]
        r.done = [s + 0.002 for s in r.submitted]
    st = M.latency_stats(tr[:10])
    assert abs(st["frame_p50_ms"] - 2.0) < 1e-6
    assert st["ttff_p99_ms"] >= st["ttff_p50_ms"] > 0


def _dpb_digest(st):
    h = hashlib.sha256()
    for slot in range(st.slots):
        for plane in st.download(slot):
            h.update(plane.tobytes())
    return h.hexdigest()


@pytest.mark.gpu
def test_batched_equals_alone(engine):
    M = ms(engine)
    specs = M.mix_specs(6, min_frames=4, max_frames=9, seed=11)
    for s in specs:  # keep the test small: no 4K streams
        if s.width > 1280:
            s.width, s.height = 854, 480
    tpl = {s.key: M.Templates(s) for s in specs}
    alone = {s.key: M.open_stream(s) for s in specs}
    mixed = {s.key: M.open_stream(s) for s in specs}
    try:
        M.run_plain(specs, tpl, alone)
        M.run_batched(specs, tpl, mixed, depth=3)
        for s in specs:
            assert _dpb_digest(alone[s.key]) == _dpb_digest(mixed[s.key]), f"stream {s.key} differs in the mix"
    finally:
        for st in list(alone.values()) + list(mixed.values()):
            st.close()


@pytest.mark.gpu
def test_schedule_changes_no_bytes(engine):
    """The autotuner's knobs (pictures queued per stream; per shape class the
    HEVC intra CTAs per launch and loop-filter tile height, the H.264
    pictures per launch) change the order and overlap of the work only."""
    M = ms(engine)
    specs = M.mix_specs(12, min_frames=4, max_frames=7, seed=21)
    for s in specs:
        if s.width > 854:
            s.width, s.height = 854, 480
    tpl = {s.key: M.Templates(s) for s in specs}
    classes = sorted({M.shape_class(s) for s in specs})
    mk = lambda scale, rows, group: tuple((c, M.ClassKnobs(scale, rows, group)) for c in classes)
    digests = []
    for schedule in (M.Schedule(1, 1.0), M.Schedule(3, classes=mk(0.25, 16, 3)),
                     M.Schedule(2, classes=mk(4.0, 32, 2))):
        streams = {s.key: M.open_stream(s) for s in specs}
        try:
            M.apply_schedule(streams, specs, schedule)
            M.run_batched(specs, tpl, streams, depth=schedule.depth)
            digests.append([_dpb_digest(streams[s.key]) for s in specs])
        finally:
            for st in streams.values():
                st.close()
    assert digests[0] == digests[1] == digests[2]


@pytest.mark.gpu
def test_batched_device_records_equal_alone(engine):
    """Many streams with device-resident records run far ahead of the GPU:
    every per-stream upload (level-scale tables included) must be ordered on
    the stream that reads it, not on the legacy default stream."""
    torch = pytest.importorskip("torch")
    M = ms(engine)
    specs = M.mix_specs(24, min_frames=6, max_frames=24, seed=13)
    for s in specs:
        if s.width > 1280:
            s.width, s.height = 854, 480
    tpl = {s.key: M.Templates(s) for s in specs}

    def upload(raw):
        d = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
        return d.data_ptr(), d

    for t in tpl.values():
        t.to_device(upload)
    torch.cuda.synchronize()
    digests = []
    for run in ("alone", "mixed", "mixed"):
        streams = {s.key: M.open_stream(s) for s in specs}
        try:
            if run == "alone":
                M.run_plain(specs, tpl, streams)
            else:
                M.run_batched(specs, tpl, streams, depth=2)
            assert all(st.error() == 0 for st in streams.values())
            digests.append({k: _dpb_digest(st) for k, st in streams.items()})
        finally:
            for st in streams.values():
                st.close()
    for s in specs:
        assert digests[0][s.key] == digests[1][s.key] == digests[2][s.key], f"stream {s.key} differs in the mix"


@pytest.mark.gpu
def test_served_equals_plain(engine):
    M = ms(engine)
    specs = M.mix_specs(5, seed=12)
    for s in specs:
        if s.width > 1280:
            s.width, s.height = 854, 480
    tpl = {s.key: M.Templates(s) for s in specs}
    trace = M.poisson_trace(400.0, 24, len(specs), seed=5, max_frames=6)
    srv = M.Server(specs, tpl, hbm_budget=1 << 40, depth=2)
    try:
        srv.run(trace)
        assert all(len(r.done) == r.frames for r in trace)
        # replay each stream's frame sequence alone and compare the DPBs
        for s in specs:
            n = sum(r.frames for r in trace if r.stream == s.key)
            if n == 0 or s.key not in srv.resident:
                continue
            with M.open_stream(s) as st:
                for k in range(n):
                    M.submit(st, s, *tpl[s.key].picture(k))
                assert st.sync() == 0
                assert _dpb_digest(st) == _dpb_digest(srv.resident[s.key]), f"stream {s.key}"
        stats = M.latency_stats(trace)
        assert stats["frames"] == sum(r.frames for r in trace)
    finally:
        srv.close()
