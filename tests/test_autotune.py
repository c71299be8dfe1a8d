"""Host logic of pito-codecs_gb300/multistream.py on fake streams (no GPU
needed): the batched form's schedule autotuner (per shape class, then the
mix's depth; its cache), and the plain server's wait for arrivals."""
from __future__ import annotations

import importlib


def ms(engine):
    return importlib.import_module("pito_codecs_gb300.multistream")


class FakeStream:
    def __init__(self, spec, default=40):
        self.spec, self.default, self.ctas, self.closed = spec, default, default, False
        self.lf_rows, self.h264_group = 64, 1

    def set_intra_ctas(self, n):
        self.ctas = self.default if n <= 0 else n

    def intra_ctas(self):
        return self.ctas

    def set_lf_tile(self, rows):
        assert rows in (16, 32, 64)
        self.lf_rows = rows

    def set_h264_group(self, n):
        self.h264_group = n
        return n

    def close(self):
        self.closed = True


def test_autotune_picks_each_class_and_the_depth_and_caches_them(engine, tmp_path):
    M = ms(engine)
    specs = M.mix_specs(12, seed=3, min_frames=20, max_frames=30)
    classes = {M.shape_class(s) for s in specs}
    opened, runs = [], []

    def open_fn(spec):
        st = FakeStream(spec)
        opened.append(st)
        return st

    def runner(prefix, templates, streams, depth):
        # fastest at depth 3, HEVC streams at half their default CTAs with
        # 32-row loop-filter tiles, H.264 streams two pictures per launch
        assert all(s.frames <= 8 for s in prefix)
        cost = 1.0 + abs(depth - 3)
        for s in prefix:
            st = streams[s.key]
            if s.codec == engine.RC_CODEC_HEVC:
                cost += abs(st.ctas - 20) / 100 + abs(st.lf_rows - 32) / 1000
            else:
                cost += abs(st.h264_group - 2) / 50
        runs.append(depth)
        return cost

    cache = tmp_path / "schedules.json"
    best, rates = M.autotune(specs, None, frames=8, open_fn=open_fn, runner=runner, cache_path=str(cache))
    assert best.depth == 3
    knobs = dict(best.classes)
    assert set(knobs) == classes
    for c, k in knobs.items():
        if c.startswith("hevc"):
            assert (k.intra_scale, k.lf_rows) == (0.5, 32)
        else:
            assert k.group == 2
    # per HEVC class: one untimed run, 3 intra scales, 2 more tile heights;
    # per H.264 class: one untimed run, 3 groups; then 4 depths on the mix
    n_hevc = sum(c.startswith("hevc") for c in classes)
    assert len(runs) == 6 * n_hevc + 4 * (len(classes) - n_hevc) + 4
    assert len(rates) == 5 * n_hevc + 3 * (len(classes) - n_hevc) + 4
    assert all(st.closed for st in opened)
    # the mix's streams got their class's knobs
    streams = {s.key: FakeStream(s) for s in specs}
    M.apply_schedule(streams, specs, best)
    for s in specs:
        st = streams[s.key]
        if s.codec == engine.RC_CODEC_HEVC:
            assert (st.ctas, st.lf_rows) == (20, 32)
        else:
            assert st.h264_group == 2
    # the same mix again: from the cache, nothing runs
    runs.clear()
    best2, rates2 = M.autotune(specs, None, open_fn=open_fn, runner=runner, cache_path=str(cache))
    assert best2 == best and rates2 == {} and not runs
    # another mix: classes already tuned come from the cache, only new
    # classes and the depth are timed
    other = M.mix_specs(16, seed=9)
    assert M.mix_signature(other) != M.mix_signature(specs)
    new = {M.shape_class(s) for s in other} - classes
    M.autotune(other, None, depths=(2,), open_fn=open_fn, runner=runner, cache_path=str(cache))
    n_new_hevc = sum(c.startswith("hevc") for c in new)
    assert len(runs) == 6 * n_new_hevc + 4 * (len(new) - n_new_hevc) + 1


def test_apply_schedule_restores_each_default_first(engine):
    M = ms(engine)
    specs = M.mix_specs(4, seed=5)
    streams = {s.key: FakeStream(s, default=30) for s in specs}
    M.apply_schedule(streams, specs, M.Schedule(2, 2.0))
    M.apply_schedule(streams, specs, M.Schedule(2, 0.5))  # relative to the default, not to the last value
    for s in specs:
        assert streams[s.key].ctas == (15 if s.codec == engine.RC_CODEC_HEVC else 30)
        assert streams[s.key].lf_rows == 64 and streams[s.key].h264_group == 1


def test_batched_runner_marks_once_per_group(engine):
    """An H.264 stream that reconstructs g pictures per launch gets one
    completion mark per g submitted pictures (a mark launches the queued
    group), and may hold g pictures even when the depth is smaller."""
    M = ms(engine)
    spec = M.StreamSpec(0, engine.RC_CODEC_H264, 64, 48, 8, 10, 1)

    class Tpl:
        def picture(self, n):
            return None, n % spec.slots

    class Stream:
        h264_group = 3

        def __init__(self):
            self.n, self.marks, self.done, self.most = 0, [], 0, 0

        def submit_h264(self, pic, slot):
            self.n += 1
            self.most = max(self.most, self.n - self.done)  # pictures held

        def mark(self):
            self.marks.append(self.n)
            return self.n

        def mark_done(self, m):
            self.done = max(self.done, m)
            return True

        def sync(self):
            return 0

    st = Stream()
    M.run_batched([spec], {0: Tpl()}, {0: st}, depth=1)
    assert st.n == 10 and st.marks == [3, 6, 9, 10] and st.most == 3


def test_plain_server_wait_survives_an_arrival_passing_mid_wait(engine):
    """serve_plain waits for each request's arrival; the clock may pass the
    arrival between the loop's test and the read that sizes the sleep, which
    must then sleep zero, not a negative time."""
    M = ms(engine)
    spec = M.StreamSpec(0, engine.RC_CODEC_H264, 64, 48, 8, 4, 1)

    class Tpl:
        def picture(self, n):
            return None, n % spec.slots

    class Stream:
        def __init__(self, s):
            self.n = 0

        def submit_h264(self, pic, slot):
            self.n += 1

        def mark(self):
            return self.n

        def mark_done(self, m):
            return True

        def close(self):
            pass

    # t0, then the loop's test (before the arrival), then the sleep's read
    # (after it), then everything later
    times = iter([0.0, 0.4, 0.6] + [0.7 + 0.01 * i for i in range(100)])
    trace = [M.Request(0, 0.5, 0, 2)]
    M.serve_plain([spec], {0: Tpl()}, trace, clock=lambda: next(times), open_fn=Stream)
    assert trace[0].admitted >= 0.5 and len(trace[0].done) == 2
