"""Host logic of pito-codecs_gb300/multistream.py on fake streams (no GPU
needed): the batched form's schedule autotuner, and the plain server's wait
for arrivals."""
from __future__ import annotations

import importlib


def ms(engine):
    return importlib.import_module("pito_codecs_gb300.multistream")


class FakeStream:
    def __init__(self, spec, default=40):
        self.spec, self.default, self.ctas, self.closed = spec, default, default, False

    def set_intra_ctas(self, n):
        self.ctas = self.default if n <= 0 else n

    def intra_ctas(self):
        return self.ctas

    def close(self):
        self.closed = True


def test_autotune_picks_the_fastest_schedule_and_caches_it(engine, tmp_path):
    M = ms(engine)
    specs = M.mix_specs(6, seed=3, min_frames=20, max_frames=30)
    opened, runs = [], []

    def open_fn(spec):
        st = FakeStream(spec)
        opened.append(st)
        return st

    def runner(prefix, templates, streams, depth):
        # fastest at depth 3 with HEVC streams at half their default CTAs
        ctas = [streams[s.key].ctas for s in prefix if s.codec == engine.RC_CODEC_HEVC]
        assert all(s.frames <= 8 for s in prefix)
        runs.append((depth, tuple(ctas)))
        return 1.0 + abs(depth - 3) + sum(abs(c - 20) for c in ctas) / 100

    cache = tmp_path / "schedules.json"
    best, rates = M.autotune(specs, None, depths=(1, 2, 3, 4), intra_scales=(0.5, 1.0, 2.0), frames=8,
                             open_fn=open_fn, runner=runner, cache_path=str(cache))
    assert best == M.Schedule(3, 0.5)
    assert len(rates) == 12 and max(rates, key=rates.get) == best
    assert len(runs) == 12 and all(st.closed for st in opened)
    # H.264 streams have no intra CTA knob; HEVC ones got default x scale
    assert {c for _, cs in runs for c in cs} == {20, 40, 80}
    # the same mix again: from the cache, nothing runs
    runs.clear()
    best2, rates2 = M.autotune(specs, None, open_fn=open_fn, runner=runner, cache_path=str(cache))
    assert best2 == best and rates2 == {} and not runs
    # another mix is tuned anew
    other = M.mix_specs(4, seed=9)
    assert M.mix_signature(other) != M.mix_signature(specs)
    M.autotune(other, None, depths=(2,), intra_scales=(1.0,), open_fn=open_fn, runner=runner, cache_path=str(cache))
    assert len(runs) == 1


def test_apply_schedule_restores_each_default_first(engine):
    M = ms(engine)
    specs = M.mix_specs(4, seed=5)
    streams = {s.key: FakeStream(s, default=30) for s in specs}
    M.apply_schedule(streams, specs, M.Schedule(2, 2.0))
    M.apply_schedule(streams, specs, M.Schedule(2, 0.5))  # relative to the default, not to the last value
    for s in specs:
        assert streams[s.key].ctas == (15 if s.codec == engine.RC_CODEC_HEVC else 30)


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
