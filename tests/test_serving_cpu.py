"""Host logic of the serving loop (pairhmm.serving) on the CPU.

The scheduler runs against a fake executor whose batches finish after a set
number of polls, so admission, memory accounting, batching and retirement
are checked without a GPU."""
import numpy as np
import pytest

from pairhmm.serving import ALIGN, Arena, Request, Scheduler, latency_summary, run_stream


class FakeExecutor:
    """Bytes per request = 1 KiB per 100 residues; batches finish after
    `polls_to_finish` calls to ready()."""

    def __init__(self, polls_to_finish=2):
        self.polls_to_finish = polls_to_finish
        self.launched = []
        self.live_bytes = 0
        self.max_live_bytes = 0
        self.max_live_batches = 0
        self.live = 0

    def request_bytes(self, r):
        return 1024 * (1 + (len(r.x) + len(r.y)) // 100) + ALIGN

    def batch_bytes(self, model, reqs):
        return sum(1024 * (1 + (len(r.x) + len(r.y)) // 100) for r in reqs) + ALIGN

    def launch(self, model, reqs, off, nbytes, slot):
        assert all(r.model == model for r in reqs)
        h = {'polls': 0, 'model': model, 'n': len(reqs), 'off': off, 'nbytes': nbytes, 'slot': slot}
        self.launched.append(h)
        self.live += 1
        self.live_bytes += nbytes
        self.max_live_bytes = max(self.max_live_bytes, self.live_bytes)
        self.max_live_batches = max(self.max_live_batches, self.live)
        return h

    def ready(self, h):
        h['polls'] += 1
        return h['polls'] >= self.polls_to_finish

    def finish(self, h, reqs):
        self.live -= 1
        self.live_bytes -= h['nbytes']
        for r in reqs:
            r.result = {'log_p': -float(len(r.x) + len(r.y)), 'model': h['model']}


def _req(i, model, lx, ly=None):
    ly = lx if ly is None else ly
    return Request(i, model, np.zeros(lx, np.int64), np.zeros(ly, np.int64), 0.5)


def test_arena_first_fit_and_coalesce():
    a = Arena(10 * ALIGN)
    x = a.alloc(3 * ALIGN)
    y = a.alloc(1)             # rounded up to one unit
    z = a.alloc(4 * ALIGN)
    assert x == (0, 3 * ALIGN) and y == (3 * ALIGN, ALIGN) and z == (4 * ALIGN, 4 * ALIGN)
    assert a.alloc(3 * ALIGN) is None and a.largest_free() == 2 * ALIGN
    a.release(*y)
    a.release(*x)              # coalesces with y's range
    assert a.free_ranges()[0] == (0, 4 * ALIGN)
    a.release(*z)              # everything back in one range
    assert a.free_ranges() == [(0, 10 * ALIGN)] and a.used == 0


def test_arena_random_alloc_release_keeps_invariants():
    rng = np.random.default_rng(0)
    a = Arena(1 << 20)
    live = []
    for _ in range(2000):
        if live and rng.random() < 0.5:
            k = int(rng.integers(len(live)))
            a.release(*live.pop(k))
        else:
            got = a.alloc(int(rng.integers(1, 40000)))
            if got:
                live.append(got)
        spans = sorted(live) + a.free_ranges()
        spans.sort()
        # live and free ranges tile the arena exactly, with no overlap
        pos = 0
        for off, n in spans:
            assert off == pos and off % ALIGN == 0
            pos += n
        assert pos == a.size
        assert a.used == sum(n for _, n in live)


def test_scheduler_batches_one_model_in_arrival_order():
    ex = FakeExecutor(polls_to_finish=1)
    s = Scheduler(ex, arena_bytes=1 << 20, max_inflight=1, max_batch=3)
    models = ['a', 'b', 'a', 'a', 'b', 'a']
    reqs = [s.submit(_req(i, m, 50), arrival=float(i)) for i, m in enumerate(models)]
    s.poll()
    # first batch: the head's model 'a', the next two 'a' requests behind it
    assert [r.rid for r in reqs if r.admitted is not None] == [0, 2, 3]
    done = s.drain()
    assert sorted(r.rid for r in done) == [0, 1, 2, 3, 4, 5]
    assert [h['model'] for h in ex.launched] == ['a', 'b', 'a']
    assert [h['n'] for h in ex.launched] == [3, 2, 1]
    assert all(r.result['log_p'] == -100.0 and r.error is None for r in reqs)


def test_scheduler_overlaps_batches_up_to_inflight_limit():
    ex = FakeExecutor(polls_to_finish=3)
    s = Scheduler(ex, arena_bytes=1 << 20, max_inflight=3, max_batch=1)
    for i in range(9):
        s.submit(_req(i, 'a', 10), arrival=float(i))
    s.poll()
    assert len(s.inflight) == 3          # three batches on the device at once
    s.drain()
    assert ex.max_live_batches == 3 and len(s.completed) == 9


def test_scheduler_admission_is_memory_bounded():
    ex = FakeExecutor(polls_to_finish=2)
    budget = 8 * 1024
    s = Scheduler(ex, arena_bytes=budget, max_inflight=8, max_batch=8)
    rng = np.random.default_rng(1)
    for i in range(40):
        s.submit(_req(i, 'ab'[i % 2], int(rng.integers(10, 250))), arrival=float(i))
    s.drain()
    assert len(s.completed) == 40 and all(r.error is None for r in s.completed)
    assert ex.max_live_bytes <= budget
    assert s.peak_bytes <= budget
    assert s.arena.used == 0 and s.arena.free_ranges() == [(0, s.arena.size)]


def test_scheduler_rejects_request_larger_than_arena():
    ex = FakeExecutor()
    s = Scheduler(ex, arena_bytes=4096, max_inflight=2, max_batch=4)
    big = s.submit(_req(0, 'a', 5000))
    ok = s.submit(_req(1, 'a', 10))
    s.drain()
    assert big.error is not None and 'arena' in big.error and big.result is None
    assert ok.error is None and ok.result is not None


def test_oldest_request_is_not_starved_by_smaller_ones():
    ex = FakeExecutor(polls_to_finish=2)
    s = Scheduler(ex, arena_bytes=6 * 1024, max_inflight=4, max_batch=1)
    small0 = s.submit(_req(0, 'a', 10), arrival=0.0)
    s.poll()                                   # small0 occupies part of the arena
    big = s.submit(_req(1, "a", 200), arrival=1.0)    # needs more than is free now
    later = [s.submit(_req(2 + i, 'a', 10), arrival=2.0 + i) for i in range(3)]
    s.poll()
    assert big.admitted is None and all(r.admitted is None for r in later)   # FIFO: wait for memory
    s.drain()
    assert big.admitted <= min(r.admitted for r in later)
    assert small0.done is not None


def test_run_stream_with_fake_clock_reports_latency():
    now = [0.0]
    clock = lambda: now[0]

    def sleep(dt):
        now[0] += dt

    class TimedExecutor(FakeExecutor):
        def ready(self, h):
            now[0] += 1e-4                    # each poll of a batch costs 0.1 ms
            return super().ready(h)

    ex = TimedExecutor(polls_to_finish=3)
    s = Scheduler(ex, arena_bytes=1 << 20, max_inflight=2, max_batch=4, clock=clock)
    reqs = [_req(i, 'ab'[i % 2], 30) for i in range(20)]
    offsets = np.arange(20) * 1e-3
    out, wall = run_stream(s, reqs, offsets, clock=clock, sleep=sleep)
    summ = latency_summary(out, wall)
    assert summ['completed'] == 20 and summ['failed'] == 0
    assert 0 < summ['p50_ms'] <= summ['p99_ms']
    assert all(r.done >= r.arrival for r in out)


def test_failed_launch_fails_its_batch_not_the_loop():
    """A launch that raises (e.g. an allocation or CUDA error in the executor)
    fails the requests of that batch, returns their memory and slot, and the
    loop serves the rest."""
    class FailingExecutor(FakeExecutor):
        def __init__(self):
            super().__init__(polls_to_finish=1)
            self.calls = 0

        def launch(self, model, reqs, off, nbytes, slot):
            self.calls += 1
            if self.calls == 1:
                raise RuntimeError('injected launch failure')
            return super().launch(model, reqs, off, nbytes, slot)

    ex = FailingExecutor()
    s = Scheduler(ex, arena_bytes=1 << 16, max_inflight=1, max_batch=2)
    reqs = [s.submit(_req(i, 'a', 20)) for i in range(6)]
    s.drain()
    failed = [r for r in reqs if r.error is not None]
    assert len(failed) == 2 and all('injected launch failure' in r.error for r in failed)
    assert all(r.result is not None for r in reqs if r.error is None)
    assert s.arena.used == 0 and s.idle()


def test_per_request_error_flag_fails_only_that_request():
    """An executor that reports a per-pair status (the kernels' status word)
    fails that request alone; its batch-mates keep their results."""
    class FlaggingExecutor(FakeExecutor):
        def finish(self, h, reqs):
            super().finish(h, reqs)
            for r in reqs:
                if r.rid == 3:
                    r.error = 'kernel status 1'

    ex = FlaggingExecutor(polls_to_finish=1)
    s = Scheduler(ex, arena_bytes=1 << 16, max_inflight=2, max_batch=4)
    reqs = [s.submit(_req(i, 'a', 15)) for i in range(8)]
    s.drain()
    assert [r.rid for r in reqs if r.error] == [3]
    summ = latency_summary(reqs, 1.0)
    assert summ['failed'] == 1 and summ['completed'] == 7
