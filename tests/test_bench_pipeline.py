"""bench.pipelined_steps, the two-context pipeline of the end-to-end
measurement, with fake contexts on the CPU: uploads and computes take turns
in step order and never overlap, a step's copy back runs outside the turn,
every context waits for its copies once at the end, and an error in one thread
stops the other and is raised (no hang)."""
import threading
import time

import pytest

import bench


class FakeContexts:
    def __init__(self, fail_at=None, copy_s=0.004):
        self.lock = threading.Lock()
        self.log = []          # (event, step or context, context, time)
        self.busy = 0          # contexts inside upload or compute
        self.max_busy = 0
        self.step = [None, None]
        self.fail_at = fail_at
        self.copy_s = copy_s
        self.copies = []       # (context, start, end) of the simulated copies
        self.finished = []
        self.compute_end = []

    def _enter(self, what, e):
        with self.lock:
            self.busy += 1
            self.max_busy = max(self.max_busy, self.busy)
            self.log.append((what, e, time.perf_counter()))

    def _leave(self):
        with self.lock:
            self.busy -= 1

    def upload(self, e):
        self._enter("upload", e)
        time.sleep(0.001)
        self._leave()

    def compute(self, e):
        self._enter("compute", e)
        n = sum(1 for ev in self.log if ev[0] == "compute")
        time.sleep(0.003)
        with self.lock:
            self.compute_end.append(time.perf_counter())
        self._leave()
        if self.fail_at is not None and n - 1 == self.fail_at:
            raise ValueError("compute failed")
        return n

    def copy_back(self, e, res):
        t0 = time.perf_counter()
        with self.lock:
            self.copies.append((e, t0, t0 + self.copy_s))
        return ("cells", e, res)

    def finish(self, e):
        with self.lock:
            self.finished.append(e)


@pytest.mark.parametrize("first,n", [(0, 16), (3, 5), (2, 1)])
def test_turns_in_step_order(first, n):
    f = FakeContexts()
    secs, recs = bench.pipelined_steps(first, n, f.upload, f.compute, f.copy_back, f.finish,
                                       timeout=10)
    assert secs > 0 and len(recs) == n
    # one context at a time inside upload + compute
    assert f.max_busy == 1
    # step i runs on context (i - first) % 2, upload then compute, in step order
    seq = [(ev[0], ev[1]) for ev in f.log]
    want = []
    for i in range(n):
        want += [("upload", i % 2), ("compute", i % 2)]
    assert seq == want
    # copy_back's values come back per step, in step order
    assert [r[3] for r in recs] == [("cells", i % 2, i + 1) for i in range(n)]
    assert all(r[0] >= 0 and r[1] > 0 and r[2] > 0 for r in recs)
    # every context waits for its copies once, after its last step (or at once)
    assert sorted(f.finished) == [0, 1]


def test_copy_back_overlaps_the_next_step():
    # simulated copies of 1 s (nothing sleeps: copy_back only queues)
    f = FakeContexts(copy_s=1.0)
    bench.pipelined_steps(0, 6, f.upload, f.compute, f.copy_back, f.finish, timeout=10)
    starts = [ev[2] for ev in f.log if ev[0] == "compute"]
    copies = sorted(f.copies, key=lambda c: c[1])
    # the copy of step i is queued before step i + 1's compute ends and is
    # still in flight while it runs: copies overlap the next step
    for i, (e, c0, c1) in enumerate(copies[:-1]):
        assert c0 < f.compute_end[i + 1] and starts[i + 1] < c1


def test_error_stops_both_threads_and_is_raised():
    f = FakeContexts(fail_at=3)
    t0 = time.perf_counter()
    with pytest.raises(ValueError, match="compute failed"):
        bench.pipelined_steps(0, 16, f.upload, f.compute, f.copy_back, f.finish, timeout=10)
    assert time.perf_counter() - t0 < 5
    # no step after the failing one and the next (which may have started)
    assert sum(1 for ev in f.log if ev[0] == "compute") <= 5
