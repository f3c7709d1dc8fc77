"""Host logic of the served form (serve.Server) on CPU, with fake reconstruction handles:
first-come admission into free slots, completion collection, error propagation from a
failed submit or poll, arrival times respected, latency summary without failed requests."""
import contextlib
import time
import types

import pytest

torch = pytest.importorskip("torch")

import psr  # noqa: E402
import serve  # noqa: E402


class FakeRecon:
    """Finishes a reconstruction after `polls` polls; can fail its submit or its poll."""

    def __init__(self, name, polls=2, fail_submit=False, fail_poll=0):
        self.name, self.polls_needed = name, polls
        self.fail_submit, self.fail_poll = fail_submit, fail_poll   # fail_poll: polls left to fail
        self.submitted = []
        self.n = 0

    def submit_device(self, xyz_ptr, nrm_ptr, rgb_ptr, n, mesh, depth=0, stream=None, location=None):
        if self.fail_submit:
            raise psr.PsrError(psr.PSR_INVALID_INPUT, "submit refused")
        self.submitted.append(n)
        self.n = 0

    def poll(self):
        if self.fail_poll:
            self.fail_poll -= 1
            raise psr.PsrError(psr.PSR_DEVICE_TIMEOUT, "bounded wait gave up")
        self.n += 1
        return self.n >= self.polls_needed

    def wait(self):
        pass

    def close(self):
        pass


class FakeStream:
    cuda_stream = 0

    def synchronize(self):
        pass


def make_server(recons):
    s = serve.Server.__new__(serve.Server)      # no CUDA: slots built by hand
    s.torch = types.SimpleNamespace(cuda=types.SimpleNamespace(stream=lambda st: contextlib.nullcontext()))
    s.vcap, s.tcap = 16, 16
    s.compute_colors, s.compute_normals = False, True
    s.host_outputs = False
    s.slots = []
    for r in recons:
        out = [torch.zeros(16, 3), torch.zeros(16, 3, dtype=torch.int32), None, torch.zeros(16, 3)]
        s.slots.append(serve._Slot(r, FakeStream(), out))
    s.queue, s.done, s.rejected = [], [], []
    return s


def req(n, tag):
    return serve.Request(xyz=torch.zeros(n, 3), normals=torch.zeros(n, 3), tag=tag)


def test_first_come_admission_and_completion():
    a, b = FakeRecon("a", polls=1), FakeRecon("b", polls=3)
    s = make_server([a, b])
    reqs = [req(10 + k, k) for k in range(5)]
    done = s.run(reqs)
    assert sorted(r.tag for r in done) == [0, 1, 2, 3, 4]
    assert all(not r.error for r in done)
    # slot a (one poll) takes requests 0, 2, 3, 4 in order; slot b (three polls) takes 1,
    # which completes in the same step as 3
    assert b.submitted == [11]
    assert a.submitted == [10, 12, 13, 14]
    assert [r.tag for r in done] == [0, 2, 3, 1, 4]
    for r in done:
        assert r.arrival <= r.admitted <= r.finished
        assert r.normals_out is not None and r.vertices.shape == (0, 3)


def test_failed_submit_and_poll_finish_with_an_error_and_free_the_slot():
    bad_submit = FakeRecon("s", fail_submit=True)
    s = make_server([bad_submit])
    done = s.run([req(5, "x"), req(6, "y")])
    assert [r.error != "" for r in done] == [True, True]
    assert "submit refused" in done[0].error
    bad_poll = FakeRecon("p", fail_poll=1)
    good = FakeRecon("g", polls=1)
    s = make_server([bad_poll, good])
    done = s.run([req(5, "x"), req(6, "y"), req(7, "z")])
    errs = {r.tag: r.error for r in done}
    assert "bounded wait" in errs["x"]
    assert errs["y"] == "" and errs["z"] == ""
    assert serve.latency_summary(done)["p50_ms"] is not None


def test_arrivals_are_respected():
    s = make_server([FakeRecon("a", polls=1)])
    t0 = time.perf_counter()
    done = s.run([req(3, "late"), req(3, "early")], arrivals=[0.05, 0.0])
    by = {r.tag: r for r in done}
    assert by["late"].admitted - t0 >= 0.05 - 1e-3
    assert by["early"].finished <= by["late"].admitted + 1e-3


def test_latency_summary_skips_failed_requests():
    ok = serve.Request(xyz=None, normals=None, arrival=1.0, finished=1.002)
    bad = serve.Request(xyz=None, normals=None, arrival=1.0, finished=9.0, error="x")
    s = serve.latency_summary([ok, bad])
    assert s["p99_ms"] == pytest.approx(2.0)
    assert serve.latency_summary([bad]) == {"p50_ms": None, "p99_ms": None}


def test_footprint_classes_first_fit_and_rejection():
    """Slots of two sizes: a large cloud waits for the large slot while small clouds queued
    behind it go to the small slot; a cloud no slot takes is rejected at once."""
    small, large = FakeRecon("small", polls=1), FakeRecon("large", polls=4)
    s = make_server([small, large])
    s.slots[0].max_points, s.slots[1].max_points = 100, 1000
    reqs = [req(500, "big0"), req(600, "big1"), req(50, "s0"), req(60, "s1"), req(5000, "huge")]
    done = s.run(reqs)
    by = {r.tag: r for r in done}
    assert "rejected" in by["huge"].error
    assert s.rejected == [by["huge"]]
    assert small.submitted == [50, 60] and large.submitted == [500, 600]
    # the small clouds did not wait behind big1, which waited for the large slot
    assert by["s1"].finished <= by["big1"].admitted + 1e-3
    assert all(by[t].error == "" for t in ("big0", "big1", "s0", "s1"))


def test_host_output_ring_hands_out_views_of_alternating_sets():
    """A finished request keeps views of the output set its slot wrote (no copy), and the
    slot's next request writes the next set of its ring."""
    a = FakeRecon("a", polls=1)
    s = make_server([a])
    s.host_outputs = True
    ring = [[torch.zeros(16, 3), torch.zeros(16, 3, dtype=torch.int32), None, torch.zeros(16, 3)] for _ in range(2)]
    sl = s.slots[0]
    sl.ring, sl.ring_at, sl.out = ring, 0, ring[0]
    done = s.run([req(4, k) for k in range(4)])
    assert [r.tag for r in done] == [0, 1, 2, 3]
    for k, r in enumerate(done):
        assert r.error == ""
        assert r.vertices.untyped_storage().data_ptr() == ring[k % 2][0].untyped_storage().data_ptr()
        assert r.triangles.untyped_storage().data_ptr() == ring[k % 2][1].untyped_storage().data_ptr()
    assert sl.out is ring[0] and sl.ring_at == 0
