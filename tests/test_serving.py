"""The render-request loop's scheduling (CPU, with stand-in renderers): every
request finishes with its own result, device memory stays within the budget,
renderers are reused per volume and evicted least recently used first,
requests that arrive while others run start without waiting for them, a
request that can never fit is refused, shortest-first admission with aging,
the per-volume renderer limit, and the memory model against the constants the
library allocates with."""
import pytest

from volview_gb300 import serving as S


class FakeRenderer:
    """The Renderer interface without a device: work takes `ticks` polls."""

    def __init__(self, volume, base, log, ticks=3):
        self.volume, self.base, self.log, self.ticks = volume, base, log, ticks
        self.w = self.h = self.spp = 0
        self.left = 0
        self.destroyed = False
        self.calls = []

    def device_bytes(self):
        assert not self.destroyed
        return self.base + (S.request_bytes(self.w, self.h, self.spp) if self.spp else 0)

    def reset_view(self):
        self.calls.append("reset")

    def resize(self, w, h):
        self.calls.append("resize")
        self.w, self.h = w, h

    def record_frames(self, first, n, params):
        self.calls.append("record")
        self.spp, self.left, self.params = n, self.ticks, params
        self.log.append(("start", params))

    def idle(self):
        self.left -= 1
        return self.left <= 0

    def read_output(self):
        return ("image", self.volume, self.params)

    def read_accumulation(self):
        return ("accumulation", self.params)

    def destroy(self):
        self.destroyed = True
        self.log.append(("destroy", self.volume))


def make_server(budget, bases, ticks=3, max_active=None, **kw):
    log, made = [], []

    def make(volume):
        r = FakeRenderer(volume, bases[volume], log, ticks)
        made.append(r)
        return r

    srv = S.Server(make, lambda v: bases[v], budget, max_active=max_active, clock=iter(range(10 ** 6)).__next__,
                   **kw)
    return srv, log, made


def run(srv, reqs):
    for q in reqs:
        srv.submit(q)
    for _ in range(10000):
        srv.step()
        if not srv.queue and not srv.active:
            return
    raise AssertionError("requests did not finish")


def test_results_are_routed_and_memory_stays_in_budget():
    bases = {"a": 10 ** 9, "b": 2 * 10 ** 9}
    budget = 40 * 10 ** 9
    srv, log, made = make_server(budget, bases)
    reqs = [S.Request("a" if k % 3 else "b", 256 << (k % 3), 256 << (k % 3), (16, 64, 256)[k % 3], params=k)
            for k in range(12)]
    run(srv, reqs)
    assert all(q.image == ("image", q.volume, q.params) for q in reqs)
    assert srv.peak_bytes <= budget
    assert srv.created < len(reqs)                      # renderers reused
    for r in made:
        assert r.calls[:3] == ["reset", "resize", "record"]  # a fresh view per request


def test_requests_overlap_and_later_ones_start_before_earlier_finish():
    bases = {"a": 10 ** 9}
    srv, log, made = make_server(100 * 10 ** 9, bases, ticks=50)
    first = S.Request("a", 512, 512, 64, params="first")
    srv.submit(first)
    srv.step()
    assert first.started is not None and first.finished is None
    second = S.Request("a", 256, 256, 16, params="second")
    srv.submit(second)
    srv.step()
    assert second.started is not None and first.finished is None  # admitted while the first runs
    assert srv.created == 2


def test_idle_renderers_are_evicted_least_recently_used():
    bases = {"a": 10 ** 9, "b": 10 ** 9, "c": 10 ** 9}
    one = bases["a"] + S.request_bytes(256, 256, 16)
    srv, log, made = make_server(2 * one + 1, bases, ticks=1, max_active=1)
    run(srv, [S.Request("a", 256, 256, 16, params=1)])
    run(srv, [S.Request("b", 256, 256, 16, params=2)])
    assert srv.created == 2 and not any(r.destroyed for r in made)
    run(srv, [S.Request("c", 256, 256, 16, params=3)])  # needs room: "a" (least recent) goes
    assert [r.volume for r in made if r.destroyed] == ["a"]
    run(srv, [S.Request("b", 256, 256, 16, params=4)])  # "b" is still resident and reused
    assert srv.created == 3


def test_a_request_that_cannot_fit_is_refused():
    srv, log, made = make_server(10 ** 6, {"a": 10 ** 9})
    srv.submit(S.Request("a", 64, 64, 16, params=0))
    with pytest.raises(MemoryError):
        srv.step()


def test_a_request_too_large_for_its_idle_renderer_is_refused():
    """The volume's renderer is resident and idle, nothing runs, and even with
    every other renderer evicted the request does not fit: refused, not polled
    for ever."""
    bases = {"a": 10 ** 9, "b": 10 ** 9}
    srv, log, made = make_server(3 * 10 ** 9, bases)
    srv.preload("a")
    srv.preload("b")
    big = S.Request("a", 8192, 8192, 16, params=0)  # ~9.5 GB of image and path state
    small = S.Request("a", 256, 256, 16, params=1)
    srv.submit(big)
    srv.submit(small)
    with pytest.raises(MemoryError):
        srv.step()
    assert [e for e in log if e[0] == "destroy"] == [("destroy", "b")]  # evicted trying
    # The refused request leaves the queue: the next steps serve the one behind it.
    assert srv.refused == [big] and big not in srv.queue
    run(srv, [])
    assert small.image == ("image", "a", 1) and big.image is None


def test_shortest_first_with_aging():
    bases = {"a": 10 ** 9}
    srv, log, made = make_server(10 ** 12, bases, ticks=5, max_active=1, order="shortest", aging_s=40)
    big = S.Request("a", 1024, 1024, 1024, params="big")
    mid = S.Request("a", 512, 512, 64, params="mid")
    small = S.Request("a", 256, 256, 16, params="small")
    for q in (big, mid, small):
        srv.submit(q)
    run(srv, [])
    assert [p for kind, p in log if kind == "start"] == ["small", "mid", "big"]
    # Past aging_s a request goes ahead of younger ones, whatever its size.
    srv, log, made = make_server(10 ** 12, bases, ticks=5, max_active=1, order="shortest", aging_s=3)
    srv.submit(S.Request("a", 1024, 1024, 1024, params="old"))
    for _ in range(5):
        srv.clock()  # time passes
    srv.submit(S.Request("a", 256, 256, 16, params="new"))
    run(srv, [])
    assert [p for kind, p in log if kind == "start"] == ["old", "new"]


def test_max_per_volume_waits_for_the_volumes_renderer():
    bases = {"a": 10 ** 9, "b": 10 ** 9}
    srv, log, made = make_server(10 ** 12, bases, ticks=4, max_per_volume=1)
    reqs = [S.Request(v, 256, 256, 16, params=k) for k, v in enumerate("aab")]
    run(srv, reqs)
    assert srv.created == 2  # one renderer per volume
    starts = [p for kind, p in log if kind == "start"]
    assert starts == [0, 2, 1]  # "b" started beside the first "a"; the second "a" waited for it


def test_request_bytes_model():
    # One pass of 16 frames at 1024^2: 16 M slots; 1024 frames: six passes of the cap.
    assert S.request_bytes(1024, 1024, 16) == 1024 * 1024 * (S.IMAGE_BYTES_PER_PIXEL + 16 * S.SLOT_BYTES)
    assert S.request_bytes(1024, 1024, 1024) == 1024 * 1024 * S.IMAGE_BYTES_PER_PIXEL + 6 * (1 << 24) * S.SLOT_BYTES
    assert S.request_bytes(4096, 4096, 1) == 4096 * 4096 * (S.IMAGE_BYTES_PER_PIXEL + S.SLOT_BYTES)


def test_request_bytes_model_follows_the_library_sources():
    """The model's constants are the ones the library allocates with: slot,
    light-map sample, stage-queue and later-flight bin bytes per path slot,
    passes in flight, frames per pass, frames' worth of slots and the slot
    cap."""
    import os
    import re
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "volview_gb300", "csrc")
    host = open(os.path.join(csrc, "vv_host.cpp")).read()
    kernels = open(os.path.join(csrc, "vv_kernels.h")).read()

    def num(pattern, text):
        m = re.search(pattern, text)
        assert m, pattern
        return int(m.group(1))

    slot = num(r"constexpr int WF_SLOT_BYTES = (\d+);", kernels)
    light = num(r"constexpr int WF_MAP_BYTES = (\d+);", kernels)
    queues = num(r"P\.queues\.alloc\(cap \* (\d+) \* sizeof\(uint32_t\)\)", host)
    binned = num(r"P\.binq\.alloc\(cap \* (\d+) \* sizeof\(uint32_t\)\)", host)
    assert S.SLOT_BYTES == slot + light + (queues + binned) * 4
    assert S.PASSES == num(r"#define VV_PASSES (\d+)", host)
    assert S.PASS_FRAMES == num(r"#define VV_SUBPASS_FRAMES (\d+)", host)
    assert S.SLOT_FRAMES == num(r"int slot_frames = (\d+);", host)
    assert S.SLOT_CAP == 1 << num(r"std::max\(px, \(size_t\)1 << (\d+)\)", host)


def test_a_pass_budget_lowers_the_model_and_reaches_the_renderers():
    """With fewer passes and frames in flight per renderer, the model asks for
    less (the dropped passes' sums and slots), and every renderer the loop
    makes gets the budget."""
    full = S.request_bytes(1024, 1024, 1024)
    lean = S.request_bytes(1024, 1024, 1024, passes=2, slot_frames=8)
    assert lean == 1024 * 1024 * (S.IMAGE_BYTES_PER_PIXEL - 48 * 4) + 2 * 8 * 1024 * 1024 * S.SLOT_BYTES
    assert lean < full / 5
    budgets = []

    class Budgeted(FakeRenderer):
        def set_pass_budget(self, passes, frames):
            budgets.append((passes, frames))

    log = []
    srv = S.Server(lambda v: Budgeted(v, 10 ** 9, log), lambda v: 10 ** 9, 10 ** 12, passes=2, slot_frames=8,
                   clock=iter(range(10 ** 6)).__next__)
    srv.preload("b")
    run(srv, [S.Request("a", 256, 256, 16, params=0), S.Request("b", 256, 256, 16, params=1)])
    assert budgets == [(2, 8), (2, 8)]


# ------------------------------------------------------------ batched passes
class FakeEngine:
    """The batch engine without a device: each queued pass takes `ticks`
    in_flight polls to finish."""

    def __init__(self, ticks=2):
        self.ticks, self.pending, self.passes = ticks, [], []

    def record(self, items):
        self.passes.append([(r.name, params, first, n, display) for r, params, first, n, display in items])
        self.pending.append([self.ticks, {id(r) for r, *_ in items}])
        for r, params, first, n, display in items:
            r.frames.append((first, n, display))
            r.params = params

    def in_flight(self):
        for p in self.pending:
            p[0] -= 1
        self.pending = [p for p in self.pending if p[0] > 0]
        return len(self.pending)

    def busy(self, r):
        return any(id(r) in p[1] for p in self.pending)

    def destroy(self):
        pass


class FakeView:
    def __init__(self, base, engine, n):
        self.base, self.engine, self.name = base, engine, f"{base.volume}{n}"
        self.w = self.h = 0
        self.frames, self.params, self.destroyed = [], None, False

    def device_bytes(self):
        return 10 ** 6 + S.view_image_bytes(self.w, self.h, 2)

    def set_pass_budget(self, passes, frames):
        pass

    def reset_view(self):
        self.frames = []

    def resize(self, w, h):
        self.w, self.h = w, h

    def idle(self):
        return not self.engine.busy(self)

    def read_output(self):
        return ("image", self.base.volume, self.params)

    def read_accumulation(self):
        return ("accumulation", self.params)

    def destroy(self):
        self.destroyed = True


class FakeBase:
    def __init__(self, volume):
        self.volume, self.destroyed = volume, False

    def device_bytes(self):
        return 10 ** 9

    def destroy(self):
        self.destroyed = True


def make_batched(budget=10 ** 12, ticks=2, **kw):
    engine = FakeEngine(ticks)
    bases, views = [], []

    def make_base(volume):
        bases.append(FakeBase(volume))
        return bases[-1]

    def make_view(base):
        views.append(FakeView(base, engine, len(views)))
        return views[-1]

    srv = S.BatchedServer(make_base, make_view, engine, budget, lambda v: 10 ** 9, lambda v: 10 ** 6, 10 ** 8,
                          clock=iter(range(10 ** 6)).__next__, **kw)
    return srv, engine, bases, views


def test_batched_passes_cover_every_frame_once_and_display_last():
    srv, engine, bases, views = make_batched(frames_per_pass=16, max_batch=3)
    reqs = [S.Request("ab"[k % 2], 64 << (k % 3), 64, (16, 40, 100)[k % 3], params=k) for k in range(9)]
    run(srv, reqs)
    assert all(q.image == ("image", q.volume, q.params) for q in reqs)
    assert len(bases) == 2 and srv.created <= len(reqs)
    for p in engine.passes:
        assert 1 <= len(p) <= 3
    assert any(len({name[0] for name, *_ in p}) == 2 for p in engine.passes)  # volumes share passes
    for q in reqs:  # the request's passes, in order, on its view
        chunks = [(first, n, display) for p in engine.passes for name, params, first, n, display in p
                  if params == q.params]
        assert [c[0] for c in chunks] == [1 + sum(c[1] for c in chunks[:k]) for k in range(len(chunks))]
        assert sum(c[1] for c in chunks) == q.spp and all(c[1] <= 16 for c in chunks)
        assert [c[2] for c in chunks] == [False] * (len(chunks) - 1) + [True]


def test_batched_requests_share_passes_and_late_ones_join():
    srv, engine, bases, views = make_batched(frames_per_pass=8, in_flight=1, ticks=3)
    first = S.Request("a", 256, 256, 64, params="first")
    srv.submit(first)
    srv.step()
    second = S.Request("a", 64, 64, 16, params="second")
    srv.submit(second)
    for _ in range(4):
        srv.step()
    assert second.started is not None and first.finished is None
    joined = [p for p in engine.passes if {"first", "second"} <= {params for _, params, *_ in p}]
    assert joined  # a later pass carries both requests
    run(srv, [])
    assert second.finished < first.finished
    assert srv.created == 2 and len(bases) == 1  # one resident volume, a view per concurrent request


def test_batched_views_are_reused_and_memory_stays_in_budget():
    one = 10 ** 8 + 10 ** 9 + 10 ** 6 + S.view_image_bytes(256, 256, 2)
    srv, engine, bases, views = make_batched(budget=one + 10 ** 6 + S.view_image_bytes(256, 256, 2) + 10,
                                             max_batch=8)
    reqs = [S.Request("a", 256, 256, 16, params=k) for k in range(6)]
    run(srv, reqs)
    assert srv.peak_bytes <= srv.budget
    assert srv.created <= 2 and all(q.image is not None for q in reqs)


def test_batched_refuses_what_cannot_fit():
    srv, engine, bases, views = make_batched(budget=10 ** 9)
    srv.submit(S.Request("a", 64, 64, 16, params=0))
    with pytest.raises(MemoryError):
        srv.step()


def test_batched_passes_stay_within_their_path_budget():
    """A pass takes about pass_paths paths: the lead request at least one
    frame, the others only frames that fit what is left."""
    srv, engine, bases, views = make_batched(pass_paths=4 * 256 * 256, max_batch=8, frames_per_pass=64)
    reqs = [S.Request("a", 256, 256, 16, params="small"), S.Request("a", 1024, 1024, 8, params="big"),
            S.Request("b", 512, 512, 4, params="mid")]
    run(srv, reqs)
    sizes = {"small": 256 * 256, "big": 1024 * 1024, "mid": 512 * 512}
    for p in engine.passes:
        paths = [sizes[params] * n for _, params, _, n, _ in p]
        # Over the budget only when the lead alone takes its one frame.
        assert sum(paths) <= 4 * 256 * 256 or (len(p) == 1 and p[0][3] == 1)
    assert all(q.image is not None for q in reqs)


def test_view_memory_model_follows_the_library_sources():
    """A view allocates the two label masks (4 bytes per bricked voxel each)
    and no volume of its own; its image holds the passes' sums it keeps."""
    import os
    import re
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "volview_gb300", "csrc")
    host = open(os.path.join(csrc, "vv_host.cpp")).read()
    view = host[host.index("vv_renderer_create_view"):host.index("extern \"C\" vv_status vv_renderer_destroy")]
    assert re.search(r"mask_a\.alloc\(elems \* sizeof\(uint32_t\)\)", view)
    assert re.search(r"mask_b\.alloc\(elems \* sizeof\(uint32_t\)\)", view)
    for shared in ("density", "normals", "labels"):
        assert f"&r->{shared}, &root->{shared}" in view  # borrowed, not allocated
    assert S.view_volume_bytes((8, 8, 8)) == 8 * 512
    assert S.view_image_bytes(64, 32, passes=2) == 64 * 32 * (S.IMAGE_BYTES_PER_PIXEL - 48 * (S.PASSES - 2))
