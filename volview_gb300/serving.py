"""A render-request loop over resident volumes (the serving workload).

Requests (a volume, an image size, paths per pixel, a camera, a clip plane and
label visibility) arrive at any time. A request is admitted when the renderers
it needs fit the device-memory budget, and it runs on a renderer of its volume
whose context stream is its own. Its frames are one `vv_record_frames` call:
passes of up to 64 frames queued at once, with a display after the last. So
the passes of every admitted request overlap on the device, and requests that
arrive while others run are admitted as memory and renderers free up, with no
barrier between them.

A renderer is reused for later requests of its volume. `vv_reset_view` restarts
its accumulation and auto exposure first, and `vv_resize` sets the request's
image, so a result depends only on its own request, alone or in any mix
(tests/test_gpu_serving.py). Idle renderers of other volumes are destroyed,
least recently used first, when a request needs their memory.

The loop itself is host logic over the C ABI: `vv_query` polls for finished
work without blocking, and `vv_renderer_memory` reports what each renderer
holds. Renderers come from a factory, so the scheduling is tested on the CPU
with stand-ins (tests/test_serving.py).

`BatchedServer` serves the same requests from one resident copy of each
volume: a request runs on a view of the volume's base renderer
(`vv_renderer_create_view`), and batched passes (`vv_batch_record`) trace the
frames of up to 8 requests, of any volumes, in the same waves, a pass at a
time, so requests that arrive while others run join the next pass.
"""
import collections
import time

# Device bytes per image pixel: the accumulation and guide images, the
# denoiser's ping/pong and guides, HDR, output and bloom, and the six passes'
# own sums (vv_resize).
IMAGE_BYTES_PER_PIXEL = 48 + 32 + 32 + 8 + 4 + 2 + 6 * 48
# Device bytes per path slot of a pass: the slot's records, the light map
# sample's direction, the ten stage queues and the later-flight bins' keys
# and sorted queue (vv_wavefront.cu).
SLOT_BYTES = 288 + 16 + 10 * 4 + 3 * 4
PASSES = 6          # passes in flight per renderer
PASS_FRAMES = 64    # frames per pass of a long vv_record_frames call
SLOT_FRAMES = 16    # frames' worth of slots a pass holds at most ...
SLOT_CAP = 1 << 24  # ... and at most this many slots, unless one frame needs more


def request_bytes(width, height, spp, passes=PASSES, slot_frames=SLOT_FRAMES):
    """Device bytes a renderer's image and path state take for one request,
    with `passes` passes in flight of up to `slot_frames` frames' worth of
    slots each (vv_set_pass_budget)."""
    px = width * height
    frames = min(spp, PASS_FRAMES)
    slots = min(min(frames, slot_frames) * px, max(SLOT_CAP, px))
    used = min(passes, -(-spp // PASS_FRAMES))
    sums = 48 * px * (PASSES - passes)  # IMAGE_BYTES_PER_PIXEL counts every pass's sums
    return px * IMAGE_BYTES_PER_PIXEL - sums + used * slots * SLOT_BYTES


class Request:
    """One render request. `params` is the vv_frame_params the request renders
    with (camera, clip plane, label visibility); `spp` its paths per pixel."""

    def __init__(self, volume, width, height, spp, params, arrival=0.0, tag=None):
        self.volume, self.width, self.height, self.spp = volume, int(width), int(height), int(spp)
        self.params, self.arrival, self.tag = params, float(arrival), tag
        self.id = None
        self.submitted = self.started = self.finished = None
        self.renderer = None
        self.image = None
        self.accumulation = None

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.submitted

    @property
    def paths(self):
        return self.width * self.height * self.spp


class Server:
    """Admits and runs requests; see the module docstring.

    `make_renderer(volume)` returns a renderer (the `renderer.Renderer`
    interface: reset_view, resize, record_frames, idle, read_output,
    read_accumulation, device_bytes, destroy) of a resident volume, its labels
    set. `base_bytes(volume)` is the device memory of such a renderer before
    any image (its volumes). `max_active` bounds the requests in flight (None:
    memory alone decides); `max_per_volume` the requests in flight per volume,
    i.e. its renderers (None: a new renderer when the others are busy).

    `order` is the admission order of queued requests: "fifo" (arrival), or
    "shortest" (fewest paths first, so short requests run beside long ones
    instead of behind them; a request queued longer than `aging_s` goes ahead
    of all younger ones, in arrival order, so long ones are not starved)."""

    def __init__(self, make_renderer, base_bytes, budget_bytes, max_active=None, keep_accumulation=False,
                 clock=time.perf_counter, order="fifo", aging_s=2.0, max_per_volume=None, passes=PASSES,
                 slot_frames=SLOT_FRAMES):
        if order not in ("fifo", "shortest"):
            raise ValueError(f"unknown admission order {order!r}")
        self.make_renderer, self.base_bytes = make_renderer, base_bytes
        self.budget, self.max_active, self.keep_accumulation = int(budget_bytes), max_active, keep_accumulation
        self.clock, self.order, self.aging_s, self.max_per_volume = clock, order, aging_s, max_per_volume
        # Each renderer's pass state (vv_set_pass_budget): fewer passes and
        # frames in flight per renderer, when several renderers serve at once.
        self.passes, self.slot_frames = passes, slot_frames
        self.queue = collections.deque()
        self.active = []
        self.idle = collections.OrderedDict()  # renderer -> volume, least recently used first
        self.owned = {}                        # renderer -> its volume
        self.next_id = 0
        self.done = []
        self.refused = []  # requests that can never fit the budget
        self.peak_bytes = 0
        self.created = 0

    # ------------------------------------------------------------- accounting
    def used_bytes(self):
        return sum(r.device_bytes() for r in self.owned)

    def _need(self, req, renderer):
        """Bytes admitting `req` adds: a new renderer's volumes and image, or
        the growth of a reused one."""
        want = request_bytes(req.width, req.height, req.spp, self.passes, self.slot_frames)
        if renderer is None:
            return self.base_bytes(req.volume) + want
        return max(0, self.base_bytes(req.volume) + want - renderer.device_bytes())

    # --------------------------------------------------------------- the loop
    def submit(self, req):
        req.id = self.next_id
        self.next_id += 1
        req.submitted = self.clock()
        self.queue.append(req)
        return req.id

    def _idle_renderer(self, volume):
        for r, v in self.idle.items():
            if v == volume:
                return r
        return None

    def _evict(self, need, keep):
        """Destroys idle renderers (least recently used first, never `keep`)
        until `need` more bytes fit; False if they cannot."""
        used = self.used_bytes()
        for r in list(self.idle):
            if used + need <= self.budget:
                break
            if r is keep:
                continue
            used -= r.device_bytes()
            del self.idle[r]
            del self.owned[r]
            r.destroy()
        return used + need <= self.budget

    def _candidates(self):
        if self.order == "fifo":
            return list(self.queue)
        now = self.clock()
        aged = [q for q in self.queue if now - q.submitted > self.aging_s]
        young = sorted((q for q in self.queue if now - q.submitted <= self.aging_s), key=lambda q: (q.paths, q.id))
        return aged + young

    def _admit(self):
        """First fit in admission order: each queued request that fits starts."""
        for req in self._candidates():
            if self.max_active is not None and len(self.active) >= self.max_active:
                return
            r = self._idle_renderer(req.volume)
            if r is None and self.max_per_volume is not None and \
                    sum(q.volume == req.volume for q in self.active) >= self.max_per_volume:
                continue
            need = self._need(req, r)
            if not self._evict(need, r):
                # Nothing runs and every other idle renderer is gone: no later
                # step frees memory (a new renderer in place of `r` would need
                # the same bytes), so the request can never start.
                if not self.active and all(x is r for x in self.idle):
                    # Refused: it leaves the queue, so the next step serves
                    # the requests behind it.
                    self.queue.remove(req)
                    self.refused.append(req)
                    raise MemoryError(f"request {req.id} needs {need} bytes, budget {self.budget}")
                continue
            self.queue.remove(req)
            if r is None:
                r = self.make_renderer(req.volume)
                if (self.passes, self.slot_frames) != (PASSES, SLOT_FRAMES):
                    r.set_pass_budget(self.passes, self.slot_frames)
                self.owned[r] = req.volume
                self.created += 1
            else:
                del self.idle[r]
            req.renderer = r
            req.started = self.clock()
            r.reset_view()
            r.resize(req.width, req.height)
            r.record_frames(1, req.spp, req.params)
            self.active.append(req)
            self.peak_bytes = max(self.peak_bytes, self.used_bytes())

    def _collect(self):
        finished = []
        for req in list(self.active):
            r = req.renderer
            if not r.idle():
                continue
            req.image = r.read_output()
            if self.keep_accumulation:
                req.accumulation = r.read_accumulation()
            req.finished = self.clock()
            self.active.remove(req)
            self.idle[r] = req.volume
            self.idle.move_to_end(r)
            req.renderer = None
            finished.append(req)
        self.done += finished
        return finished

    def step(self):
        """Collects finished requests and admits queued ones; returns the finished."""
        finished = self._collect()
        self._admit()
        return finished

    def run(self, requests, poll_s=0.0005):
        """Submits each request at its arrival time (seconds after the start)
        and runs until all have finished; returns them in submission order."""
        pending = sorted(requests, key=lambda q: q.arrival)
        t0 = self.clock()
        i = 0
        while i < len(pending) or self.queue or self.active:
            now = self.clock() - t0
            while i < len(pending) and pending[i].arrival <= now:
                self.submit(pending[i])
                i += 1
            finished = self.step()
            if not finished and poll_s > 0:
                time.sleep(poll_s)
        return sorted(pending, key=lambda q: q.id)

    def preload(self, volume):
        """Makes a renderer of `volume` resident (idle) before requests come."""
        r = self.make_renderer(volume)
        if (self.passes, self.slot_frames) != (PASSES, SLOT_FRAMES):
            r.set_pass_budget(self.passes, self.slot_frames)
        self.owned[r] = volume
        self.idle[r] = volume
        self.created += 1
        return r

    def close(self):
        for r in list(self.owned):
            r.destroy()
        self.owned.clear()
        self.idle.clear()


def view_image_bytes(width, height, passes=PASSES):
    """Device bytes of a view's image for one request in batched passes: its
    images and `passes` passes' sums, no path slots (the batch engine holds
    those)."""
    return width * height * (IMAGE_BYTES_PER_PIXEL - 48 * (PASSES - passes))


def view_volume_bytes(dims):
    """Device bytes of a view before any image: its two label masks (8 bytes
    per bricked voxel; the base's density, normals and labels are shared)."""
    bricked = 1
    for d in dims:
        bricked *= -(-int(d) // 8) * 8
    return 8 * bricked


class BatchedServer:
    """Requests served by batched passes (vv_batch_record) over shared volumes.

    Each resident volume has one base renderer (its density, normals, labels
    and transfer function on the device once); a request runs on a view of it
    (vv_renderer_create_view: its own masks, images and sums, no copy of the
    volume), reused by later requests of that volume. Requests advance in
    passes of up to `frames_per_pass` frames: every step, while fewer than
    `in_flight` batched passes are queued, one pass takes the next frames of
    up to `max_batch` admitted requests, of any volumes, so requests of any
    volume, size and paths per pixel share waves and a request that arrives
    while others run joins the next pass. A request's last pass displays it.

    Factories: `make_base(volume)` a base renderer with its labels set,
    `make_view(base)` a view of it, `engine` the batch engine (`record`,
    `in_flight`, `device_bytes`). `base_bytes(volume)` and `view_bytes(volume)`
    are the memory of a base and of a view before any image; the engine's
    path state is reserved up front (`engine_bytes`)."""

    def __init__(self, make_base, make_view, engine, budget_bytes, base_bytes, view_bytes, engine_bytes,
                 max_active=None, keep_accumulation=False, clock=time.perf_counter, order="fifo", aging_s=2.0,
                 frames_per_pass=64, max_batch=8, in_flight=4, view_passes=None, pass_paths=1 << 25):
        if order not in ("fifo", "shortest"):
            raise ValueError(f"unknown admission order {order!r}")
        self.make_base, self.make_view, self.engine = make_base, make_view, engine
        self.budget, self.base_bytes, self.view_bytes = int(budget_bytes), base_bytes, view_bytes
        self.engine_bytes = int(engine_bytes)
        self.max_active, self.keep_accumulation, self.clock = max_active, keep_accumulation, clock
        self.order, self.aging_s = order, aging_s
        self.frames_per_pass, self.max_batch, self.in_flight = frames_per_pass, max_batch, in_flight
        self.pass_paths = pass_paths
        # A view's pass sums: one per batched pass it may be in at once, so
        # that no pass waits for an earlier one to free its request's sums.
        self.view_passes = view_passes if view_passes is not None else min(PASSES, max(1, in_flight))
        self.bases = {}                        # volume -> base renderer
        self.views = {}                        # view -> volume
        self.idle = collections.OrderedDict()  # idle view -> volume, least recently used first
        self.queue = collections.deque()
        self.active = []
        self.done, self.refused = [], []
        self.next_id = 0
        self.peak_bytes = 0
        self.created = 0                       # views made
        self.passes = 0                        # batched passes queued
        self.batch_sizes = []

    # ------------------------------------------------------------- accounting
    def used_bytes(self):
        return (self.engine_bytes + sum(b.device_bytes() for b in self.bases.values()) +
                sum(v.device_bytes() for v in self.views))

    def _need(self, req, view):
        want = view_image_bytes(req.width, req.height, self.view_passes)
        fresh = self.view_bytes(req.volume) + want
        if view is not None:
            return max(0, fresh - view.device_bytes())
        return fresh + (0 if req.volume in self.bases else self.base_bytes(req.volume))

    def _evict(self, need, keep):
        """Destroys idle views (least recently used first, never `keep`), then
        bases without views, until `need` more bytes fit."""
        used = self.used_bytes()
        for v in list(self.idle):
            if used + need <= self.budget:
                break
            if v is keep:
                continue
            used -= v.device_bytes()
            del self.idle[v]
            del self.views[v]
            v.destroy()
        for name in list(self.bases):
            if used + need <= self.budget:
                break
            if any(vol == name for vol in self.views.values()):
                continue
            if any(q.volume == name for q in self.queue):
                continue
            used -= self.bases[name].device_bytes()
            self.bases.pop(name).destroy()
        return used + need <= self.budget

    # --------------------------------------------------------------- the loop
    def submit(self, req):
        req.id = self.next_id
        self.next_id += 1
        req.submitted = self.clock()
        req.queued_frames = 0
        self.queue.append(req)
        return req.id

    def preload(self, volume):
        """Makes `volume` resident (its base renderer) before requests come."""
        if volume not in self.bases:
            self.bases[volume] = self.make_base(volume)
        return self.bases[volume]

    def _candidates(self):
        if self.order == "fifo":
            return list(self.queue)
        now = self.clock()
        aged = [q for q in self.queue if now - q.submitted > self.aging_s]
        young = sorted((q for q in self.queue if now - q.submitted <= self.aging_s), key=lambda q: (q.paths, q.id))
        return aged + young

    def _idle_view(self, volume):
        for v, name in self.idle.items():
            if name == volume:
                return v
        return None

    def _admit(self):
        for req in self._candidates():
            if self.max_active is not None and len(self.active) >= self.max_active:
                return
            view = self._idle_view(req.volume)
            need = self._need(req, view)
            if not self._evict(need, view):
                if not self.active and all(v is view for v in self.idle):
                    self.queue.remove(req)
                    self.refused.append(req)
                    raise MemoryError(f"request {req.id} needs {need} bytes, budget {self.budget}")
                continue
            self.queue.remove(req)
            if view is None:
                view = self.make_view(self.preload(req.volume))
                if self.view_passes != PASSES:
                    view.set_pass_budget(self.view_passes, SLOT_FRAMES)
                self.views[view] = req.volume
                self.created += 1
            else:
                del self.idle[view]
            req.renderer = view
            req.started = self.clock()
            req.queued_frames = 0
            view.reset_view()
            view.resize(req.width, req.height)
            self.active.append(req)
            self.peak_bytes = max(self.peak_bytes, self.used_bytes())

    @staticmethod
    def _remaining(q):
        return (q.spp - q.queued_frames) * q.width * q.height

    def _lead(self, waiting):
        """The request the next pass is for: the oldest (fifo), or the one
        with the fewest paths left, requests queued longer than `aging_s`
        first in arrival order (shortest)."""
        if self.order == "fifo":
            return min(waiting, key=lambda q: q.id)
        now = self.clock()
        aged = [q for q in waiting if now - q.submitted > self.aging_s]
        if aged:
            return min(aged, key=lambda q: q.id)
        return min(waiting, key=lambda q: (self._remaining(q), q.id))

    def _dispatch(self):
        """Queues batched passes while fewer than `in_flight` are running:
        each takes the next frames of the lead request (`_lead`) and of up to
        `max_batch` - 1 more requests, of any volume, those with the fewest
        paths left first, up to about `pass_paths` paths in all (at least one
        frame of the lead). A pass ends when its longest request's frames do,
        so short passes let short requests finish in their first one while
        long ones advance over many."""
        while self.engine.in_flight() < self.in_flight:
            waiting = [q for q in self.active if q.queued_frames < q.spp]
            if not waiting:
                return
            lead = self._lead(waiting)
            rest = sorted((q for q in waiting if q is not lead), key=lambda q: (self._remaining(q), q.id))
            items, left = [], self.pass_paths
            for q in [lead] + rest:
                if len(items) == self.max_batch:
                    break
                px = q.width * q.height
                n = min(self.frames_per_pass, q.spp - q.queued_frames, left // px)
                if n < 1:
                    if items:
                        continue
                    n = 1
                items.append((q.renderer, q.params, 1 + q.queued_frames, n, q.queued_frames + n == q.spp))
                q.queued_frames += n
                left -= n * px
            self.engine.record(items)
            self.passes += 1
            self.batch_sizes.append(len(items))

    def _collect(self):
        finished = []
        for req in list(self.active):
            if req.queued_frames < req.spp or not req.renderer.idle():
                continue
            v = req.renderer
            req.image = v.read_output()
            if self.keep_accumulation:
                req.accumulation = v.read_accumulation()
            req.finished = self.clock()
            self.active.remove(req)
            self.idle[v] = req.volume
            self.idle.move_to_end(v)
            req.renderer = None
            finished.append(req)
        self.done += finished
        return finished

    def step(self):
        """Collects finished requests, admits queued ones and queues passes."""
        finished = self._collect()
        self._admit()
        self._dispatch()
        return finished

    run = Server.run

    def close(self):
        for v in list(self.views):
            v.destroy()
        self.views.clear()
        self.idle.clear()
        for b in list(self.bases.values()):
            b.destroy()
        self.bases.clear()
        self.engine.destroy()


def batched_factory(volumes, device=0, passes=4, slot_frames=16):
    """(make_base, make_view, engine, base_bytes, view_bytes, engine_bytes) for
    resident `volumes` ({name: scene config}) served by batched passes: bases
    and views each on a context (CUDA stream) of its own, and one engine."""
    from . import abi
    from . import renderer as R

    class Owned(R.Renderer):
        def destroy(self):
            super().destroy()
            self.ctx.destroy()

    def make_base(name):
        cfg = volumes[name]
        r = Owned(R.Context(device), cfg["volume"], cfg["tf"])
        soft = cfg.get("soft")
        r.set_labels(cfg["labels_vol"], abi.soft_struct(soft) if soft is not None else None)
        return r

    def make_view(base):
        return Owned(R.Context(device), None, None, view_of=base)

    class OwnedEngine(R.BatchEngine):
        def destroy(self):
            super().destroy()
            self.ctx.destroy()

    engine = OwnedEngine(R.Context(device), passes, slot_frames)

    def base(name):
        return volume_bytes(volumes[name]["volume"].dims)

    def view(name):
        return view_volume_bytes(volumes[name]["volume"].dims)

    return make_base, make_view, engine, base, view, passes * SLOT_CAP * SLOT_BYTES


def volume_bytes(dims):
    """Device bytes of a renderer's volumes before any image: bricked density,
    normals, labels and the two masks (15 bytes per bricked voxel)."""
    bricked = 1
    for d in dims:
        bricked *= -(-int(d) // 8) * 8
    return 15 * bricked


def renderer_factory(volumes, device=0, precision=None):
    """(make_renderer, base_bytes) for resident `volumes` ({name: scene
    config}): each renderer on a context (CUDA stream) of its own, owning it."""
    from . import abi
    from . import renderer as R

    class OwnedRenderer(R.Renderer):
        def destroy(self):
            super().destroy()
            self.ctx.destroy()

    measured = {}

    def make(name):
        cfg = volumes[name]
        r = OwnedRenderer(R.Context(device), cfg["volume"], cfg["tf"], precision)
        soft = cfg.get("soft")
        r.set_labels(cfg["labels_vol"], abi.soft_struct(soft) if soft is not None else None)
        measured.setdefault(name, r.device_bytes())
        return r

    def base(name):
        return measured.get(name) or volume_bytes(volumes[name]["volume"].dims)

    return make, base


def summary(requests, wall_s):
    """Throughput and latency of a finished run."""
    import numpy as np
    lat = np.array([q.latency for q in requests])
    wait = np.array([q.started - q.submitted for q in requests])
    paths = sum(q.paths for q in requests)
    by_size = {}
    for q in requests:
        by_size.setdefault(f"{q.width}x{q.height}", []).append(q.latency)
    return {"requests": len(requests), "wall_s": wall_s, "requests_per_s": len(requests) / wall_s,
            "path_samples_per_s": paths / wall_s,
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "queue_wait_p50_s": float(np.percentile(wait, 50)), "queue_wait_p99_s": float(np.percentile(wait, 99)),
            "latency_p50_s_by_image": {k: float(np.percentile(v, 50)) for k, v in sorted(by_size.items())}}
