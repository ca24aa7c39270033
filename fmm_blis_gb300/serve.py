"""Serving loop for GEMM requests on one GPU: continuous batching with
admission by HBM footprint, per-form queues, batched launches that overlap on
a pool of streams, and per-size-bucket CUDA graphs for small requests.

The reference has no serving layer (its only caller is one synchronous
bli_strassen_ab_ex call, test/test_strassen_oapi.c:166); this is the served
form of the same FMM GEMM built on the library's batched C-ABI call
(fmm_gpu_batch_dgemm) and the per-problem Tuner.

Loop (Server.tick):
  1. completions: a batch whose event has fired releases its requests'
     device memory (operands stay on the device until the request is done)
     and their footprint; cancelled requests are dropped here;
  2. admission, one queue per form, first come first served within a queue:
     a request is admitted while its footprint -- A, B, C and the FMM
     workspace of its plan -- fits the HBM budget; FP64-tagged requests may
     hold at most fp64_hbm_share of the budget, so a backlog of FP64 work
     (about 50 times slower per flop than the split form on this GPU) never
     takes the memory split requests need. Within a queue a request that
     does not fit blocks the ones behind it (no overtaking, so large requests
     are not starved);
  3. launch: the split requests admitted in this tick run as one batch on
     the next stream of the pool, so the batches of successive ticks overlap
     on the device; the FP64 requests run as one batch on their own stream
     with the persistent FP64 launch capped at fp64_ctas CTAs
     (fmm_gpu_set_f64_batch_ctas), which leaves the other SMs to the split
     form's kernels while a long FP64 batch runs.

Memory: the batched path's operands and workspaces are pieces of one device
arena allocated when the server starts (the budget plus slack), so the loop
never calls the CUDA allocator; a caching allocator under memory pressure
frees cached blocks, and cudaFree waits for every kernel on the device, long
FP64 batches included, which stalled the whole loop. FP64 requests take
their pieces from the top of the arena and split requests from the bottom,
so the long-lived FP64 pieces do not fragment the room split batches cycle
through.

Faults are handled on the host: a workspace allocation that fails (or finds
no contiguous piece of the arena) puts the batch's requests back at the
front of their queue (operands are regenerated
from the request's seed when it is launched again) and the loop goes on;
cancel(rid) withdraws a waiting request, or drops an admitted one's result
when its batch completes.

A request's result depends only on the request: its plan comes from the
deterministic Tuner and the batched call gives every problem exactly its
single-call result, so a request served in a mix returns the bits it returns
alone.

Small split requests whose plan is classical (levels 0) and whose dimensions
fit a size bucket (powers of two from 128 to graph_max_dim) run through CUDA
graphs captured once per bucket: the operands are written into a zero-padded
slot of the bucket's size and one graph launch replaces the prologue, pack,
GEMM and scatter launches. Zero padding leaves a levels-0 split result
unchanged (row and column maxima, digits and the exact integer slice products
of the real rows and columns are the same), so the graph path returns the
same bits as the batched path.
"""
from __future__ import annotations

import collections
import itertools
import time
from dataclasses import dataclass, field

from . import tune as _tune


@dataclass
class Request:
    m: int
    n: int
    k: int
    form: str = "split"               # "split" (target_rel_err) or "fp64" (drop-in)
    target_rel_err: float = 1e-10
    seed: int = 0
    arrival: float = 0.0              # perf_counter seconds
    rid: int = -1
    plan: object = None
    admitted: float | None = None
    done: float | None = None
    path: str = ""                    # "batch" or "graph"
    C: object = None                  # result (device tensor, column-major), kept after completion
    footprint: int = 0
    cancelled: bool = False
    _A: object = field(default=None, repr=False)
    _B: object = field(default=None, repr=False)
    _offs: object = field(default=None, repr=False)   # arena offsets of A, B, C on the batched path

    @property
    def latency(self) -> float | None:
        return None if self.done is None else self.done - self.arrival

    @property
    def flops(self) -> float:
        return 2.0 * self.m * self.n * self.k


def _colmajor_rand(torch, rows, cols, gen, dev):
    """uniform [-1, 1) column-major (rows x cols) tensor from a seeded
    generator (2u - 1 in place: no full-size temporaries)"""
    return torch.rand((cols, rows), generator=gen, device=dev, dtype=torch.float64).mul_(2).sub_(1).t()


def _colmajor_rand_into(torch, view, gen):
    """_colmajor_rand's values written into `view`, a column-major (rows x
    cols) view of preallocated device memory: the same generator draws, so
    the same bits"""
    torch.rand(tuple(view.t().shape), generator=gen, dtype=torch.float64, out=view.t())
    view.mul_(2).sub_(1)
    return view


class _Arena:
    """One device allocation, handed out in 256-byte aligned pieces (first fit
    over an ordered free list, neighbours merged on release). The server takes
    every request's operands and every batch's workspace from it, so serving
    never calls the CUDA allocator: a caching allocator under memory pressure
    frees cached blocks, and cudaFree waits for every kernel on the device,
    a long FP64 batch included."""

    def __init__(self, torch, dev, nbytes: int):
        self.torch = torch
        # a multiple of 256 bytes, so pieces taken from the top are as aligned as those from the bottom
        self.buf = torch.empty(max(nbytes, 256) // 256 * 256, dtype=torch.uint8, device=dev)
        self.free = [(0, self.buf.numel())]   # (offset, size), ordered by offset

    def alloc(self, nbytes: int, from_top: bool = False):
        """first fit from the bottom, or (from_top) from the top, of the arena"""
        need = (max(nbytes, 1) + 255) // 256 * 256
        order = range(len(self.free) - 1, -1, -1) if from_top else range(len(self.free))
        for x in order:
            off, size = self.free[x]
            if size < need:
                continue
            if size == need:
                del self.free[x]
                return off, need
            if from_top:
                self.free[x] = (off, size - need)
                return off + size - need, need
            self.free[x] = (off + need, size - need)
            return off, need
        return None

    def release(self, off: int, size: int):
        import bisect
        x = bisect.bisect_left(self.free, (off, 0))
        self.free.insert(x, (off, size))
        # merge with the following and the preceding piece
        if x + 1 < len(self.free) and off + size == self.free[x + 1][0]:
            self.free[x] = (off, size + self.free[x + 1][1])
            del self.free[x + 1]
        if x > 0 and self.free[x - 1][0] + self.free[x - 1][1] == off:
            self.free[x - 1] = (self.free[x - 1][0], self.free[x - 1][1] + self.free[x][1])
            del self.free[x]

    def bytes_view(self, off: int, nbytes: int):
        return self.buf[off:off + nbytes]

    def matrix(self, off: int, rows: int, cols: int):
        """a column-major rows x cols float64 view at offset off"""
        return self.buf[off:off + 8 * rows * cols].view(self.torch.float64).view(cols, rows).t()


def _bucket(x: int, lo: int = 128) -> int:
    b = lo
    while b < x:
        b *= 2
    return b


class _GraphSlot:
    """A zero-padded operand set of one bucket shape and the graph of one
    levels-0 split call over it."""

    def __init__(self, torch, fmm, dev, bm, bn, bk, slices, fmt, stream):
        self.bm, self.bn, self.bk = bm, bn, bk
        self.stream = stream
        self.A = torch.zeros((bk, bm), dtype=torch.float64, device=dev).t()
        self.B = torch.zeros((bn, bk), dtype=torch.float64, device=dev).t()
        self.C = torch.zeros((bn, bm), dtype=torch.float64, device=dev).t()
        self.ws = torch.empty(max(fmm.split_workspace_size(bm, bn, bk, None, 0, slices, fmt), 256),
                              dtype=torch.uint8, device=dev)
        self.busy_event = None
        with torch.cuda.stream(stream):
            # warm-up outside capture: tables, attributes, device error word
            fmm.split_dgemm(self.A, self.B, self.C, None, 0, slices, workspace=self.ws, stream=stream, fmt=fmt)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=stream):
            fmm.split_dgemm(self.A, self.B, self.C, None, 0, slices, workspace=self.ws,
                            stream=torch.cuda.current_stream(), fmt=fmt)
        torch.cuda.synchronize()


class Server:
    def __init__(self, hbm_budget: int | None = None, streams: int = 4, tuner: _tune.Tuner | None = None,
                 max_batch: int = 64, graph_max_dim: int = 1024, graph_slots: int = 2, use_graphs: bool = True,
                 keep_results: bool = True, device: int = 0, fp64_hbm_share: float = 0.25,
                 fp64_ctas: int | None = None, alloc_hook=None):
        import torch

        import fmm_blis_gb300 as fmm
        self.torch, self.fmm = torch, fmm
        self.dev = torch.device("cuda", device)
        if hbm_budget is None:
            free, _total = torch.cuda.mem_get_info(self.dev)
            hbm_budget = int(free * 0.8)
        self.budget = hbm_budget
        self.fp64_budget = int(hbm_budget * fp64_hbm_share)
        # operands and workspaces of the batched path live in one allocation of the budget (plus room
        # for the 256-byte rounding of each piece and a batch's own tables)
        self.arena = _Arena(torch, self.dev, hbm_budget + (64 << 20))
        self.used = 0
        self.used_fp64 = 0
        self.peak_used = 0
        self.tuner = tuner or _tune.Tuner()
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(streams)]
        self.fp64_stream = torch.cuda.Stream(device=self.dev)
        self.copy_stream = torch.cuda.Stream(device=self.dev)   # results kept out of the arena
        sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        # the FP64 batch kernel holds one SM per CTA against the split GEMM (their shared memory does not fit
        # together): an eighth of the SMs by default
        self.fp64_ctas = fp64_ctas if fp64_ctas is not None else max(1, sms // 8)
        self._next_stream = itertools.cycle(range(streams))
        self.max_batch = max_batch
        self.keep_results = keep_results
        self.graph_max_dim = graph_max_dim if use_graphs else 0
        self.graph_slots = graph_slots
        self.queues: dict[str, collections.deque[Request]] = {"split": collections.deque(),
                                                              "fp64": collections.deque()}
        self.inflight: list[tuple[object, list[Request], list]] = []   # (event, requests, arena pieces)
        self.completed: list[Request] = []
        self.cancelled: list[Request] = []
        self.alloc_hook = alloc_hook          # called before each workspace allocation; may raise (fault injection)
        self.alloc_failures = 0
        self._algs: dict = {}
        self._slots: dict = {}
        self._rid = itertools.count()
        self.launched_batches = 0

    @property
    def pending(self):
        """all waiting requests, split queue first"""
        return list(self.queues["split"]) + list(self.queues["fp64"])

    # ------------------------------------------------------------ helpers
    def _alg(self, name: str):
        if name == "classical":
            return None
        if name not in self._algs:
            self._algs[name] = self.fmm.new_fmm(_tune.COEFF_DIR / f"{name}.txt")
        return self._algs[name]

    def _workspace_bytes(self, r: Request) -> int:
        """FMM temporaries of the request's plan when it runs inside a batch:
        all products' digit slices and level accumulators at once (split), or
        its share of the FP64 problem table."""
        p = r.plan
        if p.form == "fp64":
            return 4096
        return self.fmm.batch_problem_workspace_size(r.m, r.n, r.k, self._alg(p.alg), p.levels, p.slices, p.fmt)

    def _graph_bucket(self, r: Request):
        p = r.plan
        if p.form != "split" or p.levels != 0 or max(r.m, r.n, r.k) > self.graph_max_dim:
            return None
        bucket = (_bucket(r.m), _bucket(r.n), _bucket(r.k), p.slices, p.fmt)
        if bucket not in self._slots and self._fp64_in_flight():
            # capturing a new bucket's graph synchronizes the whole device (torch.cuda.graph does, before
            # capture), which would hold the loop until the FP64 batch in flight ends, tens of seconds for a
            # large one: the request takes the batched path instead, which gives the same bits
            return None
        return bucket

    def _fp64_in_flight(self) -> bool:
        """an FP64 batch is still running (batches hold requests of one form)"""
        return any(reqs and reqs[0].plan.form == "fp64" for _ev, reqs, _pieces in self.inflight)

    # -------------------------------------------------------------- API
    def submit(self, r: Request) -> Request:
        r.rid = next(self._rid)
        if not r.arrival:
            r.arrival = time.perf_counter()
        r.plan = self.tuner.plan(r.m, r.n, r.k, r.form, r.target_rel_err)
        r.footprint = 8 * (r.m * r.k + r.k * r.n + r.m * r.n) + self._workspace_bytes(r)
        cap = self.fp64_budget if r.plan.form == "fp64" else self.budget
        if r.footprint > cap:
            raise ValueError(f"request {r.rid} needs {r.footprint} bytes, more than its HBM budget {cap}")
        self.queues[r.plan.form].append(r)
        return r

    def cancel(self, rid: int) -> bool:
        """Withdraws request rid: a waiting one leaves its queue at once, an
        admitted one is dropped (memory released, result discarded) when its
        batch completes. False if it is unknown or already done."""
        for q in self.queues.values():
            for r in q:
                if r.rid == rid:
                    q.remove(r)
                    r.cancelled = True
                    self.cancelled.append(r)
                    return True
        for _ev, reqs, _ws in self.inflight:
            for r in reqs:
                if r.rid == rid and not r.cancelled:
                    r.cancelled = True
                    return True
        return False

    def idle(self) -> bool:
        return not any(self.queues.values()) and not self.inflight

    def _admit(self, form: str) -> list[Request]:
        q, batch = self.queues[form], []
        while q and len(batch) < self.max_batch:
            r = q[0]
            if self.used + r.footprint > self.budget:
                break
            if form == "fp64" and self.used_fp64 + r.footprint > self.fp64_budget:
                break
            q.popleft()
            self.used += r.footprint
            if form == "fp64":
                self.used_fp64 += r.footprint
            self.peak_used = max(self.peak_used, self.used)
            r.admitted = time.perf_counter()
            batch.append(r)
        return batch

    def _release(self, r: Request):
        self.used -= r.footprint
        if r.plan.form == "fp64":
            self.used_fp64 -= r.footprint
        r._A = r._B = None

    def _piece(self, nbytes: int, pieces: list, from_top: bool = False):
        got = self.arena.alloc(nbytes, from_top)
        if got is None:
            for off, size in pieces:
                self.arena.release(off, size)
            pieces.clear()
            raise MemoryError(f"no contiguous {nbytes} bytes free in the serving arena")
        pieces.append(got)
        return got[0]

    def tick(self) -> int:
        """One scheduling round; returns the number of requests launched."""
        # 1. completions
        still = []
        now = time.perf_counter()
        for ev, reqs, pieces in self.inflight:
            if ev.query():
                kept = False
                for r in reqs:
                    self._release(r)
                    if r.cancelled:
                        r.C = None
                        self.cancelled.append(r)
                        continue
                    r.done = now
                    if not self.keep_results:
                        r.C = None
                    elif r.path == "batch":
                        with self.torch.cuda.stream(self.copy_stream):
                            r.C = r.C.clone()   # out of the arena, whose piece is reused next
                        kept = True
                    self.completed.append(r)
                if kept:
                    self.copy_stream.synchronize()
                for off, size in pieces:
                    self.arena.release(off, size)
            else:
                still.append((ev, reqs, pieces))
        self.inflight = still
        # 2. admission per form, 3. launch
        launched = 0
        for form in ("split", "fp64"):
            batch = self._admit(form)
            if not batch:
                continue
            st = self.fp64_stream if form == "fp64" else self.streams[next(self._next_stream)]
            try:
                ev, pieces = self._launch(batch, st, form)
            except (MemoryError, RuntimeError) as e:
                if not isinstance(e, MemoryError) and "out of memory" not in str(e).lower():
                    raise
                # nothing of the batch ran: back to the front of the queue, in order
                for r in reversed(batch):
                    self._release(r)
                    r.C = None
                    r.admitted = None
                    self.queues[form].appendleft(r)
                self.alloc_failures += 1
                continue
            self.inflight.append((ev, batch, pieces))
            self.launched_batches += 1
            launched += len(batch)
        return launched

    def _launch(self, batch, st, form):
        """operands and workspace from the arena (the allocations that may
        fail, before anything is launched: the pieces taken are returned),
        graph requests, then one batched call for the rest"""
        torch = self.torch
        pieces: list = []
        direct, graphs = [], []
        for r in batch:
            bucket = self._graph_bucket(r)
            if bucket is not None:
                graphs.append((r, bucket))
                continue
            # FP64 requests run long: their pieces come from the top of the arena, so the holes split batches
            # leave at the bottom merge back into large pieces
            top = form == "fp64"
            r._offs = (self._piece(8 * r.m * r.k, pieces, top), self._piece(8 * r.k * r.n, pieces, top),
                       self._piece(8 * r.m * r.n, pieces, top))
            direct.append(r)
        ws_off, arr, wsb = None, None, 0
        if direct:
            # the batch's workspace size from its shapes and plans alone (host-only sizing)
            wsb = max(self.fmm.batch_shapes_workspace_size(
                [(r.m, r.n, r.k, self._alg(r.plan.alg), r.plan.levels, r.plan.slices, r.plan.fmt) for r in direct]), 256)
            if self.alloc_hook is not None:
                try:
                    self.alloc_hook(wsb)
                except BaseException:
                    for off, size in pieces:
                        self.arena.release(off, size)
                    raise
            ws_off = self._piece(wsb, pieces, form == "fp64")
        with torch.cuda.stream(st):
            for r in direct:
                g = torch.Generator(device=self.dev).manual_seed(r.seed)
                oa, ob, oc = r._offs
                r._A = _colmajor_rand_into(torch, self.arena.matrix(oa, r.m, r.k), g)
                r._B = _colmajor_rand_into(torch, self.arena.matrix(ob, r.k, r.n), g)
                r.C = _colmajor_rand_into(torch, self.arena.matrix(oc, r.m, r.n), g)
                r.path = "batch"
            ws = None
            if direct:
                probs = [{"A": r._A, "B": r._B, "C": r.C, "fmm": self._alg(r.plan.alg), "levels": r.plan.levels,
                          "slices": r.plan.slices, "fmt": r.plan.fmt} for r in direct]
                arr = self.fmm.make_batch(probs)
                ws = self.arena.bytes_view(ws_off, wsb)
            for r, bucket in graphs:
                self._run_graph(r, bucket, torch.Generator(device=self.dev).manual_seed(r.seed), st)
            if direct:
                if form == "fp64":
                    prev = self.fmm.set_f64_batch_ctas(self.fp64_ctas)
                    try:
                        self.fmm.batch_dgemm(arr, workspace=ws, stream=st)
                    finally:
                        self.fmm.set_f64_batch_ctas(prev)
                else:
                    self.fmm.batch_dgemm(arr, workspace=ws, stream=st)
            ev = torch.cuda.Event()
            ev.record(st)
        return ev, pieces

    def _run_graph(self, r: Request, bucket, gen, st):
        """operands into a zero-padded slot of the bucket, one graph launch,
        the result copied out (all on stream st)"""
        torch = self.torch
        slots = self._slots.get(bucket)
        if slots is None:
            bm, bn, bk, s, fmt = bucket
            slots = [_GraphSlot(torch, self.fmm, self.dev, bm, bn, bk, s, fmt, torch.cuda.Stream(device=self.dev))
                     for _ in range(self.graph_slots)]
            self._slots[bucket] = slots
        slot = None
        while slot is None:
            for sl in slots:
                if sl.busy_event is None or sl.busy_event.query():
                    slot = sl
                    break
            if slot is None:
                slots[0].busy_event.synchronize()
        slot.stream.wait_stream(st)
        with torch.cuda.stream(slot.stream):
            slot.A.zero_()
            slot.B.zero_()
            slot.C.zero_()
            slot.A[:r.m, :r.k].copy_(_colmajor_rand(torch, r.m, r.k, gen, self.dev))
            slot.B[:r.k, :r.n].copy_(_colmajor_rand(torch, r.k, r.n, gen, self.dev))
            C = _colmajor_rand(torch, r.m, r.n, gen, self.dev)
            slot.C[:r.m, :r.n].copy_(C)
            slot.graph.replay()
            C.copy_(slot.C[:r.m, :r.n])
            ev = torch.cuda.Event()
            ev.record(slot.stream)
        slot.busy_event = ev
        st.wait_stream(slot.stream)
        r.C = C
        r.path = "graph"

    def run(self, arrivals, until_idle: bool = True, poll_s: float = 50e-6, max_s: float | None = None):
        """Serves `arrivals` (Requests with arrival offsets in seconds from
        now, sorted): each is submitted when its time comes. Returns the
        completed requests."""
        t0 = time.perf_counter()
        queue = collections.deque(sorted(arrivals, key=lambda r: r.arrival))
        while queue or (until_idle and not self.idle()):
            now = time.perf_counter()
            if max_s is not None and now - t0 > max_s:
                break
            while queue and t0 + queue[0].arrival <= now:
                r = queue.popleft()
                r.arrival = t0 + r.arrival
                self.submit(r)
            launched = self.tick()
            if not launched and (not queue or t0 + queue[0].arrival > time.perf_counter()):
                time.sleep(poll_s)
        return self.completed

    def close(self):
        self.torch.cuda.synchronize()
        self.arena = None
        for f in self._algs.values():
            self.fmm.free_fmm(f)
        self._algs.clear()


def poisson_arrivals(rate: float, duration: float, seed: int, dims=(128, 16384), split_fraction: float = 0.5,
                     target_rel_err: float = 1e-10, cap_bytes: int | None = None):
    """Seeded request stream: exponential inter-arrival times at `rate` per
    second over `duration` seconds; m, n, k log-uniform in dims; each request
    tagged split (target relative error) or FP64 drop-in. With cap_bytes, the
    dimensions are scaled down until A, B and C fit in it."""
    import numpy as np

    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    lo, hi = np.log(dims[0]), np.log(dims[1])
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        m, n, k = (int(round(float(np.exp(rng.uniform(lo, hi))))) for _ in range(3))
        if cap_bytes is not None:
            while 8 * (m * k + k * n + m * n) > cap_bytes:
                m, n, k = max(m // 2, 1), max(n // 2, 1), max(k // 2, 1)
        form = "split" if rng.uniform() < split_fraction else "fp64"
        out.append(Request(m, n, k, form=form, target_rel_err=target_rel_err,
                           seed=int(rng.integers(0, 2**31 - 1)), arrival=t))
    return out
