"""Host-side bookkeeping of the server (no GPU): the device arena that holds
the batched path's operands and workspaces, so serving never calls the CUDA
allocator (whose cudaFree, under memory pressure, waits for every kernel on
the device)."""
import random

from fmm_blis_gb300 import serve


class _Buf:
    def __init__(self, n):
        self.n = n

    def numel(self):
        return self.n


class _FakeTorch:
    uint8 = "uint8"
    float64 = "float64"

    def empty(self, n, dtype, device):
        return _Buf(n)


def test_arena_first_fit_and_merge():
    a = serve._Arena(_FakeTorch(), None, 1 << 20)
    x = a.alloc(1000)
    y = a.alloc(3000)
    z = a.alloc(1)
    assert x == (0, 1024) and y == (1024, 3072) and z == (4096, 256)   # 256-byte pieces, first fit
    a.release(*y)
    assert a.alloc(2000) == (1024, 2048)          # the freed hole is reused
    a.release(1024, 2048)
    a.release(*x)
    a.release(*z)
    assert a.free == [(0, 1 << 20)]               # neighbours merged back into one piece
    assert a.alloc((1 << 20) + 1) is None         # larger than the arena


def test_arena_random_alloc_release_keeps_pieces_disjoint():
    rng = random.Random(5)
    size = 1 << 22
    a = serve._Arena(_FakeTorch(), None, size)
    held = []
    for _ in range(2000):
        if held and rng.random() < 0.45:
            a.release(*held.pop(rng.randrange(len(held))))
        else:
            got = a.alloc(rng.randint(1, 200_000), from_top=rng.random() < 0.3)
            if got is not None:
                held.append(got)
        spans = sorted(held + a.free)
        assert sum(s for _o, s in spans) == size                         # nothing lost
        assert all(o1 + s1 <= o2 for (o1, s1), (o2, _s2) in zip(spans, spans[1:]))   # nothing overlaps
    for p in held:
        a.release(*p)
    assert a.free == [(0, size)]


def test_arena_top_pieces_keep_the_bottom_contiguous():
    """Pieces taken from the top (long-running requests) leave the bottom of
    the arena one contiguous piece for the short-lived ones."""
    a = serve._Arena(_FakeTorch(), None, 1 << 20)
    low = [a.alloc(10_000) for _ in range(5)]
    top = a.alloc(100_000, from_top=True)
    assert top[0] + top[1] == 1 << 20
    for p in low:
        a.release(*p)
    assert a.free[0] == (0, (1 << 20) - top[1])


def test_arena_pieces_are_256_byte_aligned():
    """Every piece, from either end, starts on a 256-byte boundary (the
    operands are viewed as float64 and handed to kernels), whatever the
    requested arena size."""
    rng = random.Random(7)
    a = serve._Arena(_FakeTorch(), None, 10_000_003)
    held = []
    for _ in range(500):
        if held and rng.random() < 0.4:
            a.release(*held.pop(rng.randrange(len(held))))
        else:
            got = a.alloc(rng.randint(1, 100_000), from_top=rng.random() < 0.5)
            if got is not None:
                assert got[0] % 256 == 0 and got[1] % 256 == 0
                held.append(got)


def test_new_graph_buckets_wait_while_an_fp64_batch_runs():
    """A request whose size bucket has no captured graph yet takes the batched
    path while an FP64 batch is in flight (capturing would synchronize the
    whole device and hold the loop until that batch ends); a bucket already
    captured keeps its graph path, and with no FP64 batch in flight a new
    bucket is captured as before."""
    from fmm_blis_gb300 import tune
    srv = object.__new__(serve.Server)
    srv.graph_max_dim = 1024
    srv._slots = {}
    srv.inflight = []
    t = tune.Tuner()

    def req(m, n, k, form="split"):
        r = serve.Request(m, n, k, form=form)
        r.plan = t.plan(m, n, k, form, 1e-10)
        return r

    small = req(200, 300, 250)
    assert small.plan.levels == 0
    key = srv._graph_bucket(small)
    assert key == (256, 512, 256, small.plan.slices, small.plan.fmt)   # no FP64 in flight: graph path
    srv.inflight = [(None, [req(4096, 4096, 4096, "fp64")], [])]
    assert srv._graph_bucket(small) is None                              # new bucket, FP64 running: batched
    srv._slots[key] = ["captured"]
    assert srv._graph_bucket(small) == key                               # captured bucket: graph path
    srv.inflight = [(None, [req(900, 900, 900)], [])]
    assert srv._graph_bucket(req(100, 100, 100)) is not None             # only split work in flight
    assert srv._graph_bucket(req(2000, 300, 300)) is None                # beyond the graph sizes


def test_operands_into_preallocated_memory_equal_fresh_ones():
    """The arena path writes a request's operands into preallocated memory
    with the same generator draws as a fresh allocation (CPU generator here;
    the GPU tests check the served bits against the direct calls)."""
    import torch
    rows, cols = 37, 23
    g1 = torch.Generator().manual_seed(11)
    fresh = serve._colmajor_rand(torch, rows, cols, g1, torch.device("cpu"))
    buf = torch.empty(8 * rows * cols + 256, dtype=torch.uint8)
    view = buf[256:256 + 8 * rows * cols].view(torch.float64).view(cols, rows).t()
    g2 = torch.Generator().manual_seed(11)
    into = serve._colmajor_rand_into(torch, view, g2)
    assert into.shape == (rows, cols) and into.stride() == (1, rows)
    assert torch.equal(into, fresh)
