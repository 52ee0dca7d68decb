"""Host logic of the serving loop (no GPU)."""
import threading
import time

import numpy as np

from mlau_gb300 import FP64, serve


def test_request_stream_is_seeded_and_follows_the_mix():
    a = serve.make_requests(400, rate=50.0, seed=7, n1d=(16, 32), n2d=(8, 12), n3d=(8, 8),
                            steps_3d=1)
    b = serve.make_requests(400, rate=50.0, seed=7, n1d=(16, 32), n2d=(8, 12), n3d=(8, 8),
                            steps_3d=1)
    assert [r.kind for r in a] == [r.kind for r in b]
    assert all(np.array_equal(x.state["ro"], y.state["ro"]) for x, y in zip(a, b))
    kinds = [r.kind for r in a]
    assert abs(kinds.count("1d") / 400 - 0.5) < 0.08
    assert abs(kinds.count("2d") / 400 - 0.4) < 0.08
    assert all(r.precision == FP64 for r in a if r.kind == "1d")
    arr = np.array([r.arrival for r in a])
    assert arr[0] == 0.0 and np.all(np.diff(arr) >= 0)
    assert abs(np.diff(arr).mean() - 1 / 50.0) < 0.2 / 50.0
    for r in a:
        if r.kind == "2d":
            assert 8 <= r.state["ro"].shape[0] - 8 <= 12 and 0.05 <= r.meta["t_end"] <= 0.5
            assert r.interior == (r.state["ro"].shape[0] - 8) * (r.state["ro"].shape[1] - 8)


def test_serial_schedule():
    class R:
        def __init__(self, a):
            self.arrival = a

    reqs = [R(0.0), R(0.5), R(3.0)]
    lat, end = serve.serial_schedule(reqs, [1.0, 1.0, 1.0])
    assert lat == [1.0, 1.5, 1.0] and end == 4.0


def test_block_allocator_never_oversubscribes():
    blocks = serve._Blocks(152)
    for lane, cells in (("a", 10), ("b", 30), ("c", 0)):
        blocks.set_load(lane, cells)
    peak = [0]
    inuse = [0]
    lock = threading.Lock()

    def worker(lane):
        for _ in range(50):
            g = blocks.acquire(lane)
            assert g >= 1
            with lock:
                inuse[0] += g
                peak[0] = max(peak[0], inuse[0])
            time.sleep(0.0005)
            with lock:
                inuse[0] -= g
            blocks.release(g)

    ts = [threading.Thread(target=worker, args=(n,)) for n in ("a", "b", "a", "b")]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert peak[0] <= 152 and blocks.free == 152
    blocks.set_load("a", 1)
    blocks.set_load("b", 0)
    assert blocks.acquire("a") == 152
