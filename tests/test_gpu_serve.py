"""Serving loop: each request gives the same result in the mix as alone."""
import numpy as np
import pytest

import mlau_gb300 as M
from mlau_gb300 import serve

pytestmark = pytest.mark.gpu

# small problems with moderate 2D turbulence (no request should fail)
SMALL = dict(n1d=(48, 200), n2d=(24, 56), n3d=(16, 24), t_end_2d=(0.01, 0.03), steps_3d=4,
             mach_2d=(1e-3, 0.6), beta_2d=(0.5, 10.0))
BUDGET = 2e9


def serve_all(reqs, **kw):
    with serve.Server(budget_bytes=kw.pop("budget", BUDGET), max_inst=kw.pop("max_inst", 16),
                      **kw) as srv:
        return {r.rid: r for r in srv.run(reqs, realtime=False)}


def same(a, b):
    assert a.keys() == b.keys()
    for v in a:
        assert np.array_equal(a[v], b[v], equal_nan=True), v


def test_fp64_requests_equal_the_one_at_a_time_solver():
    reqs = serve.make_requests(14, rate=1000.0, seed=1, split_frac=0.0, mix=(0.4, 0.4, 0.2),
                               **SMALL)
    done = serve_all(reqs)
    assert len(done) == len(reqs) and {r.kind for r in reqs} == {"1d", "2d", "3d"}
    for r in reqs:
        got = done[r.rid]
        assert not got.failed and got.steps > 0
        ref, steps, _ = serve.solve_alone_fp64(r)
        assert got.steps == steps, (r.kind, got.steps, steps)
        same(got.result, ref)


def test_split_requests_equal_alone_in_the_server():
    reqs = serve.make_requests(10, rate=1000.0, seed=2, split_frac=1.0, mix=(0.2, 0.6, 0.2),
                               **SMALL)
    done = serve_all(reqs)
    for r in reqs:
        alone = serve_all([r])[r.rid]
        assert not done[r.rid].failed
        assert done[r.rid].steps == alone.steps
        same(done[r.rid].result, alone.result)


def test_admission_waits_for_room_under_the_budget():
    reqs = serve.make_requests(5, rate=1000.0, seed=3, split_frac=0.0, mix=(0.0, 1.0, 0.0),
                               n2d=(48, 56), t_end_2d=(0.01, 0.02), mach_2d=(1e-3, 0.6),
                               beta_2d=(0.5, 10.0))
    # room for one 2D instance of at most 64x64 padded cells in the FP64 lane
    budget = 64 * 64 * serve.Server.BYTES_PER_CELL["2d64"] / 0.36 * 1.2
    done = serve_all(reqs, budget=budget)
    order = sorted(done.values(), key=lambda r: r.t_admit)
    for a, b in zip(order, order[1:]):
        assert b.t_admit >= a.t_done  # one at a time
    for r in reqs:
        ref, steps, _ = serve.solve_alone_fp64(r)
        assert not done[r.rid].failed and done[r.rid].steps == steps
        same(done[r.rid].result, ref)


def test_a_bad_request_fails_alone():
    reqs = serve.make_requests(8, rate=1000.0, seed=4, split_frac=0.5, mix=(0.4, 0.6, 0.0),
                               **SMALL)
    bad = next(r for r in reqs if r.kind == "2d")
    bad.state["en"][6:9, 6:9] = 0.0  # negative pressure: fault injected on the host
    done = serve_all(reqs)
    assert done[bad.rid].failed
    for r in reqs:
        if r is not bad:
            assert not done[r.rid].failed
            alone = serve_all([r])[r.rid]
            same(done[r.rid].result, alone.result)
