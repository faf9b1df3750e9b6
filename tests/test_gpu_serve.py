"""Serving form (dg_serve_*): continuous batching of solves that arrive while
others run, admitted by an HBM budget.  Every result is the same alone and in
the mix (bitwise: a problem's arithmetic never depends on its batch-mates)."""
import numpy as np
import pytest

from conftest import dg, workloads

pytestmark = pytest.mark.gpu


def requests(n=5, seed=21):
    W = workloads()
    cfgs = W.config4(seed=seed, n=n, steps=30)
    rng = np.random.default_rng(seed)
    for c in cfgs:
        c["NUM_ELEMENTS"] = [min(v, 7) for v in c["NUM_ELEMENTS"]]
        c["STEPS"] = int(rng.integers(10, 40))
    return cfgs


def alone(cfg):
    with dg().Batch([cfg]) as b:
        b.step(cfg["STEPS"])
        return b.state(0)


def test_results_same_alone_and_in_the_mix():
    m = dg()
    cfgs = requests()
    with m.Server(hbm_budget_bytes=8 << 30, keep_results=True) as srv:
        # all arrive together; the first is admitted as soon as its host
        # preparation is done, the others join it while it runs
        t0 = srv.clock
        ids = [srv.submit(c, arrival_time=t0) for c in cfgs]
        srv.run(max_seconds=120)
        res = [srv.result(i, state=True) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(cfgs)
    assert st["mean_inflight"] > 1.0  # requests overlapped on the device
    for c, r in zip(cfgs, res):
        assert r["done"] >= r["admit"] >= r["arrival"]
        ra, va = alone(c)
        assert np.array_equal(r["rho"], ra) and np.array_equal(r["vel"], va)


def test_admission_respects_the_hbm_budget():
    m = dg()
    import importlib
    cfgs = requests(n=6, seed=5)
    for c in cfgs:
        c["NUM_ELEMENTS"] = [6, 6, 6]
        c["ORDER"] = 3
        c["STEPS"] = 300  # long enough that the next request is prepared while one runs
    per = 216 * 64 * 23 * 4 + 216 * 28
    with m.Server(hbm_budget_bytes=2 * per + 100) as srv:
        for c in cfgs:
            srv.submit(c, arrival_time=0.0)
        peak = 0
        while True:
            n = srv.tick()
            peak = max(peak, n)
            if all(srv.result(i + 1)["done"] >= 0 for i in range(len(cfgs))):
                break
        st = srv.stats()
    assert peak == 2 and st["completed"] == 6


def test_request_larger_than_budget_rejected():
    m = dg()
    c = requests(n=1)[0]
    with m.Server(hbm_budget_bytes=1 << 20) as srv:
        with pytest.raises(m.DGError, match="more than the whole HBM budget"):
            srv.submit(c)


def test_steady_stream_accounting():
    """A stream of requests arriving while others run: every request completes
    after it arrived and was admitted, the device-busy time is positive and
    at most the span, and the DOF-stage updates the server counts equal the
    requests' own (4 fields x nodes x 3 stages x steps)."""
    m = dg()
    W = workloads()
    cfgs = requests(n=40, seed=9)
    rng = np.random.default_rng(9)
    with m.Server(hbm_budget_bytes=4 << 30) as srv:
        t0 = srv.clock + 0.01
        t, ids = t0, []
        for c in cfgs:
            t += float(rng.exponential(0.004))
            ids.append(srv.submit(c, arrival_time=t))
        srv.run(max_seconds=120)
        st = srv.stats()
        u = srv.utilization()
        res = [srv.result(i) for i in ids]
    assert st["completed"] == len(cfgs)
    for r in res:
        assert r["done"] >= r["admit"] >= r["arrival"]
    want = sum(W.dof_count(c) * 3 * c["STEPS"] for c in cfgs)
    assert abs(u["dof_stage_updates"] - want) <= 1e-9 * want
    assert 0.0 < u["gpu_busy_s"] <= u["span_s"] * 1.001
    assert st["p99_s"] >= st["p50_s"] > 0.0


def test_submissions_from_another_thread():
    """dg_serve_submit from a second thread while the loop thread ticks: every
    request is served, and each result is the same as alone (the submit path
    goes through the server's internal queue)."""
    import threading
    import time
    m = dg()
    cfgs = requests(n=12, seed=31)
    ids, done = [], threading.Event()
    with m.Server(hbm_budget_bytes=4 << 30, keep_results=True) as srv:
        def producer():
            for c in cfgs:
                ids.append(srv.submit(c))
                time.sleep(0.002)
            done.set()

        th = threading.Thread(target=producer)
        th.start()
        deadline = time.time() + 120
        while time.time() < deadline:
            srv.tick()
            if done.is_set() and len(ids) == len(cfgs) and all(srv.result(i)["done"] >= 0 for i in ids):
                break
        th.join()
        res = [srv.result(i, state=True) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(cfgs)
    for c, r in zip(cfgs, res):
        assert r["done"] >= r["admit"] >= r["arrival"]
        ra, va = alone(c)
        assert np.array_equal(r["rho"], ra) and np.array_equal(r["vel"], va)


def test_one_step_requests_and_budget_of_exactly_one():
    """Requests of a single RK step, under a budget of exactly one request's
    bytes: they run one at a time, each finishes, and each result equals the
    batch run alone."""
    m = dg()
    cfgs = requests(n=4, seed=17)
    for c in cfgs:
        c["NUM_ELEMENTS"] = [3, 2, 4]
        c["ORDER"] = 2
        c["STEPS"] = 1
    per = 24 * 32 * 23 * 4 + 24 * 28  # 24 elements of 27 nodes padded to 32 slots
    with m.Server(hbm_budget_bytes=per, keep_results=True) as srv:
        ids = [srv.submit(c, arrival_time=0.0) for c in cfgs]
        for _ in range(100000):
            srv.tick()  # a one-step request is admitted and retired within one tick
            if all(srv.result(i)["done"] >= 0 for i in ids):
                break
        res = [srv.result(i, state=True) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(cfgs)
    assert st["mean_inflight"] == 1.0  # every step ran with exactly one solve in flight
    for c, r in zip(cfgs, res):
        ra, va = alone(c)
        assert np.array_equal(r["rho"], ra) and np.array_equal(r["vel"], va)
