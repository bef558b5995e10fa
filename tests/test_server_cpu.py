"""Host-side logic of the request server without a GPU (dry-run planning:
kernels are compiled, nothing is launched, completions are immediate).
Failure handling is exercised on the host: rejected admissions, cancelled
and timed-out requests, injected dispatch errors."""
from __future__ import annotations

import time

import pytest

import xtensor_gb300 as xg
from xtensor_gb300.device import DeviceArray
from xtensor_gb300.server import Server


@pytest.fixture(autouse=True)
def dry():
    xg.set_option("jit.dry_run", 1)
    yield
    xg.set_option("server.paused", -1)
    xg.set_option("server.inject_fail_every", -1)
    xg.set_option("jit.dry_run", -1)


_next = [0x200000000]


def fake(shape, dtype="float32"):
    p = _next[0]
    _next[0] += 1 << 32
    return DeviceArray(shape, dtype, p)


def test_requests_complete_and_stats():
    s = Server(streams=4, hbm_budget=1 << 30)
    ids = []
    for i in range(20):
        a = fake((64, 100 + i))
        ids.append(s.submit_reduce("sum", a * a, fake((64,)), axes=[1]))
    for rid in ids:
        r = s.wait(rid, 5000)
        assert r["status"] == 0
    st = s.stats()
    assert st["completed"] == 20 and st["failed"] == 0 and st["p99_ms"] >= st["p50_ms"] >= 0
    s.close()


def test_rejection_when_larger_than_budget():
    s = Server(hbm_budget=1 << 20)
    with pytest.raises(xg.XtgError) as ei:
        s.submit_assign(fake((10,)), fake((10,)) * 2, workspace=2 << 20)
    assert ei.value.status == 11
    assert s.stats()["rejected"] == 1
    s.close()


def test_cancel_timeout_and_grouped_wave():
    s = Server(batch_min_group=4)
    xg.set_option("server.compile_inline", 1)  # batch on the first wave (this test counts launches)
    xg.set_option("server.paused", 1)
    ids = [s.submit_reduce("sum", fake((32, 64)) + fake((64,)), fake((32,)), axes=[-1]) for _ in range(10)]
    victim = s.submit_assign(fake((8, 8)), fake((8, 8)) * 3)
    with pytest.raises(xg.XtgError) as ei:
        s.wait(victim, 50)
    assert ei.value.status == 10  # timeout: still queued
    s.cancel(victim)
    with pytest.raises(xg.XtgError) as ei:
        s.wait(victim, 1000)
    assert ei.value.status == 12
    xg.set_option("server.paused", 0)
    # any new event lets the scheduler admit the held requests as one wave
    last = s.submit_assign(fake((4,)), fake((4,)) + 1)
    for rid in ids + [last]:
        assert s.wait(rid, 5000)["status"] == 0
    st = s.stats()
    assert st["batch_launches"] >= 1 and st["batched_requests"] >= 10 and st["cancelled"] == 1
    xg.set_option("server.compile_inline", 0)
    s.close()


def test_batch_kernels_compile_off_the_scheduler():
    """A group whose batch kernel is not loaded runs one request at a time
    while the kernel builds on another thread; a later group batches."""
    import time
    s = Server(batch_min_group=3)

    def wave(n, rows):
        xg.set_option("server.paused", 1)
        ids = [s.submit_reduce("sum", fake((rows, 96)) * fake((96,)), fake((rows,)), axes=[-1]) for _ in range(n)]
        xg.set_option("server.paused", 0)
        kick = s.submit_assign(fake((4,)), fake((4,)) + 1)
        for rid in ids + [kick]:
            assert s.wait(rid, 20000)["status"] == 0

    wave(6, 33)
    first = s.stats()
    assert first["batch_launches"] == 0  # the kernel was not loaded yet
    for _ in range(200):  # its background build finishes
        time.sleep(0.05)
        wave(6, 33)
        if s.stats()["batch_launches"] >= 1:
            break
    assert s.stats()["batch_launches"] >= 1
    s.close()


def test_injected_dispatch_failures_do_not_stop_the_server():
    s = Server(batch_min_group=1000)
    xg.set_option("server.inject_fail_every", 3)
    ids = [s.submit_assign(fake((16, 16)), fake((16, 16)) * 2) for _ in range(9)]
    statuses = []
    for rid in ids:
        try:
            statuses.append(s.wait(rid, 5000)["status"])
        except xg.XtgError as e:
            statuses.append(e.status)
    assert statuses.count(6) == 3 and statuses.count(0) == 6
    assert s.stats()["failed"] == 3
    s.close()


def test_budget_accounting_returns_to_zero():
    s = Server(hbm_budget=1 << 24, max_inflight=2)
    ids = [s.submit_assign(fake((100,)), fake((100,)) + 1, workspace=1 << 22) for _ in range(12)]
    for rid in ids:
        s.wait(rid, 5000)
    s.drain(5000)
    st = s.stats()
    assert st["inflight"] == 0 and st["hbm_reserved"] == 0 and st["completed"] == 12
    s.close()
