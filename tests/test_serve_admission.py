"""Host logic of the request server: memory-budget admission (FIFO, head of line waits, requests that can
never fit are rejected) and release.  No GPU: the server is constructed but not started."""
import pytest


def _server(budget):
    pytest.importorskip("torch")
    from spectraldoublediffusiveconvection_gb300 import serve
    return serve, serve.Server(device="cpu", memory_budget=budget)


def test_admission_counts_state_and_operators():
    serve, srv = _server(10 ** 9)
    r = serve.Request("integrate", 30, 256, 8000.0)
    assert srv._try_admit(r) is True
    assert srv.used == srv.request_bytes(r) and srv.resident == srv.plan_bytes(r)
    r2 = serve.Request("integrate", 30, 256, 8000.0)
    assert srv._try_admit(r2) is True                 # same shape: operators counted once
    assert srv.resident == srv.plan_bytes(r) and srv.used == 2 * srv.request_bytes(r)
    srv._release(r)
    srv._release(r2)
    assert srv.used == 0


def test_continuation_holds_more_than_integration():
    serve, srv = _server(10 ** 9)
    a = serve.Request("integrate", 48, 512, 9000.0)
    b = serve.Request("continue", 48, 512, 9000.0)
    assert srv.request_bytes(b) > srv.request_bytes(a)


def test_waits_when_full_and_rejects_what_never_fits():
    serve, probe = _server(1)
    big = serve.Request("continue", 48, 512, 9000.0)
    small = serve.Request("integrate", 20, 64, 9000.0)
    _, srv = _server(probe.plan_bytes(small) + int(1.5 * probe.request_bytes(small)))
    assert srv._try_admit(big) == "reject"
    assert srv._try_admit(small) is True
    s2 = serve.Request("integrate", 20, 64, 9000.0)
    assert srv._try_admit(s2) is False                # fits alone, not now: waits
    srv._release(small)
    assert srv._try_admit(s2) is True


def test_admit_kind_is_fifo_and_reports_rejections():
    serve, srv = _server(10 ** 7)
    reqs = [serve.Request("integrate", 20, 64, 9000.0) for _ in range(3)]
    huge = serve.Request("integrate", 48, 512, 9000.0)
    for r in [reqs[0], huge, reqs[1], reqs[2]]:
        srv.submit(r)
    got = srv._admit_kind("integrate")
    assert huge.error is not None and huge.done.is_set() and srv.stats["rejected"] == 1
    n = len(got)
    assert got == reqs[:n] and n >= 1
    assert list(srv._pending["integrate"]) == reqs[n:]


def test_failed_worker_fails_its_requests_and_drain_returns():
    serve, srv = _server(10 ** 9)
    a = serve.Request("continue", 20, 64, 9000.0)
    b = serve.Request("continue", 20, 64, 9000.0)
    srv.submit(a)
    srv.submit(b)
    got = srv._admit_kind("continue")                  # a and b admitted; move a into the waiting list
    assert got == [a, b]
    srv._waiting.setdefault(a.shape, []).append(a)
    srv._pending["continue"].append(b)                 # b back in the queue (admitted bytes kept)
    srv._worker_failed("continue", RuntimeError("device lost"))
    assert a.done.is_set() and b.done.is_set()
    assert "device lost" in a.error and "device lost" in b.error
    assert srv.drain(timeout=1.0) is False and srv.worker_error
    assert srv.used == 0


def test_cancel_queued_and_waiting_requests():
    """Server.cancel on the host: a request still in the queue is retired at once without touching the
    budget; an admitted request waiting for its batch (continuation) or its group's boundary (integration)
    returns its bytes; a request in flight is only marked (its worker retires it)."""
    serve, srv = _server(10 ** 9)
    q = serve.Request("integrate", 20, 64, 9000.0)
    srv.submit(q)
    assert srv.cancel(q) is True
    assert q.done.is_set() and q.error == "cancelled" and not srv._pending["integrate"] and srv.used == 0
    assert srv.cancel(q) is False                      # already completed
    a = serve.Request("continue", 20, 64, 9000.0)
    b = serve.Request("integrate", 24, 128, 9000.0)
    srv.submit(a)
    srv.submit(b)
    assert srv._admit_kind("continue") == [a] and srv._admit_kind("integrate") == [b]
    srv._waiting.setdefault(a.shape, []).append(a)
    srv._int_joining.setdefault(b.shape, []).append(b)
    assert srv.used == srv.request_bytes(a) + srv.request_bytes(b) and srv._active == 2
    assert srv.cancel(a) and srv.cancel(b)
    assert a.error == b.error == "cancelled" and a.done.is_set() and b.done.is_set()
    assert srv.used == 0 and srv._active == 0 and not srv._waiting[a.shape] and not srv._int_joining[b.shape]
    c = serve.Request("integrate", 20, 64, 9000.0)
    srv.submit(c)
    srv._admit_kind("integrate")                       # admitted and handed to a group (in flight)
    assert srv.cancel(c) is True and c.cancelled and not c.done.is_set()
    srv._finish(c, error="cancelled")                  # what the worker does at the next boundary
    assert srv.used == 0 and srv._active == 0


def test_latency_report_splits_queue_and_device_time():
    serve, _ = _server(10 ** 9)
    reqs = []
    for i in range(10):
        r = serve.Request("integrate", 20, 64, 9000.0)
        r.t_submit, r.t_start, r.t_done = 0.0, 0.01 * i, 0.01 * i + 0.1
        reqs.append(r)
    bad = serve.Request("integrate", 20, 64, 9000.0)
    bad.t_submit, bad.t_start, bad.t_done, bad.error = 0.0, 0.0, 5.0, "non-finite state"
    rep = serve.latency_report(reqs + [bad])
    assert rep["n"] == 10
    assert rep["device_p50_ms"] == pytest.approx(100.0) and rep["device_p99_ms"] == pytest.approx(100.0)
    assert rep["queue_p50_ms"] == pytest.approx(45.0)
    assert rep["max_ms"] == pytest.approx(190.0)
