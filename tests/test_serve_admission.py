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
