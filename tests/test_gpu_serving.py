"""Serving on the GPU: every request's result is the same when served in a continuously
batched mix, served alone one at a time, and computed by the oracle port."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload():
    """Sessions of varied sizes and request sequences (frames, edits), one starting at frame
    0 (its first frame clears), arriving in a burst."""
    from sandengine_gb300 import workloads as wl
    sizes = [(256, 256), (300, 130), (64, 64), (1000, 700), (77, 190), (512, 128), (130, 67)]
    sessions = []
    for i, (w, h) in enumerate(sizes):
        g = wl.patch_fill(w, h, 40 + i, *wl.twelve_fill_spec(), patch=16)
        sessions.append((w, h, g, 0 if i == 2 else 1 + i))
    reqs = []  # (session, nframes, mods, arrival_ms)
    for i, (w, h) in enumerate(sizes):
        for j in range(1 + i % 3):
            nf = [1, 13, 40, 9, 70][(i + j) % 5]
            mods = wl.circle_edits(w, h, 5, 10 * i + j, (i + j) % 4, [0, 3, 14]) if (i + j) % 2 == 0 else []
            reqs.append((i, nf, mods, 0.0 if j == 0 else 0.5 * j))
    return sessions, reqs


def _serve(se, rs, sessions, reqs, budget, plain):
    from sandengine_gb300.serving import Server
    srv = Server(rs, budget)
    for (w, h, g, f) in sessions:
        srv.open_session(w, h, g, f)
    ids = [srv.submit(s, nf, [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in mods], arr)
           for (s, nf, mods, arr) in reqs]
    srv.run(plain=plain)
    return srv, ids


def _oracle(ports, sessions, reqs):
    port = ports["twelve_materials"]
    out = []
    for i, (w, h, g, f) in enumerate(sessions):
        g = g.copy()
        for (s, nf, mods, _) in reqs:
            if s == i:
                port.run(g, f, nf, mods, nthreads=8)
                f += nf
        out.append((g, f))
    return out


def test_mixed_equals_alone_equals_oracle(se, ports, rulesets):
    rs = se.parse_string(rulesets["twelve_materials"])
    sessions, reqs = _workload()
    want = _oracle(ports, sessions, reqs)
    mixed, ids = _serve(se, rs, sessions, reqs, 256 << 20, plain=False)
    alone, _ = _serve(se, rs, sessions, reqs, 256 << 20, plain=True)
    for i, (g, f) in enumerate(want):
        assert np.array_equal(mixed.grid(i), g), f"session {i}: batched result differs from the oracle"
        assert np.array_equal(alone.grid(i), g), f"session {i}: one-at-a-time result differs from the oracle"
        assert mixed.frame(i) == f and alone.frame(i) == f
    st = mixed.stats()
    assert st["requests"] == len(reqs) and st["iterations"] > 0
    assert st["p99_ms"] >= st["p50_ms"] >= 0
    # the iterations' GPU time lies within the run (they run in order on one stream)
    assert 0 < st["kernel_ms"] <= st["wall_ms"] * 1.001
    assert all(mixed.latency_ms(r) >= 0 for r in ids)


def test_eviction_under_a_tight_budget(se, ports, rulesets):
    """A budget that holds only a few sessions forces LRU eviction to host and restores;
    results stay exact."""
    rs = se.parse_string(rulesets["twelve_materials"])
    sessions, reqs = _workload()
    want = _oracle(ports, sessions, reqs)
    # all sessions need 7.18 MB together; the largest 5.6 MB (2 x 1000 x 700 x 4 B)
    srv, _ = _serve(se, rs, sessions, reqs, 6 << 20, plain=False)
    st = srv.stats()
    assert st["evictions"] > 0, st
    assert st["peak_resident_bytes"] <= 6 << 20
    for i, (g, f) in enumerate(want):
        assert np.array_equal(srv.grid(i), g), f"session {i}"
    # a second round revisits every session: evicted ones come back from host memory
    port = ports["twelve_materials"]
    for i in range(len(sessions)):
        srv.submit(i, 11, [], 0.0)
    srv.run()
    st = srv.stats()
    assert st["restores"] > 0, st
    for i, (g, f) in enumerate(want):
        g = g.copy()
        port.run(g, f, 11, None, nthreads=8)
        assert np.array_equal(srv.grid(i), g), f"session {i}, second round"


def test_session_larger_than_budget_is_rejected(se, rulesets):
    from sandengine_gb300.serving import Server
    rs = se.parse_string(rulesets["four_materials"])
    srv = Server(rs, 1 << 20)
    with pytest.raises(se.SandengineError) as e:
        srv.open_session(1024, 1024)
    assert e.value.kind == "Budget"


@pytest.mark.parametrize("plain", [False, True])
def test_cancelled_requests_are_skipped(se, ports, rulesets, plain):
    """Host-side fault injection: requests withdrawn before the run are skipped (their
    sessions do not advance for them), the others are served exactly; a request that has
    run cannot be cancelled, and a cancelled one has no latency."""
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.serving import Server
    rs = se.parse_string(rulesets["twelve_materials"])
    P = ports["twelve_materials"]
    sizes = [(200, 150), (64, 64), (333, 120)]
    grids = [wl.patch_fill(w, h, 70 + i, *wl.twelve_fill_spec(), patch=16) for i, (w, h) in enumerate(sizes)]
    srv = Server(rs, 1 << 30)
    sids = [srv.open_session(w, h, g, 3) for (w, h), g in zip(sizes, grids)]
    plan = [(0, 10), (1, 7), (2, 12), (0, 5), (1, 9), (2, 4)]
    rids = [srv.submit(s, n) for s, n in plan]
    cancelled = {rids[1], rids[3], rids[5]}
    for r in cancelled:
        srv.cancel(r)
    srv.run(plain=plain)
    frames = [3, 3, 3]
    for r, (s, n) in zip(rids, plan):
        if r in cancelled:
            continue
        P.run(grids[s], frames[s], n)
        frames[s] += n
    for s in sids:
        assert np.array_equal(srv.grid(s), grids[s]), f"session {s}"
        assert srv.frame(s) == frames[s]
    with pytest.raises(se.SandengineError):
        srv.cancel(rids[0])  # already run
    with pytest.raises(se.SandengineError):
        srv.latency_ms(rids[1])  # cancelled
    assert srv.latency_ms(rids[0]) >= 0


@pytest.mark.parametrize("plain,budget", [(False, 256 << 20), (True, 256 << 20), (False, 6 << 20)])
def test_live_loop_requests_from_another_thread(se, ports, rulesets, plain, budget):
    """The live loop: requests submitted from a second thread while the loop runs (and while
    earlier requests are on the GPU) are admitted and served; each session's result equals
    the oracle's, as served alone; a request withdrawn before it starts is skipped; wait()
    and poll() report completion.  With a 6 MB budget sessions are evicted to host memory
    and restored while the loop runs."""
    import threading
    from sandengine_gb300.serving import Server
    rs = se.parse_string(rulesets["twelve_materials"])
    sessions, reqs = _workload()
    srv = Server(rs, budget)
    for (w, h, g, f) in sessions:
        srv.open_session(w, h, g, f)
    srv.start(plain=plain)
    ids, cancelled = [None] * len(reqs), set()
    # a long request ahead of the one to cancel keeps the latter queued behind it
    srv.submit(3, 300, [], 0.0)
    victim = srv.submit(3, 17, [], 0.0)
    try:
        srv.cancel(victim)
        cancelled.add(victim)
    except se.SandengineError:
        pass  # it had started already: then it is served like any other request

    def client(lo, hi):
        for i in range(lo, hi):
            s, nf, mods, _ = reqs[i]
            ids[i] = srv.submit(s, nf, [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in mods])

    # one thread submits the first half at once; this one the rest, after the loop is busy
    t = threading.Thread(target=client, args=(0, len(reqs) // 2))
    t.start()
    t.join()
    client(len(reqs) // 2, len(reqs))
    lat = [srv.wait(r, 60000.0) for r in ids]
    assert all(x >= 0 for x in lat)
    assert srv.poll(ids[-1]) is not None
    if cancelled:
        with pytest.raises(se.SandengineError) as e:
            srv.wait(victim, 0.0)
        assert e.value.kind == "Cancelled"
    srv.stop()
    # the oracle: session 3 first advanced 300 frames (and 17 more when not cancelled)
    extra = [(3, 300, [], 0.0)] + ([] if cancelled else [(3, 17, [], 0.0)])
    order = []
    for i in range(len(sessions)):
        order += [r for r in extra if r[0] == i] + [r for r in reqs if r[0] == i]
    want = _oracle(ports, sessions, order)
    for i, (g, f) in enumerate(want):
        assert np.array_equal(srv.grid(i), g), f"session {i}: live result differs from the oracle"
        assert srv.frame(i) == f
    st = srv.stats()
    assert st["requests"] == len(reqs) + 2 - len(cancelled)
    if budget < (7 << 20):
        assert st["evictions"] > 0 and st["restores"] > 0, st
