"""Host logic of the propagator-solve service, in dry-run mode (no device work: each
request holds its memory for dry_seconds).  Checks continuous batching: requests that
arrive while others run are admitted as slots and memory free up, the HBM budget is never
exceeded, admission goes in arrival order but lets a request that fits pass one that
does not (until the oldest reaches its age bound), oversized requests are solved in
chunks of sources or rejected at submission, queued requests can be shed, and the queue
depth is traced."""
import time

import numpy as np

import grid_gb300 as g

GB = 1 << 30


def req(dims=(8, 8, 8, 8), Ls=8, nsrc=1, dry=0.05, **kw):
    return g.make_request(dims, Ls, 0.01, 0.5, 1, nsrc, 2, dry_seconds=dry, **kw)


def test_budget_never_exceeded_and_slots_overlap():
    r = req(dims=(16, 16, 16, 16), Ls=16, nsrc=4, dry=0.2)
    one = g.request_bytes(r)
    budget = int(2.5 * one)  # two fit, the third must wait
    s = g.Server(budget, slots=4, flags=g.Server.DRY_RUN)
    for _ in range(6):
        s.submit(req(dims=(16, 16, 16, 16), Ls=16, nsrc=4, dry=0.2))
    assert s.wait(6, 30)
    st = s.stats()
    assert st.peak_used_bytes <= budget
    assert st.max_running == 2  # memory, not slots, limited the concurrency
    res = sorted(s.results(), key=lambda x: x.id)
    assert all(x.status == 0 for x in res)
    # first come, first served: start times follow submission order
    starts = [x.t_start for x in res]
    assert starts == sorted(starts)
    s.close()


def test_continuous_admission_while_running():
    s = g.Server(64 * GB, slots=2, flags=g.Server.DRY_RUN)
    s.submit(req(dry=0.3))
    s.submit(req(dry=0.3))
    time.sleep(0.05)
    st = s.stats()
    assert st.running == 2
    late = s.submit(req(dry=0.05))  # arrives while both slots are busy
    assert s.wait(3, 10)
    res = {x.id: x for x in s.results()}
    # the late request started as soon as a slot freed, before the others had all ended
    first_end = min(res[0].t_end, res[1].t_end)
    assert res[late].t_start >= first_end - 1e-3
    assert res[late].t_start - first_end < 0.1
    s.close()


def test_oversized_request_is_chunked_or_rejected():
    big = req(dims=(24, 24, 24, 24), Ls=16, nsrc=12, dry=0.01)
    one_src = g.request_bytes(req(dims=(24, 24, 24, 24), Ls=16, nsrc=1))
    full = g.request_bytes(big)
    budget = int(full * 0.4)
    s = g.Server(budget, slots=2, flags=g.Server.DRY_RUN)
    s.submit(big)
    s.submit(req(dims=(24, 24, 24, 24), Ls=16, nsrc=1, dry=0.01))
    assert s.wait(2, 10)
    res = sorted(s.results(), key=lambda x: x.id)
    assert res[0].status == 0 and 1 <= res[0].chunk < 12
    assert g.request_bytes(req(dims=(24, 24, 24, 24), Ls=16, nsrc=res[0].chunk)) <= budget
    s.close()
    tiny = g.Server(one_src // 2, slots=1, flags=g.Server.DRY_RUN)
    tiny.submit(req(dims=(24, 24, 24, 24), Ls=16, nsrc=1, dry=0.01))
    assert tiny.wait(1, 10)
    (r,) = tiny.results()
    assert r.status == 3  # GB_ERR_OOM: does not fit even one source, rejected at submission
    assert tiny.stats().rejected == 1
    tiny.close()


def test_request_bytes_scale_with_sources_and_volume():
    a = g.request_bytes(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1))
    b = g.request_bytes(req(dims=(8, 8, 8, 8), Ls=8, nsrc=4))
    c = g.request_bytes(req(dims=(16, 8, 8, 8), Ls=8, nsrc=4))
    assert a < b < c
    assert abs(c / b - 2) < 0.01


def test_skip_ahead_then_age_bound():
    """A large request that does not fit what is left of the budget is passed by a small
    one that does; once the large one has waited age_limit nothing passes it."""
    small = g.request_bytes(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1))
    large = g.request_bytes(req(dims=(16, 16, 16, 16), Ls=16, nsrc=4))
    budget = large + small // 2  # the large one fits only when nothing else runs
    s = g.Server(budget, slots=4, flags=g.Server.DRY_RUN)
    s.set_age_limit(0.25)
    hold = s.submit(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1, dry=0.6))  # runs, blocking the large one
    time.sleep(0.05)
    big = s.submit(req(dims=(16, 16, 16, 16), Ls=16, nsrc=4, dry=0.05))
    time.sleep(0.02)
    passer = s.submit(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1, dry=0.05))  # fits beside `hold`
    time.sleep(0.4)  # the large request is now older than the age bound
    late = s.submit(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1, dry=0.05))
    assert s.wait(4, 10)
    res = {x.id: x for x in s.results()}
    assert res[passer].t_start < res[big].t_start  # passed the large request
    assert res[big].t_start < res[late].t_start  # the age bound held the late one back
    assert res[big].t_start >= res[hold].t_end - 1e-3
    assert s.stats().peak_used_bytes <= budget
    s.close()


def test_fifo_and_shortest_first_policies():
    small = g.request_bytes(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1))
    large = g.request_bytes(req(dims=(16, 16, 16, 16), Ls=16, nsrc=4))
    # FIFO: the small request waits behind the large one that does not fit yet
    s = g.Server(large + small // 2, slots=4, flags=g.Server.DRY_RUN | g.Server.FIFO)
    hold = s.submit(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1, dry=0.3))
    time.sleep(0.05)
    big = s.submit(req(dims=(16, 16, 16, 16), Ls=16, nsrc=4, dry=0.05))
    small_id = s.submit(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1, dry=0.05))
    assert s.wait(3, 10)
    res = {x.id: x for x in s.results()}
    assert res[big].t_start <= res[small_id].t_start
    assert res[big].t_start >= res[hold].t_end - 1e-3
    s.close()
    # shortest first: with one slot busy, the queued requests start smallest first
    s = g.Server(64 * GB, slots=1, flags=g.Server.DRY_RUN | g.Server.SHORTEST_FIRST)
    s.set_age_limit(60.0)
    s.submit(req(dry=0.2))
    time.sleep(0.05)
    ids = [s.submit(req(dims=d, Ls=8, nsrc=1, dry=0.02)) for d in ((16, 16, 16, 16), (8, 8, 8, 8), (12, 12, 12, 12))]
    assert s.wait(4, 10)
    res = {x.id: x for x in s.results()}
    order = sorted(ids, key=lambda i: res[i].t_start)
    assert order == [ids[1], ids[2], ids[0]]
    s.close()


def test_cancel_queued_and_trace():
    s = g.Server(64 * GB, slots=1, flags=g.Server.DRY_RUN)
    run = s.submit(req(dry=0.3))
    time.sleep(0.05)
    queued = [s.submit(req(dry=0.01)) for _ in range(5)]
    assert s.cancel_queued() == 5
    assert s.wait(6, 10)
    res = {x.id: x for x in s.results()}
    assert res[run].status == 0
    assert all(res[i].status == 10 for i in queued)  # GB_ERR_CANCELLED
    st = s.stats()
    assert st.cancelled == 5 and st.max_queued == 5
    t, q, r = s.trace()
    assert len(t) >= 8 and all(np.diff(t) >= 0)
    assert q.max() == 5 and q[-1] == 0 and r.max() == 1
    s.close()
