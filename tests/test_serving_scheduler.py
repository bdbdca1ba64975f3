"""Host logic of the propagator-solve service, in dry-run mode (no device work: each
request holds its memory for dry_seconds).  Checks continuous batching: requests that
arrive while others run are admitted as slots and memory free up, the HBM budget is never
exceeded, admission is first-come first-served, oversized requests are solved in chunks
of sources or rejected."""
import time

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
    assert r.status == 3  # GB_ERR_OOM: does not fit even one source
    tiny.close()


def test_request_bytes_scale_with_sources_and_volume():
    a = g.request_bytes(req(dims=(8, 8, 8, 8), Ls=8, nsrc=1))
    b = g.request_bytes(req(dims=(8, 8, 8, 8), Ls=8, nsrc=4))
    c = g.request_bytes(req(dims=(16, 8, 8, 8), Ls=8, nsrc=4))
    assert a < b < c
    assert abs(c / b - 2) < 0.01
