"""Host model of the window ring of the hub-row SpMV kernel (k_hubwin, gg_spmv_hub.cu).

A CTA's 32 warps share kHwBufs window buffers.  The copy of window q lands in buffer
q mod kHwBufs and completes on that buffer's mbarrier; the last warp to leave window q
issues the copy of window q + kHwBufs after the copy it held has landed.  A warp waits
for every window before it leaves it and leaves windows in order, and an item may read
up to kHwBufs consecutive windows after the warp has left every window before its
first.  The model runs random schedules of warps with random items and checks what the
kernel relies on: no deadlock, the arrivals counted for a buffer always belong to one
window, a buffer holds the window an item reads while the item runs, and every wait is
on the phase right after the last one the warp saw (mbarrier parity waits cannot tell
phases two apart).  It also checks that leaving a window without waiting for it (the
protocol of an earlier build, which faulted) breaks these rules."""
import random

import pytest

BUFS = 4


def _items(rnd, units, nwarps):
    out = []
    for _ in range(nwarps):
        lst, q = [], 0
        for b, e in units:
            nw = e - b
            x = 0
            while x < nw:
                x += rnd.choice([0, 0, 1, 1, 2, 5])
                if x >= nw:
                    break
                span = min(rnd.choice([1, 1, 2, 3, 4]), nw - x)
                lst.append((q + x, q + x + span, q))
                x += span - 1 if span > 1 else rnd.choice([0, 1])
            q += nw
        out.append(lst)
    return out


def _warp(items, units, wait_before_leave):
    waited = arrived = 0
    q0 = 0
    for b, e in units:
        us, ue = q0, q0 + e - b
        q0 = ue
        for f, l, u in items:
            if u != us:
                continue
            while arrived < f:
                if wait_before_leave and waited == arrived:
                    yield ("wait", waited)
                    waited += 1
                yield ("leave", arrived)
                arrived += 1
                waited = max(waited, arrived)
            while waited < l:
                yield ("wait", waited)
                waited += 1
            yield ("work", f, l)
        while arrived < ue:
            if wait_before_leave and waited == arrived:
                yield ("wait", waited)
                waited += 1
            yield ("leave", arrived)
            arrived += 1
            waited = max(waited, arrived)


def _run(seed, wait_before_leave, nwarps=32, units=((0, 9), (9, 20), (20, 23))):
    rnd = random.Random(seed)
    total = sum(e - b for b, e in units)
    items = _items(rnd, units, nwarps)
    issued, landed = [0] * BUFS, [0] * BUFS
    in_flight = []
    issued_q = set()
    for q in range(min(BUFS, total)):
        issued[q % BUFS] += 1
        issued_q.add(q)
        in_flight.append(q)
    count = [0] * BUFS
    left = {}
    gens = [_warp(items[w], units, wait_before_leave) for w in range(nwarps)]
    pending = [next(g, None) for g in gens]
    for _ in range(10 ** 6):
        if all(p is None for p in pending) and not in_flight:
            break
        if in_flight and rnd.random() < 0.3:
            q = in_flight.pop(0)
            landed[q % BUFS] += 1
        ready = []
        for w, p in enumerate(pending):
            if p is None:
                continue
            if p[0] == "wait":
                q = p[1]
                b, k = q % BUFS, q // BUFS
                assert landed[b] >= k, "waiting two phases ahead"
                if landed[b] >= k + 1:
                    ready.append(w)
            else:
                ready.append(w)
        if not ready:
            assert in_flight, "deadlock"
            continue
        w = rnd.choice(ready)
        p = pending[w]
        if p[0] == "leave":
            q = p[1]
            b = q % BUFS
            assert q in issued_q, "left a window before its copy was issued"
            left[q] = left.get(q, 0) + 1
            count[b] += 1
            if count[b] == nwarps:
                assert left[q] == nwarps, "arrivals of two windows in one counter"
                count[b] = 0
                if q + BUFS < total:
                    assert landed[b] == issued[b]
                    issued[b] += 1
                    issued_q.add(q + BUFS)
                    in_flight.append(q + BUFS)
        elif p[0] == "work":
            for q in range(p[1], p[2]):
                b = q % BUFS
                assert landed[b] == q // BUFS + 1 and issued[b] == q // BUFS + 1, "buffer not holding its window"
        pending[w] = next(gens[w], None)
    else:
        raise AssertionError("did not finish")
    assert all(left.get(q, 0) == nwarps for q in range(total))


@pytest.mark.parametrize("seed", range(40))
def test_ring_protocol_holds(seed):
    _run(seed, wait_before_leave=True)


def test_leaving_without_waiting_breaks_the_ring():
    bad = 0
    for seed in range(20):
        try:
            _run(seed, wait_before_leave=False)
        except AssertionError:
            bad += 1
    assert bad > 0
