"""Model of the two-warp barrier protocol of k_levi_civita_pair (nsg_integrate.cu):
the leading warp publishes tau-step records, the trailing warp decides when the
particle ends; over random interleavings and every stop point, both warps must leave
and every named-barrier phase must complete (a phase that never completes would hang
the GPU, so this is checked on the CPU before the kernel runs)."""
import random

FULL, EMPTY = 1, 3


def leader(shared):
    m = 0
    while True:
        b = m & 1
        if m >= 2:
            yield ("sync", EMPTY + b)
            yield ("run", 0)                 # the stop flag may be read any time after the sync
            if shared["stop"]:
                shared["term_at"] = m
                yield ("arrive", FULL + b)   # termination token
                yield ("sync", EMPTY + (b ^ 1))
                return
        yield ("run", 0)                     # tau-step m
        yield ("arrive", FULL + b)
        m += 1


def trailer(stop_at, shared):
    m = 0
    stopped = False
    while True:
        b = m & 1
        yield ("sync", FULL + b)
        if shared["term_at"] == m:
            return
        if not stopped:
            yield ("run", 0)
            if m == stop_at:
                stopped = True
                shared["stop"] = True
        yield ("arrive", EMPTY + b)
        m += 1


def simulate(stop_at, rng):
    shared = {"stop": False, "term_at": -1}
    warps = {"lead": leader(shared), "trail": trailer(stop_at, shared)}
    count = {k: 0 for k in (1, 2, 3, 4)}
    phase = {k: 0 for k in (1, 2, 3, 4)}
    members = {k: set() for k in (1, 2, 3, 4)}
    waiting, done, idle = {}, set(), 0
    while len(done) < 2:
        w = rng.choice([x for x in warps if x not in done])
        if w in waiting:
            bar, ph = waiting[w]
            if phase[bar] > ph:
                del waiting[w]
                idle = 0
            else:
                idle += 1
                if idle > 1000:
                    return "deadlock at stop %d: %s" % (stop_at, waiting)
            continue
        idle = 0
        try:
            op, bar = next(warps[w])
        except StopIteration:
            done.add(w)
            continue
        if op == "run":
            continue
        if w in members[bar]:
            return "warp %s arrives twice in one phase of barrier %d" % (w, bar)
        members[bar].add(w)
        count[bar] += 1
        if count[bar] == 2:
            count[bar], members[bar] = 0, set()
            phase[bar] += 1
        elif op == "sync":
            waiting[w] = (bar, phase[bar])
    if any(count.values()):
        return "unfinished phases at stop %d: %s" % (stop_at, count)
    return None


def test_protocol_completes_for_every_stop_point():
    rng = random.Random(11)
    errors = [e for stop_at in range(12) for _ in range(500) for e in [simulate(stop_at, rng)] if e]
    assert not errors, errors[:3]
