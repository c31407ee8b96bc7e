"""The ring protocol of the TMA residual-restriction (k_resid_restrict_tma,
mg_tma.cu), emulated on the CPU.

A producer lane fills e slots (planes i0-1 .. i1) and r slots (planes
i0 .. i1-1) and waits on a slot's "empty" barrier before refilling it.
Consumer warps, each at its own pace, wait on the "full" barriers of the
planes a step reads (found with the kernel's incremental slot and phase
counters), and arrive on the "empty" barriers of e(p-1) and r(p) once their
step is done.  The loads land at arbitrary later times.  Mbarriers are
modelled with their phase-parity waits.

Bars, over many random interleavings and chunk lengths: every wait returns
only once its fill has landed and never sees a barrier two phases ahead (a
parity wait would then pass or block wrongly); no slot is refilled while a
warp still reads it; every step reads the planes it expects; the schedule
ends without deadlock.
"""
import random

import pytest

ESLOTS, RSLOTS = 5, 4  # RR_ESLOTS, RR_RSLOTS


class Barrier:
    """An mbarrier: `count` arrivals (or one arrival plus the transaction
    bytes of a load) complete a phase; phase-parity waits."""

    def __init__(self, count):
        self.count = count
        self.pending = count
        self.completed = 0  # phases completed so far

    def arrive(self):
        self.pending -= 1
        assert self.pending >= 0
        if self.pending == 0:
            self.completed += 1
            self.pending = self.count

    def passes(self, parity, fill):
        """A phase-parity wait as the hardware does it: true when the current
        (incomplete) phase's parity differs from `parity`.  It names phase
        `fill` exactly only while the barrier is at most one phase past the
        one before it: that is the protocol's invariant, checked here."""
        assert fill <= self.completed <= fill + 1, "a parity wait would name the wrong phase"
        return (self.completed & 1) != (parity & 1)


def emulate(i0, i1, warps, seed, wrap_bug=False):
    rng = random.Random(seed)
    P0 = i0 - 1
    efull = [Barrier(1) for _ in range(ESLOTS)]
    eempty = [Barrier(warps) for _ in range(ESLOTS)]
    rfull = [Barrier(1) for _ in range(RSLOTS)]
    rempty = [Barrier(warps) for _ in range(RSLOTS)]
    etag = [None] * ESLOTS  # plane held by each slot once its load landed
    rtag = [None] * RSLOTS
    readers = {}  # (kind, slot) -> warps still to release the slot's current plane
    in_flight = []  # loads issued, not landed: (kind, slot, plane)

    def producer():
        for P in range(P0, i1 + 1):
            u = P - P0
            s = u % ESLOTS
            if u >= ESLOTS:
                parity = (u // ESLOTS - 1) & 1
                while not eempty[s].passes(parity, u // ESLOTS - 1):
                    yield
                assert readers.get(("e", s), 0) == 0, "e slot refilled while a warp reads it"
            in_flight.append(("e", s, P))
            Q = P - 1
            if i0 <= Q < i1:
                v = Q - i0
                sr = v % RSLOTS
                if v >= RSLOTS:
                    parity = (v // RSLOTS - 1) & 1
                    while not rempty[sr].passes(parity, v // RSLOTS - 1):
                        yield
                    assert readers.get(("r", sr), 0) == 0, "r slot refilled while a warp reads it"
                in_flight.append(("r", sr, Q))
            yield

    def consumer():
        # the kernel's counters: e(i0) is fill 1 of slot 1, r(i0) fill 0 of slot 0
        se, ne_ph, sr, nr_ph = 1, 0, 0, 0
        for b, f in ((efull[0], 0), (efull[1], 0)):
            while not b.passes(f, f):
                yield
        for p in range(i0, i1):
            sp = 0 if se == ESLOTS - 1 else se + 1
            sm1 = ESLOTS - 1 if se == 0 else se - 1
            # e(p+1): the next slot, one phase on when the ring wrapped
            ph = ne_ph + 1 if sp == 0 and not wrap_bug else ne_ph
            while not efull[sp].passes(ph, ph):
                yield
            while not rfull[sr].passes(nr_ph, nr_ph):
                yield
            # the step reads e(p-1), e(p), e(p+1) and r(p)
            assert (etag[sm1], etag[se], etag[sp]) == (p - 1, p, p + 1)
            assert rtag[sr] == p
            yield  # the step's arithmetic, interleaved with the others
            assert (etag[sm1], etag[se], etag[sp], rtag[sr]) == (p - 1, p, p + 1, p)
            # release e(p-1) and r(p)
            readers[("e", sm1)] -= 1
            readers[("r", sr)] -= 1
            eempty[sm1].arrive()
            rempty[sr].arrive()
            se = sp
            if sp == 0:
                ne_ph += 1
            sr = 0 if sr == RSLOTS - 1 else sr + 1
            if sr == 0:
                nr_ph += 1
            yield

    tasks = [producer()] + [consumer() for _ in range(warps)]
    alive = list(tasks)
    steps = 0
    while alive or in_flight:
        steps += 1
        assert steps < 200000, "deadlock"
        # a load lands, or a task advances by one wait or action
        if in_flight and (not alive or rng.random() < 0.4):
            kind, s, plane = in_flight.pop(rng.randrange(len(in_flight)))
            if kind == "e":
                etag[s] = plane
                readers[("e", s)] = warps
                efull[s].arrive()
            else:
                rtag[s] = plane
                readers[("r", s)] = warps
                rfull[s].arrive()
            continue
        t = rng.choice(alive)
        try:
            next(t)
        except StopIteration:
            alive.remove(t)


@pytest.mark.parametrize("chunk", [2, 4, 6, 10, 20, 30, 64])
def test_resid_restrict_ring_protocol(chunk):
    for seed in range(40):
        i0 = 2 * (seed % 3)
        emulate(i0, i0 + chunk, warps=3, seed=1000 * chunk + seed)


def test_emulation_catches_a_wrong_phase():
    """The emulation itself: a consumer that forgets the phase step when the
    e ring wraps waits on the wrong phase of slot 0, which the checks flag."""
    with pytest.raises(AssertionError):
        for seed in range(20):
            emulate(0, 20, warps=2, seed=seed, wrap_bug=True)
