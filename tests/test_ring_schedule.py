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


# ---- the fused red-black iteration's ring (k_rbgs_fused) ----
FU_ESLOTS, FU_RSLOTS = 6, 4


def emulate_fused(i0, i1, seed, early_release=False):
    """k_rbgs_fused's protocol: e planes i0-2 .. i1+1 and r planes i0-1 .. i1
    through rings of 6 and 4 slots.  The consumers move in step (a block
    barrier per plane step q): R(q) reads e(q-1..q+1) and r(q); after the
    barrier one thread issues the TMA store of plane q-2, waits until the
    store issued one step earlier (plane q-3) has read its slot, and releases
    e(q-3) and r(q-2); then K(q-1) reads e(q-2..q) and r(q-1).  A store
    reads its slot at an arbitrary later time."""
    rng = random.Random(seed)
    P0, Q0 = i0 - 2, i0 - 1
    efull = [Barrier(1) for _ in range(FU_ESLOTS)]
    eempty = [Barrier(1) for _ in range(FU_ESLOTS)]
    rfull = [Barrier(1) for _ in range(FU_RSLOTS)]
    rempty = [Barrier(1) for _ in range(FU_RSLOTS)]
    etag = [None] * FU_ESLOTS
    rtag = [None] * FU_RSLOTS
    in_flight = []  # loads: (kind, slot, plane)
    stores = []  # stores not done reading: (slot, plane)

    def eslot(p):
        return (p - P0) % FU_ESLOTS

    def rslot(p):
        return (p - Q0) % FU_RSLOTS

    def producer():
        for P in range(P0, i1 + 2):
            u = P - P0
            s = u % FU_ESLOTS
            if u >= FU_ESLOTS:
                k = u // FU_ESLOTS - 1
                while not eempty[s].passes(k & 1, k):
                    yield
                assert all(slot != s for slot, _ in stores), "e slot refilled while a store reads it"
            in_flight.append(("e", s, P))
            Q = P - 1
            if Q0 <= Q <= i1:
                v = Q - Q0
                sr = v % FU_RSLOTS
                if v >= FU_RSLOTS:
                    k = v // FU_RSLOTS - 1
                    while not rempty[sr].passes(k & 1, k):
                        yield
                in_flight.append(("r", sr, Q))
            yield

    def wait(bars, p, base, n):
        u = p - base
        f = u // n
        while not bars[u % n].passes(f & 1, f):
            yield

    def consumers():
        yield from wait(efull, P0, P0, FU_ESLOTS)
        yield from wait(efull, P0 + 1, P0, FU_ESLOTS)
        for q in range(i0 - 1, i1 + 1):
            yield from wait(efull, q + 1, P0, FU_ESLOTS)
            yield from wait(rfull, q, Q0, FU_RSLOTS)
            # R(q)
            assert [etag[eslot(x)] for x in (q - 1, q, q + 1)] == [q - 1, q, q + 1] and rtag[rslot(q)] == q
            yield
            # barrier, then the store of plane q-2 and the releases
            if q - 2 >= i0:
                stores.append((eslot(q - 2), q - 2))
            if q - 3 >= P0:
                if q - 3 >= i0 and not early_release:
                    while any(pl == q - 3 for _, pl in stores):  # cp.async.bulk.wait_group.read 1
                        yield
                eempty[eslot(q - 3)].arrive()
            if q - 2 >= Q0:
                rempty[rslot(q - 2)].arrive()
            # K(q-1)
            p = q - 1
            if p >= i0:
                assert [etag[eslot(x)] for x in (p - 1, p, p + 1)] == [p - 1, p, p + 1] and rtag[rslot(p)] == p
            yield
        # the last plane's store; the block waits for every store to finish
        stores.append((eslot(i1 - 1), i1 - 1))
        while stores:
            yield

    tasks = [producer(), consumers()]
    alive = list(tasks)
    steps = 0
    while alive or in_flight or stores:
        steps += 1
        assert steps < 200000, "deadlock"
        r = rng.random()
        if in_flight and (not alive or r < 0.3):
            kind, s, plane = in_flight.pop(rng.randrange(len(in_flight)))
            if kind == "e":
                etag[s] = plane
                efull[s].arrive()
            else:
                rtag[s] = plane
                rfull[s].arrive()
            continue
        if stores and r < 0.5:
            slot, plane = stores.pop(rng.randrange(len(stores)))
            assert etag[slot] == plane, "a store read a refilled slot"
            continue
        if not alive:
            continue
        t = rng.choice(alive)
        try:
            next(t)
        except StopIteration:
            alive.remove(t)


@pytest.mark.parametrize("chunk", [1, 2, 3, 8, 29, 64])
def test_fused_ring_protocol(chunk):
    for seed in range(30):
        emulate_fused(seed % 4, seed % 4 + chunk, seed=500 * chunk + seed)


def test_fused_emulation_catches_an_early_release():
    """The emulation itself: releasing e(q-3) without waiting for its store
    to have read the slot lets the producer refill it under the store."""
    with pytest.raises(AssertionError):
        for seed in range(200):
            emulate_fused(0, 29, seed=seed, early_release=True)
