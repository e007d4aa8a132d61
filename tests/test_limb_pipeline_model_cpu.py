"""A CPU model of the mbarrier protocol of limb_gemm_kernel
(inspire_gb300/csrc/limb_gemm.cu), run under seeded random interleavings.

The model follows the kernel's roles and waits one for one: the TMA producer
(one thread), the MMA issuer (one thread, its tcgen05 commits landing in
issue order), the converter warps of the converting forms (four, two per box
pair) and the epilogue warps (four per row block), over the two row blocks,
two box pairs per row block, three request slots and, in the staged
converting form (narrow request tiles), a ring of raw-tile staging slots.
Barriers follow PTX mbarrier semantics: a phase completes when its expected
arrivals and transaction bytes are all in, and a parity wait passes while
the barrier's current phase has the other parity, so it cannot tell phases
two apart.

Every box, staging slot, request slot and accumulator records what was last
written to it and what its reader last finished with, and the model checks
that nothing is read before it is written or overwritten before it is
freed, that every role runs to its end, and that the producer's drain
leaves no copy in flight when it exits. Two orderings of the staged
form are checked both ways: its converter warps wait for the freed box
before the raw tile (the other order reads stale tiles once copies land out
of order), and its producer waits on the converter warps before the first
pack-unit box (needed once the request ring is deeper than three slots).
"""
import random

import pytest


class Violation(Exception):
    pass


class Deadlock(Exception):
    pass


class Bar:
    """An mbarrier: `count` arrivals and the expected transaction units."""

    def __init__(self, name, count):
        self.name, self.count = name, count
        self.pending, self.tx, self.phase = count, 0, 0

    def arrive(self):
        if self.pending == 0:
            raise Violation("%s: an arrival beyond the phase's count" % self.name)
        self.pending -= 1
        self._complete()

    def expect_tx(self, n):
        self.tx += n
        self.arrive()

    def complete_tx(self, n):
        self.tx -= n
        self._complete()

    def _complete(self):
        if self.pending == 0 and self.tx == 0:
            self.phase += 1
            self.pending = self.count

    def passed(self, parity):
        return (self.phase & 1) != parity


ROW_BLOCKS, PAIRS = 2, 2


class Kernel:
    """One CTA's pipeline over `n_db` DB units followed by `n_pk` pack units.

    form: "planes" (digit planes loaded by TMA), "inplace" (full request
    tiles: raw u16 tiles land in their own box and are converted there) or
    "staged" (narrow tiles: raw tiles go through `stages` staging slots).
    """

    def __init__(self, form, n_db, n_pk, stages=9, conv_done=True, b_slots=3,
                 box_first=True, lenient=False):
        self.form, self.n_db, self.nu = form, n_db, n_db + n_pk
        # lenient: record stale reads and early overwrites in `log` and go
        # on, to see where they lead.
        self.lenient, self.log = lenient, []
        self.conv = form != "planes"
        self.staged = form == "staged"
        self.use_conv_done = conv_done
        self.box_first = box_first  # staged converter: box wait, then tile wait
        self.ns = stages
        self.nb = b_slots
        nslot = ROW_BLOCKS * PAIRS
        self.a_full = [Bar("a_full%d" % s, 2 if self.conv else 1) for s in range(nslot)]
        self.a_empty = [Bar("a_empty%d" % s, 1) for s in range(nslot)]
        self.b_full = [Bar("b_full%d" % s, 1) for s in range(b_slots)]
        self.b_empty = [Bar("b_empty%d" % s, 1) for s in range(b_slots)]
        self.acc_full = [Bar("acc_full%d" % e, 1) for e in range(ROW_BLOCKS)]
        self.acc_empty = [Bar("acc_empty%d" % e, 4) for e in range(ROW_BLOCKS)]
        nst = self.ns if self.staged else nslot
        self.st_full = [Bar("st_full%d" % j, 1) for j in range(nst)]
        self.st_empty = [Bar("st_empty%d" % j, 1) for j in range(nst)]
        self.conv_done = Bar("conv_done", 4)
        # State: box (slot, half) -> (what, unit); last unit the MMA pipe
        # freed per slot; staging slot contents and last read; request slot
        # contents and last freed; accumulator contents and reads.
        self.box = {}
        self.freed = [-1] * nslot
        self.stage = [None] * nst
        self.stage_read = [-1] * nst
        self.bslot = [None] * b_slots
        self.b_freed = [-1] * b_slots
        self.acc = [None] * ROW_BLOCKS
        self.acc_reads = [dict() for _ in range(ROW_BLOCKS)]
        self.tma = []      # copies in flight: completions in any order
        self.commits = []  # tcgen05 commits: land in issue order

    # ---- checks ------------------------------------------------------
    def fail(self, msg):
        if not self.lenient:
            raise Violation(msg)
        self.log.append(msg)

    def box_free(self, s, i):
        if self.freed[s] < i - 1:
            self.fail("box pair %d overwritten for unit %d while unit %d "
                      "is not freed" % (s, i, self.freed[s] + 1))

    def box_ready(self, s, i):
        for h in (0, 1):
            if self.box.get((s, h)) != ("A", i):
                self.fail("MMA read box (%d, %d) for unit %d holding %r"
                          % (s, h, i, self.box.get((s, h))))

    # ---- roles -------------------------------------------------------
    def producer(self):
        seq = 0
        conv_seen = False
        nslot = ROW_BLOCKS * PAIRS
        a_last, a_raw = [-1] * nslot, [False] * nslot
        b_last = [-1] * self.nb
        st_last = [-1] * self.ns

        def load_pair(rb, p, i):
            nonlocal seq, conv_seen
            s = rb * PAIRS + p
            db = i < self.n_db
            if self.staged and db:
                for hh in range(2):
                    j = seq % self.ns
                    yield (self.st_empty[j], ((seq // self.ns) & 1) ^ 1)
                    if self.stage_read[j] != seq - self.ns and seq >= self.ns:
                        self.fail("staging slot %d overwritten by tile %d "
                                  "before tile %d was read" % (j, seq, seq - self.ns))
                    self.st_full[j].expect_tx(1)
                    self.tma.append(("stage", j, seq))
                    st_last[j] = seq
                    seq += 1
                return
            if self.staged and self.use_conv_done and not conv_seen:
                yield (self.conv_done, 0)
                conv_seen = True
            yield (self.a_empty[s], (i & 1) ^ 1)
            self.box_free(s, i)
            if self.conv and db:  # in place: raw tiles into the boxes
                self.st_full[s].expect_tx(2)
                for h in (0, 1):
                    self.tma.append(("raw", s, h, i))
                a_last[s], a_raw[s] = i, True
                return
            if self.conv:
                self.a_full[s].arrive()
            self.a_full[s].expect_tx(2)
            for h in (0, 1):
                self.tma.append(("box", s, h, i))
            a_last[s], a_raw[s] = i, False

        for i in range(self.nu):
            for p in range(PAIRS):
                yield from load_pair(0, p, i)
            for p in range(PAIRS):
                n = 2 * i + p
                slot = n % self.nb
                yield (self.b_empty[slot], ((n // self.nb) & 1) ^ 1)
                if self.b_freed[slot] < n - self.nb:
                    raise Violation("request slot %d overwritten by %d" % (slot, n))
                self.b_full[slot].expect_tx(1)
                self.tma.append(("b", slot, n))
                b_last[slot] = n
                yield from load_pair(1, p, i)
        # Drain: every copy this thread issued has landed before it exits.
        for s in range(nslot):
            if a_last[s] >= 0:
                yield ((self.st_full if a_raw[s] else self.a_full)[s], a_last[s] & 1)
        for slot in range(self.nb):
            if b_last[slot] >= 0:
                yield (self.b_full[slot], (b_last[slot] // self.nb) & 1)
        for j in range(self.ns if self.staged else 0):
            if st_last[j] >= 0:
                yield (self.st_full[j], (st_last[j] // self.ns) & 1)
        if self.tma:
            raise Violation("producer exits with %d copies in flight" % len(self.tma))

    def converter(self, cw):
        p, h = cw >> 1, cw & 1
        for i in range(self.nu):
            if i >= self.n_db:
                break
            for rb in range(ROW_BLOCKS):
                s = rb * PAIRS + p
                if self.staged:
                    sq = 8 * i + 4 * rb + cw
                    j = sq % self.ns
                    if self.box_first:
                        yield (self.a_empty[s], (i & 1) ^ 1)
                        yield (self.st_full[j], (sq // self.ns) & 1)
                    else:
                        yield (self.st_full[j], (sq // self.ns) & 1)
                        yield (self.a_empty[s], (i & 1) ^ 1)
                    if self.stage[j] != sq:
                        self.fail("converter read staging slot %d for tile "
                                  "%d holding %r" % (j, sq, self.stage[j]))
                    self.stage_read[j] = sq
                    self.st_empty[j].arrive()
                    self.box_free(s, i)
                else:
                    yield (self.st_full[s], i & 1)
                    if self.box.get((s, h)) != ("raw", i):
                        self.fail("converter read box (%d, %d) for unit %d "
                                  "holding %r" % (s, h, i, self.box.get((s, h))))
                yield None
                self.box[(s, h)] = ("A", i)
                self.a_full[s].arrive()
        if self.staged:
            self.conv_done.arrive()

    def mma(self):
        for i in range(self.nu):
            for rb in range(ROW_BLOCKS):
                yield (self.acc_empty[rb], (i & 1) ^ 1)
                if i > 0 and self.acc_reads[rb].get(i - 1, 0) != 4:
                    raise Violation("accumulator %d rewritten before unit %d was "
                                    "read" % (rb, i - 1))
                for p in range(PAIRS):
                    n = 2 * i + p
                    slot = n % self.nb
                    if rb == 0:
                        yield (self.b_full[slot], (n // self.nb) & 1)
                        if self.bslot[slot] != n:
                            raise Violation("MMA read request slot %d for %d holding %r"
                                            % (slot, n, self.bslot[slot]))
                    s = rb * PAIRS + p
                    yield (self.a_full[s], i & 1)
                    self.box_ready(s, i)
                    self.commits.append(("a", s, i))
                    if rb == ROW_BLOCKS - 1:
                        self.commits.append(("b", slot, n))
                self.commits.append(("acc", rb, i))

    def epilogue(self, e):
        for i in range(self.nu):
            yield (self.acc_full[e], i & 1)
            if self.acc[e] != i:
                raise Violation("epilogue read accumulator %d for unit %d holding %r"
                                % (e, i, self.acc[e]))
            self.acc_reads[e][i] = self.acc_reads[e].get(i, 0) + 1
            self.acc_empty[e].arrive()

    # ---- asynchronous completions ------------------------------------
    def land(self, ev):
        kind = ev[0]
        if kind == "stage":
            _, j, seq = ev
            self.stage[j] = seq
            self.st_full[j].complete_tx(1)
        elif kind == "raw":
            _, s, h, i = ev
            self.box[(s, h)] = ("raw", i)
            self.st_full[s].complete_tx(1)
        elif kind == "box":
            _, s, h, i = ev
            self.box[(s, h)] = ("A", i)
            self.a_full[s].complete_tx(1)
        else:
            _, slot, n = ev
            self.bslot[slot] = n
            self.b_full[slot].complete_tx(1)

    def commit(self, ev):
        kind, x, i = ev
        if kind == "a":
            self.freed[x] = i
            self.a_empty[x].arrive()
        elif kind == "b":
            self.b_freed[x] = i
            self.b_empty[x].arrive()
        else:
            self.acc[x] = i
            self.acc_full[x].arrive()


def simulate(kernel, seed):
    """Runs every role to its end under a schedule drawn from `seed`;
    raises Violation or Deadlock. The seed also draws how fast each role,
    the copies and the MMA pipe's commits move relative to one another, and
    how far the oldest copy in flight may lag the younger ones (copies land
    in any order)."""
    rng = random.Random(seed)
    speed = {"producer": 1.0, "converter": rng.choice([0.2, 1.0, 5.0]),
             "mma": rng.choice([0.02, 0.1, 1.0]), "epilogue": rng.choice([0.02, 0.1, 1.0]),
             "tma": rng.choice([0.2, 1.0, 5.0]), "commit": rng.choice([0.01, 0.05, 0.3, 1.0]),
             "oldest": rng.choice([1.0, 0.1, 0.01])}
    roles = {kernel.producer(): "producer", kernel.mma(): "mma"}
    for e in range(ROW_BLOCKS):
        for _ in range(4):
            roles[kernel.epilogue(e)] = "epilogue"
    if kernel.conv:
        for cw in range(4):
            roles[kernel.converter(cw)] = "converter"
    waits = {r: None for r in roles}
    live = list(roles)
    while live or kernel.tma or kernel.commits:
        choices = [("role", r, speed[roles[r]]) for r in live
                   if waits[r] is None or waits[r][0].passed(waits[r][1])]
        choices += [("tma", k, speed["tma"] * (speed["oldest"] if k == 0 else 1.0))
                    for k in range(len(kernel.tma))]
        if kernel.commits:
            choices.append(("commit", 0, speed["commit"]))
        if not choices:
            raise Deadlock("blocked on %s" % [(waits[r][0].name, waits[r][1])
                                              for r in live if waits[r] is not None])
        x = rng.random() * sum(c[2] for c in choices)
        for kind, what, weight in choices:
            x -= weight
            if x <= 0:
                break
        if kind == "role":
            try:
                waits[what] = next(what)
            except StopIteration:
                live.remove(what)
        elif kind == "tma":
            kernel.land(kernel.tma.pop(what))
        else:
            kernel.commit(kernel.commits.pop(0))


def violations(make, seeds):
    """Violation messages over `seeds` schedules of kernels made by
    make(rng); a deadlock fails the test."""
    found = []
    for seed in range(seeds):
        k = make(random.Random(10_000 + seed))
        try:
            simulate(k, seed)
        except Violation as e:
            found.append(str(e))
    return found


@pytest.mark.parametrize("form,stages", [("planes", 9), ("inplace", 9), ("staged", 4),
                                         ("staged", 8), ("staged", 9)])
def test_pipeline_protocol_holds(form, stages):
    """The kernel's protocol: no read before a write, no overwrite before a
    release, no deadlock, for CTAs of 0-4 DB units and 0-3 pack units."""
    def make(rng):
        n_db, n_pk = rng.choice([0, 1, 2, 4]), rng.choice([0, 1, 3])
        return Kernel(form, n_db, n_pk or (0 if n_db else 1), stages=stages)
    assert violations(make, 600) == []


def test_staged_converter_waits_for_the_box_before_the_tile():
    """With nine staging slots a slot's consecutive tiles belong to
    different converter warps. Waiting for the raw tile first, a warp can
    meet the slot a phase early (the previous tile not landed yet, copies
    landing out of order), pass the parity wait and read the old tile.
    Waiting for the freed box first rules it out, and so do staging slots
    in a multiple of four (each warp then owns its slots)."""
    def make(stages, box_first):
        return lambda rng: Kernel("staged", rng.choice([2, 3, 4]), rng.choice([0, 1, 2]),
                                  stages=stages, box_first=box_first)
    found = violations(make(9, False), 800)
    assert found and all("converter read staging slot" in f for f in found)
    assert violations(make(9, True), 800) == []
    assert violations(make(8, False), 800) == []


@pytest.mark.parametrize("stages", [4, 5, 6, 7, 8, 10, 12, 16])
def test_staged_ring_sizes(stages):
    """The staging ring sizes the kernel admits (a multiple of 4, or 8 and
    more) keep the converter's waits exact; 5 to 7 slots would not, in
    either wait order."""
    found = violations(lambda rng: Kernel("staged", rng.choice([2, 3, 4]),
                                          rng.choice([0, 1, 2]), stages=stages), 500)
    if stages % 4 == 0 or stages >= 8:
        assert found == []
    else:
        assert found and all("converter read staging slot" in f for f in found)


def test_staged_producer_waits_for_the_converters_before_pack_boxes():
    """The producer waits on no box during the DB units. With three request
    slots its request-slot waits keep it within a unit of the MMA pipe, so
    its first pack-box wait is exact even without the wait on the converter
    warps; with a deeper request ring it is not, and the wait on the
    converter warps is what keeps it exact."""
    def make(b_slots, conv_done):
        return lambda rng: Kernel("staged", rng.choice([2, 3, 4, 5]), rng.choice([1, 2]),
                                  stages=9, conv_done=conv_done, b_slots=b_slots)
    assert violations(make(3, False), 600) == []
    found = violations(make(6, False), 600)
    assert found and all("overwritten" in f for f in found)
    assert violations(make(6, True), 600) == []


def outcomes(make, seeds):
    """Counts of how lenient runs end: clean, with stale reads or early
    overwrites logged, with a broken barrier (an arrival beyond a phase's
    count) or stalled (every role blocked, which the kernel's bounded waits
    report as a pipeline timeout)."""
    out = {"clean": 0, "logged": 0, "broken": 0, "stalled": 0}
    for seed in range(seeds):
        k = make(random.Random(10_000 + seed))
        try:
            simulate(k, seed)
            out["logged" if k.log else "clean"] += 1
        except Deadlock:
            out["stalled"] += 1
        except Violation:
            out["broken"] += 1
    return out


def test_inexact_staging_waits_can_stall_the_pipe():
    """A six-slot staging ring (what the shared memory left for narrow
    request tiles over Z_2^64, eight digit planes a request) lets converter
    warps pass their staging waits a phase early in either wait order; the
    stale reads free slots early, and schedules end with an arrival beyond a
    barrier's count (undefined in PTX) or with every role blocked, i.e. a
    pipeline timeout. Nine slots with the box waited first run clean."""
    def make(stages, box_first):
        return lambda rng: Kernel("staged", rng.choice([2, 3, 4, 6]), rng.choice([0, 1, 2]),
                                  stages=stages, box_first=box_first, lenient=True)
    for box_first in (False, True):
        out = outcomes(make(6, box_first), 600)
        assert out["stalled"] > 0 and out["broken"] > 0
    assert outcomes(make(9, True), 600) == {"clean": 600, "logged": 0, "broken": 0,
                                            "stalled": 0}
