"""Model check of the exchange handshake of the FP32 cycle kernel
(k_cycles32 in csrc/ptmc_cycles32.cu, one CTA per run, a warp per walker).

The kernel replaces the per-cycle CTA barrier by a handshake between the two
walkers of the drawn exchange pair.  This test runs the same protocol as a
state machine under many adversarial interleavings (every shared-memory access
is a separate scheduling point; a random scheduler with skewed walker speeds
picks which walker runs next) and checks the properties the kernel relies on:

  * no deadlock: every walker finishes every cycle;
  * every record a walker reads is its partner's record of the same cycle
    (no record is overwritten before the partner has read it);
  * the slot updates at the end of a cycle (step adaptation, sampling) see the
    move counters of the walker that held the slot during the cycle;
  * the holder of every slot after every cycle, and the order of the per-slot
    updates, equal the CTA-barrier form's (parallel_tempering_exchange!,
    src/Exchange.jl:132-180, one pair attempted per cycle).

The exchange decision is a deterministic function of the two energies and the
run-level draw, as in the kernel (both walkers evaluate it with the same
inputs).
"""
import random

import pytest


def energy(w, c):
    """Deterministic stand-in for a walker's energy after the moves of cycle c."""
    return ((w * 7919 + c * 104729) % 1009) / 1009.0


def draws(R, cycles, p_exch, seed):
    """Run-level exchange draws: the pair k (or None) and the acceptance uniform."""
    rng = random.Random(seed)
    out = []
    for _ in range(cycles):
        if R > 1 and rng.random() < p_exch:
            out.append((rng.randrange(R - 1), rng.random()))
        else:
            out.append((None, 0.0))
    return out


def accept(e_lo, e_hi, u):
    """Symmetric decision from the lower slot's and the upper slot's energies."""
    return min(1.0, 2.0 ** (e_lo - e_hi)) > u


def barrier_form(R, cycles, dr):
    """The CTA-barrier schedule: holder of each slot after each cycle."""
    wos = list(range(R))  # slot -> walker
    hist = []
    for c in range(cycles):
        k, u = dr[c]
        if k is not None:
            w1, w2 = wos[k], wos[k + 1]
            if accept(energy(w1, c), energy(w2, c), u):
                wos[k], wos[k + 1] = w2, w1
        hist.append(list(wos))
    return hist


def handshake_form(R, cycles, dr, sched_seed):
    """The handshake protocol, one generator per walker; returns the per-slot
    (cycle, walker) sequence of end-of-cycle updates."""
    flag = [0] * R                # s_xflag: 2 cyc + 1 written, 2 cyc + 2 partner read
    rec = [None] * R              # s_xen / s_xbox: (energy, cycle)
    cnt = [[] for _ in range(R)]  # move counters per slot: (cycle, walker)
    epi = [[] for _ in range(R)]  # end-of-cycle slot updates: (cycle, walker)

    def walker(w):
        slot = w
        for c in range(cycles):
            yield None                        # the moves of cycle c
            e = energy(w, c)
            cnt[slot].append((c, w))          # counters of the slot the moves were made in
            yield None
            k, u = dr[c]
            if k is not None and slot in (k, k + 1):
                other = k + 1 if slot == k else k
                rec[slot] = (e, c)            # record, fence, flag
                yield None
                flag[slot] = 2 * c + 1
                yield ("wait", other, 2 * c + 1)
                yield None                    # fence, then the read: a separate access
                eo, co = rec[other]
                assert co == c, "partner record overwritten or stale"
                yield None
                flag[slot] = 2 * c + 2        # read done
                yield ("wait", other, 2 * c + 2)
                lo_side = slot == k
                if accept(e if lo_side else eo, eo if lo_side else e, u):
                    slot = other
            assert cnt[slot] and cnt[slot][-1][0] == c, "slot update before the holder's counters"
            epi[slot].append((c, w))          # adaptation + sampling of the slot held now
            yield None

    rng = random.Random(sched_seed)
    speed = [rng.choice([1, 1, 2, 5, 20]) for _ in range(R)]  # skewed: some walkers lag
    gens = [walker(w) for w in range(R)]
    waiting = [None] * R
    done = [False] * R
    while not all(done):
        ready = [w for w in range(R) if not done[w]
                 and (waiting[w] is None or flag[waiting[w][0]] >= waiting[w][1])]
        assert ready, "deadlock"
        w = rng.choices(ready, weights=[speed[v] for v in ready])[0]
        waiting[w] = None
        try:
            ev = next(gens[w])
        except StopIteration:
            done[w] = True
            continue
        if ev is not None:
            waiting[w] = (ev[1], ev[2])
    return epi


@pytest.mark.parametrize("R,p_exch", [(2, 1.0), (3, 1.0), (5, 0.7), (8, 1.0), (8, 0.3)])
def test_handshake_equals_barrier_form(R, p_exch):
    cycles = 25
    for trial in range(150):
        dr = draws(R, cycles, p_exch, 1000 * R + trial)
        ref = barrier_form(R, cycles, dr)
        epi = handshake_form(R, cycles, dr, 7 * trial + R)
        for s in range(R):
            # one update per cycle, in cycle order, by the walker the barrier form puts there
            assert [c for c, _ in epi[s]] == list(range(cycles))
            assert [w for _, w in epi[s]] == [ref[c][s] for c in range(cycles)]


def test_model_detects_a_missing_ack():
    """Without the second wait a walker leaves the exchange as soon as it has
    read its partner's record; it can then reach a later exchange in the same
    slot and overwrite its record before the slower partner has read it.  The
    model must find that race under some schedule, so the check above is not
    vacuous."""
    R, cycles = 4, 25

    def no_ack_form(dr, sched_seed):
        flag = [0] * R
        rec = [None] * R
        bad = []

        def walker(w):
            slot = w
            for c in range(cycles):
                yield None
                e = energy(w, c)
                k, u = dr[c]
                if k is not None and slot in (k, k + 1):
                    other = k + 1 if slot == k else k
                    rec[slot] = (e, c)
                    yield None
                    flag[slot] = 2 * c + 1
                    yield ("wait", other, 2 * c + 1)
                    yield None                # the read happens a step later
                    eo, co = rec[other]
                    if co != c:
                        bad.append((w, c))
                    lo_side = slot == k
                    if accept(e if lo_side else eo, eo if lo_side else e, u):
                        slot = other
                yield None

        rng = random.Random(sched_seed)
        speed = [rng.choice([1, 50]) for _ in range(R)]
        gens = [walker(w) for w in range(R)]
        waiting = [None] * R
        done = [False] * R
        while not all(done):
            ready = [w for w in range(R) if not done[w]
                     and (waiting[w] is None or flag[waiting[w][0]] >= waiting[w][1])]
            if not ready:
                return bad
            w = rng.choices(ready, weights=[speed[v] for v in ready])[0]
            waiting[w] = None
            try:
                ev = next(gens[w])
            except StopIteration:
                done[w] = True
                continue
            if ev is not None:
                waiting[w] = (ev[1], ev[2])
        return bad

    found = False
    for trial in range(200):
        if no_ack_form(draws(R, cycles, 1.0, trial), trial):
            found = True
            break
    assert found, "the model should expose the race the second wait prevents"
