"""The barrier protocol of the tensor-core complex128 pass (k_txpipe in
quantumflow_gb300/csrc/tcfx.cu), model-checked on the CPU.

The kernel's roles -- 8 converter warps, one MMA-issuing thread, the
tensor core (in-order MMA completion), 8 epilogue warps -- are run as
agents under random interleavings, with the kernel's mbarriers (arrival
counts, phases, parity waits), its three A-operand stages, two
accumulator stages and five row-exponent slots.  Every schedule must
finish (no deadlock), no parity wait may be made on a barrier already two
phases past the awaited one (parity would then read the wrong phase), and
no stage or slot may be overwritten while a reader still needs it.  A
planted flaw -- the issuer arriving on e_ready before it waits for the
accumulators -- must be caught.
"""
import random

import pytest

AST, ESL, CW, EW = 3, 5, 8, 8  # A stages, row-exponent slots, converter and epilogue warps


class Bar:
    """mbarrier: `count` arrivals complete a phase; `phase` = phases completed."""

    def __init__(self, count):
        self.count, self.pending, self.phase = count, count, 0

    def arrive(self):
        self.pending -= 1
        if self.pending == 0:
            self.phase += 1
            self.pending = self.count

    def done(self, k, who):
        """try_wait.parity on phase k (parity k & 1)."""
        if self.phase >= k + 2:
            raise AssertionError(f"parity alias: {who} waits phase {k}, barrier at {self.phase}")
        return self.phase > k


def run(ntiles, seed, e_ready_early=False):
    rnd = random.Random(seed)
    a_full = [Bar(CW) for _ in range(AST)]     # converters -> issuer
    a_free = [Bar(1) for _ in range(AST)]      # MMA commit -> converters
    mma_done = [Bar(1) for _ in range(2)]      # MMA commit -> epilogue
    e_ready = [Bar(1) for _ in range(2)]       # issuer -> epilogue (row exponents)
    tmem_free = [Bar(EW) for _ in range(2)]    # epilogue -> issuer
    a_reading = [False] * AST                  # an MMA in flight reads the A stage
    t_tile = [None] * 2                        # tile whose accumulators a stage holds
    t_readers = [0] * 2
    e_tile, e_need = [None] * ESL, [0] * ESL   # row-exponent slot owner and pending readers
    conv = [dict(it=0, st=0) for _ in range(CW)]
    epi = [dict(it=0, st=0) for _ in range(EW)]
    iss = dict(it=0, st=0)
    tc = []
    while True:
        acts = [("c", w) for w, c in enumerate(conv) if c["it"] < ntiles]
        acts += [("e", w) for w, e in enumerate(epi) if e["it"] < ntiles]
        if iss["it"] < ntiles:
            acts.append(("i", 0))
        if tc:
            acts.append(("t", 0))
        if not acts:
            return
        rnd.shuffle(acts)
        for kind, w in acts:
            if kind == "t":                    # the tensor core finishes the oldest tile's MMAs
                it = tc.pop(0)
                a_reading[it % AST] = False
                a_free[it % AST].arrive()
                mma_done[it & 1].arrive()
                break
            if kind == "c":
                c = conv[w]
                it = c["it"]
                a, ar = it % AST, it // AST
                if c["st"] == 0:               # wait until the MMAs of tile it - 3 have read the stage
                    if ar > 0 and not a_free[a].done(ar - 1, f"conv{w}"):
                        continue
                    c["st"] = 1
                    break
                if c["st"] == 1:               # write the A stage and the row-exponent slot
                    assert not a_reading[a], f"A stage {a} overwritten under an MMA (tile {it})"
                    sl = it % ESL
                    if e_tile[sl] != it:
                        assert e_need[sl] == 0, f"row-exponent slot {sl} overwritten (tile {it})"
                        e_tile[sl], e_need[sl] = it, EW
                    c["st"] = 2
                    break
                a_full[a].arrive()
                c["it"], c["st"] = it + 1, 0
                break
            if kind == "i":
                it = iss["it"]
                a, ar, t = it % AST, it // AST, it & 1
                if iss["st"] == 0:
                    if not a_full[a].done(ar, "issuer a_full"):
                        continue
                    if e_ready_early:
                        e_ready[t].arrive()
                    iss["st"] = 1
                    break
                if it >= 2 and not tmem_free[t].done((it >> 1) - 1, "issuer tmem_free"):
                    continue
                assert t_readers[t] == 0, f"accumulators {t} overwritten under the epilogue (tile {it})"
                if not e_ready_early:
                    e_ready[t].arrive()
                t_tile[t], t_readers[t] = it, EW
                a_reading[a] = True
                tc.append(it)
                iss["it"], iss["st"] = it + 1, 0
                break
            if kind == "e":
                e = epi[w]
                it = e["it"]
                t, par = it & 1, it >> 1
                if e["st"] == 0:
                    if not e_ready[t].done(par, f"epi{w} e_ready"):
                        continue
                    if not mma_done[t].done(par, f"epi{w} mma_done"):
                        continue
                    assert t_tile[t] == it
                    assert e_tile[it % ESL] == it, "row exponent of another tile"
                    e_need[it % ESL] -= 1
                    e["st"] = 1
                    break
                t_readers[t] -= 1              # last tensor-memory read done: release
                tmem_free[t].arrive()
                e["it"], e["st"] = it + 1, 0
                break
        else:
            raise AssertionError("deadlock")


def test_protocol_random_schedules():
    for seed in range(600):
        run(random.Random(seed).randint(1, 30), seed)


def test_protocol_catches_early_e_ready():
    with pytest.raises(AssertionError, match="parity alias"):
        for seed in range(600):
            run(random.Random(seed).randint(1, 30), seed, e_ready_early=True)
