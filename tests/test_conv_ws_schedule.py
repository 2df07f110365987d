"""Host model of the persistent warp-specialised convolution's handshake
(k_conv3x3_tma_ws in fingering_dynamics_gb300/csrc/sg_tcgen05.cu), no GPU.

Agents, interleaved at random: the producer/MMA thread (its program order as
in the kernel: prologue fills of S chunks, then per chunk c = j * nk + kc: for
the first chunk of tile j >= 2 wait acce[j % 2], wait full[c % S], MMAs,
commit empty[c % S], after the last chunk of a tile commit accf[j % 2], then
refill the stage of chunk c - 1 once empty says its MMAs are done), the
epilogue warps (per tile: wait accf[j % 2], read the accumulators, one arrival
per warp, eight warps, on acce[j % 2]), the TMA engine (completes the boxes of a stage, in
issue order, at any time) and the tensor-core engine (completes MMAs and their
commits in issue order at any time).  mbarriers count completed phases; a
parity wait for phase i must never find the barrier two phases on (it would
then wait for a phase that is already over).  The model checks that every run
ends (no deadlock), that no wait aliases, that no stage is refilled before the
MMAs that read it are done, and that no accumulator buffer is written by a
tile's MMAs before the epilogue of the tile two earlier has read it.
"""
import random

import pytest


class Bar:
    def __init__(self, count):
        self.count, self.arrived, self.phases = count, 0, 0

    def arrive(self):
        self.arrived += 1
        assert self.arrived <= self.count
        if self.arrived == self.count:
            self.arrived, self.phases = 0, self.phases + 1


def run(tiles, nk, S, seed, mistake=None):
    rng = random.Random(seed)
    full = [Bar(1) for _ in range(S)]
    empty = [Bar(1) for _ in range(S)]
    accf = [Bar(1) for _ in range(2)]
    acce = [Bar(8) for _ in range(2)]
    tma_q, mma_q = [], []         # in-order engines: pending completions
    stage_chunk = [None] * S      # chunk whose boxes a stage holds
    stage_reads = [0] * S         # MMAs issued on a stage and not completed
    buf_tile = [None, None]       # tile whose accumulators a buffer holds
    buf_read = [True, True]       # the epilogue has read the buffer
    nc = tiles * nk

    def ready(bar, i):
        assert bar.phases <= i + 1, "parity wait would alias"
        return bar.phases > i

    def producer():
        def issue(c):
            st = c % S
            assert stage_reads[st] == 0, "stage refilled while its MMAs may read it"
            stage_chunk[st] = c
            tma_q.append(("full", st, c))
        for c in range(min(S, nc)):
            issue(c)
        for c in range(nc):
            j, kc, b, st = c // nk, c % nk, (c // nk) % 2, c % S
            if kc == 0:
                if j >= 2 and mistake != "no_acce_wait":
                    while not ready(acce[b], (j - 2) // 2):
                        yield
                assert buf_read[b] or buf_tile[b] is None, "accumulator overwritten before it was read"
                buf_tile[b], buf_read[b] = j, False
            while not ready(full[st], c // S):
                yield
            assert stage_chunk[st] == c
            stage_reads[st] += 1
            mma_q.append(("mma", st, c))
            mma_q.append(("empty", st, c))
            if kc == nk - 1:
                mma_q.append(("accf", b, j))
            if c >= 1 and c - 1 + S < nc:
                ps = (c - 1) % S
                if mistake != "refill_without_wait":
                    while not ready(empty[ps], (c - 1) // S):
                        yield
                issue(c - 1 + S)
            yield

    def epilogue():
        for j in range(tiles):
            b = j % 2
            while not ready(accf[b], j // 2):
                yield
            assert buf_tile[b] == j
            buf_read[b] = True
            for _ in range(8):  # one arrival per epilogue warp
                acce[b].arrive()
            yield

    agents = {"p": producer(), "e": epilogue()}
    done = set()
    steps = 0
    while len(done) < 2 or tma_q or mma_q:
        steps += 1
        assert steps < 100000, "no progress"
        choices = [a for a in agents if a not in done] + (["tma"] if tma_q else []) + (["mma"] if mma_q else [])
        assert choices, "deadlock"
        pick = rng.choice(choices)
        if pick == "tma":
            _, st, c = tma_q.pop(0)
            full[st].arrive()
        elif pick == "mma":
            kind, i, c = mma_q.pop(0)
            if kind == "mma":
                stage_reads[i] -= 1
            elif kind == "empty":
                empty[i].arrive()
            else:
                accf[i].arrive()
        else:
            try:
                next(agents[pick])
            except StopIteration:
                done.add(pick)
    assert all(r == 0 for r in stage_reads)


@pytest.mark.parametrize("S", [4, 5, 6])
@pytest.mark.parametrize("nk", [1, 2, 3, 24])
def test_ws_handshake(S, nk):
    for tiles in (1, 2, 3, 4, 7):
        for seed in range(25):
            run(tiles, nk, S, seed)


@pytest.mark.parametrize("mistake", ["no_acce_wait", "refill_without_wait"])
def test_model_catches_planted_mistakes(mistake):
    """Dropping the wait on acce (MMAs overwrite a buffer the epilogue has not
    read) or the wait on empty before a refill (a stage overwritten under its
    MMAs) fails on some interleaving."""
    with pytest.raises(AssertionError):
        for seed in range(200):
            run(4, 2, 4, seed, mistake)
