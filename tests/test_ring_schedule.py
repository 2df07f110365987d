"""Host model of the copy schedule of the FP32 staged kernel's split ring
(tma_strip_split in fingering_dynamics_gb300/csrc/fd_fused_tma.cuh), no GPU.

The kernel keeps four slots; the g half of ring row r (g_0, the g_i planes
and the mask row, the mask into a 6-row mask ring) and its f half complete
on separate mbarriers (0..3 g, 4..7 f).  The model replays, in program order,
the prologue and the per-row loop: fills issued by the copy thread after each
CTA barrier, waits with the parity bit of the next fill, and every read of a
slot or mask row.  It checks, for every strip height and for consecutive
strips of the persistent batch kernel (phases carried over), that each wait
returns the fill it expects with the right parity, that no slot half or mask
row is refilled while a later read still needs it, and that every issued fill
is waited for before the strip ends.
"""
import pytest


MASK_ROWS = 6  # TmaSmem<float, NT, 4>::MASK_ROWS


def run_strips(strips, mistake=None, mask_rows=MASK_ROWS):
    phase = 0
    fills = {b: [] for b in range(8)}
    waited = {b: 0 for b in range(8)}
    for y0, y1 in strips:
        first, last = y0 - 2, y1 + 1
        g_slot, f_slot, m_row, done_g, done_f = {}, {}, {}, set(), set()

        def issue_g(r):
            if r > last:
                return
            b = (r - first) & 3
            fills[b].append(("g", r))
            g_slot[b] = r
            m_row[(r - first) % mask_rows] = r

        def issue_f(r):
            if r > y1:
                return
            b = 4 + ((r - first) & 3)
            fills[b].append(("f", r))
            f_slot[b - 4] = r

        def wait(b, kind, r):
            nonlocal phase
            n = waited[b]
            assert fills[b][n] == (kind, r), (b, fills[b][n], kind, r)
            assert ((phase >> b) & 1) == (n & 1)
            phase ^= 1 << b
            waited[b] += 1
            (done_g if kind == "g" else done_f).add(r)

        def wait_g(r):
            wait((r - first) & 3, "g", r)

        def wait_f(r):
            wait(4 + ((r - first) & 3), "f", r)

        def read_g(r):
            assert g_slot[(r - first) & 3] == r and r in done_g, ("g", r)

        def read_f(r):
            assert f_slot[(r - first) & 3] == r and r in done_f, ("f", r)

        def read_mask(r):
            assert m_row[(r - first) % mask_rows] == r and r in done_g, ("mask", r)

        def psi_of(r):  # psi of row r: g of rows r-1 .. r+1, mask of row r
            for k in (r - 1, r, r + 1):
                read_g(k)
            read_mask(r)

        for r in range(first, first + 4):
            issue_g(r)
        for r in range(y0 - 1, y0 + 3):
            issue_f(r)
        wait_g(y0 - 2), wait_g(y0 - 1), wait_g(y0)
        psi_of(y0 - 1)
        issue_g(y0 + 2)  # after a CTA barrier
        wait_g(y0 + 1)
        psi_of(y0)
        issue_g(y0 + 3)  # after a CTA barrier
        wait_f(y0 - 1), wait_f(y0)
        for y in range(y0, y1):
            wait_g(y + 2)
            psi_of(y + 1)
            issue_g(y + 4 if mistake != "g_fill_one_row_early" else y + 5)  # after the row's CTA barrier
            if y > y0:
                issue_f(y + 2 if mistake != "f_fill_one_row_early" else y + 3)
            if mistake != "f_wait_after_the_pull":
                wait_f(y + 1)
            for k in (y - 1, y, y + 1):  # the f pull of row y
                read_f(k)
            read_mask(y)
            if mistake == "f_wait_after_the_pull":
                wait_f(y + 1)
        for b in range(8):
            assert waited[b] == len(fills[b]), (b, waited[b], len(fills[b]))


@pytest.mark.parametrize("H", [1, 2, 3, 4, 5, 7, 8, 16, 33, 64])
def test_split_ring_schedule(H):
    for R in range(1, H + 2):
        strips = [(y0, min(y0 + R, H)) for y0 in range(0, H, R)]
        run_strips(strips)
        run_strips(strips[::-1] + strips)  # a persistent CTA taking several strips in a row


@pytest.mark.parametrize("mistake", ["f_wait_after_the_pull", "g_fill_one_row_early", "f_fill_one_row_early",
                                     "mask_ring_of_4_rows"])
def test_model_catches_planted_mistakes(mistake):
    """The model is not vacuous: each schedule mistake planted in it (a wait
    moved after the reads it guards, a fill issued one row early into a slot
    still being read, a mask ring too short for the rows in flight) fails on
    some strip."""
    rows = 4 if mistake == "mask_ring_of_4_rows" else MASK_ROWS
    with pytest.raises((AssertionError, KeyError, IndexError)):
        for H in (8, 16, 33):
            for R in range(1, H + 1):
                run_strips([(y0, min(y0 + R, H)) for y0 in range(0, H, R)], mistake, mask_rows=rows)
