"""Host model of the copy schedule of the FP32 staged kernel's split ring
(tma_strip_split in fingering_dynamics_gb300/csrc/fd_fused_tma.cuh), no GPU.

The kernel keeps four slots; the g half of ring row r (g_0, the g_i planes
and the mask row, the mask into a 6-row mask ring) and its f half complete
on separate mbarriers (0..3 g, 4..7 f).  The model replays, in program order,
the prologue and the per-row loop: fills issued by the copy thread after each
CTA barrier, waits with the parity bit of the next fill, and every read of a
slot or mask row.  It checks, for every strip height, for strips walked up
and down, and for consecutive strips of the persistent batch kernel (phases
carried over), that each wait
returns the fill it expects with the right parity, that no slot half or mask
row is refilled while a later read still needs it, and that every issued fill
is waited for before the strip ends.
"""
import pytest


MASK_ROWS = 6  # TmaSmem<float, NT, 4>::MASK_ROWS


def run_strips(strips, mistake=None, mask_rows=MASK_ROWS):
    """`strips`: (y0, y1) or (y0, y1, down) entries; a strip walked down takes
    its rows from the top (local row l is lattice row y1 - 1 - l), and every
    read checks the lattice row it needs."""
    phase = 0
    fills = {b: [] for b in range(8)}
    waited = {b: 0 for b in range(8)}
    for strip in strips:
        y0, y1 = strip[0], strip[1]
        down = len(strip) > 2 and strip[2]
        n = y1 - y0

        def lat(l):
            return y1 - 1 - l if down else y0 + l

        g_slot, f_slot, m_row, done_g, done_f = {}, {}, {}, set(), set()

        def issue_g(l):
            if l > n + 1:
                return
            b = (l + 2) & 3
            fills[b].append(("g", l))
            g_slot[b] = lat(l)
            m_row[(l + 2) % mask_rows] = lat(l)

        def issue_f(l):
            if l > n:
                return
            b = 4 + ((l + 2) & 3)
            fills[b].append(("f", l))
            f_slot[b - 4] = lat(l)

        def wait(b, kind, l):
            nonlocal phase
            k = waited[b]
            assert fills[b][k] == (kind, l), (b, fills[b][k], kind, l)
            assert ((phase >> b) & 1) == (k & 1)
            phase ^= 1 << b
            waited[b] += 1
            (done_g if kind == "g" else done_f).add(lat(l))

        def wait_g(l):
            wait((l + 2) & 3, "g", l)

        def wait_f(l):
            wait(4 + ((l + 2) & 3), "f", l)

        def rows_of(l):  # slots of the lattice rows below, at and above local row l
            return [(k + 2) & 3 for k in ((l + 1, l, l - 1) if down else (l - 1, l, l + 1))]

        def read_g(b, r):
            assert g_slot[b] == r and r in done_g, ("g", r)

        def read_f(b, r):
            assert f_slot[b] == r and r in done_f, ("f", r)

        def read_mask(l):
            assert m_row[(l + 2) % mask_rows] == lat(l) and lat(l) in done_g, ("mask", lat(l))

        def psi_of(l):  # psi of local row l: g of lattice rows y-1 .. y+1, mask of row y
            y = lat(l)
            for b, r in zip(rows_of(l), (y - 1, y, y + 1)):
                read_g(b, r)
            read_mask(l)

        for l in range(-2, 2):
            issue_g(l)
        for l in range(-1, 3):
            issue_f(l)
        wait_g(-2), wait_g(-1), wait_g(0)
        psi_of(-1)
        issue_g(2)  # after a CTA barrier
        wait_g(1)
        psi_of(0)
        issue_g(3)  # after a CTA barrier
        wait_f(-1), wait_f(0)
        for l in range(n):
            wait_g(l + 2)
            psi_of(l + 1)
            issue_g(l + 4 if mistake != "g_fill_one_row_early" else l + 5)  # after the row's CTA barrier
            if l > 0:
                issue_f(l + 2 if mistake != "f_fill_one_row_early" else l + 3)
            if mistake != "f_wait_after_the_pull":
                wait_f(l + 1)
            y = lat(l)
            for b, r in zip(rows_of(l), (y - 1, y, y + 1)):  # the f pull of lattice row y
                read_f(b, r)
            read_mask(l)
            if mistake == "f_wait_after_the_pull":
                wait_f(l + 1)
        for b in range(8):
            assert waited[b] == len(fills[b]), (b, waited[b], len(fills[b]))


@pytest.mark.parametrize("H", [1, 2, 3, 4, 5, 7, 8, 16, 33, 64])
def test_split_ring_schedule(H):
    for R in range(1, H + 2):
        strips = [(y0, min(y0 + R, H)) for y0 in range(0, H, R)]
        run_strips(strips)
        run_strips(strips[::-1] + strips)  # a persistent CTA taking several strips in a row
        # the single-lattice kernel walks odd strips down
        run_strips([(y0, y1, (y0 // R) % 2 == 1) for y0, y1 in strips])
        run_strips([(y0, y1, True) for y0, y1 in strips] + strips)


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
                run_strips([(y0, min(y0 + R, H), down) for y0 in range(0, H, R) for down in (False, True)],
                           mistake, mask_rows=rows)
