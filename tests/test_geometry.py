"""Host geometry against the reference's Createblock / Bounce_back (CPU)."""
import numpy as np
import pytest

from fixtures import circle_lists, corner_dicts, load
from fingering_dynamics_gb300 import geometry as geo


def test_circle_outline_symmetric_and_connected():
    for r in range(0, 20):
        pts = {tuple(p) for p in geo.circle_outline(0, 0, r)}
        for x, y in list(pts):
            assert (-x, y) in pts and (x, -y) in pts and (y, x) in pts
        if r >= 1:
            # 8-connected closed curve: every point has exactly two 8-neighbours
            for x, y in pts:
                n = sum((x + dx, y + dy) in pts for dx in (-1, 0, 1) for dy in (-1, 0, 1) if dx or dy)
                assert n >= 2


def test_createblock_matches_reference():
    fx = load("geometry_masks")
    H, W = int(fx["H"]), int(fx["W"])
    cb = geo.Createblock(H, W)
    circles = [((int(c[0]), int(c[1])), int(c[2])) for c in fx["circles"]]
    rects = [((int(r[0]), int(r[1])), (int(r[2]), int(r[3]))) for r in fx["rects"]]
    bpa, side, conc, vex = cb.setCirleblock(circles)
    assert np.array_equal(bpa, fx["bpa_circles"])
    for got, ref in zip(side + conc + vex, fx["circle_masks"]):
        assert np.array_equal(got, ref)
    bpa_r, corners = cb.setblock(rects)
    assert np.array_equal(bpa_r, fx["bpa_rects"])
    assert corners == corner_dicts(fx["corners"])


def test_link_bits_reproduce_reference_bounce_back():
    """Applying the packed link bits must equal the reference's mask-by-mask
    bounce-back (restated in the oracle) on random populations."""
    from oracle import lbm_oracle as O
    fx = load("geometry_masks")
    H, W = int(fx["H"]), int(fx["W"])
    side, conc, vex = circle_lists(fx["circle_masks"])
    corners = corner_dicts(fx["corners"])
    bits = (geo.circle_link_bits(side, conc, vex) | geo.rect_link_bits(corners, H, W)
            | geo.wall_row_link_bits(H, W))
    rng = np.random.default_rng(5)
    fb = rng.standard_normal((9, H, W)); gb = rng.standard_normal((9, H, W))
    f = rng.standard_normal((9, H, W)); g = rng.standard_normal((9, H, W))
    f_ref, g_ref = f.copy(), g.copy()
    O.halfway_bounceback_circle(side, conc, vex, fb, gb, f_ref, g_ref)
    O.halfway_bounceback_rec(corners, fb, gb, f_ref, g_ref)
    O.bottom_top_wall(fb[:, 1:-1], gb[:, 1:-1], f_ref[:, 1:-1], g_ref[:, 1:-1])
    f_bits, g_bits = f.copy(), g.copy()
    for i in range(1, 9):
        m = ((bits >> (i - 1)) & 1).astype(bool)
        f_bits[i][m] = fb[geo.OPPOSITE[i]][m]
        g_bits[i][m] = gb[geo.OPPOSITE[i]][m]
    assert np.array_equal(f_bits, f_ref) and np.array_equal(g_bits, g_ref)


@pytest.mark.parametrize("name", ["periodic_circles_24x48", "walls_rects_24x48"])
def test_build_geometry_matches_fixture(name):
    fx = load(name)
    H, W = int(fx["H"]), int(fx["W"])
    rects = [((int(r[0]), int(r[1])), (int(r[2]), int(r[3]))) for r in fx["rects"]]
    circles = [((int(c[0]), int(c[1])), int(c[2])) for c in fx["circles"]]
    g = geo.build_geometry(H, W, rects=rects, circles=circles, walls=str(fx["variant"]) == "walls")
    assert np.array_equal(g.block_psi_all, fx["block_psi_all"])
    assert np.array_equal(g.solid, fx["block_psi_all"] == 1)
    assert np.array_equal((g.mask_word & geo.SOLID_BIT) != 0, g.solid)


def test_random_blocks_seeded_and_porosity():
    r1 = geo.random_blocks(256, 512, 0.75, 6, 14, seed=3)
    r2 = geo.random_blocks(256, 512, 0.75, 6, 14, seed=3)
    assert r1 == r2
    g = geo.build_geometry(256, 512, rects=r1[0], circles=r1[1], walls=True)
    assert 0.70 < g.porosity < 0.80
    # blocks never overlap, so every solid cell is covered exactly once
    assert g.block_psi_all.max() == 1
