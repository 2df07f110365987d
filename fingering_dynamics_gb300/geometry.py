"""Host-side block geometry: rasterised obstacles, the reference's bounce-back
link sets, and the packed per-cell mask word the CUDA kernels read.

The reference builds its obstacles in ``lattice_boltzmann/create_block.py``
(class ``Createblock``) by drawing one-pixel outlines with OpenCV, filling them
with ``scipy.ndimage.binary_fill_holes`` and scanning the first quadrant of
each circle to classify the fluid cells next to the outline
(create_block.py:51-220, 395-407).  ``lattice_boltzmann/bounce_back.py`` then
turns those cell lists into per-direction boolean masks (bounce_back.py:25-167).

This module restates that behaviour with these choices:

* OpenCV is not available, so outlines come from this module's own integer
  rasterisers (:func:`circle_outline`, :func:`rectangle_outline`); the same
  rasteriser also backs the ``cv2`` stand-in used when the reference itself is
  run to produce test fixtures, so both sides see identical outlines.
* Each shape is rasterised in a small local window instead of a full H x W
  image per shape, so thousands of blocks on a 4096 x 2048 lattice take
  seconds.
* The twelve circle masks and eight rectangle masks are folded into one
  per-cell, per-direction *link bit*: bit ``i-1`` set means "after streaming,
  population ``i`` of this cell is replaced by the post-collision population
  ``opposite(i)`` of the same cell", which is exactly what every assignment
  in bounce_back.py does.  Several masks writing the same (cell, direction)
  write the same value, so the union is order independent.

Mask word layout (uint16 per cell, row-major (H, W)):

====== ===========================================================
bits   meaning
====== ===========================================================
0..7   bounce-back link for populations 1..8
8      solid cell (``block_psi_all == 1``, create_block.py / fingering_periodic.py:450)
====== ===========================================================
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
from scipy.ndimage import binary_fill_holes

__all__ = [
    "SOLID_BIT",
    "OPPOSITE",
    "circle_outline",
    "rectangle_outline",
    "Createblock",
    "rect_link_bits",
    "circle_link_bits",
    "wall_row_link_bits",
    "pack_mask",
    "Geometry",
    "random_blocks",
]

SOLID_BIT = 1 << 8
# D2Q9 opposite directions (fingering_periodic.py:50-89 ordering).
OPPOSITE = (0, 3, 4, 1, 2, 7, 8, 5, 6)


# ----------------------------------------------------------------------------
# rasterisers (stand-ins for cv2.circle / cv2.rectangle, thickness 1)
# ----------------------------------------------------------------------------
def circle_outline(cx: int, cy: int, r: int) -> np.ndarray:
    """Integer outline of a circle as an (N, 2) array of (x, y) points.

    Midpoint (Bresenham-type) circle: walk one octant with an integer decision
    variable and mirror it eight ways.  The outline is 8-connected and
    symmetric under x/y reflection through the centre, which the quadrant scan
    in :meth:`Createblock.setCirleblock` relies on.
    """
    r = int(r)
    if r < 0:
        raise ValueError("negative radius")
    pts = set()
    x, y, d = r, 0, 1 - r
    while x >= y:
        for px, py in ((x, y), (y, x), (-y, x), (-x, y), (-x, -y), (-y, -x), (y, -x), (x, -y)):
            pts.add((cx + px, cy + py))
        y += 1
        if d < 0:
            d += 2 * y + 1
        else:
            x -= 1
            d += 2 * (y - x) + 1
    return np.array(sorted(pts), dtype=np.int64).reshape(-1, 2)


def rectangle_outline(p0, p1) -> np.ndarray:
    """One-pixel outline of the axis-aligned box with corners p0, p1 (inclusive)."""
    x0, x1 = sorted((int(p0[0]), int(p1[0])))
    y0, y1 = sorted((int(p0[1]), int(p1[1])))
    pts = set()
    for x in range(x0, x1 + 1):
        pts.add((x, y0))
        pts.add((x, y1))
    for y in range(y0, y1 + 1):
        pts.add((x0, y))
        pts.add((x1, y))
    return np.array(sorted(pts), dtype=np.int64).reshape(-1, 2)


def _np_index(v: int, n: int) -> int:
    """Index the way numpy does for one scalar: negatives wrap once, overflow raises."""
    if -n <= v < 0:
        return v + n
    if 0 <= v < n:
        return v
    raise IndexError(f"index {v} is out of bounds for axis with size {n}")


def _points_to_mask(points, H: int, W: int) -> np.ndarray:
    m = np.zeros((H, W), dtype=bool)
    if len(points):
        p = np.asarray(points, dtype=np.int64).reshape(-1, 2)
        # numpy fancy indexing: negative wraps, overflow raises IndexError
        m[p[:, 1], p[:, 0]] = True
    return m


# ----------------------------------------------------------------------------
# Createblock restatement
# ----------------------------------------------------------------------------
class Createblock:
    """Obstacle builder with the reference's interface (create_block.py:7-407).

    ``setblock(rect_corner_list)`` returns ``(block_psi_all, corner_list)`` and
    ``setCirleblock(circle_list)`` returns ``(block_psi_all, side_list,
    concave_list, convex_list)`` with the same meanings, orderings and numpy
    indexing behaviour as the reference.  ``block_psi_all`` counts how many
    filled shapes cover a cell; only cells covered exactly once are solid
    (fingering_periodic.py:450).
    """

    def __init__(self, H: int, W: int):
        self.H = int(H)
        self.W = int(W)

    # create_block.py:39-48 (cv2.findNonZero + cv2.boundingRect)
    @staticmethod
    def getCorner(outline_points: np.ndarray) -> dict:
        xs, ys = outline_points[:, 0], outline_points[:, 1]
        x, y = int(xs.min()), int(ys.min())
        w, h = int(xs.max()) - x + 1, int(ys.max()) - y + 1
        return {
            "top_left": (x, y + h - 1),
            "bottom_left": (x, y),
            "top_right": (x + w - 1, y + h - 1),
            "bottom_right": (x + w - 1, y),
        }

    def _check_inside(self, pts: np.ndarray, what: str):
        if pts.size and (pts[:, 0].min() < 0 or pts[:, 1].min() < 0
                         or pts[:, 0].max() >= self.W or pts[:, 1].max() >= self.H):
            raise ValueError(f"{what} outline leaves the {self.H}x{self.W} lattice")

    # create_block.py:395-407
    def setblock(self, rect_corner_list):
        block_psi_all = np.zeros((self.H, self.W), dtype=np.int64)
        corner_list = []
        for p0, p1 in rect_corner_list:
            pts = rectangle_outline(p0, p1)
            self._check_inside(pts, "rectangle")
            c = self.getCorner(pts)
            corner_list.append(c)
            x0, y0 = c["bottom_left"]
            x1, y1 = c["top_right"]
            # a filled rectangle outline is the inclusive box
            block_psi_all[y0:y1 + 1, x0:x1 + 1] += 1
        return block_psi_all, corner_list

    # create_block.py:51-220
    def setCirleblock(self, circle_list):
        H, W = self.H, self.W
        block_psi_all = np.zeros((H, W), dtype=np.int64)
        side_top, side_bottom, side_left, side_right = [], [], [], []
        cave_tr, cave_tl, cave_br, cave_bl = [], [], [], []
        vex_tr, vex_tl, vex_br, vex_bl = [], [], [], []
        for (cx, cy), r in circle_list:
            cx, cy, r = int(cx), int(cy), int(r)
            pts = circle_outline(cx, cy, r)
            self._check_inside(pts, "circle")
            # local window big enough for the outline and for the quadrant
            # scan below, which can reach x + 2r + 2 in the worst case
            R = 2 * r + 4
            ox, oy = cx - R, cy - R
            win = np.zeros((2 * R + 1, 2 * R + 1), dtype=bool)
            win[pts[:, 1] - oy, pts[:, 0] - ox] = True
            filled = binary_fill_holes(win)
            fy, fx = np.nonzero(filled)
            gy, gx = fy + oy, fx + ox
            block_psi_all[gy, gx] += 1

            def outline(xg, yg):
                # the reference indexes its full-size outline image here;
                # points past the top/right edge raise IndexError there
                if xg >= W or yg >= H:
                    raise IndexError(f"circle scan at ({xg},{yg}) leaves the lattice")
                return bool(win[yg - oy, xg - ox])

            st, sl, ctr, vtr = [], [], [], []
            jj = r
            for i in range(1, r + 2):
                for j in range(jj, 0, -1):
                    if outline(cx + j, cy + i):
                        jj = j + 1
                        break
                    fb = outline(cx + j, cy + i - 1)
                    fl = outline(cx + j - 1, cy + i)
                    flb = outline(cx + j - 1, cy + i - 1)
                    if fl and fb:
                        ctr.append((cx + j, cy + i))
                    elif fl:
                        sl.append((cx + j, cy + i))
                    elif fb:
                        st.append((cx + j, cy + i))
                    elif flb:
                        vtr.append((cx + j, cy + i))
            # mirror the first quadrant (create_block.py:114-152)
            for tx, ty in st:
                side_top.append((2 * cx - tx, ty))
                side_bottom.append((tx, 2 * cy - ty))
                side_bottom.append((2 * cx - tx, 2 * cy - ty))
            side_top.append((cx, cy + r + 1))
            side_top.extend(st)
            side_bottom.append((cx, cy - r - 1))
            for lx, ly in sl:
                side_right.append((2 * cx - lx, ly))
                side_left.append((lx, 2 * cy - ly))
                side_right.append((2 * cx - lx, 2 * cy - ly))
            side_left.extend(sl)
            side_left.append((cx + r + 1, cy))
            side_right.append((cx - r - 1, cy))
            for qx, qy in ctr:
                cave_tl.append((2 * cx - qx, qy))
                cave_br.append((qx, 2 * cy - qy))
                cave_bl.append((2 * cx - qx, 2 * cy - qy))
            cave_tr.extend(ctr)
            for vx, vy in vtr:
                vex_tl.append((2 * cx - vx, vy))
                vex_br.append((vx, 2 * cy - vy))
                vex_bl.append((2 * cx - vx, 2 * cy - vy))
            vex_tr.extend(vtr)

        m = lambda pts: _points_to_mask(pts, H, W)  # noqa: E731
        concave_list = [m(cave_tr), m(cave_tl), m(cave_br), m(cave_bl)]
        side_list = [m(side_top), m(side_bottom), m(side_right), m(side_left)]
        convex_list = [m(vex_tr), m(vex_tl), m(vex_br), m(vex_bl)]
        return block_psi_all, side_list, concave_list, convex_list


# ----------------------------------------------------------------------------
# link bits
# ----------------------------------------------------------------------------
def rect_link_bits(corner_list, H: int, W: int) -> np.ndarray:
    """Per-direction bounce-back links of ``halfway_bounceback_rec``
    (bounce_back.py:25-86) as a uint16 word per cell (bits 0..7 = dirs 1..8).

    The barrier and corner masks are built with numpy slicing exactly as the
    reference does, so wrap-around at negative indices and IndexError at
    overflow behave the same.
    """
    n = np.zeros((H, W), bool); s = np.zeros((H, W), bool)
    e = np.zeros((H, W), bool); w = np.zeros((H, W), bool)
    nw = np.zeros((H, W), bool); ne = np.zeros((H, W), bool)
    sw = np.zeros((H, W), bool); se = np.zeros((H, W), bool)
    for c in corner_list:
        tlx, tly = c["top_left"]
        blx, bly = c["bottom_left"]
        trx, _ = c["top_right"]
        brx, _ = c["bottom_right"]
        n[tly + 1, tlx:trx + 1] = True
        s[bly - 1, tlx:trx + 1] = True
        w[bly:tly + 1, tlx - 1] = True
        e[bly:tly + 1, trx + 1] = True
        nw[tly + 1, tlx - 1] = True
        ne[tly + 1, trx + 1] = True
        sw[bly - 1, blx - 1] = True
        se[bly - 1, brx + 1] = True
    per_dir = {
        1: e, 2: n, 3: w, 4: s,
        5: ne | n | e, 6: nw | n | w, 7: sw | s | w, 8: se | s | e,
    }
    return _fold(per_dir, H, W)


def circle_link_bits(side_list, concave_list, convex_list) -> np.ndarray:
    """Per-direction links of ``halfway_bounceback_circle`` (bounce_back.py:89-167)."""
    sd, cc, vx = side_list, concave_list, convex_list
    H, W = sd[0].shape
    per_dir = {
        1: sd[3] | cc[0] | cc[2],
        2: sd[0] | cc[0] | cc[1],
        3: sd[2] | cc[1] | cc[3],
        4: sd[1] | cc[2] | cc[3],
        5: vx[0] | cc[0] | sd[0] | sd[3],
        6: vx[1] | cc[1] | sd[0] | sd[2],
        7: vx[3] | cc[3] | sd[1] | sd[2],
        8: vx[2] | cc[2] | sd[1] | sd[3],
    }
    return _fold(per_dir, H, W)


def wall_row_link_bits(H: int, W: int) -> np.ndarray:
    """Links of ``bottom_top_wall`` as called by the walled driver.

    fingering.py:573 passes ``f[:, 1:-1]`` for a (9, H, W) array, which slices
    the *row* axis, so inside fingering.py:432-451 row ``0`` is lattice row 1
    and row ``-1`` is lattice row H-2: populations 2, 5, 6 bounce on row 1 and
    4, 7, 8 on row H-2, across every column.
    """
    per_dir = {d: np.zeros((H, W), bool) for d in range(1, 9)}
    if H >= 3:
        for d in (2, 5, 6):
            per_dir[d][1, :] = True
        for d in (4, 7, 8):
            per_dir[d][H - 2, :] = True
    return _fold(per_dir, H, W)


def _fold(per_dir, H, W) -> np.ndarray:
    out = np.zeros((H, W), dtype=np.uint16)
    for d, m in per_dir.items():
        out |= (m.astype(np.uint16) << (d - 1))
    return out


def pack_mask(solid: np.ndarray, *link_bit_arrays) -> np.ndarray:
    """Combine a solid flag array and any number of link-bit arrays into the
    uint16 mask word the kernels read."""
    out = np.where(np.asarray(solid, bool), SOLID_BIT, 0).astype(np.uint16)
    for lb in link_bit_arrays:
        out |= np.asarray(lb, np.uint16) & 0xFF
    return out


# ----------------------------------------------------------------------------
# assembled geometry + seeded generators
# ----------------------------------------------------------------------------
@dataclass
class Geometry:
    """A complete obstacle description for one lattice.

    ``solid`` is True where ``block_psi_all == 1``; ``mask_word`` is the packed
    uint16 array (H, W) consumed by the kernels; the reference-format lists are
    kept so the oracle can apply bounce-back the reference's way.
    """
    H: int
    W: int
    block_psi_all: np.ndarray
    solid: np.ndarray
    mask_word: np.ndarray
    corner_list: list = field(default_factory=list)
    circle_masks: tuple | None = None   # (side_list, concave_list, convex_list)
    walls: bool = False
    rects: list = field(default_factory=list)     # ((x0, y0), (x1, y1)) as given
    circles: list = field(default_factory=list)   # ((cx, cy), r) as given

    @property
    def fluid(self) -> np.ndarray:
        return ~self.solid

    @property
    def porosity(self) -> float:
        return float(self.fluid.mean())


def build_geometry(H: int, W: int, rects=(), circles=(), walls: bool = False) -> Geometry:
    """Rasterise rectangles (``((x0, y0), (x1, y1))``) and circles
    (``((cx, cy), r)``) the reference's way and pack the mask word."""
    cb = Createblock(H, W)
    bpa = np.zeros((H, W), dtype=np.int64)
    links = []
    corner_list = []
    circle_masks = None
    if rects:
        b, corner_list = cb.setblock(list(rects))
        bpa += b
        links.append(rect_link_bits(corner_list, H, W))
    if circles:
        b, sl, cl, vl = cb.setCirleblock(list(circles))
        bpa += b
        circle_masks = (sl, cl, vl)
        links.append(circle_link_bits(sl, cl, vl))
    if walls:
        links.append(wall_row_link_bits(H, W))
    solid = bpa == 1
    return Geometry(H, W, bpa, solid, pack_mask(solid, *links), corner_list, circle_masks, walls,
                    list(rects), list(circles))


def square_blocks(H: int, W: int, n: int, side: int, seed: int, gap: int = 2, margin: int = 2,
                  max_tries: int = 100000):
    """``n`` non-overlapping squares of ``side`` cells placed uniformly at
    random from a seeded generator, at least ``gap`` free cells apart and
    ``margin`` cells from the lattice edges; ``setblock`` corner pairs
    (inclusive, create_block.py:395-407)."""
    rng = np.random.default_rng(seed)
    occ = np.zeros((H, W), dtype=bool)
    rects = []
    tries = 0
    while len(rects) < n and tries < max_tries:
        tries += 1
        x0 = int(rng.integers(margin, W - margin - side + 1))
        y0 = int(rng.integers(margin, H - margin - side + 1))
        if occ[max(y0 - gap, 0):y0 + side + gap, max(x0 - gap, 0):x0 + side + gap].any():
            continue
        occ[y0:y0 + side, x0:x0 + side] = True
        rects.append(((x0, y0), (x0 + side - 1, y0 + side - 1)))
    if len(rects) < n:
        raise ValueError(f"placed only {len(rects)} of {n} squares")
    return rects


def random_blocks(H: int, W: int, porosity: float, rmin: int, rmax: int, seed: int,
                  kinds=("circle", "square"), gap: int = 2, x_margin: int = 0,
                  max_tries: int = 200000, max_blocks: int | None = None):
    """Seeded rejection placement of non-overlapping circles and squares.

    Shapes get a radius / half-side drawn uniformly from ``[rmin, rmax]``,
    keep ``gap`` free cells between each other and stay ``r + 2`` away from
    the lattice edges (the circle scan of create_block.py:81-112 reads
    ``r + 1`` cells past the outline).  Placement stops when the solid
    fraction reaches ``1 - porosity`` or after ``max_blocks`` shapes.
    Returns ``(rects, circles)`` in the reference's list formats.
    """
    rng = np.random.default_rng(seed)
    occ = np.zeros((H, W), dtype=bool)
    target = (1.0 - porosity) * H * W
    covered = 0
    rects, circles = [], []
    tries = 0
    while covered < target and tries < max_tries:
        if max_blocks is not None and len(rects) + len(circles) >= max_blocks:
            break
        tries += 1
        r = int(rng.integers(rmin, rmax + 1))
        kind = kinds[int(rng.integers(0, len(kinds)))]
        m = r + 2
        lo_x = m + x_margin
        if W - m - 1 < lo_x or H - m - 1 < m:
            continue
        cx = int(rng.integers(lo_x, W - m))
        cy = int(rng.integers(m, H - m))
        y0, y1 = cy - r - gap, cy + r + gap + 1
        x0, x1 = cx - r - gap, cx + r + gap + 1
        if occ[max(y0, 0):y1, max(x0, 0):x1].any():
            continue
        occ[cy - r:cy + r + 1, cx - r:cx + r + 1] = True
        if kind == "circle":
            circles.append(((cx, cy), r))
            covered += math.pi * r * r
        else:
            rects.append(((cx - r, cy - r), (cx + r, cy + r)))
            covered += (2 * r + 1) ** 2
    return rects, circles
