"""CPU oracle for the two-phase (free-energy) D2Q9 lattice-Boltzmann step.

TEST INFRASTRUCTURE ONLY.  This module is the oracle the CUDA path is
compared against; it is imported by ``tests/``, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py`` and by nothing else.  The product
path never calls it.

It restates, in vectorised numpy, the algorithm of the reference scripts
``lattice_boltzmann/fingering_periodic.py`` (periodic in y, Gaussian inlet;
"periodic" variant) and ``lattice_boltzmann/fingering.py`` (walls at the
bottom and top, plug inlet, corner nodes; "walls" variant), together with the
bounce-back rules of ``lattice_boltzmann/bounce_back.py``.  Each function names
the reference lines it follows.

Every floating-point expression keeps the reference's operand order
(left-to-right evaluation of the numpy expressions, sequential sums over the
nine directions), so on the same inputs this oracle is bit-for-bit equal to
the reference; the golden fixtures under ``tests/golden`` (made by running the
reference itself) pin that.

Macroscopic fields (rho, ux, uy, p, mu, mix_tau) are kept, as in the
reference, as 1-D arrays over fluid cells in row-major order; psi and the
three stencils are full (H, W) arrays.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# D2Q9 lattice (fingering_periodic.py:50-89)
EX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.float64)
EY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], dtype=np.float64)
W9 = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36])
OPP = (0, 3, 4, 1, 2, 7, 8, 5, 6)


@dataclass
class OracleParams:
    H: int
    W: int
    variant: str            # "periodic" (fingering_periodic.py) or "walls" (fingering.py)
    tau: float              # g relaxation time (fingering_periodic.py:26)
    eta_n: float            # Eta_n (fingering_periodic.py:34)
    M: float                # viscosity ratio (fingering_periodic.py:22)
    a: float                # bulk free-energy coefficient (fingering_periodic.py:39)
    kappa: float            # gradient coefficient (fingering_periodic.py:38)
    gamma: float            # mobility (fingering_periodic.py:40)
    psi_wall: float         # psi written into solid cells (fingering_periodic.py:18)
    inlet_ux: np.ndarray    # (H,) inlet velocity per row (fingering_periodic.py:270-271 / fingering.py:299)
    outlet_coef: float      # 2/3 (fingering_periodic.py:317) or 1.5 (fingering.py:378)
    # variant "periodic_xy" (an extension the reference does not have, so
    # parity with it is unpinned): periodic in x too, no Zou-He, and a body
    # force per unit mass added to mu grad psi in the velocity and the forcing
    force_x: float = 0.0
    force_y: float = 0.0
    # outlet "pressure" (also an extension): rho = 1 imposed at x = W-1, u_x from
    # the known populations, coefficient 2/3, instead of the velocity-type outlet
    outlet: str = "velocity"


def gaussian_inlet_profile(H: int, u0: float) -> np.ndarray:
    """u_x(y) of fingering_periodic.py:270-271 (H must be even)."""
    temp = np.array([i * 3 / (H / 2) for i in range(int(-H / 2), int(H / 2))])
    return u0 * np.exp(- (temp ** 2) / 2)


# ----------------------------------------------------------------------------
# psi stencils (fingering_periodic.py:214-256, fingering.py:219-286)
# ----------------------------------------------------------------------------
def _padded_psi(psi, solid, prm: OracleParams):
    """psi with psi_wall on solid cells and one ghost cell on every side.

    x ghosts are +1 (left) and -1 (right) (fingering_periodic.py:94-95,218).
    In the periodic variant the y ghosts are the wrapped rows
    (np.roll on the unpadded axis); in the walled variant they are rows of
    psi_wall, corners included (fingering.py:102,224).
    """
    H, W = psi.shape
    p = psi.copy()
    p[solid] = prm.psi_wall
    t = np.empty((H + 2, W + 2))
    t[1:-1, 1:-1] = p
    if prm.variant == "periodic_xy":
        t[1:-1, 0] = p[:, -1]
        t[1:-1, -1] = p[:, 0]
    else:
        t[1:-1, 0] = 1.0
        t[1:-1, -1] = -1.0
    if prm.variant == "walls":
        t[0, :] = prm.psi_wall
        t[-1, :] = prm.psi_wall
    else:
        t[0, :] = t[-2, :]
        t[-1, :] = t[1, :]
    return t


def _nbrs(t):
    c = t[1:-1, 1:-1]
    E, Wn = t[1:-1, 2:], t[1:-1, :-2]
    N, S = t[2:, 1:-1], t[:-2, 1:-1]
    NE, NW = t[2:, 2:], t[2:, :-2]
    SE, SW = t[:-2, 2:], t[:-2, :-2]
    return c, E, Wn, N, S, NE, NW, SE, SW


def stencils(psi, solid, prm):
    """(d psi/dx, d psi/dy, laplacian) with the reference's summation order."""
    c, E, Wn, N, S, NE, NW, SE, SW = _nbrs(_padded_psi(psi, solid, prm))
    z = np.zeros_like(c)
    gx = ((((((z + 4 * E) + (-4 * Wn)) + NE) + (-NW)) + (-SW)) + SE) / 12
    gy = ((((((z + 4 * N) + (-4 * S)) + NE) + NW) + (-SW)) + (-SE)) / 12
    lap = (((((((((z + (-20 * c)) + 4 * N) + 4 * E) + 4 * Wn) + 4 * S) + NE) + NW) + SW) + SE) / 6
    return gx, gy, lap


def mu_plain(psi, lap, prm):
    """fingering_periodic.py:146-149 (full grid)."""
    return prm.a * psi * (np.ones_like(psi) - np.power(psi, 2)) - prm.kappa * lap


# ----------------------------------------------------------------------------
# state
# ----------------------------------------------------------------------------
class OracleState:
    """Full lattice state in the reference's layout."""

    def __init__(self, prm: OracleParams, solid: np.ndarray, psi0: np.ndarray,
                 rho0: np.ndarray | None = None, init_mu: bool = False, init_uy: bool = False):
        """Compute.__init__ (fingering_periodic.py:48-121, fingering.py:54-127).

        ``psi0`` is the initial order parameter before solid cells are set to
        psi_wall; ``rho0`` (H, W) is the initial density (None -> 1.0,
        fingering_periodic.py:103; fingering.py:106-107 draws it at random).
        ``init_mu``/``init_uy`` select fingering.py:122-123, which compute mu
        and u_y before the equilibria; the periodic script leaves both at zero.
        """
        H, W = prm.H, prm.W
        self.prm = prm
        self.solid = np.asarray(solid, bool)
        self.mask = ~self.solid
        m = self.mask
        self.psi = np.array(psi0, dtype=np.float64, copy=True)
        self.psi[self.solid] = prm.psi_wall
        self.rho = (np.ones((H, W)) if rho0 is None else np.asarray(rho0, np.float64))[m].copy()
        self.ux = np.zeros((H, W))[m]
        self.uy = np.zeros((H, W))[m]
        self.mu = np.zeros((H, W))[m]
        self.f = np.zeros((9, H, W))
        self.g = np.zeros((9, H, W))
        self.npx, self.npy, self.np2 = stencils(self.psi, self.solid, prm)
        self.p = self._p()
        if init_mu:
            self.mu = self._mu()
        if init_uy:
            # fingering.py:123 evaluates getUy while f is still zero
            self.uy = (np.zeros((H, W))[m] + self.mu * self.npy[m] / 2) / self.rho
        self.mix_tau = self._mix_tau()
        feq, geq = self._equilibria()
        self.f[:, m] = feq
        self.g[:, m] = geq
        self.steps = 0

    # fingering_periodic.py:123-124
    def _p(self):
        return 1 / 3 * self.rho + self.psi[self.mask] * self.mu

    # fingering_periodic.py:141-144
    def _mu(self):
        ps = self.psi[self.mask]
        return self.prm.a * ps * (np.ones_like(ps) - np.power(ps, 2)) - self.prm.kappa * self.np2[self.mask]

    # fingering_periodic.py:201-208
    def _mix_tau(self):
        prm = self.prm
        ps = self.psi[self.mask]
        ones = np.ones_like(ps)
        v1 = prm.eta_n / self.rho
        v2 = prm.eta_n * prm.M / self.rho
        mix_v = np.divide(2 * v1 * v2, (v1 * (ones - ps) + v2 * (ones + ps)))
        return 3 * mix_v + 0.5

    # fingering_periodic.py:126-139
    def _u(self):
        m = self.mask
        f = self.f
        tx = np.zeros(int(m.sum()))
        ty = np.zeros(int(m.sum()))
        for i in range(9):
            tx = tx + f[i][m] * EX[i]
        for i in range(9):
            ty = ty + f[i][m] * EY[i]
        if self.prm.variant == "periodic_xy":
            ux = ((tx + self.mu * self.npx[m] / 2) + self.rho * self.prm.force_x / 2) / self.rho
            uy = ((ty + self.mu * self.npy[m] / 2) + self.rho * self.prm.force_y / 2) / self.rho
            return ux, uy
        ux = (tx + self.mu * self.npx[m] / 2) / self.rho
        uy = (ty + self.mu * self.npy[m] / 2) / self.rho
        return ux, uy

    def _eu_q(self):
        ux, uy = self.ux, self.uy
        eu = EX[:, None] * ux[None, :] + EY[:, None] * uy[None, :]
        q = 3 * eu + 4.5 * eu ** 2 - 1.5 * (ux ** 2 + uy ** 2)
        return eu, q

    # fingering_periodic.py:155-192
    def _equilibria(self):
        prm = self.prm
        ps = self.psi[self.mask]
        _, q = self._eu_q()
        A = np.empty_like(q)
        A[0] = (self.rho - 3.0 * (1.0 - W9[0]) * self.p) / W9[0]
        A[1:] = 3 * self.p
        B = np.empty_like(q)
        B[0] = (ps - 3.0 * (1.0 - W9[0]) * prm.gamma * self.mu) / W9[0]
        B[1:] = 3 * prm.gamma * self.mu
        feq = W9[:, None] * (A + self.rho * q)
        geq = W9[:, None] * (B + ps * q)
        return feq, geq

    # fingering_periodic.py:194-199
    def _forcing(self):
        m = self.mask
        eu, _ = self._eu_q()
        ux, uy = self.ux, self.uy
        gx, gy = self.npx[m], self.npy[m]
        pref = self.mu * W9[:, None] * (1 - 1 / (2 * self.mix_tau))
        ax = (EX[:, None] - ux) * 3 + EX[:, None] * eu * 9
        ay = (EY[:, None] - uy) * 3 + EY[:, None] * eu * 9
        F = pref * (ax * gx + ay * gy)
        if self.prm.variant == "periodic_xy":  # body force density rho b
            prb = self.rho * W9[:, None] * (1 - 1 / (2 * self.mix_tau))
            F = F + prb * (ax * self.prm.force_x + ay * self.prm.force_y)
        return F

    # ------------------------------------------------------------------
    # one step: fingering_periodic.py:454-479 / fingering.py:558-585
    # ------------------------------------------------------------------
    def collide(self):
        """fingering_periodic.py:455-460 and 258-264 (fluid cells only)."""
        m = self.mask
        F = self._forcing()
        feq, geq = self._equilibria()
        fm = self.f[:, m]
        gm = self.g[:, m]
        self.f[:, m] = fm - 1.0 / self.mix_tau * (fm - feq) + F
        self.g[:, m] = gm - 1.0 / self.prm.tau * (gm - geq)

    def step(self, bb_rect=None, bb_circle=None):
        """Advance one reference iteration.

        ``bb_rect`` is a ``corner_list`` (bounce_back.py:25-86) and
        ``bb_circle`` a ``(side_list, concave_list, convex_list)`` triple
        (bounce_back.py:89-167); either may be None.
        """
        self.collide()
        fb = self.f.copy()
        gb = self.g.copy()
        self.f, self.g = stream(self.f), stream(self.g)
        if bb_rect:
            halfway_bounceback_rec(bb_rect, fb, gb, self.f, self.g)
        if bb_circle is not None:
            halfway_bounceback_circle(*bb_circle, fb, gb, self.f, self.g)
        if self.prm.variant == "walls":
            bottom_top_wall(fb[:, 1:-1], gb[:, 1:-1], self.f[:, 1:-1], self.g[:, 1:-1])
        self.zou_he()
        self.macros()
        self.steps += 1

    def boundary_fields(self):
        """psi_x, psi_y and mu_plain from the current psi and stored laplacian
        (fingering_periodic.py:273-275, 309-311)."""
        gx, gy, _ = stencils(self.psi, self.solid, self.prm)
        return gx, gy, mu_plain(self.psi, self.np2, self.prm)

    def zou_he(self):
        if self.prm.variant == "periodic_xy":
            return
        gx, gy, mu = self.boundary_fields()
        if self.prm.variant == "walls":
            zou_he_inlet_walls(self.f, self.g, gx, gy, mu, self.prm)
            zou_he_outlet_walls(self.f, self.g, gx[:, -1], gy[:, -1], mu[:, -1], self.prm)
        else:
            zou_he_inlet_periodic(self.f, self.g, gx, gy, mu, self.prm)
            zou_he_outlet_periodic(self.f, self.g, gx[:, -1], gy[:, -1], mu[:, -1], self.prm)

    def macros(self):
        """fingering_periodic.py:470-479."""
        m = self.mask
        acc = self.f[0].copy()
        for i in range(1, 9):
            acc = acc + self.f[i]
        self.rho = acc[m]
        acc = self.g[0].copy()
        for i in range(1, 9):
            acc = acc + self.g[i]
        self.psi[m] = acc[m]
        self.psi[self.solid] = self.prm.psi_wall
        self.npx, self.npy, self.np2 = stencils(self.psi, self.solid, self.prm)
        self.mu = self._mu()
        self.ux, self.uy = self._u()
        self.p = self._p()
        self.mix_tau = self._mix_tau()

    def full(self, name):
        """A compacted fluid field expanded to (H, W) with NaN on solid cells."""
        out = np.full((self.prm.H, self.prm.W), np.nan)
        out[self.mask] = getattr(self, name)
        return out


# ----------------------------------------------------------------------------
# streaming and bounce-back
# ----------------------------------------------------------------------------
def stream(a):
    """fingering_periodic.py:327-343: every cell, periodic in x and y."""
    out = np.empty_like(a)
    for i in range(9):
        out[i] = np.roll(np.roll(a[i], int(EX[i]), axis=1), int(EY[i]), axis=0)
    return out


def halfway_bounceback_rec(corner_list, fb, gb, f, g):
    """bounce_back.py:25-86."""
    H, W = f[0].shape
    n, s, e, w, nw, ne, sw, se = (np.zeros((H, W), bool) for _ in range(8))
    for c in corner_list:
        tlx, tly = c["top_left"]
        blx, bly = c["bottom_left"]
        trx = c["top_right"][0]
        brx = c["bottom_right"][0]
        n[tly + 1, tlx:trx + 1] = True
        s[bly - 1, tlx:trx + 1] = True
        w[bly:tly + 1, tlx - 1] = True
        e[bly:tly + 1, trx + 1] = True
        nw[tly + 1, tlx - 1] = True
        ne[tly + 1, trx + 1] = True
        sw[bly - 1, blx - 1] = True
        se[bly - 1, brx + 1] = True
    plan = {1: [e], 2: [n], 3: [w], 4: [s], 5: [ne, n, e], 6: [nw, n, w],
            7: [sw, s, w], 8: [se, s, e]}
    _apply_bb(plan, fb, gb, f, g)


def halfway_bounceback_circle(side_list, concave_list, convex_list, fb, gb, f, g):
    """bounce_back.py:89-167 (list positions as the reference indexes them)."""
    sd, cc, vx = side_list, concave_list, convex_list
    plan = {1: [sd[3], cc[0], cc[2]], 2: [sd[0], cc[0], cc[1]], 3: [sd[2], cc[1], cc[3]],
            4: [sd[1], cc[2], cc[3]], 5: [vx[0], cc[0], sd[0], sd[3]],
            6: [vx[1], cc[1], sd[0], sd[2]], 7: [vx[3], cc[3], sd[1], sd[2]],
            8: [vx[2], cc[2], sd[1], sd[3]]}
    _apply_bb(plan, fb, gb, f, g)


def _apply_bb(plan, fb, gb, f, g):
    for i, masks in plan.items():
        o = OPP[i]
        for mk in masks:
            f[i][mk] = fb[o][mk]
            g[i][mk] = gb[o][mk]


def bottom_top_wall(fb, gb, f, g):
    """fingering.py:432-451 (called with row-sliced views, fingering.py:573)."""
    for i, o, row in ((2, 4, 0), (4, 2, -1), (5, 7, 0), (6, 8, 0), (7, 5, -1), (8, 6, -1)):
        f[i][row, :] = fb[o][row, :]
        g[i][row, :] = gb[o][row, :]


# ----------------------------------------------------------------------------
# Zou-He boundaries
# ----------------------------------------------------------------------------
def zou_he_inlet_periodic(f, g, gx, gy, mu, prm):
    """fingering_periodic.py:268-302: column 0, every row."""
    ux = prm.inlet_ux
    px, py, m = gx[:, 0], gy[:, 0], mu[:, 0]
    rho_in = 1 / (1 - ux) * (f[0][:, 0] + f[2][:, 0] + f[4][:, 0]
                             + 2 * (f[3][:, 0] + f[6][:, 0] + f[7][:, 0]) - px * m / 2)
    psi_in = 1.0 - (g[0][:, 0] + g[2][:, 0] + g[3][:, 0] + g[4][:, 0] + g[6][:, 0] + g[7][:, 0])
    wsum = W9[1] + W9[5] + W9[8]
    f[1][:, 0] = f[3][:, 0] + 2 / 3 * ux * rho_in - px * m / 6
    g[1][:, 0] = W9[1] * psi_in / wsum
    f[5][:, 0] = f[7][:, 0] - 0.5 * (f[2][:, 0] - f[4][:, 0]) + 1.0 / 6.0 * ux * rho_in - px * m / 6 - py * m / 4
    g[5][:, 0] = W9[5] * psi_in / wsum
    f[8][:, 0] = f[6][:, 0] + 0.5 * (f[2][:, 0] - f[4][:, 0]) + 1.0 / 6.0 * ux * rho_in - px * m / 6 + py * m / 4
    g[8][:, 0] = W9[8] * psi_in / wsum


def _outlet_body(f, g, px, py, m, prm):
    ux = prm.inlet_ux
    c = prm.outlet_coef
    S = (f[0][:, -1] + f[2][:, -1] + f[4][:, -1] + 2 * (f[1][:, -1] + f[5][:, -1] + f[8][:, -1]) + px * m / 2)
    if prm.outlet == "pressure":
        rho_out = np.ones_like(S)
        ux = S - 1.0
        c = 2 / 3
    else:
        rho_out = 1 / (1 + ux) * S
    psi_out = -1.0 - (g[0][:, -1] + g[1][:, -1] + g[2][:, -1] + g[4][:, -1] + g[5][:, -1] + g[8][:, -1])
    wsum = W9[3] + W9[6] + W9[7]
    f[3][:, -1] = f[1][:, -1] - c * ux * rho_out + px * m / 6
    g[3][:, -1] = W9[3] * psi_out / wsum
    f[6][:, -1] = f[8][:, -1] - 0.5 * (f[2][:, -1] - f[4][:, -1]) - 1.0 / 6.0 * ux * rho_out + py * m / 4 + px * m / 6
    g[6][:, -1] = W9[6] * psi_out / wsum
    f[7][:, -1] = f[5][:, -1] + 0.5 * (f[2][:, -1] - f[4][:, -1]) - 1.0 / 6.0 * ux * rho_out - py * m / 4 + px * m / 6
    g[7][:, -1] = W9[7] * psi_out / wsum


def zou_he_outlet_periodic(f, g, px, py, m, prm):
    """fingering_periodic.py:305-324: column W-1, every row."""
    _outlet_body(f, g, px, py, m, prm)


def zou_he_inlet_walls(f, g, gx, gy, mu, prm):
    """fingering.py:298-364: rows 1..H-2 plus the two inlet corner nodes."""
    ux = prm.inlet_ux
    px, py, m = gx[:, 0], gy[:, 0], mu[:, 0]
    rho_in = 1 / (1 - ux) * (f[0][:, 0] + f[2][:, 0] + f[4][:, 0]
                             + 2 * (f[3][:, 0] + f[6][:, 0] + f[7][:, 0]) - px * m / 2)
    psi_in = 1.0 - (g[0][:, 0] + g[2][:, 0] + g[3][:, 0] + g[4][:, 0] + g[6][:, 0] + g[7][:, 0])
    wsum = W9[1] + W9[5] + W9[8]
    r = slice(1, -1)
    f[1][r, 0] = f[3][r, 0] + (2 / 3) * ux[r] * rho_in[r] - px[r] * m[r] / 6
    g[1][r, 0] = W9[1] * psi_in[r] / wsum
    f[5][r, 0] = (f[7][r, 0] - 0.5 * (f[2][r, 0] - f[4][r, 0]) + 1.0 / 6.0 * ux[r] * rho_in[r]
                  - px[r] * m[r] / 6 - py[r] * m[r] / 4)
    g[5][r, 0] = W9[5] * psi_in[r] / wsum
    f[8][r, 0] = (f[6][r, 0] + 0.5 * (f[2][r, 0] - f[4][r, 0]) + 1.0 / 6.0 * ux[r] * rho_in[r]
                  - px[r] * m[r] / 6 + py[r] * m[r] / 4)
    g[8][r, 0] = W9[8] * psi_in[r] / wsum
    # bottom-left corner (fingering.py:334-348)
    f[1][0, 0] = f[3][0, 0]; g[1][0, 0] = g[3][0, 0]
    f[2][0, 0] = f[4][0, 0]; g[2][0, 0] = g[4][0, 0]
    f[5][0, 0] = f[7][0, 0]; g[5][0, 0] = g[7][0, 0]
    f[6][0, 0] = 0.5 * (rho_in[1] - (f[0][0, 0] + f[1][0, 0] + f[2][0, 0] + f[3][0, 0]
                                    + f[4][0, 0] + f[5][0, 0] + f[7][0, 0]))
    g[6][0, 0] = W9[6] * (1.0 - (g[0][0, 0] + g[1][0, 0] + g[2][0, 0] + g[3][0, 0]
                                 + g[4][0, 0] + g[5][0, 0] + g[7][0, 0])) / (W9[6] + W9[8])
    f[8][0, 0] = f[6][0, 0]; g[8][0, 0] = g[6][0, 0]
    # top-left corner (fingering.py:350-364)
    f[1][-1, 0] = f[3][-1, 0]; g[1][-1, 0] = g[3][-1, 0]
    f[4][-1, 0] = f[2][-1, 0]; g[4][-1, 0] = g[2][-1, 0]
    f[8][-1, 0] = f[6][-1, 0]; g[8][-1, 0] = g[6][-1, 0]
    f[5][-1, 0] = 0.5 * (rho_in[-2] - (f[0][-1, 0] + f[1][-1, 0] + f[2][-1, 0] + f[3][-1, 0]
                                      + f[4][-1, 0] + f[6][-1, 0] + f[8][-1, 0]))
    g[5][-1, 0] = W9[5] * (1.0 - (g[0][-1, 0] + g[1][-1, 0] + g[2][-1, 0] + g[3][-1, 0]
                                  + g[4][-1, 0] + g[6][-1, 0] + g[8][-1, 0])) / (W9[5] + W9[7])
    f[7][-1, 0] = f[5][-1, 0]; g[7][-1, 0] = g[5][-1, 0]


def zou_he_outlet_walls(f, g, px, py, m, prm):
    """fingering.py:369-390: column W-1 plus the two outlet corner copies."""
    _outlet_body(f, g, px, py, m, prm)
    f[2][0, -1] = f[4][0, -1]; g[2][0, -1] = g[4][0, -1]
    f[4][-1, -1] = f[2][-1, -1]; g[4][-1, -1] = g[2][-1, -1]


def diagnostics(st: OracleState) -> dict:
    """FP64 colour masses, saturation, finger tip and breakthrough of an
    oracle state: the same definitions as the library's fd_diag (the reference
    defines none of them)."""
    m = st.mask
    rho = st.rho
    psi = st.psi[m]
    xs = np.nonzero(m)[1]
    inv = psi > 0
    return {
        "mass_r": float(np.sum(rho * (1.0 + psi) * 0.5)),
        "mass_b": float(np.sum(rho * (1.0 - psi) * 0.5)),
        "invaded": int(inv.sum()),
        "fluid": int(m.sum()),
        "saturation": float(inv.sum() / max(int(m.sum()), 1)),
        "tip_x": int(xs[inv].max()) if inv.any() else -1,
        "breakthrough": int(bool(inv[xs >= st.prm.W - 5].any())),
    }


def nonequilibrium(rho, psi, ux, uy, mix_tau, solid, prm: OracleParams):
    """First-order non-equilibrium part of a restart from fields (an extension
    with no reference counterpart, restating fd_add_nonequilibrium):
    f_i^(1) = -3 w_i tau_mix Q_i : S(rho u), g_i^(1) = -3 w_i tau Q_i : S(psi u),
    Q_i = e_i e_i - I/3, S the symmetric part of the gradient by central
    differences over fluid neighbours (one-sided next to solid cells or
    lattice edges, zero without a fluid neighbour).  Inputs are full (H, W)
    arrays; returns (df, dg) of shape (9, H, W), zero on solid cells."""
    H, W = solid.shape
    fluid = ~np.asarray(solid, bool)
    v = np.stack([rho * ux, rho * uy, psi * ux, psi * uy])

    def neighbour(dx, dy):
        ys, xs = np.mgrid[0:H, 0:W]
        yy, xx = ys + dy, xs + dx
        ok = np.ones((H, W), bool)
        if prm.variant == "walls":
            ok &= (yy >= 0) & (yy < H)
        yy = np.mod(yy, H)
        if prm.variant == "periodic_xy":
            xx = np.mod(xx, W)
        else:
            ok &= (xx >= 0) & (xx < W)
            xx = np.clip(xx, 0, W - 1)
        ok &= fluid[yy, xx]
        return ok, v[:, yy, xx]

    def deriv(dx, dy):
        okp, vp = neighbour(dx, dy)
        okm, vm = neighbour(-dx, -dy)
        return np.where(okp & okm, 0.5 * (vp - vm), np.where(okp, vp - v, np.where(okm, v - vm, 0.0)))

    dxv, dyv = deriv(1, 0), deriv(0, 1)
    fxx, fyy, fxy = dxv[0], dyv[1], 0.5 * (dyv[0] + dxv[1])
    gxx, gyy, gxy = dxv[2], dyv[3], 0.5 * (dyv[2] + dxv[3])
    df = np.zeros((9, H, W))
    dg = np.zeros((9, H, W))
    for i in range(9):
        qxx, qyy, qxy = EX[i] ** 2 - 1 / 3, EY[i] ** 2 - 1 / 3, EX[i] * EY[i]
        df[i] = -3 * W9[i] * mix_tau * (qxx * fxx + qyy * fyy + 2 * qxy * fxy)
        dg[i] = -3 * W9[i] * prm.tau * (qxx * gxx + qyy * gyy + 2 * qxy * gxy)
    df[:, ~fluid] = 0
    dg[:, ~fluid] = 0
    return df, dg
