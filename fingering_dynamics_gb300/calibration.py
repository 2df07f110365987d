"""psi_wall <-> contact angle calibration by a droplet experiment.

The reference sets wettability by the order parameter written into solid
cells (psi_wall, fingering_periodic.py:18,93) and carries no formula for the
contact angle it produces; its droplet check (validation.py:43-190, 387-425)
does not run as committed.  This module repeats that experiment on the GPU:
a semicircular droplet of invading fluid (psi = +1) is placed on a solid block
in defending fluid (psi = -1), equilibrated with the reference's periodic-
variant constants and no inflow, and the contact angle is read from a circle
fitted to the psi = 0 contour:

    cos(theta) = -(y_c - y_s) / R

with (x_c, y_c, R) the fitted circle and y_s the substrate surface (half a
cell above the last solid row, where half-way bounce-back places the wall);
theta is measured through the droplet.  All psi_wall values run as one
batched ensemble.

``python -m fingering_dynamics_gb300.calibration`` regenerates
``contact_angle_table.json`` (needs a GPU).
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import replace

import numpy as np

from .geometry import build_geometry
from .params import LBMParams, periodic_reference_params

TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "contact_angle_table.json")


def droplet_case(psi_wall: float, H: int = 128, W: int = 256, radius: int = 24, substrate: int = 24,
                 M: float = 1.0):
    """(params, geometry, psi0, substrate surface y) of one droplet run."""
    prm = periodic_reference_params().with_size(H, W)
    prm = replace(prm, psi_wall=psi_wall, M=M, u0=0.0, inlet_ux=np.zeros(H))
    g = build_geometry(H, W, rects=[((8, 4), (W - 9, substrate))])
    ys = substrate + 0.5
    yy, xx = np.mgrid[0:H, 0:W]
    # equilibrium interface profile of the model, psi = tanh(distance / xi), xi = 2
    # (fingering_periodic.py:37); a sharp +-1 edge excites a transient the
    # strong interfacial tension of the reference constants does not survive
    d = np.sqrt((xx - W / 2) ** 2 + (yy - ys) ** 2) - radius
    psi0 = -np.tanh(d / 2.0)
    psi0[yy <= substrate] = -1.0
    # the inlet column is held at psi = +1 by zou_he_boundary_inlet
    # (fingering_periodic.py:278-302); start with the reference's slab there
    psi0[:, :prm.slab] = 1.0
    return prm, g, psi0, ys


def fit_circle(x: np.ndarray, y: np.ndarray):
    """Algebraic least-squares circle (x - a)^2 + (y - b)^2 = r^2 through points."""
    A = np.column_stack([x, y, np.ones_like(x)])
    rhs = -(x ** 2 + y ** 2)
    (D, E, F), *_ = np.linalg.lstsq(A, rhs, rcond=None)
    a, b = -D / 2, -E / 2
    return a, b, math.sqrt(max(a * a + b * b - F, 0.0))


def contact_angle(psi: np.ndarray, ys: float, x_center: float, min_height: float = 3.0) -> float:
    """Contact angle (degrees, through the psi > 0 phase) of a droplet sitting
    on the surface y = ys, from the psi = 0 crossings along each row."""
    H, W = psi.shape
    if not np.isfinite(psi).all():
        return float("nan")
    px, py = [], []
    xc = int(round(x_center))
    for y in range(int(math.ceil(ys + min_height)), H):
        row = psi[y]
        if row[xc] <= 0:
            continue
        for step in (-1, 1):  # walk out of the droplet to its left / right edge
            x = xc
            while 0 <= x + step < W and row[x + step] > 0:
                x += step
            if not 0 <= x + step < W:
                continue
            a, b = row[x], row[x + step]
            px.append(x + step * a / (a - b))
            py.append(float(y))
    if len(px) < 6:
        return float("nan")
    _, b, r = fit_circle(np.array(px), np.array(py))
    c = np.clip(-(b - ys) / r, -1.0, 1.0)
    return math.degrees(math.acos(c))


def calibrate(psi_walls=(-0.7, -0.5, -0.3, 0.0, 0.3, 0.5, 0.7), steps: int = 8000, dtype: str = "f32",
              H: int = 128, W: int = 256, radius: int = 24, substrate: int = 24) -> dict:
    """Run one droplet per psi_wall (one batched ensemble) and measure angles."""
    from .ensemble import Ensemble
    cases = [droplet_case(pw, H=H, W=W, radius=radius, substrate=substrate) for pw in psi_walls]
    ens = Ensemble([(p, g, psi0) for p, g, psi0, _ in cases], dtype=dtype)
    ens.step(steps)
    angles = []
    for lat, (prm, _, _, ys) in zip(ens.lattices, cases):
        psi = lat.macroscopic()["psi"]
        angles.append(contact_angle(psi, ys, prm.W / 2))
    ens.close()
    return {"psi_wall": [float(p) for p in psi_walls], "theta_deg": angles, "steps": steps,
            "setup": f"{H}x{W} periodic variant, reference constants, M = 1, no inflow, droplet R = {radius} on a "
                     f"block up to row {substrate}"}


def psi_wall_for_angle(theta_deg: float, table: dict | None = None) -> float:
    """psi_wall giving contact angle theta (degrees) by monotone interpolation
    of the calibration table."""
    if table is None:
        with open(TABLE) as fh:
            table = json.load(fh)
    th = np.asarray(table["theta_deg"], float)
    pw = np.asarray(table["psi_wall"], float)
    ok = np.isfinite(th)
    th, pw = th[ok], pw[ok]
    order = np.argsort(th)
    return float(np.interp(theta_deg, th[order], pw[order]))


if __name__ == "__main__":
    res = calibrate()
    with open(TABLE, "w") as fh:
        json.dump(res, fh, indent=1)
    print(json.dumps(res))
