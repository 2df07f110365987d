"""Host logic of the model parameters (no GPU): the reference's constant
chains reproduced exactly (tests/golden/reference_constants.json, recorded by
importing the reference scripts, tests/golden/make_reference_constants.py),
the lattice-quantity mapping, the inlet profiles, the contact-angle table and
the circle fit behind it."""
import json
import math
import os

import numpy as np
import pytest

from fingering_dynamics_gb300.calibration import contact_angle, fit_circle, psi_wall_for_angle
from fingering_dynamics_gb300.params import (from_relaxation_times, inlet_profile, periodic_reference_params,
                                             walls_reference_params)

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = {"tau": "tau", "Eta_n": "eta_n", "M": "M", "a": "a", "kappa": "kappa", "gamma": "gamma",
          "psi_wall": "psi_wall", "u0": "u0"}


@pytest.fixture(scope="module")
def ref():
    with open(os.path.join(HERE, "golden", "reference_constants.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("variant", ["periodic", "walls"])
def test_reference_constant_chains_exact(ref, variant):
    r = ref[variant]
    fn = periodic_reference_params if variant == "periodic" else walls_reference_params
    prm = fn(H=int(r["H"]), W=int(r["W"]))
    for name, attr in FIELDS.items():
        assert getattr(prm, attr) == r[name], (variant, name, getattr(prm, attr), r[name])


def test_from_relaxation_times_mapping():
    prm = from_relaxation_times(64, 128, 0.6, 1.0, 5e-4, 90.0, 0.01, variant="walls", angle_map="cos")
    # psi = +1 relaxes with tau_inv and psi = -1 with tau_def (mixing rule at rho = 1)
    assert math.isclose(3 * prm.eta_n + 0.5, 0.6, rel_tol=1e-15)
    assert math.isclose(3 * prm.M * prm.eta_n + 0.5, 1.0, rel_tol=1e-15)
    assert prm.kappa == 0.75 * 5e-4 * 2.0 and prm.a == -2.0 * prm.kappa / 4.0
    assert math.isclose(prm.gamma, 0.01 * 20.0 / ((-prm.a * 15.0) * (prm.tau - 0.5)), rel_tol=1e-15)
    assert abs(prm.psi_wall) < 1e-15  # cos(90 deg)
    assert prm.variant == "walls" and prm.outlet_coef == 1.5


def test_inlet_profiles():
    H, u0 = 24, 0.01
    g = inlet_profile(H, u0, "gaussian")
    s = (np.arange(H) - H / 2) * 3 / (H / 2)
    np.testing.assert_allclose(g, u0 * np.exp(-s * s / 2), rtol=1e-15, atol=0)
    assert g.argmax() == H // 2 and g.max() == u0
    np.testing.assert_array_equal(inlet_profile(7, u0, "plug"), np.full(7, u0))
    with pytest.raises(ValueError):
        inlet_profile(7, u0, "gaussian")


def test_contact_angle_table_interpolation():
    table = {"psi_wall": [-0.5, 0.0, 0.5], "theta_deg": [150.0, 90.0, 30.0]}
    assert psi_wall_for_angle(90.0, table) == 0.0
    assert psi_wall_for_angle(120.0, table) == pytest.approx(-0.25)
    assert psi_wall_for_angle(10.0, table) == 0.5  # clamped to the table
    # the committed table is monotone: wetter walls (larger psi_wall) give smaller angles
    pw = [psi_wall_for_angle(t) for t in (40, 60, 90, 120, 150)]
    assert all(a > b for a, b in zip(pw, pw[1:]))


def test_circle_fit_and_contact_angle():
    t = np.linspace(0.2, 2.9, 40)
    a, b, r = fit_circle(10 + 7 * np.cos(t), -3 + 7 * np.sin(t))
    assert (a, b, r) == pytest.approx((10.0, -3.0, 7.0), abs=1e-9)
    # a cap of the circle of radius 20 centred 10 below the surface y = 50: the angle through the
    # droplet is acos(10 / 20) = 60 degrees
    H, W, ys, xc, R, depth = 120, 160, 50.0, 80.0, 20.0, 10.0
    y, x = np.mgrid[0:H, 0:W].astype(float)
    # a smooth profile across the interface (tanh of the signed distance) for sub-cell crossings
    dist = R - np.sqrt((x - xc) ** 2 + (y - (ys - depth)) ** 2)
    psi = np.where(y < ys, -1.0, np.tanh(dist / 2.0))
    assert contact_angle(psi, ys, xc, min_height=1.0) == pytest.approx(60.0, abs=1.5)
