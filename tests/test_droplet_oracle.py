"""The contact-angle calibration's droplet experiment in the CPU oracle
(tests/golden/make_droplet_angles.py): a rerun reproduces the committed
golden angle, and the golden angles fall monotonically with psi_wall."""
import json
import os

from golden.make_droplet_angles import OUT, oracle_angle


def test_golden_droplet_angles_reproduce():
    with open(OUT) as fh:
        rec = json.load(fh)
    th = rec["theta_deg"]
    assert th[0] > th[1] > th[2], th
    k = rec["psi_wall"].index(0.0)
    assert abs(oracle_angle(0.0) - th[k]) < 1e-9
