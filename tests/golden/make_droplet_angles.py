"""Golden droplet angles from the CPU oracle (test infrastructure).

The contact-angle calibration (fingering_dynamics_gb300.calibration) runs a
droplet on a solid block on the GPU and reads the angle from a circle fitted
to the psi = 0 contour.  This script runs the same experiment, smaller
(64 x 128 lattice, droplet R = 12 on a block up to row 12, 2000 iterations)
in the FP64 numpy oracle, which restates the reference's step, and records
the angles for psi_wall in {-0.5, 0, 0.5}:

    python tests/golden/make_droplet_angles.py   # writes droplet_angles_64x128.json
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

CASE = {"H": 64, "W": 128, "radius": 12, "substrate": 12, "steps": 2000, "psi_wall": [-0.5, 0.0, 0.5]}
OUT = os.path.join(HERE, "droplet_angles_64x128.json")


def oracle_droplet(psi_wall, H, W, radius, substrate, steps):
    """psi of the droplet case after `steps` oracle iterations, and the substrate surface y."""
    import numpy as np
    from fingering_dynamics_gb300.calibration import droplet_case
    from oracle.lbm_oracle import OracleParams, OracleState
    prm, g, psi0, ys = droplet_case(psi_wall, H=H, W=W, radius=radius, substrate=substrate)
    op = OracleParams(H=H, W=W, variant="periodic", tau=prm.tau, eta_n=prm.eta_n, M=prm.M, a=prm.a,
                      kappa=prm.kappa, gamma=prm.gamma, psi_wall=prm.psi_wall,
                      inlet_ux=np.asarray(prm.inlet_ux, np.float64), outlet_coef=prm.outlet_coef)
    st = OracleState(op, g.solid, psi0)
    for _ in range(steps):
        st.step(g.corner_list, None)
    return st.psi, ys


def oracle_angle(psi_wall, case=CASE):
    from fingering_dynamics_gb300.calibration import contact_angle
    psi, ys = oracle_droplet(psi_wall, case["H"], case["W"], case["radius"], case["substrate"], case["steps"])
    return contact_angle(psi, ys, case["W"] / 2)


if __name__ == "__main__":
    rec = dict(CASE)
    rec["theta_deg"] = [oracle_angle(pw) for pw in CASE["psi_wall"]]
    rec["made_by"] = "tests/golden/make_droplet_angles.py (FP64 numpy oracle)"
    with open(OUT, "w") as fh:
        json.dump(rec, fh, indent=1)
    print(rec)
