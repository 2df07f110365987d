"""The psi_wall -> contact angle droplet calibration: the angle falls
monotonically as the wall favours the droplet's phase, and the committed
table agrees with a fresh (shorter) run."""
import json
import math

import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_droplet_angles_monotone_and_table_consistent():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()
    from fingering_dynamics_gb300.calibration import TABLE, calibrate, psi_wall_for_angle
    res = calibrate(psi_walls=(-0.5, 0.0, 0.5), steps=6000)
    th = res["theta_deg"]
    assert all(math.isfinite(t) for t in th), th
    assert th[0] > th[1] > th[2], th
    with open(TABLE) as fh:
        table = json.load(fh)
    for pw, t in zip(res["psi_wall"], th):
        ref = dict(zip(table["psi_wall"], table["theta_deg"])).get(pw)
        if ref is not None and math.isfinite(ref):
            assert abs(t - ref) < 6.0, (pw, t, ref)
    # the inverse map reproduces the table
    assert abs(psi_wall_for_angle(table["theta_deg"][3], table) - table["psi_wall"][3]) < 1e-6


def test_gpu_droplet_angles_match_the_oracle():
    """The calibration experiment on the GPU (batched FP32 kernels) against the
    same experiment in the FP64 CPU oracle (tests/golden/droplet_angles_64x128.json,
    made by tests/golden/make_droplet_angles.py): 64 x 128, droplet R = 12,
    2000 iterations, psi_wall in {-0.5, 0, 0.5}; angles within 1.5 degrees."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()
    from fingering_dynamics_gb300.calibration import calibrate
    from golden.make_droplet_angles import OUT
    with open(OUT) as fh:
        gold = json.load(fh)
    res = calibrate(psi_walls=tuple(gold["psi_wall"]), steps=gold["steps"], H=gold["H"], W=gold["W"],
                    radius=gold["radius"], substrate=gold["substrate"])
    for pw, t, ref in zip(gold["psi_wall"], res["theta_deg"], gold["theta_deg"]):
        assert abs(t - ref) < 1.5, (pw, t, ref)
