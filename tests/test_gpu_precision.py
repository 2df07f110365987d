"""Reduced-precision storage against the FP64 path (short run of the error study)."""
import math

import pytest

pytestmark = pytest.mark.gpu


def test_precision_study_short():
    from bench import workload
    from fingering_dynamics_gb300.precision import precision_study
    prm, g = workload(64, 256)
    res = precision_study(prm, g, dtypes=("f32", "f16", "bf16", "f16/nearest"), steps=1000, every=250, window=500)
    per = res["per_dtype"]
    assert len(res["checkpoints"]["iteration"]) == 4
    for d in ("f32", "f16", "bf16"):
        assert per[d]["finite"]
    # tolerances of the storage formats over the first 500 iterations
    assert per["f32"]["max_dpsi_window"] <= 1e-5
    assert per["f16"]["max_dpsi_window"] <= 1e-3
    assert per["bf16"]["max_dpsi_window"] <= 5e-2
    # colour masses follow the FP64 run closely
    assert per["f32"]["mass_drift_r_max"] <= 1e-4 and per["f16"]["mass_drift_r_max"] <= 1e-3
    # stochastic rounding: smaller phase error than round to nearest on this workload
    assert per["f16"]["max_dpsi_run"] < per["f16/nearest"]["max_dpsi_run"]
    assert not math.isnan(per["f16"]["sat_err_max"])
