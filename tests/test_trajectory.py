"""Trajectory shard format round trip (CPU)."""
import numpy as np

from fingering_dynamics_gb300.trajectory import TrajectoryWriter, read_shards


def test_shards_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    solid = rng.random((8, 12)) < 0.2
    w = TrajectoryWriter(str(tmp_path), solid, meta={"H": 8, "W": 12}, frames_per_shard=3)
    frames = [{k: rng.standard_normal((8, 12)) for k in ("psi", "ux", "uy")} for _ in range(7)]
    for i, f in enumerate(frames):
        w.add(f, 200 * i)
    w.close()
    shards = list(read_shards(str(tmp_path)))
    assert [len(s["iteration"]) for s in shards] == [3, 3, 1]
    psi = np.concatenate([s["psi"] for s in shards])
    assert np.array_equal(psi, np.stack([f["psi"] for f in frames]).astype(np.float32))
    assert np.array_equal(np.concatenate([s["iteration"] for s in shards]), 200 * np.arange(7))
    assert all(np.array_equal(s["solid"], solid) and s["meta"]["W"] == 12 for s in shards)
