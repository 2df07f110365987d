"""Trajectory shards: (psi, u_x, u_y) frames of a lattice at fixed intervals,
with its solid mask, written as compressed .npz shards.

The reference keeps psi frames in an in-memory list every ``mabiki`` steps
(fingering.py:565-566) and pickles it for a movie (openmovie.py:14-15).  Here
frames go to disk in shards of ``frames_per_shard`` so long runs and large
ensembles stream out; they are the training data of a surrogate and the
record of a run.  Shard layout: ``psi``, ``ux``, ``uy`` (n, H, W) float32,
``iteration`` (n,), ``solid`` (H, W) bool, ``meta`` (JSON text).
"""
from __future__ import annotations

import glob
import json
import os

import numpy as np


class TrajectoryWriter:
    def __init__(self, directory: str, solid: np.ndarray, meta: dict | None = None, frames_per_shard: int = 64,
                 prefix: str = "shard"):
        os.makedirs(directory, exist_ok=True)
        self.directory = directory
        self.solid = np.asarray(solid, bool)
        self.meta = dict(meta or {})
        self.frames_per_shard = int(frames_per_shard)
        self.prefix = prefix
        self._frames = {"psi": [], "ux": [], "uy": [], "iteration": []}
        self._n_shards = 0

    def add(self, fields: dict, iteration: int):
        """Append one frame; ``fields`` has psi, ux, uy (H, W) arrays
        (e.g. ``Lattice.macroscopic()``)."""
        for k in ("psi", "ux", "uy"):
            self._frames[k].append(np.asarray(fields[k], np.float32))
        self._frames["iteration"].append(int(iteration))
        if len(self._frames["iteration"]) >= self.frames_per_shard:
            self.flush()

    def add_lattice(self, lattice):
        self.add(lattice.macroscopic(), lattice.iteration)

    def flush(self):
        if not self._frames["iteration"]:
            return
        path = os.path.join(self.directory, f"{self.prefix}_{self._n_shards:05d}.npz")
        np.savez_compressed(path, psi=np.stack(self._frames["psi"]), ux=np.stack(self._frames["ux"]),
                            uy=np.stack(self._frames["uy"]), iteration=np.array(self._frames["iteration"]),
                            solid=self.solid, meta=np.array(json.dumps(self.meta)))
        self._n_shards += 1
        self._frames = {"psi": [], "ux": [], "uy": [], "iteration": []}

    def close(self):
        self.flush()


def read_shards(directory: str, prefix: str = "shard"):
    """Yield the shards of a directory in order, as dicts of arrays (meta parsed)."""
    for path in sorted(glob.glob(os.path.join(directory, f"{prefix}_*.npz"))):
        with np.load(path, allow_pickle=False) as z:
            d = {k: z[k] for k in z.files}
        d["meta"] = json.loads(str(d["meta"]))
        yield d
