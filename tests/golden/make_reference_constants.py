"""Record the reference scripts' own model constants in reference_constants.json.

Run from the repository root in a checkout where the reference is available:

    python tests/golden/make_reference_constants.py /root/reference

Imports lattice_boltzmann/fingering_periodic.py and lattice_boltzmann/fingering.py
unmodified (with the stand-ins of make_golden.py for matplotlib and cv2) and
writes the module globals their constant chains compute at import time
(fingering_periodic.py:15-44, fingering.py:16-50) before anything overrides
them, so that tests can pin this package's parameter functions to them.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden import import_reference  # noqa: E402

NAMES = ("H", "W", "tau", "Eta_n", "M", "a", "kappa", "gamma", "psi_wall", "u0", "sigma")


def main(ref_root):
    fp, fw, _, _ = import_reference(ref_root)
    out = {}
    for key, mod in (("periodic", fp), ("walls", fw)):
        out[key] = {n: float(getattr(mod, n)) for n in NAMES if hasattr(mod, n)}
    path = os.path.join(HERE, "reference_constants.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
