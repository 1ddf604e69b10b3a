"""Regenerates the golden fixtures in this folder from the reference checkout.

Run with the reference checkout named by SANDENGINE_REF:

    SANDENGINE_REF=<reference checkout> python tests/golden/make_golden.py

Writes
  reference_materials.yaml   the reference's data/materials.yaml (the rule-set fixture whose
                             generated GLSL is the reference's known answer)
  reference_gen.json         SHA-256 and length of the reference's checked-in
                             shaders/compute/gen/{materials,rules,falling_sand}.glsl
  grids.json                 per-frame digests of grids advanced by the reference's own
                             compute shader compiled on the CPU (oracle/_ref)
"""
import hashlib
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.build import Ref, reference_root  # noqa: E402
from sandengine_gb300.simulation import grid_digest  # noqa: E402
from sandengine_gb300 import workloads as wl  # noqa: E402
from tests.golden.cases import CASES  # noqa: E402


def main():
    ref = reference_root()
    if ref is None:
        sys.exit("no reference checkout")
    shutil.copyfile(os.path.join(ref, "data", "materials.yaml"), os.path.join(HERE, "reference_materials.yaml"))
    gen = {}
    for name in ("materials.glsl", "rules.glsl", "falling_sand.glsl"):
        data = open(os.path.join(ref, "shaders", "compute", "gen", name), "rb").read()
        gen[name] = {"sha256": hashlib.sha256(data).hexdigest(), "bytes": len(data)}
    with open(os.path.join(HERE, "reference_gen.json"), "w") as f:
        json.dump(gen, f, indent=1)
    out = {}
    for case in CASES:
        R = Ref(case.ruleset_text())
        g = case.initial_grid()
        digests = []
        for i in range(case.frames):
            f = case.frame0 + 1 + i
            g = R.step(g, f, case.mods_at(i), nthreads=os.cpu_count() or 1)
            digests.append(str(grid_digest(g)))
        out[case.name] = {"frames": case.frames, "frame0": case.frame0, "digests": digests}
        print(case.name, "done", flush=True)
    with open(os.path.join(HERE, "grids.json"), "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    main()
