"""Generate golden outputs of the reference's z-plane post-processing.

Run where the reference is checked out (its src directory given by
--reference-src or CTRAJ_REFERENCE_SRC); GPU machines only read the .npz files this writes.

    python tests/golden/make_golden_post.py --reference-src <reference>/src

For the fixture cases ``config0``, ``config1`` and ``example_lens`` (initial
conditions from their .npz files, made by make_golden.py) it re-propagates the
molecules credited to the apertures of interest with the reference itself,
builds the reference's ``SimulationResult`` from those ``Molecule`` objects and
calls the reference's ``post_processing.find_radial_pos_dist`` and
``find_vel_dist`` at several planes, with and without an element filter.
Stored per case: the molecule indices (into the case's initial conditions, in
result order), and per (plane, filter) the returned arrays.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
import refstubs  # noqa: E402

HERE = Path(__file__).resolve().parent

CASES = {
    # case: (apertures of interest, planes, filters)
    "config0": (["Detected", "A2"], [0.0, 0.3, 0.7, 1.0005, 2.5, 3.0, 3.5], [None, ["Detected"]]),
    "config1": (["Detected", "Inside lens"], [0.3, 0.9, 1.1, 1.4, 2.0, 3.0], [None, ["Inside lens"]]),
    "example_lens": (["Detected"], [0.5, 0.9, 1.2, 2.0], [None]),
}


def main():
    ap = argparse.ArgumentParser()
    refstubs.add_argument(ap)
    args = ap.parse_args()
    sys.path.insert(0, str(HERE))
    import make_golden
    refstubs.install(refstubs.require(args.reference_src))
    from trajectories.molecule import Molecule
    from trajectories.post_processing import find_radial_pos_dist, find_vel_dist
    from trajectories.trajectory_simulator import Counter, SimulationResult

    tables = make_golden.make_tables()
    for name, (aoi, planes, filters) in CASES.items():
        fx = np.load(HERE / f"{name}.npz")
        specs = json.loads(str(fx["spec"]))["elements"]
        names = [str(s) for s in fx["label_names"]]
        labels = [names[k] for k in fx["label"]]
        ids = np.array([i for i, s in enumerate(labels) if s in aoi], dtype=np.int64)
        beamline = make_golden.build_reference_beamline(specs, tables)
        lenses = [(e, s) for e, s in zip(beamline.elements, sorted(specs, key=lambda s: s["z0"]))
                  if s["cls"] == "ElectrostaticLens"]
        ics = fx["ics"]
        molecules = []
        for i in ids:
            for e, s in lenses:
                if s.get("dt") is not None:
                    e.dz = ics[5, i] * s["dt"]
            m = Molecule()
            m.init_trajectory(beamline, ics[:3, i], ics[3:, i])
            beamline.propagate_through(m)
            assert m.aperture_hit == labels[i], (name, i, m.aperture_hit, labels[i])
            molecules.append(m)
        result = SimulationResult(Counter(), beamline, None, None, molecules)
        out = dict(ids=ids, planes=np.array(planes))
        for k, z in enumerate(planes):
            for f, flt in enumerate(filters):
                out[f"pos_{k}_{f}"] = np.asarray(find_radial_pos_dist(result, z, flt), dtype=np.float64)
                out[f"vel_{k}_{f}"] = np.asarray(find_vel_dist(result, z, flt), dtype=np.float64)
        out["filters"] = np.array(json.dumps(filters))
        np.savez_compressed(HERE / f"post_{name}.npz", **out)
        print(f"post_{name}: {ids.size} molecules, {len(planes)} planes", flush=True)


if __name__ == "__main__":
    main()
