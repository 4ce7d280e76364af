"""Record the HDF5 layout the reference writes for a simulation result.

Run where the reference is checked out (its src directory given by
--reference-src or CTRAJ_REFERENCE_SRC).  h5py is replaced by the in-memory recorder fake_h5py.py
(h5py is not installed here), the reference's own classes propagate a few
molecules of the ``config1`` fixture (aperture + hexapole lens), and the
reference's ``SimulationResult.save_to_hdf`` writes them; the recorded groups,
attributes and datasets go to hdf_layout.npz.

    python tests/golden/make_golden_hdf.py --reference-src <reference>/src
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
N_MOLECULES = 40


def to_json(v):
    if isinstance(v, (np.floating, float)):
        return float(v)
    if isinstance(v, (np.integer, int, np.bool_, bool)):
        return v.item() if hasattr(v, "item") else v
    return str(v)


def main():
    ap = argparse.ArgumentParser()
    refstubs.add_argument(ap)
    args = ap.parse_args()
    sys.path.insert(0, str(HERE))
    import fake_h5py

    sys.modules["h5py"] = fake_h5py  # before the reference imports it
    import make_golden
    refstubs.install(refstubs.require(args.reference_src))
    from trajectories.distributions import CeNTREXVelocityDistribution, GaussianPositionDistribution
    from trajectories.molecule import Molecule
    from trajectories.trajectory_simulator import Counter, SimulationResult

    fx = np.load(HERE / "config1.npz")
    specs = json.loads(str(fx["spec"]))["elements"]
    beamline = make_golden.build_reference_beamline(specs, make_golden.make_tables())
    lenses = [(e, s) for e, s in zip(beamline.elements, sorted(specs, key=lambda s: s["z0"]))
              if s["cls"] == "ElectrostaticLens"]
    names = [str(s) for s in fx["label_names"]]
    labels = [names[k] for k in fx["label"]]
    # a mix of labels: the first molecules of each kind
    ids = []
    for want in sorted(set(labels)):
        ids += [i for i, s in enumerate(labels) if s == want][: N_MOLECULES // len(set(labels)) + 1]
    ids = sorted(ids)[:N_MOLECULES]
    ics = fx["ics"]
    counter = Counter()
    molecules = []
    for i in ids:
        for e, s in lenses:
            if s.get("dt") is not None:
                e.dz = ics[5, i] * s["dt"]
        m = Molecule()
        m.init_trajectory(beamline, ics[:3, i], ics[3:, i])
        beamline.propagate_through(m)
        counter.increment_counter(m.aperture_hit)
        molecules.append(m)
    result = SimulationResult(counter, beamline, GaussianPositionDistribution(1.5e-3, 1.5e-3, 0.0),
                              CeNTREXVelocityDistribution(sigmax=20.0, sigmay=20.0), molecules)
    path = "reference.h5"
    result.save_to_hdf(path, "run")
    store = fake_h5py.snapshot(path)
    groups = {g: {k: to_json(v) for k, v in d["attrs"].items()} for g, d in store.items()}
    out = {"groups": np.array(json.dumps(groups)), "ids": np.array(ids, np.int64)}
    for g, d in store.items():
        for name, arr in d["datasets"].items():
            out[f"ds::{g}::{name}"] = arr
    np.savez_compressed(HERE / "hdf_layout.npz", **out)
    print(f"hdf_layout: {len(groups)} groups, {sum(len(d['datasets']) for d in store.values())} datasets")


if __name__ == "__main__":
    main()
