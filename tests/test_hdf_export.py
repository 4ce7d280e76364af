"""HDF5 export of a simulation result in the reference's layout.

h5py is not installed here or on the GPU machines; both this package and the
reference write through the in-memory recorder tests/golden/fake_h5py.py.
hdf_layout.npz holds what the reference's SimulationResult.save_to_hdf wrote
for 40 molecules of the config1 fixture (make_golden_hdf.py); the same result
rebuilt from this package's classes must write the same groups, attributes
and datasets.  Excluded: the lens's ``state`` (a TlF state object in the
reference, its repr stored), its ``dz`` (the reference realises the fixed
time step by rewriting dz per molecule, so it stores the last molecule's),
and this package's lens extensions ``dt`` / ``scheme``.
"""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

import fixtures

GOLDEN = Path(__file__).resolve().parent / "golden"
LENS_SKIP = {"state", "dz", "dt", "scheme"}


@pytest.fixture()
def fake_h5py(monkeypatch):
    import fake_h5py as fk

    monkeypatch.setitem(sys.modules, "h5py", fk)
    fk.STORES.clear()
    return fk


def golden():
    z = np.load(GOLDEN / "hdf_layout.npz")
    groups = json.loads(str(z["groups"]))
    data = {k[4:]: z[k] for k in z.files if k.startswith("ds::")}
    return groups, data, z["ids"]


def rebuild(groups, data):
    """The reference's result, from this package's classes."""
    import ctraj
    from ctraj.molecule import Molecule, Trajectory

    fx = fixtures.load("config1")
    bl = fixtures.build_beamline(fx)
    counter = ctraj.Counter()
    counter.counter_dict = dict(groups["run/counter"])
    mols = []
    k = 0
    while f"run/trajectories/molecule_{k}" in groups:
        g = f"run/trajectories/molecule_{k}"
        m = Molecule(alive=bool(groups[g]["alive"]))
        m.trajectory = Trajectory(data[f"{g}::x"], data[f"{g}::v"], data[f"{g}::a"], data[f"{g}::t"])
        m.set_aperture_hit(groups[g]["aperture_hit"])
        mols.append(m)
        k += 1
    return ctraj.SimulationResult(counter, bl, ctraj.GaussianPositionDistribution(1.5e-3, 1.5e-3, 0.0),
                                  ctraj.CeNTREXVelocityDistribution(sigmax=20.0, sigmay=20.0), mols)


def test_result_layout_matches_the_reference(fake_h5py):
    groups, data, _ = golden()
    res = rebuild(groups, data)
    res.save_to_hdf("ours.h5", "run")
    store = fake_h5py.snapshot("ours.h5")
    assert set(store) == set(groups)
    for g, attrs in groups.items():
        ours = store[g]["attrs"]
        skip = LENS_SKIP if attrs.get("class") == "ElectrostaticLens" else set()
        want = {k: v for k, v in attrs.items() if k not in skip}
        got = {k: v for k, v in ours.items() if k not in skip}
        assert set(got) == set(want), (g, set(got) ^ set(want))
        for k, v in want.items():
            assert (got[k] == v) or (isinstance(v, float) and np.isclose(float(got[k]), v, rtol=0, atol=0)), (g, k)
        for name, arr in store[g]["datasets"].items():
            np.testing.assert_array_equal(arr, data[f"{g}::{name}"])
    assert sum(len(d["datasets"]) for d in store.values()) == len(data)


def test_existing_run_asks_before_overwriting(fake_h5py, monkeypatch):
    groups, data, _ = golden()
    res = rebuild(groups, data)
    res.save_to_hdf("twice.h5", "run")
    monkeypatch.setattr("builtins.input", lambda prompt: "n")
    res.save_to_hdf("twice.h5", "run")  # declined: nothing changes
    monkeypatch.setattr("builtins.input", lambda prompt: "y")
    res.save_to_hdf("twice.h5", "run")  # overwritten
    assert "run/trajectories/molecule_0" in fake_h5py.snapshot("twice.h5")
    with pytest.raises(ValueError, match="counter"):
        res.counter.save_to_hdf("twice.h5", "run")


def test_gaussian_distribution_is_not_saved(fake_h5py):
    import ctraj

    with pytest.raises(NotImplementedError):
        ctraj.GaussianDistribution(0.0, 1.0).save_to_hdf("x.h5", "run", "g")
