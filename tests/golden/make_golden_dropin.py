"""Pin the drop-in boundary: what this package's beamline compiler and
distribution descriptors make of the reference's own objects.

Run where the reference is checked out (its src directory given by
--reference-src or CTRAJ_REFERENCE_SRC); the GPU machines never run this.

    python tests/golden/make_golden_dropin.py --reference-src <reference>/src

The drop-in promise is that a user hands ``TrajectorySimulator.run_simulation``
the reference's own ``Beamline``, element and ``Distribution`` objects and gets
the same run as with this package's mirror classes.  The run sees those
objects only through ``ctraj.compiler.compile_beamline`` (the C element table,
the counter labels and the force / mesh tables) and
``ctraj.distributions.device_spec`` (the device-draw descriptors), so this
script builds, from the reference's classes:

* the beamline of every golden fixture (its spec; the lens-only extension
  field ``dt`` is left out, since the reference's lens has none, so its own
  ``dz`` default applies), with the fixture's force tables in ``a_interp``;
* a beamline of elements constructed with only name, z0 and L, so every other
  field is the reference's default -- including an ``ElectrostaticLens`` with
  an interp1d ``a_interp`` and the reference's ``d``, ``dz``, ``V`` and
  ``mass`` defaults;
* distribution objects with default and with explicit fields;

and stores what the compiler and ``device_spec`` return for them in
dropin.npz.  tests/test_dropin_reference.py requires this package's mirror
classes, built from the same arguments, to give the same bytes.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT / "centrex-molecule-trajectories_gb300"))
import refstubs  # noqa: E402

# fixtures whose beamlines are compiled (every golden case)
CASES = ["config0", "config1", "example_lens", "kat_circle", "kat_rect", "kat_plates", "kat_lens",
         "kat_honeycomb"]

# distributions: (role, class name, keyword arguments)
DISTRIBUTIONS = [
    ("position", "GaussianPositionDistribution", {}),
    ("position", "GaussianPositionDistribution", {"sigmax": 1.5e-3, "sigmay": 1.5e-3, "z": 0.0}),
    ("position", "CeNTREXPositionDistribution", {}),
    ("position", "CeNTREXPositionDistribution", {"d": 0.01, "z": 0.002}),
    ("velocity", "CeNTREXVelocityDistribution", {}),
    ("velocity", "CeNTREXVelocityDistribution", {"sigmax": 20.0, "sigmay": 20.0}),
    ("velocity", "CeNTREXVelocityDistribution", {"vx": 1.0, "sigmax": 2.0, "vy": -3.0, "sigmay": 4.0,
                                                 "vz": 150.0, "sigmaz": 12.0}),
]


def defaults_spec():
    """Elements given only name, z0 and L (and the lens its interp1d table):
    every other field is the class's default."""
    return [
        dict(cls="CircularAperture", name="Aperture", z0=0.1, L=0.01),
        dict(cls="RectangularAperture", name="Rectangle", z0=0.3, L=0.01),
        dict(cls="ElectrostaticLens", name="ES lens", z0=0.6, L=0.6, force=dict(table="radial")),
        dict(cls="FieldPlates", name="Field plates", z0=1.5, L=1.0),
        dict(cls="Honeycomb", name="Honeycomb", z0=2.6, L=0.02),
        dict(cls="CircularAperture", name="Detection plane", z0=3.0, L=0.0, d=float("inf")),
    ]


def defaults_fixture():
    """A fixture-shaped dict for defaults_spec: its lens takes example_lens's radial table."""
    import fixtures

    ex = fixtures.load("example_lens")
    spec = json.loads(str(ex["spec"]))
    lens = [s for s in spec["elements"] if s["cls"] == "ElectrostaticLens"][0]
    table = lens["force"]["table"]
    elems = defaults_spec()
    for e in elems:
        if e["cls"] == "ElectrostaticLens":
            e["force"]["table"] = table
    return {"spec": np.array(json.dumps({"elements": elems})),
            f"table_{table}_knots": ex[f"table_{table}_knots"],
            f"table_{table}_values": ex[f"table_{table}_values"]}


def reference_classes():
    import trajectories.beamline as beamline
    import trajectories.beamline_elements as elements
    import trajectories.distributions as distributions

    def cls(name):
        for mod in (elements, beamline, distributions):
            if hasattr(mod, name):
                return getattr(mod, name)
        raise KeyError(name)

    return cls


def compiled(cb, prefix):
    """The compiler's output as npz entries."""
    out = {f"{prefix}_elements": np.frombuffer(bytes(cb.elements), np.uint8),
           f"{prefix}_labels": np.array(cb.labels, dtype=str),
           f"{prefix}_n_tables": np.array(len(cb.tables))}
    for k, t in enumerate(cb.tables):
        out[f"{prefix}_table{k}_kind"] = np.array(t.kind)
        out[f"{prefix}_table{k}_knots"] = t.knots
        for f in ("coef", "values"):
            v = getattr(t, f)
            if v is not None:
                out[f"{prefix}_table{k}_{f}"] = v
    return out


def dist_bytes(spec):
    return np.frombuffer(bytes(spec), np.uint8) if spec is not None else np.zeros(0, np.uint8)


def main():
    ap = argparse.ArgumentParser()
    refstubs.add_argument(ap)
    ap.add_argument("--out", default=str(HERE / "dropin.npz"))
    args = ap.parse_args()
    refstubs.install(refstubs.require(args.reference_src))
    import make_golden

    make_golden.install_mesh_stand_ins()
    import fixtures
    from ctraj.compiler import compile_beamline
    from ctraj.distributions import device_spec

    cls = reference_classes()
    out = {"cases": np.array(CASES + ["defaults"], dtype=str)}
    for name in CASES:
        bl = fixtures.build_beamline(fixtures.load(name), classes=cls, drop=("dt",))
        assert type(bl).__module__.startswith("trajectories"), type(bl)
        out.update(compiled(compile_beamline(bl), name))
    bl = fixtures.build_beamline(defaults_fixture(), classes=cls)
    out.update(compiled(compile_beamline(bl), "defaults"))
    for k, (role, name, kw) in enumerate(DISTRIBUTIONS):
        d = cls(name)(**kw)
        out[f"dist_{k}"] = dist_bytes(device_spec(d, role))
    out["distributions"] = np.array(json.dumps(DISTRIBUTIONS))
    np.savez_compressed(args.out, **out)
    print(f"dropin: {len(CASES) + 1} beamlines, {len(DISTRIBUTIONS)} distributions")


if __name__ == "__main__":
    main()
