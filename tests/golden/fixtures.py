"""Load the golden fixtures written by make_golden.py and rebuild their
beamlines from this package's classes (no reference import needed)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CASES = ["config0", "config1", "example_lens", "kat_circle", "kat_rect", "kat_plates", "kat_lens",
         "kat_honeycomb"]


def available():
    return [c for c in CASES if (HERE / f"{c}.npz").exists()]


def load(name):
    z = np.load(HERE / f"{name}.npz", allow_pickle=False)
    return {k: z[k] for k in z.files}


def build_beamline(fx, V=None, classes=None, drop=()):
    """Beamline from a fixture's spec: of this package's element classes, or,
    with ``classes`` (a function from class name to class, e.g. the
    reference's), of those; fields named in ``drop`` are left to the class's
    default.  Lens forces are this package's StarkForce (the reference's
    public ``a_interp`` field takes any callable) or a scipy interp1d."""
    import ctraj
    from scipy.interpolate import interp1d

    spec = json.loads(str(fx["spec"]))
    cls = classes or (lambda name: getattr(ctraj, name))
    elems = []
    for s in spec["elements"]:
        kw = {k: v for k, v in s.items() if k not in ("cls", "force") and k not in drop}
        if s["cls"] == "ElectrostaticLens":
            f = s["force"]
            knots = fx[f"table_{f['table']}_knots"]
            if f"table_{f['table']}_coef" in fx:
                kw["a_interp"] = ctraj.StarkForce(knots, fx[f"table_{f['table']}_coef"], V=f["V"],
                                                  R=f["R"], mass=f["mass"], field_order=f["order"])
            else:
                kw["a_interp"] = interp1d(knots, fx[f"table_{f['table']}_values"])
        elems.append(cls(s["cls"])(**kw))
    return cls("Beamline")(elems)


def expected_labels(fx):
    names = [str(s) for s in fx["label_names"]]
    return [names[i] for i in fx["label"]]


def traces(fx):
    """{molecule index: (rows, row_index or None, full length)}"""
    out = {}
    for k in fx:
        if k.startswith("trace_") and k.count("_") == 1:
            j = int(k.split("_")[1])
            idx = fx.get(f"trace_{j}_idx")
            n = int(fx[f"trace_{j}_len"]) if f"trace_{j}_len" in fx else fx[k].shape[0]
            out[j] = (fx[k], idx, n)
    return out
