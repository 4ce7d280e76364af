"""The drop-in boundary with the reference's own objects.

A user switching from the reference hands TrajectorySimulator.run_simulation
the reference's Beamline, element and Distribution instances.  The run sees
them only through ctraj.compiler.compile_beamline (C element table, counter
labels, force and mesh tables) and ctraj.distributions.device_spec (device
draw descriptors), so the reference's objects and this package's mirror
classes, built from the same arguments, must compile to the same bytes:

* tests/golden/dropin.npz holds what the reference's objects compiled to
  (tests/golden/make_golden_dropin.py, run against the reference), for every
  golden beamline, a beamline of default-constructed elements (including a
  lens with an interp1d table and the reference's d, dz, V and mass
  defaults) and seven distributions -- checked here without the reference;
* where the reference's src directory is available (CTRAJ_REFERENCE_SRC), the
  same is redone live from the reference's classes in a subprocess.

Reference classes: beamline.py:12-55, apertures.py:22-210,
electrostatic_lens.py:23-46, meshes.py:26-62, distributions.py:55-185.
"""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import fixtures
import make_golden_dropin as gen
import refstubs
from ctraj.compiler import compile_beamline
from ctraj.distributions import device_spec

HERE = Path(__file__).resolve().parent
GOLDEN = HERE / "golden" / "dropin.npz"


def _mirror(name):
    """This package's classes, built from the arguments the fixture gave the reference's."""
    fx = gen.defaults_fixture() if name == "defaults" else fixtures.load(name)
    return compile_beamline(fixtures.build_beamline(fx, drop=("dt",)))


def _check(z, name, cb):
    assert bytes(cb.elements) == z[f"{name}_elements"].tobytes(), name
    assert list(cb.labels) == [str(s) for s in z[f"{name}_labels"]], name
    assert len(cb.tables) == int(z[f"{name}_n_tables"]), name
    for k, t in enumerate(cb.tables):
        assert t.kind == int(z[f"{name}_table{k}_kind"])
        np.testing.assert_array_equal(t.knots, z[f"{name}_table{k}_knots"])
        for f in ("coef", "values"):
            key = f"{name}_table{k}_{f}"
            assert (getattr(t, f) is None) == (key not in z), key
            if key in z:
                np.testing.assert_array_equal(getattr(t, f), z[key])


def _check_distributions(z):
    import ctraj

    for k, (role, name, kw) in enumerate(json.loads(str(z["distributions"]))):
        spec = device_spec(getattr(ctraj, name)(**kw), role)
        assert spec is not None, name
        assert bytes(spec) == z[f"dist_{k}"].tobytes(), (name, kw)


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN)
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("name", gen.CASES + ["defaults"])
def test_mirror_compiles_like_the_reference_objects(golden, name):
    _check(golden, name, _mirror(name))


def test_distributions_give_the_reference_objects_descriptors(golden):
    _check_distributions(golden)


def test_defaults_beamline_covers_the_reference_lens_defaults(golden):
    """The default-constructed lens: interp1d table, field order 0, and the
    reference's own d, dz, V and mass (electrostatic_lens.py:29-46)."""
    from ctraj import _abi

    raw = golden["defaults_elements"].tobytes()
    n = len(raw) // __import__("ctypes").sizeof(_abi.Element)
    els = (_abi.Element * n).from_buffer_copy(raw)
    lens = [e for e in els if e.type == _abi.ELECTROSTATIC_LENS][0]
    assert lens.field_order == 0 and lens.step_mode == _abi.STEP_DZ
    assert lens.p[0] == 1.75 * 0.0254 and lens.p[1] == 1e-3          # d, dz
    assert lens.p[3] == 27.6e3 and lens.p[5] == (204.38 + 19.00) * 1.67e-27  # V, mass
    assert lens.p[4] == lens.p[0] / 2


@pytest.mark.skipif(refstubs.reference_src() is None,
                    reason="the reference's src directory is not available (set CTRAJ_REFERENCE_SRC)")
def test_live_reference_objects(tmp_path):
    out = tmp_path / "dropin_live.npz"
    subprocess.run([sys.executable, str(HERE / "golden" / "make_golden_dropin.py"), "--reference-src",
                    refstubs.reference_src(), "--out", str(out)], check=True, capture_output=True)
    z = np.load(out)
    live = {k: z[k] for k in z.files}
    for name in gen.CASES + ["defaults"]:
        _check(live, name, _mirror(name))
    _check_distributions(live)
