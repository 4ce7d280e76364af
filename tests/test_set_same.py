"""Setting a force table or the beamline that a context already holds, bit for
bit, changes nothing (the drop-in compiles and sets them before every
run_simulation): the next runs give the same results as before, and a table
or beamline that differs in one value is taken as new (ctraj_set_force_table,
ctraj_set_beamline)."""
import ctypes

import numpy as np
import pytest

from ctraj import _abi
from ctraj.compiler import compile_beamline
from ctraj.workloads import lens_beamline, source

pytestmark = pytest.mark.gpu


def _specs():
    from ctraj.distributions import device_spec

    xd, vd = source()
    return device_spec(xd, "position"), device_spec(vd, "velocity")


def _set(eng, cb):
    for tid, t in enumerate(cb.tables):
        st = t.as_struct()
        _abi.check(eng.lib.ctraj_set_force_table(eng.ctx, tid, ctypes.byref(st)), eng.lib)
    _abi.check(eng.lib.ctraj_set_beamline(eng.ctx, cb.elements, cb.n_elements, len(cb.labels)), eng.lib)


def test_setting_the_same_table_and_beamline_again_changes_nothing():
    from ctraj.engine import Engine

    xs, vs = _specs()
    eng = Engine(0)
    try:
        bl = lens_beamline()
        cb = compile_beamline(bl)
        first = eng.run(cb, 200_000, xdist=xs, vdist=vs, seed=3)
        for _ in range(2):  # a freshly compiled copy of the same beamline, set by hand and by the engine
            again = compile_beamline(bl)
            _set(eng, again)
            r = eng.run(again, 200_000, xdist=xs, vdist=vs, seed=3)
            np.testing.assert_array_equal(r.counts, first.counts)
            assert (r.molecule_steps, r.lens_steps) == (first.molecule_steps, first.lens_steps)
        # one coefficient changed: a new table, rebuilt (the lens steps change)
        changed = compile_beamline(bl)
        t = changed.tables[0]
        t.coef = np.array(t.coef, dtype=np.float64, copy=True)
        t.coef[:, 2] *= 1.5
        _set(eng, changed)
        r = eng.run(changed, 200_000, xdist=xs, vdist=vs, seed=3)
        assert r.lens_steps != first.lens_steps
        # and back to the original table: the original results
        _set(eng, cb)
        r = eng.run(cb, 200_000, xdist=xs, vdist=vs, seed=3)
        np.testing.assert_array_equal(r.counts, first.counts)
        assert r.lens_steps == first.lens_steps
        # a beamline with one element moved is taken as new
        moved = compile_beamline(bl)
        moved.elements[0].p[0] = moved.elements[0].p[0] * 0.5  # half the first aperture's diameter
        _set(eng, moved)
        r = eng.run(moved, 200_000, xdist=xs, vdist=vs, seed=3)
        assert r.counts[0] != first.counts[0]
    finally:
        eng.close()
