"""z-plane post-processing (ctraj_plane, ctraj.post_processing) against the
reference's own find_radial_pos_dist / find_vel_dist outputs
(tests/golden/post_*.npz, made by make_golden_post.py with the reference).

FP64 replays follow the reference's trajectory rows exactly; the step to the
plane uses dt * dt where the reference's numpy scalar ``dt ** 2`` may differ in
the last bit, so states are compared to 1e-13 relative (and most are equal).
"""
from pathlib import Path

import numpy as np
import pytest

import fixtures

GOLDEN = Path(__file__).resolve().parent / "golden"
POST_CASES = [c for c in ("config0", "config1", "example_lens") if (GOLDEN / f"post_{c}.npz").exists()]
REL = 1e-13


def load_post(case):
    import json

    z = np.load(GOLDEN / f"post_{case}.npz")
    out = {k: z[k] for k in z.files}
    out["filters"] = json.loads(str(out["filters"]))
    return out


def test_take_timestep_matches_the_formula():
    from ctraj.post_processing import take_timestep

    x, v = take_timestep(np.array([1.0, 2.0, 3.0]), np.array([0.1, 0.2, 10.0]), np.array([0.0, -9.8, 0.0]), 0.5)
    np.testing.assert_allclose(x, [1.05, 2.1 - 9.8 * 0.125, 8.0])
    np.testing.assert_allclose(v, [0.1, 0.2 - 4.9, 10.0])


@pytest.mark.gpu
@pytest.mark.parametrize("case", POST_CASES)
def test_plane_states_match_reference_post_processing(case):
    from ctraj.compiler import compile_beamline
    from ctraj.engine import Engine

    fx = fixtures.load(case)
    post = load_post(case)
    cb = compile_beamline(fixtures.build_beamline(fx))
    labels = fixtures.expected_labels(fx)
    ids = post["ids"]
    n = fx["ics"].shape[1]
    eng = Engine(0)
    try:
        n_exact = n_total = 0
        for k, z in enumerate(post["planes"]):
            st = eng.plane(cb, n, ids, float(z), precision=64, ics=fx["ics"])
            for f, flt in enumerate(post["filters"]):
                keep = np.ones(ids.size, bool) if flt is None else np.isin([labels[i] for i in ids], flt)
                got = st[keep]
                got = got[got[:, 6] > 0]
                ref_pos, ref_vel = post[f"pos_{k}_{f}"], post[f"vel_{k}_{f}"]
                assert got.shape[0] == ref_pos.shape[0], (case, z, flt)
                if got.shape[0] == 0:
                    continue
                np.testing.assert_allclose(got[:, 0:2], ref_pos, rtol=REL, atol=1e-18)
                np.testing.assert_allclose(got[:, 3:6], ref_vel, rtol=REL, atol=1e-18)
                n_exact += int(np.sum(got[:, 0:2] == ref_pos) + np.sum(got[:, 3:6] == ref_vel))
                n_total += ref_pos.size + ref_vel.size
        assert n_exact >= 0.95 * n_total
    finally:
        eng.close()


@pytest.mark.gpu
def test_drop_in_post_processing_api():
    import ctraj
    from ctraj.post_processing import find_radial_pos_dist, find_vel_dist

    case = "config1"
    fx = fixtures.load(case)
    post = load_post(case)
    bl = fixtures.build_beamline(fx)
    sim = ctraj.TrajectorySimulator(precision=64)
    n = fx["ics"].shape[1]
    sim.run_simulation(bl, "post", N_traj=n, apertures_of_interest=["Detected", "Inside lens"], ics=fx["ics"])
    np.testing.assert_array_equal(sim.result.replay["ids"], post["ids"])
    for k, z in enumerate(post["planes"]):
        for f, flt in enumerate(post["filters"]):
            np.testing.assert_allclose(find_radial_pos_dist(sim.result, float(z), flt), post[f"pos_{k}_{f}"],
                                       rtol=REL, atol=1e-18)
            np.testing.assert_allclose(find_vel_dist(sim.result, float(z), flt), post[f"vel_{k}_{f}"],
                                       rtol=REL, atol=1e-18)
