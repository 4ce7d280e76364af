"""Stark-table generation (stark_potential.py:9-88, electrostatic_lens.py:191-209).

The reference diagonalises centrex_TlF's TlF Hamiltonian, absent here; the
fixture tests/golden/stark_synthetic.npz holds what the reference's own
stark_potential and lens_acceleration computed for a synthetic Hamiltonian of
the same form (make_golden_stark.py).  The oracle's numpy restatement must
reproduce it exactly; the GPU implementation (batched eigensolves, overlaps
on the device, permutations composed on the host) to rounding.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import stark_reference as ref

GOLDEN = Path(__file__).resolve().parent / "golden" / "stark_synthetic.npz"
REL = 1e-10  # GPU vs LAPACK eigenvalues: energies ~1e10 rad/s agree to ~1e-15 relative


def golden():
    z = np.load(GOLDEN)
    return {k: z[k] for k in z.files}


def state_vector(g):
    basis = [tuple(b) for b in g["basis"]]
    v = np.zeros(len(basis), complex)
    v[basis.index(tuple(g["state"]))] = 1.0
    return v


def test_oracle_matches_the_reference_run():
    g = golden()
    V = ref.stark_potential(g["H0"], g["HE"], g["HB"], state_vector(g), g["Ezs"])
    np.testing.assert_allclose(V, g["V_array"], rtol=1e-13, atol=0)
    W = lambda E: ref.stark_potential(g["H0"], g["HE"], g["HB"], state_vector(g), E / 100)
    r, a = ref.lens_table(W, float(g["lens_V"]), float(g["lens_d"]), float(g["lens_mass"]))
    np.testing.assert_array_equal(r, g["table_r"])
    np.testing.assert_allclose(a, g["table_a"], rtol=1e-9, atol=0)


def test_tracking_follows_the_state_through_crossings():
    """The J=2, m=0 curve crosses other states' energies: without the
    reordering, the energy at a fixed index of the sorted spectrum would jump
    to another state."""
    g = golden()
    H0, HE, HB = g["H0"], g["HE"], g["HB"]
    from scipy.constants import hbar

    _, V0 = np.linalg.eigh(H0 + 100.0 * HE + 1e-4 * HB)
    idx = int(np.argmax(np.abs(state_vector(g) @ V0)))
    sorted_only = np.array([np.linalg.eigh(H0 + Ez * HE + 1e-4 * HB)[0][idx] for Ez in g["Ezs"]]) * hbar
    assert not np.allclose(sorted_only, g["V_array"], rtol=1e-6, atol=0)
    # the tracked curve is smooth: no jumps between neighbouring fields
    assert np.max(np.abs(np.diff(g["V_array"], 2))) < 0.01 * np.ptp(g["V_array"])


def test_product_reorder_matches_the_reference_rule():
    from ctraj.stark import reorder_evecs

    rng = np.random.default_rng(0)
    A = rng.normal(size=(6, 6)) + 1j * rng.normal(size=(6, 6))
    E, V = np.linalg.eigh(A + A.conj().T)
    perm = rng.permutation(6)
    E2, V2 = reorder_evecs(V[:, perm], E[perm], V)
    np.testing.assert_array_equal(E2, E)
    E3, V3 = ref.reorder(V[:, perm], E[perm], V)
    np.testing.assert_array_equal(E2, E3)


def test_hamiltonian_shapes_are_checked():
    from ctraj.stark import LinearHamiltonian

    with pytest.raises(ValueError):
        LinearHamiltonian(np.eye(3), np.eye(3), np.eye(2))


@pytest.mark.gpu
def test_gpu_curve_matches_the_reference_run():
    from ctraj.stark import LinearHamiltonian, stark_potential

    g = golden()
    H = LinearHamiltonian(g["H0"], g["HE"], g["HB"])
    V = stark_potential(state_vector(g), g["Ezs"], H)
    np.testing.assert_allclose(V, g["V_array"], rtol=REL, atol=0)


@pytest.mark.gpu
def test_gpu_lens_table_matches_the_reference_run():
    import ctraj
    from ctraj.stark import LinearHamiltonian, lens_table_from_hamiltonian

    g = golden()
    H = LinearHamiltonian(g["H0"], g["HE"], g["HB"])
    lens = ctraj.ElectrostaticLens(name="ES lens", z0=1.0, L=0.6, d=float(g["lens_d"]), V=float(g["lens_V"]))
    assert lens.mass == float(g["lens_mass"])
    f = lens_table_from_hamiltonian(lens, state_vector(g), H)
    np.testing.assert_array_equal(f.x, g["table_r"])
    # a = -gradient(V) / m: differences of neighbouring energies, ~1e-4 of V
    np.testing.assert_allclose(f.y, g["table_a"], rtol=1e-6, atol=1e-9 * np.abs(g["table_a"]).max())


@pytest.mark.gpu
def test_lens_built_from_the_hamiltonian_propagates():
    """The generated table drives a lens on the device (FP64 equals the oracle)."""
    import ctraj
    from ctraj.compiler import compile_beamline
    from ctraj.engine import Engine
    from ctraj.stark import LinearHamiltonian, lens_table_from_hamiltonian
    from oracle import oracle

    g = golden()
    H = LinearHamiltonian(g["H0"], g["HE"], g["HB"])
    lens = ctraj.ElectrostaticLens(name="ES lens", z0=0.5, L=0.3, d=float(g["lens_d"]), V=float(g["lens_V"]))
    lens.a_interp = lens_table_from_hamiltonian(lens, state_vector(g), H)
    bl = ctraj.Beamline([lens, ctraj.CircularAperture("Detection plane", 1.5, 0.0, d=np.inf)])
    cb = compile_beamline(bl)
    rng = np.random.default_rng(5)
    n = 2000
    ics = np.vstack([rng.normal(0, 3e-3, n), rng.normal(0, 3e-3, n), np.zeros(n), rng.normal(0, 3, n),
                     rng.normal(0, 3, n), rng.normal(184, 16, n)])
    eng = Engine(0)
    try:
        r = eng.run(cb, n, precision=64, ics=ics, outputs=True)
    finally:
        eng.close()
    o = oracle.run(cb, ics)
    np.testing.assert_array_equal(r.label, o["label"])
    np.testing.assert_array_equal(r.final, o["final"])
