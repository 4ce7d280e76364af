"""Golden outputs of the reference's Stark-table generation on a synthetic
Hamiltonian.

Run where the reference is checked out (its src directory given by
--reference-src or CTRAJ_REFERENCE_SRC); the GPU machines only read the .npz this writes.

    python tests/golden/make_golden_stark.py --reference-src <reference>/src

The reference builds Stark curves from the TlF Hamiltonian of the third-party
package centrex_TlF (stark_potential.py:5-7,22-27), which is not installed and
whose version the reference does not pin.  This script injects, through a stub
``centrex_TlF`` module, a synthetic Hamiltonian of the same form -- H(E, B) =
H0 + E_z HE + B_z HB in rad/s on a basis of rotor states |J, m> (rigid-rotor
energies, the dipole coupling of J and J +- 1 at equal m, a small Zeeman term
that lifts the +-m degeneracy, as the reference's B = 1e-4 T does) -- and runs
the reference's own code on it:

* ``stark_potential(state, Ezs)`` (stark_potential.py:9-67): the diagonalisation
  at every field, the adiabatic reordering ``reorder_evecs`` (:78-88), the
  state index and the energies in J;
* ``ElectrostaticLens.lens_acceleration`` with ``a_interp = None``
  (electrostatic_lens.py:174-213): the r grid, |E| = 2 V r / R^2, the Stark
  curve, ``-np.gradient(V_stark, dr) / mass`` and the interp1d it keeps.

centrex_TlF's ``find_closest_vector_idx`` is restated (the index of the
largest |<state|v_k>|).  What the fixture pins is the reference's algorithm
around the Hamiltonian, not TlF's Hamiltonian itself.
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
import refstubs  # noqa: E402

HERE = Path(__file__).resolve().parent
J_MAX = 4
STATE = (2, 0)  # |J, m> followed


def rotor_basis(j_max: int = J_MAX):
    return [(J, m) for J in range(j_max + 1) for m in range(-J, J + 1)]


def synthetic_hamiltonian(j_max: int = J_MAX):
    """(H0, HE, HB) in rad/s, rad/s per V/cm and rad/s per T."""
    from scipy.constants import c, hbar, pi

    basis = rotor_basis(j_max)
    n = len(basis)
    index = {s: k for k, s in enumerate(basis)}
    b_rot = 2 * pi * 6.686e9 / 2          # rad/s, E_J = B J (J + 1)
    dipole = 4.2283 * 1e-21 / c           # C m
    d_cm = dipole * 100.0 / hbar          # rad/s per (V/cm)
    H0 = np.zeros((n, n), complex)
    HE = np.zeros((n, n), complex)
    HB = np.zeros((n, n), complex)
    for (J, m), k in index.items():
        # rotor energy plus a small J- and m-dependent shift (hyperfine stand-in)
        H0[k, k] = b_rot * J * (J + 1) + 2 * pi * 1.3e5 * (J + 1) * m * m
        HB[k, k] = 2 * pi * 7.6e5 * m      # Zeeman, rad/s per T
        if (J + 1, m) in index:
            kk = index[(J + 1, m)]
            me = -d_cm * np.sqrt(((J + 1) ** 2 - m ** 2) / ((2 * J + 1) * (2 * J + 3)))
            HE[k, kk] = me
            HE[kk, k] = np.conj(me)
    return H0, HE, HB


class StubState:
    """Stands in for centrex_TlF's State: the basis vector of |J, m>."""

    def __init__(self, J, m):
        self.J, self.mJ = J, m

    def state_vector(self, QN):
        v = np.zeros(len(QN), complex)
        v[QN.index((self.J, self.mJ))] = 1.0
        return v

    def find_largest_component(self):
        return self

    def __mul__(self, k):  # the reference writes 1 * UncoupledBasisState(...)
        return self

    __rmul__ = __mul__

    def __repr__(self):
        return f"|J={self.J}, mJ={self.mJ}>"


def find_closest_vector_idx(state_vec, vector_array):
    """The column of vector_array with the largest |<state|v_k>|."""
    return int(np.argmax(np.abs(np.conj(state_vec) @ vector_array)))


def install_tlf_stub():
    H0, HE, HB = synthetic_hamiltonian()
    tlf = types.ModuleType("centrex_TlF")
    states = types.ModuleType("centrex_TlF.states")
    utils = types.ModuleType("centrex_TlF.states.utils")
    ham = types.ModuleType("centrex_TlF.hamiltonian")
    states.generate_uncoupled_states_ground = lambda Js: rotor_basis(J_MAX)
    states.UncoupledBasisState = lambda **kw: StubState(kw.get("J", 0), kw.get("mJ", 0))
    states.State = StubState
    utils.find_closest_vector_idx = find_closest_vector_idx
    ham.generate_uncoupled_hamiltonian_X = lambda QN: (H0, HE, HB)
    ham.generate_uncoupled_hamiltonian_X_function = (
        lambda parts: (lambda E, B: parts[0] + E[2] * parts[1] + B[2] * parts[2]))
    tlf.states, tlf.hamiltonian = states, ham
    states.utils = utils
    sys.modules.update({"centrex_TlF": tlf, "centrex_TlF.states": states, "centrex_TlF.states.utils": utils,
                        "centrex_TlF.hamiltonian": ham})
    return H0, HE, HB


class _Axes:
    def plot(self, *a, **k):
        pass


def main():
    ap = argparse.ArgumentParser()
    refstubs.add_argument(ap)
    args = ap.parse_args()
    sys.path.insert(0, str(HERE))
    H0, HE, HB = install_tlf_stub()  # before refstubs, so the stub modules above are used
    refstubs.install(refstubs.require(args.reference_src))
    import trajectories.stark_potential as sp
    from trajectories.beamline_elements.electrostatic_lens import ElectrostaticLens

    sp.plt = types.SimpleNamespace(subplots=lambda *a, **k: (None, _Axes()), show=lambda: None)
    state = StubState(*STATE)
    Ezs = np.linspace(0, 70000, 400)
    V_array = sp.stark_potential(state, Ezs)

    # the lens's table: lens_acceleration with a_interp = None
    d, V, mass = 1.75 * 0.0254, 27.6e3, (204.38 + 19.00) * 1.67e-27
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        os.mkdir("interpolation_functions")
        try:
            lens = ElectrostaticLens(name="ES lens", z0=1.0, L=0.6, d=d, V=V, mass=mass, state=state)
            lens.a_interp = None
            lens.lens_acceleration(np.array([1e-3, 0.0, 0.0]))
        finally:
            os.chdir(cwd)
    f = lens.a_interp
    np.savez_compressed(HERE / "stark_synthetic.npz", H0=H0, HE=HE, HB=HB, basis=np.array(rotor_basis()),
                        state=np.array(STATE), Ezs=Ezs, V_array=V_array, lens_d=d, lens_V=V, lens_mass=mass,
                        table_r=np.asarray(f.x), table_a=np.asarray(f.y))
    print(f"stark_synthetic: {len(rotor_basis())} states, {Ezs.size} fields, table {np.asarray(f.x).size} knots")


if __name__ == "__main__":
    main()
