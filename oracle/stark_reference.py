"""TEST INFRASTRUCTURE, NOT PRODUCT CODE: numpy restatement of the reference's
Stark-curve generation, the checker of ctraj.stark.stark_potential.

stark_potential   stark_potential.py:9-67 -- eigh of H(E, B) = H0 + E_z HE +
                  B_z HB at each field in turn, the basis reordered against the
                  previous one (reorder_evecs, :78-88), the state's index from
                  the eigenbasis at 100 V/cm, energies times hbar
lens_table        electrostatic_lens.py:191-209 -- the a(r) interp1d the lens
                  builds from that curve when a_interp is None

Pinned by tests/golden/stark_synthetic.npz (make_golden_stark.py runs the
reference's own code on a synthetic Hamiltonian).  Only tests/ import it.
"""
from __future__ import annotations

import numpy as np


def reorder(V_in, E_in, V_ref):
    overlap = np.absolute(np.matmul(np.conj(V_in.T), V_ref))
    index = np.argsort(np.argmax(overlap, axis=1))
    return E_in[index], V_in[:, index]


def stark_potential(H0, HE, HB, state_vec, Ezs, B=1e-4, E_start=100.0):
    from scipy.constants import hbar

    def H(Ez):
        return H0 + Ez * HE + B * HB

    _, V_ref = np.linalg.eigh(H(E_start))
    V_ref_0 = V_ref
    energies_all = np.zeros((len(Ezs), H0.shape[0]))
    for i, Ez in enumerate(Ezs):
        D, V = np.linalg.eigh(H(Ez))
        energies, evecs = reorder(V, D, V_ref)
        energies_all[i, :] = energies
        V_ref = evecs
    state_i = int(np.argmax(np.abs(np.conj(state_vec) @ V_ref_0)))
    return energies_all[:, state_i] * hbar


def lens_table(W, V, d, mass, dr=1e-4):
    """(r_values, a_values) of the lens table from W(E in V/m) in J."""
    r_values = np.linspace(0, d / 2 * 1.01, int(np.round(d / 2 / dr)))
    E_values = 2 * V / ((d / 2) ** 2) * r_values
    a_values = -np.gradient(W(E_values), dr) / mass
    return r_values, a_values
