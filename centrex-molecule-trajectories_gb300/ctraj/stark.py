"""Stark-shift tables and the lens force laws built from them.

The reference turns a Stark curve into a radial acceleration table once per
lens (electrostatic_lens.py:194-213): r grid, |E| = 2 V r / R^2, W(E) from the
TlF Hamiltonian (stark_potential.py:9-67, needs the absent ``centrex_TlF``),
a(r) = -dW/dr / m, then a linear ``interp1d``.  This module supplies:

* :class:`TwoLevelStark` -- the analytic two-level curve
  W(E) = -(sqrt(a^2 + (d E)^2) - a) used by the lens workloads (a = h * f,
  d the dipole moment), in joules for E in V/m;
* :class:`StarkForce` -- a cubic-spline table of W(E) on uniform knots plus
  the lens field model |E| = alpha r^n.  It is a callable r -> a_r that the
  reference accepts as ``ElectrostaticLens.a_interp`` and that the compiler
  uploads as a piecewise-cubic table;
* :func:`reference_radial_table` -- the reference's own interp1d
  construction (:194-209) fed from any W(E) instead of ``stark_potential``;
* :func:`stark_potential` -- the reference's Stark curve of a state
  (stark_potential.py:9-88) for any Hamiltonian of the form H0 + E_z HE +
  B_z HB (:class:`LinearHamiltonian`), with the eigensolves batched on the
  GPU, and :func:`lens_table_from_hamiltonian`, the lens table the reference
  builds from it when ``a_interp`` is None.  centrex_TlF, which supplies the
  TlF matrices in the reference, is not available here: the caller brings
  the matrices.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
from scipy.constants import h as PLANCK
from scipy.constants import c as LIGHT
from scipy.interpolate import CubicSpline, interp1d

DEBYE = 1e-21 / LIGHT  # C m
TLF_MASS = (204.38 + 19.00) * 1.67e-27  # kg, electrostatic_lens.py:44-46

__all__ = ["DEBYE", "TLF_MASS", "TwoLevelStark", "StarkForce", "hexapole_force",
           "reference_radial_table", "field_coefficient", "LinearHamiltonian", "reorder_evecs",
           "stark_potential", "lens_table_from_hamiltonian"]


@dataclass(frozen=True)
class TwoLevelStark:
    """W(E) = sign (sqrt(a^2 + (d E)^2) - a) with a = h * splitting_hz, d =
    dipole_debye * D; sign -1 (the workloads' curve) is the high-field-seeking
    state, which a hexapole defocuses, +1 the low-field-seeking one, which it
    focuses."""

    splitting_hz: float = 6.7e9
    dipole_debye: float = 4.2
    sign: float = -1.0

    @property
    def a(self) -> float:
        return PLANCK * self.splitting_hz

    @property
    def d(self) -> float:
        return self.dipole_debye * DEBYE

    def __call__(self, E):
        E = np.asarray(E, dtype=np.float64)
        return self.sign * (np.sqrt(self.a ** 2 + (self.d * E) ** 2) - self.a)

    def spline(self, n_knots: int = 4096, E_max: float = 1e7) -> CubicSpline:
        """Cubic spline (scipy default not-a-knot) of W on n_knots uniform knots in [0, E_max]."""
        E = np.linspace(0.0, E_max, n_knots)
        return CubicSpline(E, self(E))


def field_coefficient(V: float, R: float, order: int) -> float:
    """alpha in |E| = alpha r^n: 2 V / R^2 for n = 1 (the reference's model,
    electrostatic_lens.py:200) and 3 V / R^3 for n = 2 (hexapole)."""
    if order == 1:
        return 2.0 * V / R ** 2
    if order == 2:
        return 3.0 * V / R ** 3
    raise ValueError(f"field order must be 1 or 2, got {order}")


@dataclass
class StarkForce:
    """Radial acceleration a_r(r) = -W'(|E|) d|E|/dr / m with |E| = alpha r^n.

    ``knots`` (uniform) and ``coef`` ((n_knots - 1, 4), scipy PPoly order per
    interval) define W(E).  Calling the object evaluates a_r exactly like the
    device's FP64 path: E = alpha*(r*r) (n = 2) or alpha*r (n = 1), W' by the
    PPoly nu = 1 evaluation, then -(W' * dE/dr) / mass.
    """

    knots: np.ndarray
    coef: np.ndarray
    V: float
    R: float
    mass: float = TLF_MASS
    field_order: int = 2
    alpha: float = field(init=False)

    def __post_init__(self):
        self.knots = np.ascontiguousarray(self.knots, dtype=np.float64)
        self.coef = np.ascontiguousarray(self.coef, dtype=np.float64)
        if self.coef.shape != (self.knots.size - 1, 4):
            raise ValueError("coef must have shape (n_knots - 1, 4)")
        dk = np.diff(self.knots)
        if not np.allclose(dk, dk[0], rtol=1e-9, atol=0.0):
            raise ValueError("Stark table knots must be uniformly spaced")
        self.alpha = field_coefficient(self.V, self.R, self.field_order)
        self._pp = None

    @classmethod
    def from_spline(cls, spline: CubicSpline, V: float, R: float, mass: float = TLF_MASS,
                    field_order: int = 2) -> "StarkForce":
        return cls(knots=spline.x, coef=np.ascontiguousarray(spline.c.T), V=V, R=R, mass=mass,
                   field_order=field_order)

    def with_voltage(self, V: float) -> "StarkForce":
        return StarkForce(self.knots, self.coef, V, self.R, self.mass, self.field_order)

    def dWdE(self, E):
        if self._pp is None:
            from scipy.interpolate import PPoly

            self._pp = PPoly(np.ascontiguousarray(self.coef.T), self.knots)
        return self._pp(E, 1)

    def __call__(self, r):
        if self.field_order == 2:
            E = self.alpha * (r * r)
            return -(self.dWdE(E) * (2.0 * self.alpha * r)) / self.mass
        E = self.alpha * r
        return -(self.dWdE(E) * self.alpha) / self.mass


def hexapole_force(V: float = 30e3, R: float = 17.5e-3, splitting_hz: float = 6.7e9,
                   dipole_debye: float = 4.2, n_knots: int = 4096, E_max: float = 1e7,
                   mass: float = TLF_MASS, low_field_seeker: bool = False) -> StarkForce:
    """Hexapole lens, |E| = 3 V r^2 / R^3, with the two-level Stark table on
    n_knots knots over 0..E_max V/m (the electrostatic-lens workload; with
    low_field_seeker the curve's other sign, a state the lens focuses)."""
    sp = TwoLevelStark(splitting_hz, dipole_debye, 1.0 if low_field_seeker else -1.0).spline(n_knots, E_max)
    return StarkForce.from_spline(sp, V=V, R=R, mass=mass, field_order=2)


def reference_radial_table(W, V: float, d: float, mass: float = TLF_MASS,
                           dr: float = 1e-4) -> interp1d:
    """The reference's a(r) table (electrostatic_lens.py:194-209) from W(E) in J, E in V/m.

    Kept as the reference writes it, including np.gradient with spacing ``dr``
    on a grid whose actual spacing is (1.01 d/2) / (n - 1).
    """
    r_values = np.linspace(0, d / 2 * 1.01, int(np.round(d / 2 / dr)))
    E_values = 2 * V / ((d / 2) ** 2) * r_values
    V_stark = W(E_values)
    a_values = -np.gradient(V_stark, dr) / mass
    return interp1d(r_values, a_values)


# ---------------------------------------------------------------------------
# Stark curves from a Hamiltonian (stark_potential.py:9-88)
# ---------------------------------------------------------------------------


@dataclass
class LinearHamiltonian:
    """H(E, B) = H0 + E_z HE + B_z HB in rad/s (E in V/cm, B in T): the form of
    the TlF ground-state Hamiltonian the reference diagonalises
    (stark_potential.py:26-27; centrex_TlF's function is linear in the field
    components).  Any basis and size; the matrices are Hermitian."""

    H0: np.ndarray
    HE: np.ndarray
    HB: np.ndarray

    def __post_init__(self):
        self.H0, self.HE, self.HB = (np.asarray(a, dtype=np.complex128) for a in (self.H0, self.HE, self.HB))
        n = self.H0.shape[0]
        if any(a.shape != (n, n) for a in (self.H0, self.HE, self.HB)):
            raise ValueError("H0, HE and HB must be square matrices of one size")

    def __call__(self, E, B):
        return self.H0 + E[2] * self.HE + B[2] * self.HB


def reorder_evecs(V_in, E_in, V_ref):
    """stark_potential.py:78-88: order eigenpairs so that index k follows the
    reference vector k (largest overlap), E_out, V_out."""
    overlap = np.abs(np.conj(V_in.T) @ V_ref)
    index = np.argsort(np.argmax(overlap, axis=1))
    return E_in[index], V_in[:, index]


def stark_potential(state, Ezs, hamiltonian: LinearHamiltonian, basis=None, B: float = 1e-4,
                    E_start: float = 100.0) -> np.ndarray:
    """Stark energy (J) of ``state`` at the field magnitudes ``Ezs`` (V/cm),
    stark_potential.py:9-67, on the GPU.

    All the Hamiltonians H(Ez z^, B z^) are diagonalised in one batched
    Hermitian eigensolve (cuSOLVER through torch.linalg.eigh, complex128), the
    overlaps |V_i^H V_(i-1)| of consecutive eigenbases in one batched product
    on the device.  The reference's adiabatic reordering (each step's
    eigenpairs sorted by the reference vector they overlap most, the reference
    being the previous step's reordered basis, reorder_evecs) is then a chain
    of index permutations composed on the host: with perm the previous step's
    order, the largest overlap of new vector k among the reordered columns is
    column inv(perm)[argmax_c |V_i^H V_(i-1)|[k, c]].  The state is the
    eigenvector at E = E_start V/cm (the reference's 100 V/cm and B = 1e-4 T)
    with the largest |<state|v>| (centrex_TlF's find_closest_vector_idx).

    ``state``: a state vector in the Hamiltonian's basis, or an object with
    ``state_vector(basis)`` (centrex_TlF's State).  Needs a CUDA GPU.
    """
    import torch
    from scipy.constants import hbar

    if not torch.cuda.is_available():
        raise RuntimeError("stark_potential runs its eigensolves on a CUDA GPU; none is available")
    H = hamiltonian
    vec = np.asarray(state.state_vector(basis) if hasattr(state, "state_vector") else state, np.complex128)
    Ezs = np.asarray(Ezs, dtype=np.float64)
    n = H.H0.shape[0]
    if vec.shape != (n,):
        raise ValueError(f"state vector of length {vec.shape} for a {n}-state Hamiltonian")
    dev = torch.device("cuda")
    H0, HE, HB = (torch.as_tensor(a, device=dev) for a in (H.H0, H.HE, H.HB))
    Ez = torch.as_tensor(Ezs, device=dev)
    # H0 + E_z HE + B_z HB, in the reference's order of operations
    Hs = (H0 + Ez[:, None, None] * HE) + B * HB
    evals, evecs = torch.linalg.eigh(Hs)
    _, V0 = torch.linalg.eigh((H0 + E_start * HE) + B * HB)
    prev = torch.cat([V0[None], evecs[:-1]]) if Ezs.size else V0[None]
    best = (evecs.mH @ prev).abs().argmax(dim=2).cpu().numpy()
    E = evals.cpu().numpy()
    out = np.empty_like(E)
    inv = np.arange(n)
    for i in range(Ezs.size):
        order = np.argsort(inv[best[i]])
        out[i] = E[i][order]
        inv = np.empty(n, dtype=np.int64)
        inv[order] = np.arange(n)
    state_i = int(np.argmax(np.abs(np.conj(vec) @ V0.cpu().numpy())))
    return out[:, state_i] * hbar


def lens_table_from_hamiltonian(lens, state, hamiltonian: LinearHamiltonian, basis=None) -> interp1d:
    """The lens's a(r) table as ``ElectrostaticLens.lens_acceleration`` builds it
    when ``a_interp`` is None (electrostatic_lens.py:191-209): r grid, |E| =
    2 V r / (d/2)^2, the Stark curve of ``state`` (``stark_potential``, E in
    V/cm), a = -np.gradient(V_stark, dr) / mass, linear interp1d.  Assign the
    result to ``lens.a_interp``."""
    return reference_radial_table(lambda E: stark_potential(state, E / 100, hamiltonian, basis), V=lens.V,
                                  d=lens.d, mass=lens.mass)
