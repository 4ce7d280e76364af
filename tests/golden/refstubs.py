"""Import shims that let the reference package load in a container without its
plotting / HDF5 / TlF-Hamiltonian dependencies.

Test infrastructure only: used by ``make_golden.py`` to run the reference's own
``Beamline.propagate_through`` on injected initial conditions.  The reference
imports ``h5py``, ``matplotlib``, ``centrex_TlF`` and ``hexalattice`` at module
top level (``src/trajectories/molecule.py:2-3``, ``beamline.py:5-6``,
``beamline_elements/apertures.py:7-11``, ``electrostatic_lens.py:7-10``,
``meshes.py:9-15``, ``stark_potential.py:1-7``) but the propagation path never
calls into them once ``ElectrostaticLens.a_interp`` is supplied.
"""
import sys
import types


class _AnyMeta(type):
    def __getattr__(cls, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Any


class _Any(metaclass=_AnyMeta):
    """Placeholder that absorbs calls, attribute access and products.

    Dunder lookups raise so that ``abc`` does not mistake a class-level default
    built from it (``ElectrostaticLens.state``) for an abstract method.
    """

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Any()

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Any()

    def __mul__(self, other):
        return self

    __rmul__ = __mul__

    def __repr__(self):
        return "<stub>"


def _module_getattr(name):
    if name.startswith("__"):
        raise AttributeError(name)
    return _Any


def _stub(name):
    mod = types.ModuleType(name)
    mod.__getattr__ = _module_getattr
    sys.modules[name] = mod
    parent, _, child = name.rpartition(".")
    if parent:
        setattr(sys.modules[parent], child, mod)
    return mod


_STUBS = [
    "h5py", "h5py._hl",
    "matplotlib", "matplotlib.pyplot", "matplotlib.patches", "matplotlib.collections",
    "centrex_TlF", "centrex_TlF.states", "centrex_TlF.states.utils", "centrex_TlF.hamiltonian",
    "hexalattice", "hexalattice.hexalattice",
]


ENV = "CTRAJ_REFERENCE_SRC"


def reference_src(explicit=None):
    """The reference's ``src`` directory: ``explicit`` if given, else the
    environment variable CTRAJ_REFERENCE_SRC; None when neither names an
    existing directory."""
    import os

    path = explicit or os.environ.get(ENV)
    return path if path and os.path.isdir(path) else None


def add_argument(ap):
    """--reference-src for the fixture generators (defaults to CTRAJ_REFERENCE_SRC)."""
    import os

    ap.add_argument("--reference-src", default=os.environ.get(ENV),
                    help=f"the reference's src directory (default: ${ENV})")


def require(path):
    if not reference_src(path):
        raise SystemExit(f"the reference's src directory is required: pass --reference-src or set {ENV}")
    return reference_src(path)


def install(reference_src):
    """Install the stubs and put the reference's ``src`` directory on sys.path."""
    for name in _STUBS:
        if name not in sys.modules:
            _stub(name)
    if reference_src not in sys.path:
        sys.path.insert(0, reference_src)
