"""Differentiable soft transmission of a lens beamline.

The reference only counts hard hits (Counter, trajectory_simulator.py:106-158),
which has no useful gradient.  ``ctraj_soft_transmission`` replaces each hard
aperture test up to the end of the lens by a sigmoid of the edge distance
(width ``width``) and returns the mean product of the weights together with
its exact gradient from a discrete-adjoint backward pass on the GPU (lens
states checkpointed every ``checkpoint`` RK4 steps and recomputed segment by
segment).  ``SoftTransmission`` wraps it as a torch.autograd.Function so the
beamline can be tuned with torch optimisers:

    prob = SoftProblem.from_beamline(lens_beamline(), n=1_000_000, aperture="A1")
    p = torch.tensor(prob.initial_params(), dtype=torch.float64, requires_grad=True)
    loss = soft_loss(p, prob)      # soft detected fraction
    loss.backward()                # p.grad = d loss / d (V, lens z0, r_A1, r_bore, sigma_vx, sigma_vy)

Hard counts (ctraj_run) remain the reported figure; the soft loss tends to the
detected fraction as the width goes to zero.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .compiler import CompiledBeamline, compile_beamline
from .distributions import device_spec
from .engine import G, default_engine

PARAM_NAMES = ("V", "lens_z0", "aperture_r", "bore_r", "sigma_vx", "sigma_vy")

__all__ = ["PARAM_NAMES", "SoftProblem", "SoftOutput", "soft_transmission", "SoftTransmission", "soft_loss"]


@dataclass
class SoftProblem:
    cb: CompiledBeamline
    n: int
    xdist: _abi.Distribution
    vdist: _abi.Distribution
    aperture: int = -1                  # element index of the aperture-radius parameter
    width: float = 0.2e-3               # sigmoid width (m)
    log_floor: float = -30.0
    checkpoint: int = 64
    precision: int = 32
    seed: int = 0
    offset: int = 0
    g: float = G
    normals: np.ndarray | None = None   # (5, n) unit normals instead of device draws
    extra: dict = field(default_factory=dict)

    @classmethod
    def from_beamline(cls, beamline, n: int, xdist=None, vdist=None, aperture: str | None = None, **kw):
        """``aperture`` names the circular aperture whose radius is a parameter."""
        from .workloads import source

        cb = beamline if isinstance(beamline, CompiledBeamline) else compile_beamline(beamline)
        if xdist is None or vdist is None:
            xd, vd = source()
            xdist = xdist or xd
            vdist = vdist or vd
        xs = xdist if isinstance(xdist, _abi.Distribution) else device_spec(xdist, "position")
        vs = vdist if isinstance(vdist, _abi.Distribution) else device_spec(vdist, "velocity")
        if xs is None or xs.kind != _abi.DIST_GAUSSIAN_POSITION or vs is None or vs.kind != _abi.DIST_GAUSSIAN_VELOCITY:
            raise TypeError("the soft transmission needs Gaussian position and velocity distributions")
        idx = -1
        if aperture is not None:
            names = [cb.labels[e.label] if 0 <= e.label < len(cb.labels) else None for e in cb.elements]
            hits = [i for i, e in enumerate(cb.elements) if e.type == _abi.CIRCULAR_APERTURE and names[i] == aperture]
            if not hits:
                raise ValueError(f"no circular aperture named {aperture!r}")
            idx = hits[0]
        return cls(cb=cb, n=int(n), xdist=xs, vdist=vs, aperture=idx, **kw)

    def lens(self):
        return [e for e in self.cb.elements if e.type == _abi.ELECTROSTATIC_LENS][0]

    def param_bounds(self) -> np.ndarray:
        """(6, 2) physical limits: V >= 0; the lens stays between the element in
        front of it and the one behind it (1 mm clear); radii and velocity
        spreads positive."""
        els = list(self.cb.elements)
        li = [i for i, e in enumerate(els) if e.type == _abi.ELECTROSTATIC_LENS][0]
        L = els[li].z1 - els[li].z0
        lo_z = (els[li - 1].z1 + 1e-3) if li > 0 else -np.inf
        hi_z = (els[li + 1].z0 - L - 1e-3) if li + 1 < len(els) else np.inf
        tiny = 1e-6
        return np.array([[0.0, np.inf], [lo_z, hi_z], [tiny, np.inf], [tiny, np.inf], [tiny, np.inf],
                         [tiny, np.inf]])

    def initial_params(self) -> np.ndarray:
        L = self.lens()
        r_ap = self.cb.elements[self.aperture].p[0] / 2 if self.aperture >= 0 else 0.0
        return np.array([L.p[3], L.z0, r_ap, L.p[0] / 2, self.vdist.p[1], self.vdist.p[3]], dtype=np.float64)


@dataclass
class SoftOutput:
    loss: float
    grad: np.ndarray | None
    lens_molecules: int
    lens_steps: int
    dropped: int
    kernels: int
    extra: dict = field(default_factory=dict)


def soft_transmission(prob: SoftProblem, params, want_grad: bool = True, engine=None,
                      timing: bool = False) -> SoftOutput:
    eng = engine or default_engine()
    eng.load(prob.cb)
    a = _abi.SoftArgs()
    a.n = prob.n
    a.precision = prob.precision
    keep = None
    if prob.normals is not None:
        keep = np.ascontiguousarray(prob.normals, dtype=np.float64)
        if keep.shape != (5, prob.n):
            raise ValueError(f"normals must have shape (5, {prob.n})")
        a.ic_mode = _abi.IC_HOST
        a.normals = keep.ctypes.data
    else:
        a.ic_mode = _abi.IC_DEVICE_DRAW
    a.seed = int(prob.seed) & 0xFFFFFFFFFFFFFFFF
    a.offset = int(prob.offset) & 0xFFFFFFFFFFFFFFFF
    a.xdist = prob.xdist
    a.vdist = prob.vdist
    a.g = float(prob.g)
    a.width = float(prob.width)
    a.log_floor = float(prob.log_floor)
    a.aperture = int(prob.aperture)
    a.checkpoint = int(prob.checkpoint)
    a.want_grad = 1 if want_grad else 0
    a.timing = 1 if timing else 0
    p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1))
    if p.size != _abi.SOFT_NPARAMS:
        raise ValueError(f"params must have {_abi.SOFT_NPARAMS} entries {PARAM_NAMES}")
    r = _abi.SoftResult()
    status = eng.lib.ctraj_soft_transmission(eng.ctx, ctypes.byref(a), p.ctypes.data, ctypes.byref(r))
    del keep
    _abi.check(status, eng.lib)
    extra = {"front_ms": float(r.front_ms), "lens_ms": float(r.lens_ms)} if r.timed else {}
    return SoftOutput(loss=float(r.loss), grad=np.array(r.grad[:]) if want_grad else None,
                      lens_molecules=int(r.lens_molecules), lens_steps=int(r.lens_steps),
                      dropped=int(r.dropped), kernels=int(r.kernels), extra=extra)


def _torch_function():
    import torch

    class SoftTransmission(torch.autograd.Function):
        """loss = SoftTransmission.apply(params, problem[, engine]); params: (6,) tensor."""

        @staticmethod
        def forward(ctx, params, prob, engine=None):
            want = bool(ctx.needs_input_grad[0])
            out = soft_transmission(prob, params.detach().to("cpu", torch.float64).numpy(), want_grad=want,
                                    engine=engine)
            g = out.grad if want else np.zeros(_abi.SOFT_NPARAMS)
            ctx.save_for_backward(torch.as_tensor(g, dtype=params.dtype, device=params.device))
            ctx.soft_output = out
            return torch.tensor(out.loss, dtype=params.dtype, device=params.device)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None, None

    return SoftTransmission


try:
    SoftTransmission = _torch_function()
except ImportError:  # pragma: no cover - torch is part of the supported environment
    SoftTransmission = None


def soft_loss(params, prob: SoftProblem, engine=None):
    """Soft transmission as a differentiable torch scalar."""
    return SoftTransmission.apply(params, prob, engine)
