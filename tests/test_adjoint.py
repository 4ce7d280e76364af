"""Soft transmission and its discrete adjoint (ctraj_soft_transmission).

CPU: the FP64 torch reference (oracle/soft_reference.py) differentiated by
autograd agrees with its own central finite differences (h = 1e-4 relative).
GPU: the CUDA FP64 forward and adjoint against that reference on the same unit
normals; the CUDA FP32 adjoint against the FP64 reference; the FP64 adjoint
against central finite differences of the CUDA FP64 forward at 1e5
molecules; checkpoint-interval independence; the torch.autograd.Function;
and the zero-width limit against the hard detected fraction.
"""
import numpy as np
import pytest

from ctraj.adjoint import PARAM_NAMES, SoftProblem
from ctraj.workloads import lens_beamline

# Tolerances (relative, per parameter, against the largest of the compared values)
FD_REL = 1e-4       # adjoint vs central finite differences, h = 1e-4 relative
FP64_REL = 1e-9     # CUDA FP64 vs torch FP64 (same arithmetic up to rounding order)
FP32_REL = 1e-4     # CUDA FP32 adjoint vs the FP64 reference
CKPT_REL = 3e-4     # FP32 gradients of two checkpoint intervals: the backward maps compose
                    # over other segments, so their rounding differs (up to 1.2e-4 seen)
V_TEST = 8e3        # lens voltage of the small cases: enough molecules pass to give a signal


def problem(n, detector=False, aperture="A1", **kw):
    """The lens beamline; detector: a 10 mm detector aperture at 3.0 m behind
    a lens focusing the molecules onto it (the low-field-seeking state;
    aperture="Detection plane" makes the detector's radius the parameter)."""
    bl = lens_beamline(detector_d=10e-3, low_field_seeker=True) if detector else lens_beamline()
    return SoftProblem.from_beamline(bl, n=n, aperture=aperture, **kw)


def params(prob, V=V_TEST):
    p = prob.initial_params()
    p[0] = V
    return p


def rel_err(a, b, floor=1e-300):
    """|a - b| relative to the larger magnitude; differences of two values both
    below `floor` (a gradient that vanishes for the case) count as zero."""
    a, b = np.asarray(a), np.asarray(b)
    d = np.abs(a - b)
    return np.where(d <= floor, 0.0, d / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-300))


NEGLIGIBLE = 1e-15  # a gradient below this (per unit of its parameter) is zero for these cases


def test_initial_params_follow_the_beamline():
    prob = problem(10)
    p = prob.initial_params()
    assert PARAM_NAMES == ("V", "lens_z0", "aperture_r", "bore_r", "sigma_vx", "sigma_vy")
    np.testing.assert_allclose(p, [30e3, 0.80, 6e-3, 17.5e-3, 20.0, 20.0])
    with pytest.raises(ValueError):
        SoftProblem.from_beamline(lens_beamline(), n=10, aperture="nope")
    lim = prob.param_bounds()
    assert lim[0, 0] == 0.0  # V >= 0
    # the 0.60 m lens stays between A1 (ends at 0.301 m) and the 3.0 m plane, 1 mm clear
    np.testing.assert_allclose(lim[1], [0.302, 3.0 - 0.6 - 1e-3])


def test_torch_reference_autograd_matches_finite_differences():
    from oracle import soft_reference as sr

    n = 1500
    prob = problem(n)
    p0 = params(prob)
    nrm = np.random.default_rng(1).standard_normal((5, n))
    kw = dict(aperture=prob.aperture, width=prob.width, log_floor=prob.log_floor)
    loss, g = sr.soft_grad(prob.cb, nrm, prob.xdist, prob.vdist, p0, **kw)
    fd = sr.soft_fd(prob.cb, nrm, prob.xdist, prob.vdist, p0, **kw)
    assert loss > 0
    assert rel_err(g, fd).max() < FD_REL, (g, fd)


# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def engine():
    from ctraj.engine import Engine

    e = Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("aperture", ["A1", "Detection plane"])
def test_torch_reference_behind_the_lens_matches_finite_differences(aperture):
    """A detector aperture behind the lens: the reference's own gradient,
    including the aperture-radius parameter on either side of the lens."""
    from oracle import soft_reference as sr

    n = 1500
    prob = problem(n, detector=True, aperture=aperture)
    p0 = params(prob)
    nrm = np.random.default_rng(2).standard_normal((5, n))
    kw = dict(aperture=prob.aperture, width=prob.width, log_floor=prob.log_floor)
    loss, g = sr.soft_grad(prob.cb, nrm, prob.xdist, prob.vdist, p0, **kw)
    fd = sr.soft_fd(prob.cb, nrm, prob.xdist, prob.vdist, p0, **kw)
    import torch

    open_plane = SoftProblem.from_beamline(lens_beamline(low_field_seeker=True), n=n, aperture="A1")
    free = sr.soft_loss(open_plane.cb, nrm, prob.xdist, prob.vdist, torch.tensor(p0),
                        aperture=open_plane.aperture, width=prob.width, log_floor=prob.log_floor)
    assert 0 < loss < 0.5 * float(free)  # the detector takes part of what reaches 3 m
    # (the bore radius does not limit a focused beam: its gradient vanishes)
    assert rel_err(g, fd, NEGLIGIBLE).max() < FD_REL, (g, fd)


@pytest.fixture(scope="module")
def reference_1e4():
    from oracle import soft_reference as sr

    n = 10_000
    prob = problem(n)
    nrm = np.random.default_rng(7).standard_normal((5, n))
    p0 = params(prob)
    kw = dict(aperture=prob.aperture, width=prob.width, log_floor=prob.log_floor)
    loss, g = sr.soft_grad(prob.cb, nrm, prob.xdist, prob.vdist, p0, **kw)
    return n, nrm, p0, loss, g


@pytest.mark.gpu
def test_fp64_adjoint_matches_torch_autograd(engine, reference_1e4):
    from ctraj.adjoint import soft_transmission

    n, nrm, p0, loss, g = reference_1e4
    prob = problem(n, precision=64, normals=nrm)
    out = soft_transmission(prob, p0, engine=engine)
    assert rel_err(out.loss, loss) < FP64_REL
    assert rel_err(out.grad, g).max() < FP64_REL, (out.grad, g)


@pytest.mark.gpu
@pytest.mark.parametrize("aperture", ["A1", "Detection plane"])
def test_adjoint_behind_the_lens_matches_torch_autograd(engine, aperture):
    """A 10 mm detector aperture behind the lens: the CUDA FP64 loss and
    gradient against the torch FP64 reference, the FP32 gradient within its
    tolerance."""
    from ctraj.adjoint import soft_transmission
    from oracle import soft_reference as sr

    n = 10_000
    prob = problem(n, detector=True, aperture=aperture)
    nrm = np.random.default_rng(11).standard_normal((5, n))
    p0 = params(prob)
    kw = dict(aperture=prob.aperture, width=prob.width, log_floor=prob.log_floor)
    loss, g = sr.soft_grad(prob.cb, nrm, prob.xdist, prob.vdist, p0, **kw)
    out64 = soft_transmission(problem(n, detector=True, aperture=aperture, precision=64, normals=nrm), p0,
                              engine=engine)
    assert rel_err(out64.loss, loss) < FP64_REL
    assert rel_err(out64.grad, g, NEGLIGIBLE).max() < FP64_REL, (out64.grad, g)
    out32 = soft_transmission(problem(n, detector=True, aperture=aperture, precision=32, normals=nrm), p0,
                              engine=engine)
    assert rel_err(out32.grad, g, NEGLIGIBLE).max() < FP32_REL, (out32.grad, g)
    assert abs(g[1]) > 0  # the lens position matters to the detector


@pytest.mark.gpu
def test_fp32_adjoint_matches_fp64_reference(engine, reference_1e4):
    from ctraj.adjoint import soft_transmission

    n, nrm, p0, loss, g = reference_1e4
    prob = problem(n, precision=32, normals=nrm)
    out = soft_transmission(prob, p0, engine=engine)
    assert rel_err(out.loss, loss) < 1e-5
    assert rel_err(out.grad, g).max() < FP32_REL, (out.grad, g)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_adjoint_matches_finite_differences_on_device_draws(engine, precision):
    from ctraj.adjoint import soft_transmission

    prob64 = problem(100_000, precision=64, seed=3)
    p0 = params(prob64)
    fd = np.zeros(6)
    for k in range(6):
        h = 1e-4 * abs(p0[k])
        pp, pm = p0.copy(), p0.copy()
        pp[k] += h
        pm[k] -= h
        fd[k] = (soft_transmission(prob64, pp, want_grad=False, engine=engine).loss
                 - soft_transmission(prob64, pm, want_grad=False, engine=engine).loss) / (2 * h)
    out = soft_transmission(problem(100_000, precision=precision, seed=3), p0, engine=engine)
    assert rel_err(out.grad, fd).max() < FD_REL, (precision, out.grad, fd)


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_the_gradient(engine):
    from ctraj.adjoint import soft_transmission

    p0 = params(problem(1))
    outs = [soft_transmission(problem(50_000, seed=5, checkpoint=k), p0, engine=engine) for k in (64, 17, 1)]
    for o in outs[1:]:
        # the forward pass is the same; the backward maps compose over
        # different segments, so only rounding differs
        assert o.loss == outs[0].loss
        assert rel_err(o.grad, outs[0].grad).max() < CKPT_REL, (o.grad, outs[0].grad)
    # in FP64 the intervals agree to rounding
    o64 = [soft_transmission(problem(20_000, seed=5, checkpoint=k, precision=64), p0, engine=engine)
           for k in (64, 17)]
    assert o64[1].loss == o64[0].loss
    assert rel_err(o64[1].grad, o64[0].grad).max() < FP64_REL, (o64[1].grad, o64[0].grad)
    again = soft_transmission(problem(50_000, seed=5, checkpoint=64), p0, engine=engine)
    np.testing.assert_array_equal(again.grad, outs[0].grad)  # deterministic
    # the forward-only call gives the same loss
    f = soft_transmission(problem(50_000, seed=5), p0, want_grad=False, engine=engine)
    assert f.loss == outs[0].loss and f.grad is None


@pytest.mark.gpu
def test_autograd_function(engine):
    import torch

    from ctraj.adjoint import soft_loss, soft_transmission

    prob = problem(50_000, seed=9)
    p = torch.tensor(params(prob), dtype=torch.float64, requires_grad=True)
    loss = soft_loss(p, prob, engine)
    (2.0 * loss).backward()
    ref = soft_transmission(prob, params(prob), engine=engine)
    assert float(loss.detach()) == ref.loss
    np.testing.assert_array_equal(p.grad.numpy(), 2.0 * ref.grad)
    with torch.no_grad():
        assert float(soft_loss(p, prob, engine)) == ref.loss


@pytest.mark.gpu
def test_zero_width_limit_is_the_hard_detected_fraction(engine):
    from ctraj.adjoint import soft_transmission
    from ctraj.distributions import device_spec
    from ctraj.workloads import source

    n = 200_000
    prob = problem(n, precision=64, seed=4, width=1e-9, log_floor=-700.0)
    p = prob.initial_params()
    soft = soft_transmission(prob, p, want_grad=False, engine=engine).loss
    xd, vd = source()
    hard = engine.run(prob.cb, n, precision=64, xdist=device_spec(xd, "position"),
                      vdist=device_spec(vd, "velocity"), seed=4, outputs=True)
    detected = hard.counts[-1] / n
    near = np.count_nonzero(hard.margin < 1e-7) / n  # molecules within 100 widths of an edge
    assert abs(soft - detected) <= near + 1e-12, (soft, detected, near)


@pytest.mark.gpu
def test_soft_argument_checks(engine):
    from ctraj.adjoint import soft_transmission
    from ctraj.compiler import compile_beamline
    from ctraj.workloads import ballistic_beamline

    prob = problem(100)
    p = prob.initial_params()
    with pytest.raises(ValueError, match="checkpoint"):
        soft_transmission(problem(100, checkpoint=65), p, engine=engine)
    with pytest.raises(ValueError, match="width"):
        soft_transmission(problem(100, width=0.0), p, engine=engine)
    bad = p.copy()
    bad[0] = np.inf
    with pytest.raises(ValueError, match="finite"):
        soft_transmission(prob, bad, engine=engine)
    nolens = SoftProblem.from_beamline(ballistic_beamline(), n=100)
    with pytest.raises(ValueError, match="lens"):
        soft_transmission(nolens, p, engine=engine)
