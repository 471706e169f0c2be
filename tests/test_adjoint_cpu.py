"""CPU checks of the adjoint's test reference and of the checkpointed rollout.

* The torch restatement of one step (adjoint_ref) equals the oracle's step
  (which is pinned bit-exact to the reference) to 1e-12, for both models and
  both boundary maps, noise included.
* The checkpoint/replay logic of adjoint._Rollout, driven by a CPU stepper
  built on adjoint_ref + torch.autograd, gives the same gradients as
  differentiating the unrolled loop directly, for several checkpoint
  spacings.
"""
import numpy as np
import pytest
import torch

import adjoint_ref as R
import oracle_bind as ob
from w3914777_gb300 import adjoint, amps


class _P:
    """Attribute bag standing in for amps.Params in the torch reference."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def _kob_p(bc, noise):
    return _P(nx=24, ny=20, bc=bc, dx=0.03, dy=0.03, tau=0.0003, epsb=0.01, kappa=1.8, delta=0.02, aniso=6.0,
              alpha=0.9, gama=10.0, teq=1.0, theta0=0.2, dt=1e-4, pi=3.1415926, noise=noise, seed=77, model=0)


def _kob_state(p, seed=1):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:p.ny, 0:p.nx]
    phi = 0.5 * (1 - np.tanh((np.hypot(x - 11.3, y - 9.6) - 5) / 2)) + 1e-3 * rng.standard_normal((p.ny, p.nx))
    T = 0.01 * rng.standard_normal((p.ny, p.nx))
    return phi, T


def test_noise_stream_matches_oracle():
    u = R.noise_u01(1234, 17, 50)
    for i in (0, 1, 7, 49):
        assert u[i] == ob.lib().orc_uniform01(1234, 17, i)


@pytest.mark.parametrize("bc", [0, 1])
@pytest.mark.parametrize("noise", [0.0, 0.01])
def test_kobayashi_torch_step_matches_oracle(bc, noise):
    p = _kob_p(bc, noise)
    phi, T = _kob_state(p)
    op = ob.kob_params(p.nx, p.ny, bc=bc, theta0=p.theta0, noise=noise, seed=p.seed)
    ophi, oT = ob.kob_run(op, phi, T, 1, step0=3)
    st = torch.tensor(np.stack([phi, T]))
    out = R.kob_step(st, p, torch.tensor(p.delta, dtype=torch.float64), torch.tensor(p.kappa, dtype=torch.float64),
                     torch.tensor(p.epsb, dtype=torch.float64), 3).numpy()
    assert np.abs(out[0] - ophi).max() <= 1e-12
    assert np.abs(out[1] - oT).max() <= 1e-12


@pytest.mark.parametrize("bc,stencil", [(0, 0), (1, 0), (1, 1)])
def test_graingrowth_torch_step_matches_oracle(bc, stencil):
    rng = np.random.default_rng(2)
    eta = rng.uniform(0, 1, (3, 18, 22))
    op = ob.gg_params(22, 18, q=3, bc=bc, stencil=stencil)
    ref = np.stack(ob.gg_run(op, list(eta), 1))
    p = _P(nx=22, ny=18, bc=bc, stencil=stencil, dx=op.dx, dy=op.dy, dt=op.dt)
    out = R.gg_step(torch.tensor(eta), p, op.mobil, op.grcoef, op.gamma).numpy()
    assert np.abs(out - ref).max() <= 1e-12


class _TorchStepper:
    """The Stepper interface over adjoint_ref on the CPU (autograd per step)."""

    def __init__(self, p):
        self.params = p
        self.dtype = torch.float64
        self.vals = [p.delta, p.kappa, p.epsb]

    def set_param_values(self, values):
        self.vals = list(values)

    def _f(self, state, step, pv):
        return R.kob_step(state, self.params, pv[0], pv[1], pv[2], step)

    def forward(self, state, step, out=None):
        with torch.no_grad():
            r = self._f(state, step, torch.tensor(self.vals, dtype=torch.float64))
        if out is None:
            return r
        out.copy_(r)
        return out

    def adjoint(self, state, grad_out, step, grad_params, grad_in=None):
        with torch.enable_grad():
            x = state.detach().clone().requires_grad_(True)
            pv = torch.tensor(self.vals, dtype=torch.float64, requires_grad=True)
            gx, gp = torch.autograd.grad(self._f(x, step, pv), (x, pv), grad_out)
        grad_params += gp
        if grad_in is None:
            return gx
        grad_in.copy_(gx)
        return grad_in


@pytest.mark.parametrize("segment", [1, 3, 4, 10])
def test_rollout_checkpointing_matches_unrolled(segment):
    p = _kob_p(1, 0.01)
    phi, T = _kob_state(p)
    x0 = torch.tensor(np.stack([phi, T]))
    n = 10
    tgt = torch.zeros_like(x0[0])
    # direct: autograd through the unrolled loop
    pv = torch.tensor([p.delta, p.kappa, p.epsb], dtype=torch.float64, requires_grad=True)
    xa = x0.clone().requires_grad_(True)
    s = xa
    for k in range(n):
        s = R.kob_step(s, p, pv[0], pv[1], pv[2], 5 + k)
    (0.5 * ((s[0] - tgt) ** 2).sum()).backward()
    # checkpointed
    pv2 = torch.tensor([p.delta, p.kappa, p.epsb], dtype=torch.float64, requires_grad=True)
    xb = x0.clone().requires_grad_(True)
    out = adjoint._Rollout.apply(xb, pv2, _TorchStepper(p), n, 5, segment)
    (0.5 * ((out[0] - tgt) ** 2).sum()).backward()
    assert torch.allclose(xb.grad, xa.grad, rtol=1e-12, atol=1e-14)
    assert torch.allclose(pv2.grad, pv.grad, rtol=1e-12, atol=0)


def test_param_names_cover_models():
    assert adjoint.PARAM_NAMES[amps.KOBAYASHI] == ("delta", "kappa", "epsb")
    assert adjoint.PARAM_NAMES[amps.GRAINGROWTH] == ("mobil", "grcoef", "gamma")
