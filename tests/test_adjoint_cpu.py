"""CPU checks of the adjoint's test reference and of the checkpointed rollout.

* The torch restatement of one step (adjoint_ref) equals the oracle's step
  (which is pinned bit-exact to the reference) to 1e-12, for both models and
  both boundary maps, noise included.
* The checkpointed rollout's device-memory layout (host-side arithmetic of
  amps_adjoint_memory_bytes) and its argument checks.
"""
import ctypes

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


@pytest.mark.parametrize("nsteps,segment,nseg,seg", [(1000, 0, 32, 32), (1000, 32, 32, 32), (24, 0, 5, 5),
                                                      (10, 1, 10, 1), (10, 50, 1, 10)])
def test_rollout_memory_layout(nsteps, segment, nseg, seg):
    """Checkpoints: ceil(N/segment) states, plus segment-1 replay states and
    four ping-pong states (each rounded up to 256 B), plus 256 B of scalars."""
    p = amps.Params.preset(amps.KOBAYASHI, 0, nx=256, ny=256)
    sb = 2 * 256 * 256 * 4
    got = amps.lib().amps_adjoint_memory_bytes(ctypes.byref(p), amps.F32, nsteps, segment)
    assert got == sb * (nseg + seg - 1 + 4) + 256


def test_adjoint_abi_rejects_sintering():
    p = amps.Params.preset(amps.SINTERING, 0, nx=64, ny=64, tile=16)
    assert amps.lib().amps_adjoint_memory_bytes(ctypes.byref(p), amps.F64, 10, 0) == 0
    h = ctypes.c_void_p()
    assert amps.lib().amps_adjoint_create(ctypes.byref(p), amps.F64, 10, 0, ctypes.byref(h)) == 6
    assert not h.value


def test_param_names_cover_models():
    assert adjoint.PARAM_NAMES[amps.KOBAYASHI] == ("delta", "kappa", "epsb")
    assert adjoint.PARAM_NAMES[amps.GRAINGROWTH] == ("mobil", "grcoef", "gamma")
