"""Differentiable rollouts of the explicit phase-field step.

The reference runs forward only; this module adds reverse-mode gradients of
a loss on the state after N explicit steps with respect to the initial state
and three model parameters, through the hand-written adjoint kernels of the
libamps C ABI:

  Kobayashi dendrite (snowflake/function.h:5-60): state [phi, T],
      parameters ("delta", "kappa", "epsb") -- anisotropy strength, latent
      heat K, mean interface energy.
  Grain growth (graingrowth/function.h:5-30): state [eta_0 .. eta_{Q-1}],
      parameters ("mobil", "grcoef", "gamma") -- L, kappa, cross-coupling.

`Stepper` wraps one step and its adjoint (amps_step_forward /
amps_step_adjoint).  `Rollout` wraps the native checkpointed rollout
(amps_adjoint_*): the forward sweep keeps every `segment`-th state
(segment = ceil(sqrt(N)) by default, so O(sqrt N) states are held; 1 keeps
all and replays nothing), the backward sweep replays one segment at a time
from its checkpoint and runs that segment's adjoint steps in reverse; each
sweep is one CUDA graph launch.  `rollout()` is the torch.autograd entry.
Each step's noise (Kobayashi) is a function of the step index alone, so the
replay reproduces the forward exactly.

All computation is on the device, in float64 or float32 (the state tensor's
dtype).  There is no CPU path: the library must be built.
"""
import ctypes

import torch

from . import amps

PARAM_NAMES = {amps.KOBAYASHI: ("delta", "kappa", "epsb"), amps.GRAINGROWTH: ("mobil", "grcoef", "gamma")}


def _code(dtype):
    if dtype == torch.float64:
        return amps.F64
    if dtype == torch.float32:
        return amps.F32
    raise TypeError(f"state must be float64 or float32, not {dtype}")


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _nfields(params):
    return 2 if params.model == amps.KOBAYASHI else params.nfields


def _check_model(params):
    if params.model not in PARAM_NAMES:
        raise ValueError("the adjoint covers the Kobayashi and grain-growth models")


class Stepper:
    """One explicit step and its adjoint for fixed parameters and grid."""

    def __init__(self, params, dtype=torch.float64, device="cuda"):
        _check_model(params)
        self.params = params.replace()
        self.dtype = dtype
        self.code = _code(dtype)
        self.device = torch.device(device)
        self.shape = (_nfields(params), params.ny, params.nx)

    def set_param_values(self, values):
        for name, v in zip(PARAM_NAMES[self.params.model], values):
            setattr(self.params, name, float(v))

    def forward(self, state, step, out=None):
        if out is None:
            out = torch.empty_like(state)
        rc = amps.lib().amps_step_forward(ctypes.byref(self.params), self.code, _ptr(state), _ptr(out), int(step),
                                          _stream())
        amps._check(rc, None, "amps_step_forward")
        return out

    def adjoint(self, state, grad_out, step, grad_params, grad_in=None):
        if grad_in is None:
            grad_in = torch.empty_like(state)
        rc = amps.lib().amps_step_adjoint(ctypes.byref(self.params), self.code, _ptr(state), _ptr(grad_out),
                                          _ptr(grad_in), _ptr(grad_params), int(step), _stream())
        amps._check(rc, None, "amps_step_adjoint")
        return grad_in


class Rollout:
    """Native checkpointed rollout of `nsteps` steps (an amps_adjoint handle).

    One forward must precede each backward; a second forward replaces the
    checkpoints of the first.
    """

    def __init__(self, params, nsteps, dtype=torch.float64, segment=0, graphs=True, device="cuda"):
        _check_model(params)
        self.params = params.replace()
        self.dtype = dtype
        self.code = _code(dtype)
        self.device = torch.device(device)
        self.nsteps = int(nsteps)
        self.shape = (_nfields(params), params.ny, params.nx)
        h = ctypes.c_void_p()
        rc = amps.lib().amps_adjoint_create(ctypes.byref(self.params), self.code, self.nsteps, int(segment),
                                            ctypes.byref(h))
        amps._check(rc, None, "amps_adjoint_create")
        self.h = h
        if not graphs:
            amps.lib().amps_adjoint_set_graphs(self.h, 0)
        self.segment = amps.lib().amps_adjoint_segment(self.h)

    @staticmethod
    def memory_bytes(params, nsteps, dtype=torch.float64, segment=0):
        return amps.lib().amps_adjoint_memory_bytes(ctypes.byref(params), _code(dtype), int(nsteps), int(segment))

    def _ck(self, rc, what):
        if rc != 0:
            msg = amps.lib().amps_adjoint_last_error(self.h).decode()
            raise amps.AmpsError(rc, f"{what}: {msg or amps.lib().amps_status_string(rc).decode()}")

    def _validate(self, t, what):
        if not t.is_cuda or t.dtype != self.dtype or tuple(t.shape) != self.shape or not t.is_contiguous():
            raise ValueError(f"{what} must be a contiguous CUDA {self.dtype} tensor {self.shape}")

    def forward(self, state0, param_values=None, step0=0):
        self._validate(state0, "state0")
        if param_values is None:
            param_values = [getattr(self.params, n) for n in PARAM_NAMES[self.params.model]]
        pv = (ctypes.c_double * 3)(*[float(v) for v in param_values])
        out = torch.empty_like(state0)
        amps.lib().amps_adjoint_set_stream(self.h, _stream())
        self._ck(amps.lib().amps_adjoint_forward(self.h, pv, _ptr(state0), _ptr(out), int(step0)),
                 "amps_adjoint_forward")
        return out

    def backward(self, grad_final):
        self._validate(grad_final, "grad_final")
        g0 = torch.empty_like(grad_final)
        gp = torch.empty(3, dtype=torch.float64, device=grad_final.device)
        amps.lib().amps_adjoint_set_stream(self.h, _stream())
        self._ck(amps.lib().amps_adjoint_backward(self.h, _ptr(grad_final), _ptr(g0), _ptr(gp)),
                 "amps_adjoint_backward")
        return g0, gp

    def close(self):
        if getattr(self, "h", None):
            amps.lib().amps_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state0, pvals, runner, step0):
        ctx.runner = runner
        return runner.forward(state0.detach().contiguous(), pvals.tolist(), step0)

    @staticmethod
    def backward(ctx, grad_out):
        g0, gp = ctx.runner.backward(grad_out.detach().to(ctx.runner.dtype).contiguous())
        return g0, gp.cpu(), None, None


def rollout(state0, params, nsteps, param_values=None, step0=0, segment=0, runner=None, graphs=True):
    """State after `nsteps` explicit steps from `state0`, differentiable.

    state0: CUDA tensor [nf, ny, nx] (float64 or float32, contiguous);
    params: `amps.Params` of the model (grid and fixed coefficients);
    param_values: CPU float64 tensor of the three parameters of PARAM_NAMES
      (requires_grad for their gradient), or None to use the values in params;
    step0: noise step index of the first step;
    segment: steps between checkpoints (0: ceil(sqrt(nsteps)); 1: keep all);
    runner: a `Rollout` to reuse (its checkpoints are overwritten).
    """
    if runner is None:
        runner = Rollout(params, nsteps, dtype=state0.dtype, segment=segment, graphs=graphs,
                         device=state0.device)
    if param_values is None:
        param_values = torch.tensor([getattr(params, n) for n in PARAM_NAMES[params.model]], dtype=torch.float64)
    if param_values.dtype != torch.float64:
        raise TypeError("param_values must be float64")
    return _RolloutFn.apply(state0, param_values, runner, int(step0))
