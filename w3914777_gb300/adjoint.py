"""Differentiable rollouts of the explicit phase-field step.

The reference runs forward only; this module adds reverse-mode gradients of
a loss on the state after N explicit steps with respect to the initial state
and three model parameters, through the hand-written adjoint kernels behind
`amps_step_forward` / `amps_step_adjoint` (libamps C ABI):

  Kobayashi dendrite (snowflake/function.h:5-60): state [phi, T],
      parameters ("delta", "kappa", "epsb") -- anisotropy strength, latent
      heat K, mean interface energy.
  Grain growth (graingrowth/function.h:5-30): state [eta_0 .. eta_{Q-1}],
      parameters ("mobil", "grcoef", "gamma") -- L, kappa, cross-coupling.

`rollout` is a `torch.autograd.Function`: the forward keeps only every
`segment`-th state (segment = ceil(sqrt(N)) by default, so O(sqrt N) states
are held), and the backward replays one segment at a time from its
checkpoint, then runs the adjoint steps of that segment in reverse.  Each
step's noise (Kobayashi) is a function of the step index alone, so the replay
reproduces the forward exactly.

All computation is on the device, in float64 or float32 (the state tensor's
dtype).  There is no CPU path: the library must be built.
"""
import ctypes
import math

import torch

from . import amps

PARAM_NAMES = {amps.KOBAYASHI: ("delta", "kappa", "epsb"), amps.GRAINGROWTH: ("mobil", "grcoef", "gamma")}


def _dtype_code(t):
    if t.dtype == torch.float64:
        return amps.F64
    if t.dtype == torch.float32:
        return amps.F32
    raise TypeError(f"state must be float64 or float32, not {t.dtype}")


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class Stepper:
    """One explicit step and its adjoint for fixed parameters and grid."""

    def __init__(self, params, dtype=torch.float64, device="cuda"):
        if params.model not in PARAM_NAMES:
            raise ValueError("the adjoint covers the Kobayashi and grain-growth models")
        self.params = params.replace()
        self.dtype = dtype
        self.device = torch.device(device)
        self.nf = 2 if params.model == amps.KOBAYASHI else params.nfields
        self.shape = (self.nf, params.ny, params.nx)
        code = amps.F64 if dtype == torch.float64 else amps.F32
        nbytes = amps.lib().amps_adjoint_workspace_bytes(ctypes.byref(self.params), code)
        self.work = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=self.device)
        self.code = code

    def set_param_values(self, values):
        for name, v in zip(PARAM_NAMES[self.params.model], values):
            setattr(self.params, name, float(v))

    def forward(self, state, step, out=None):
        if out is None:
            out = torch.empty_like(state)
        rc = amps.lib().amps_step_forward(ctypes.byref(self.params), self.code, _ptr(state), _ptr(out),
                                          _ptr(self.work), int(step), _stream())
        amps._check(rc, None, "amps_step_forward")
        return out

    def adjoint(self, state, grad_out, step, grad_params, grad_in=None):
        if grad_in is None:
            grad_in = torch.empty_like(state)
        rc = amps.lib().amps_step_adjoint(ctypes.byref(self.params), self.code, _ptr(state), _ptr(grad_out),
                                          _ptr(grad_in), _ptr(grad_params), _ptr(self.work), int(step),
                                          _stream())
        amps._check(rc, None, "amps_step_adjoint")
        return grad_in


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state0, pvals, stepper, nsteps, step0, segment):
        stepper.set_param_values(pvals.tolist())
        checkpoints = [state0.detach().clone()]
        a, b = state0.detach().clone(), torch.empty_like(state0)
        for k in range(nsteps):
            stepper.forward(a, step0 + k, out=b)
            a, b = b, a
            if (k + 1) % segment == 0 and k + 1 < nsteps:
                checkpoints.append(a.clone())
        ctx.stepper, ctx.nsteps, ctx.step0, ctx.segment = stepper, nsteps, step0, segment
        ctx.pvals = pvals.tolist()
        ctx.checkpoints = checkpoints
        return a

    @staticmethod
    def backward(ctx, grad_out):
        st, seg = ctx.stepper, ctx.segment
        st.set_param_values(ctx.pvals)
        gp = torch.zeros(3, dtype=torch.float64, device=grad_out.device)
        g = grad_out.detach().to(st.dtype).contiguous().clone()
        g2 = torch.empty_like(g)
        nseg = len(ctx.checkpoints)
        for s in reversed(range(nseg)):
            first = s * seg
            count = min(seg, ctx.nsteps - first)
            # replay the segment, keeping the input state of every step
            states = [ctx.checkpoints[s]]
            for k in range(count - 1):
                states.append(st.forward(states[-1], ctx.step0 + first + k))
            for k in reversed(range(count)):
                st.adjoint(states[k], g, ctx.step0 + first + k, gp, grad_in=g2)
                g, g2 = g2, g
            ctx.checkpoints[s] = None
        return g, gp.cpu(), None, None, None, None


def rollout(state0, params, nsteps, param_values=None, step0=0, segment=None, stepper=None):
    """State after `nsteps` explicit steps from `state0`, differentiable.

    state0: device tensor [nf, ny, nx] (float64 or float32, contiguous);
    params: `amps.Params` of the model (grid and fixed coefficients);
    param_values: CPU float64 tensor of the three parameters of PARAM_NAMES
      (requires_grad for their gradient), or None to use the values in params;
    step0: noise step index of the first step;
    segment: steps between checkpoints (default ceil(sqrt(nsteps))).
    """
    if state0.dim() != 3 or not state0.is_cuda or not state0.is_contiguous():
        raise ValueError("state0 must be a contiguous CUDA tensor [nf, ny, nx]")
    if stepper is None:
        stepper = Stepper(params, dtype=state0.dtype, device=state0.device)
    if tuple(state0.shape) != stepper.shape or state0.dtype != stepper.dtype:
        raise ValueError(f"state0 must be {stepper.shape} {stepper.dtype}")
    if param_values is None:
        param_values = torch.tensor([getattr(params, n) for n in PARAM_NAMES[params.model]], dtype=torch.float64)
    if nsteps < 1:
        raise ValueError("nsteps must be >= 1")
    if segment is None:
        segment = max(1, math.ceil(math.sqrt(nsteps)))
    return _Rollout.apply(state0, param_values, stepper, int(nsteps), int(step0), int(segment))
