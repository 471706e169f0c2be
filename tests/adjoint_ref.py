"""Plain-PyTorch float64 restatement of one explicit step (test reference).

Differentiated by torch.autograd, it is the reference the hand-written
adjoint kernels are checked against: same neighbour maps (periodic wrap or
zero-flux mirror), same stencils and the same per-step noise stream as
amps_step_forward.  Kobayashi: snowflake/function.h:5-60; grain growth:
graingrowth/function.h:5-30.  Used by tests only.
"""
import numpy as np
import torch

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix(z):
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def noise_u01(seed, step, n):
    """The noise stream of the Kobayashi step: uniform [0,1) per cell index."""
    with np.errstate(over="ignore"):
        a = _mix(np.array([step], dtype=np.uint64))
        k = _mix(np.array([seed], dtype=np.uint64) ^ a)
        z = _mix(k + np.arange(n, dtype=np.uint64))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def nbmap(n, k, bc):
    i = np.arange(n) + k
    if bc == 0:
        return torch.as_tensor(np.mod(i, n))
    i = np.where(i < 0, -i - 1, i)
    return torch.as_tensor(np.where(i >= n, 2 * n - i - 1, i))


def _shift(f, kx, ky, bc):
    ny, nx = f.shape[-2:]
    return f[..., nbmap(ny, ky, bc), :][..., nbmap(nx, kx, bc)]


def kob_step(state, p, delta, kappa, epsb, step):
    """state [2, ny, nx]; delta/kappa/epsb scalar tensors; returns [2, ny, nx]."""
    phi, T = state[0], state[1]
    bc = p.bc
    s = lambda f, kx, ky: _shift(f, kx, ky, bc)
    px = (s(phi, 1, 0) - s(phi, -1, 0)) * (0.5 / p.dx)
    py = (s(phi, 0, 1) - s(phi, 0, -1)) * (0.5 / p.dy)
    a = p.aniso * (torch.atan2(py, px) - p.theta0)
    eps = epsb * (1 + delta * torch.cos(a))
    epd = -epsb * p.aniso * delta * torch.sin(a)

    def lap(f):
        return ((s(f, -1, 0) + s(f, 1, 0)) + (s(f, -2, 0) + s(f, 2, 0)) + (s(f, 0, -1) + s(f, 0, 1))
                + (s(f, 0, -2) + s(f, 0, 2)) - 8 * f) * (1.0 / (p.dx * p.dy))

    P1, P2 = eps * epd * px, eps * epd * py
    term1 = (s(P1, 0, 1) - s(P1, 0, -1)) * (0.5 / p.dy)
    term2 = -(s(P2, 1, 0) - s(P2, -1, 0)) * (0.5 / p.dx)
    m = (p.alpha / p.pi) * torch.atan(p.gama * (p.teq - T))
    drive = phi - 0.5 + m
    if p.noise != 0.0:
        u = torch.as_tensor(noise_u01(p.seed, step, phi.numel()).reshape(phi.shape), device=phi.device)
        drive = drive + p.noise * (u - 0.5)
    d = (p.dt / p.tau) * (term1 + term2 + eps * eps * lap(phi) + phi * (1 - phi) * drive)
    return torch.stack([phi + d, T + p.dt * lap(T) + kappa * d])


def gg_step(eta, p, mobil, grcoef, gamma):
    """eta [q, ny, nx]; returns [q, ny, nx]."""
    bc = p.bc
    s = lambda f, kx, ky: _shift(f, kx, ky, bc)
    if p.stencil == 0:
        lap = sum(s(eta, kx, ky) for ky in (-1, 0, 1) for kx in (-1, 0, 1) if kx or ky) - 8 * eta
    else:
        lap = s(eta, -1, 0) + s(eta, 1, 0) + s(eta, 0, -1) + s(eta, 0, 1) - 4 * eta
    lap = lap * (1.0 / (p.dx * p.dy))
    S = (eta * eta).sum(0, keepdim=True)
    dfd = eta * (eta * eta - 1 + 2 * gamma * (S - eta * eta))
    return eta - p.dt * mobil * (dfd - grcoef * lap)
