"""The grain-growth ensemble workload: many independent Fan-Chen runs of
different sizes, field counts and coefficients advanced together by
`amps.Ensemble` (one launch per group of members a step, the groups as
parallel branches of each period's CUDA graph).

No reference counterpart: the reference runs one grid per process
(graingrowth/end2end_mix.cu).  Each member is the 1024^2 Q=8 Fan-Chen
workload's physics (gamma = 1.5, dx = 1, eta ~ U[-1e-3, 1e-3] seeded) with
  side  = round(exp(U[ln 128, ln 1024])) (any integer: the edge tiles of a
          side that is not a multiple of the tile are partial),
  Q     in {4, 8, 12, 16},
  kappa ~ U[1, 3],  L ~ U[0.5, 2],
  dt    = stable_dt(L, kappa).
"""
import math

import numpy as np

from . import amps


def stable_dt(mobil, grcoef, dx=1.0, dt_max=0.05, safety=0.9):
    """Largest explicit-Euler step the member's diffusion allows, capped at 0.05.

    The reference's 8-neighbour Laplacian (graingrowth/function.h:20, every
    neighbour weight 1, centre -8) has the Fourier symbol
    2cos kx + 2cos ky + 4cos kx cos ky - 8, whose minimum is -12 (at kx = 0,
    ky = pi).  Explicit Euler on d eta/dt = L kappa lap eta is stable while
    dt * L * kappa * 12 / dx^2 <= 2; the step keeps a 0.9 margin.  With
    L * kappa up to 6 the rule gives dt down to 0.025, so members with
    L * kappa > 3 run below the workload's dt = 0.05.
    """
    return min(dt_max, safety * 2.0 * dx * dx / (12.0 * mobil * grcoef))


def member_params(count=64, seed=2024, tile=32, overrides=None, round_to_tile=False):
    """Parameters of `count` seeded ensemble members (list of amps.Params);
    round_to_tile: sides rounded to multiples of the tile (no partial tiles)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        side = int(round(math.exp(rng.uniform(math.log(128), math.log(1024)))))
        if round_to_tile:
            side = max(tile, int(round(side / tile)) * tile)
        q = int(rng.choice([4, 8, 12, 16]))
        kappa = float(rng.uniform(1.0, 3.0))
        mobil = float(rng.uniform(0.5, 2.0))
        p = amps.Params.preset(amps.GRAINGROWTH, 0, nx=side, ny=side, nfields=q, grcoef=kappa, mobil=mobil,
                               tile=tile, seed=seed * 1000 + i)
        p.dt = stable_dt(mobil, kappa, p.dx)
        for k, v in (overrides or {}).items():
            setattr(p, k, v)
        out.append(p)
    return out


def cells(params_list):
    """Cells per step summed over the members."""
    return sum(p.nx * p.ny for p in params_list)
