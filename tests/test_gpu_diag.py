"""Microstructure diagnostics on the device (amps_interface, amps_grains,
amps_boundary_lengths, amps_compare_all) against the numpy restatement
tests/diag_ref.py on synthetic states: exact integer counts and lengths,
errors to 1e-15 relative."""
import numpy as np
import pytest

import diag_ref as D
from w3914777_gb300 import amps

pytestmark = pytest.mark.gpu


def voronoi_etas(n, q, seeds, rng, periodic=True):
    pts = rng.uniform(0, n, (seeds, 2))
    lab = rng.integers(0, q, seeds)
    y, x = np.mgrid[0:n, 0:n].astype(float)
    d = []
    for px, py in pts:
        dx, dy = np.abs(x - px), np.abs(y - py)
        if periodic:
            dx, dy = np.minimum(dx, n - dx), np.minimum(dy, n - dy)
        d.append(dx * dx + dy * dy)
    owner = lab[np.argmin(np.array(d), axis=0)]
    etas = 0.05 * rng.uniform(0, 1, (q, n, n))
    for k in range(q):
        etas[k][owner == k] += 0.9
    etas[:, rng.uniform(0, 1, (n, n)) < 0.03] = 0.2  # unlabelled specks below the threshold
    return etas


@pytest.mark.parametrize("bc", [amps.BC_PERIODIC, amps.BC_NOFLUX])
def test_grains_and_boundaries_match_numpy(bc):
    rng = np.random.default_rng(5)
    n, q = 64, 4
    etas = voronoi_etas(n, q, 14, rng, periodic=bc == amps.BC_PERIODIC)
    p = amps.Params.preset(amps.GRAINGROWTH, 0, nx=n, ny=n, nfields=q, tile=32, bc=bc, mode=amps.PUREHIGH,
                           high_tier=amps.TIER_FP64)
    with amps.Simulation(p) as s:
        s.set_fields(etas)
        g = s.grains(threshold=0.5)
        bl = s.boundary_lengths()
    lab = D.labels(etas, 0.5)
    ng, cells = D.components(lab, bc)
    assert (g["grains"], g["cells"]) == (ng, cells)
    assert g["mean_area"] == pytest.approx(cells * p.dx * p.dy / ng, rel=1e-15)
    np.testing.assert_array_equal(bl, D.boundaries(D.labels(etas, -1e300), q, p.dx, p.dy, bc))


def test_sintering_neck_widths_match_numpy():
    n = 96
    p = amps.Params.preset(amps.SINTERING, 0, nx=n, ny=n, nfields=3, tile=32, mode=amps.PUREHIGH,
                           high_tier=amps.TIER_FP64)
    y, x = np.mgrid[0:n, 0:n].astype(float)
    discs = [(30, 48, 18), (62, 48, 16), (46, 24, 14)]
    etas = np.array([((x - cx) ** 2 + (y - cy) ** 2 <= r * r).astype(float) for cx, cy, r in discs])
    c = np.clip(etas.sum(0), 0, 1)
    state = np.concatenate([c[None], etas])
    with amps.Simulation(p) as s:
        s.set_fields(state)
        bl = s.boundary_lengths(level=0.5)
        g = s.grains(threshold=0.5, level=0.5)
    ref = D.boundaries(D.labels(etas, -1e300, conc=c), 3, p.dx, p.dy, p.bc)
    np.testing.assert_array_equal(bl, ref)
    assert bl[0, 1] > 0 and bl[0, 2] > 0  # the discs touch: necks
    assert g["grains"] == 3


def test_interface_and_errors_match_numpy():
    p = amps.Params.preset(amps.KOBAYASHI, 0, nx=128, ny=128, tile=32, mode=amps.PUREHIGH,
                           high_tier=amps.TIER_FP64)
    rng = np.random.default_rng(1)
    y, x = np.mgrid[0:128, 0:128].astype(float)
    r = np.hypot(x - 60.3, y - 70.1) * (1 + 0.3 * np.cos(6 * np.arctan2(y - 70.1, x - 60.3)))
    phi = 0.5 * (1 - np.tanh(r - 25))
    T = rng.uniform(0, 0.1, phi.shape)
    with amps.Simulation(p) as s:
        s.set_fields(np.stack([phi, T]))
        got = s.interface(0, 0.5)
        other = phi + rng.normal(0, 1e-3, phi.shape)
        err = s.compare_all(0, other)
    cells, area, per, box = D.interface(phi, 0.5, p.dx, p.dy, p.bc)
    assert (got["cells"], (got["xmin"], got["xmax"], got["ymin"], got["ymax"])) == (cells, box)
    assert got["area"] == pytest.approx(area, rel=1e-15)
    assert got["perimeter"] == pytest.approx(per, rel=1e-15)
    d = phi - other
    assert err["max_abs"] == np.abs(d).max()
    assert err["rms"] == pytest.approx(np.sqrt((d * d).mean()), rel=1e-13)
    assert err["mean_abs"] == pytest.approx(np.abs(d).mean(), rel=1e-13)
