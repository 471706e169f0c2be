"""Host-side checks of the ensemble workload: seeded member parameters and
the per-member stable time step (no GPU needed)."""
from w3914777_gb300 import ensemble


def test_members_are_seeded_in_range_and_stable():
    ps = ensemble.member_params(count=64, seed=2024)
    assert len(ps) == 64
    for p in ps:
        assert p.nx == p.ny and 128 <= p.nx <= 1024
        assert p.nfields in (4, 8, 12, 16)
        assert 1.0 <= p.grcoef <= 3.0 and 0.5 <= p.mobil <= 2.0
        # explicit Euler on the 8-neighbour Laplacian: dt * L * kappa * 12 <= 2 (with a 0.9 margin)
        assert p.dt * p.mobil * p.grcoef * 12 <= 2 * 0.9 + 1e-12
        assert p.dt <= 0.05
    again = ensemble.member_params(count=64, seed=2024)
    key = lambda q: [(p.nx, p.nfields, p.grcoef, p.mobil, p.dt, p.seed) for p in q]
    assert key(ps) == key(again)
    assert key(ps) != key(ensemble.member_params(count=64, seed=7))
    assert len({p.nfields for p in ps}) == 4
    # any integer side, as drawn: most are not multiples of the tile
    assert sum(p.nx % 32 != 0 for p in ps) > 32
    assert all(p.nx % 32 == 0 for p in ensemble.member_params(count=64, seed=2024, round_to_tile=True))


def test_stable_dt_caps_at_the_workload_step():
    assert ensemble.stable_dt(0.5, 1.0) == 0.05
    assert abs(ensemble.stable_dt(2.0, 3.0) - 0.9 * 2 / 72) < 1e-15
