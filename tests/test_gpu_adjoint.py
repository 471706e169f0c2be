"""Hand-written adjoint of the explicit step (amps_step_forward / amps_step_adjoint).

The reference has no gradients; these tests pin the adjoint to the forward it
differentiates:
  * the forward step agrees with amps_run's PUREHIGH FP64 step (<= 1e-12);
  * one adjoint step against torch.autograd of the plain-PyTorch float64
    restatement (tests/adjoint_ref.py) on a noisy dendrite seed: relative
    1e-10 (rounding order only);
  * dot-product test <J^T g, u> against a central finite difference of
    <g, f(x + h u)> (relative 1e-6 in FP64; the requirement is 1e-5), and
    parameter gradients against central differences (relative 1e-6).  The
    Kobayashi anisotropy angle atan2(py, px) is ill-conditioned where
    grad phi ~ 0, so these finite-difference states keep |grad phi| away from
    zero (a ramp with a smooth modulation);
  * a 24-step L2-misfit rollout through torch.autograd with sqrt(N)
    checkpoints: gradients w.r.t. the parameters and the initial temperature
    against finite differences of the whole rollout (relative 1e-5), and
    the same gradients with other checkpoint spacings (state gradients
    bit-identical);
  * FP32 adjoint against FP64 (relative 2e-3).
"""
import numpy as np
import pytest
import torch

import adjoint_ref as R
from w3914777_gb300 import adjoint, amps

pytestmark = pytest.mark.gpu

DEV = "cuda"


def kob_params(n=64, **kw):
    return amps.Params.preset(amps.KOBAYASHI, 0, nx=n, ny=n, tile=16, mode=amps.PUREHIGH, **kw)


def gg_params(n=64, q=4, **kw):
    return amps.Params.preset(amps.GRAINGROWTH, 0, nx=n, ny=n, nfields=q, tile=16, mode=amps.PUREHIGH, **kw)


def kob_disc_state(p, seed=3):
    """Off-centre tanh disc with small noise; small random T."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:p.ny, 0:p.nx].astype(np.float64)
    r = np.hypot(x - p.nx / 2 + 0.37, y - p.ny / 2 - 0.21) * p.dx
    phi = 0.5 * (1 - np.tanh((r - 10 * p.dx) / (2 * p.dx))) + 1e-3 * rng.standard_normal(r.shape)
    T = 0.005 * rng.standard_normal(r.shape)
    return np.stack([phi, T])


def kob_state(p, seed=3):
    """|grad phi| bounded away from 0: a ramp with a smooth modulation; smooth T."""
    y, x = np.mgrid[0:p.ny, 0:p.nx].astype(np.float64)
    n = p.nx
    phi = 0.2 + 0.4 * (x + 0.7 * y) / n + 0.01 * np.sin(4 * np.pi * x / n) * np.sin(6 * np.pi * y / n)
    T = 0.05 * np.cos(2 * np.pi * x / n) * np.sin(2 * np.pi * (y + 3) / n)
    return np.stack([phi, T])


def gg_state(p, seed=4):
    """Smooth random grains: each eta a blurred uniform field."""
    rng = np.random.default_rng(seed)
    e = rng.uniform(0, 1, (p.nfields, p.ny, p.nx))
    for _ in range(4):
        e = (e + np.roll(e, 1, 1) + np.roll(e, -1, 1) + np.roll(e, 1, 2) + np.roll(e, -1, 2)) / 5
    return e


def dev(a, dtype=torch.float64):
    return torch.tensor(a, dtype=dtype, device=DEV).contiguous()


def one_step_sim(p, state):
    with amps.Simulation(p.replace(high_tier=amps.TIER_FP64), graphs=False) as s:
        s.set_fields(state)
        s.run(1)
        return s.fields()


@pytest.mark.parametrize("model", ["kob", "kob_periodic", "gg", "gg5"])
def test_forward_matches_run(model):
    if model.startswith("kob"):
        p = kob_params(bc=amps.BC_PERIODIC) if model == "kob_periodic" else kob_params()
        x = kob_state(p)
    else:
        p = gg_params(stencil=1 if model == "gg5" else 0, bc=amps.BC_NOFLUX if model == "gg5" else amps.BC_PERIODIC)
        x = gg_state(p)
    ref = one_step_sim(p, x)
    st = adjoint.Stepper(p)
    out = st.forward(dev(x), 0).cpu().numpy()
    assert np.abs(out - ref).max() <= 1e-12


def _autograd_ref(p, x, g, step):
    xs = torch.tensor(x, requires_grad=True)
    names = adjoint.PARAM_NAMES[p.model]
    pv = torch.tensor([getattr(p, nm) for nm in names], dtype=torch.float64, requires_grad=True)
    if p.model == amps.KOBAYASHI:
        out = R.kob_step(xs, p, pv[0], pv[1], pv[2], step)
    else:
        out = R.gg_step(xs, p, pv[0], pv[1], pv[2])
    gx, gp = torch.autograd.grad(out, (xs, pv), torch.tensor(g))
    return out.detach().numpy(), gx.numpy(), gp.numpy()


@pytest.mark.parametrize("case", ["kob_noflux", "kob_periodic", "gg8_periodic", "gg8_noflux", "gg5_noflux"])
def test_adjoint_matches_autograd(case):
    if case.startswith("kob"):
        p = kob_params(bc=amps.BC_NOFLUX if case.endswith("noflux") else amps.BC_PERIODIC)
        x = kob_disc_state(p)
    else:
        p = gg_params(stencil=1 if case.startswith("gg5") else 0,
                      bc=amps.BC_NOFLUX if case.endswith("noflux") else amps.BC_PERIODIC)
        x = gg_state(p)
    g = np.random.default_rng(9).standard_normal(x.shape)
    ref_out, ref_gx, ref_gp = _autograd_ref(p, x, g, 7)
    st = adjoint.Stepper(p)
    gp = torch.zeros(3, dtype=torch.float64, device=DEV)
    out = st.forward(dev(x), 7).cpu().numpy()
    gx = st.adjoint(dev(x), dev(g), 7, gp).cpu().numpy()
    assert np.abs(out - ref_out).max() <= 1e-12
    assert np.abs(gx - ref_gx).max() <= 1e-10 * np.abs(ref_gx).max()
    np.testing.assert_allclose(gp.cpu().numpy(), ref_gp, rtol=1e-10)


def _dot_test(p, x, h, seed=7):
    rng = np.random.default_rng(seed)
    st = adjoint.Stepper(p)
    xd = dev(x)
    u = dev(rng.standard_normal(x.shape))
    g = dev(rng.standard_normal(x.shape))
    gp = torch.zeros(3, dtype=torch.float64, device=DEV)
    jt_g = st.adjoint(xd, g, 5, gp)
    lhs = float((jt_g * u).sum())
    fp = float((g * st.forward(xd + h * u, 5)).sum())
    fm = float((g * st.forward(xd - h * u, 5)).sum())
    fd = (fp - fm) / (2 * h)
    assert abs(lhs - fd) <= 1e-6 * abs(fd), (lhs, fd)
    # parameters
    names = adjoint.PARAM_NAMES[p.model]
    for k, name in enumerate(names):
        v = getattr(p, name)
        hp = 1e-4 * abs(v)
        vals = []
        for s in (+1, -1):
            st.set_param_values([getattr(p, nm) + (s * hp if nm == name else 0.0) for nm in names])
            vals.append(float((g * st.forward(xd, 5)).sum()))
        st.set_param_values([getattr(p, nm) for nm in names])
        fdp = (vals[0] - vals[1]) / (2 * hp)
        assert abs(float(gp[k]) - fdp) <= 1e-6 * abs(fdp) + 1e-9, (name, float(gp[k]), fdp)


@pytest.mark.parametrize("bc", [amps.BC_NOFLUX, amps.BC_PERIODIC])
def test_kobayashi_dot_product(bc):
    p = kob_params(bc=bc)
    _dot_test(p, kob_state(p), 1e-6)


@pytest.mark.parametrize("stencil,bc", [(0, amps.BC_PERIODIC), (0, amps.BC_NOFLUX), (1, amps.BC_NOFLUX)])
def test_graingrowth_dot_product(stencil, bc):
    p = gg_params(stencil=stencil, bc=bc)
    _dot_test(p, gg_state(p), 1e-6)


def _misfit_setup(dtype=torch.float64, nsteps=24):
    p = kob_params()
    x = kob_state(p)
    # target: the same rollout with delta = 0.04, K = 1.8
    tgt = adjoint.rollout(dev(x), p.replace(delta=0.04, kappa=1.8), nsteps)[0].detach()
    return p, x, tgt.to(dtype)


def _misfit(p, x, tgt, nsteps, pv, dtype=torch.float64, segment=0, t0_dir=None, eps=0.0):
    x0 = dev(x, dtype)
    if t0_dir is not None:
        x0[1] += eps * t0_dir.to(dtype)
    out = adjoint.rollout(x0, p, nsteps, param_values=pv, segment=segment)
    return 0.5 * ((out[0] - tgt) ** 2).sum()


def _grads(p, x, tgt, nsteps, dtype=torch.float64, segment=0, graphs=True):
    pv = torch.tensor([p.delta, p.kappa, p.epsb], dtype=torch.float64, requires_grad=True)
    x0 = dev(x, dtype).requires_grad_(True)
    out = adjoint.rollout(x0, p, nsteps, param_values=pv, segment=segment, graphs=graphs)
    loss = 0.5 * ((out[0] - tgt) ** 2).sum()
    loss.backward()
    return pv.grad.clone(), x0.grad.clone(), float(loss.detach())


def test_rollout_misfit_gradients_vs_fd():
    n = 24
    p, x, tgt = _misfit_setup(nsteps=n)
    gpar, gx, _ = _grads(p, x, tgt, n)
    base = [p.delta, p.kappa, p.epsb]
    for k in range(3):
        h = 1e-4 * abs(base[k])
        vp = torch.tensor([b + (h if i == k else 0) for i, b in enumerate(base)], dtype=torch.float64)
        vm = torch.tensor([b - (h if i == k else 0) for i, b in enumerate(base)], dtype=torch.float64)
        fd = (float(_misfit(p, x, tgt, n, vp)) - float(_misfit(p, x, tgt, n, vm))) / (2 * h)
        assert abs(float(gpar[k]) - fd) <= 1e-5 * abs(fd), (k, float(gpar[k]), fd)
    # initial temperature, along a random direction
    rng = np.random.default_rng(11)
    d = dev(rng.standard_normal((p.ny, p.nx)))
    pv = torch.tensor(base, dtype=torch.float64)
    h = 1e-6
    fd = (float(_misfit(p, x, tgt, n, pv, t0_dir=d, eps=h)) - float(_misfit(p, x, tgt, n, pv, t0_dir=d, eps=-h))) / (2 * h)
    ad = float((gx[1] * d).sum())
    assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)


def test_rollout_matches_unrolled_autograd():
    """Noisy dendrite seed, 24 steps: checkpointed CUDA adjoint vs autograd of
    the unrolled plain-PyTorch reference (float64 on the CPU)."""
    n = 24
    p = kob_params()
    x = kob_disc_state(p)
    tgt = torch.tensor(np.random.default_rng(2).uniform(0, 1, (p.ny, p.nx)))
    pv = torch.tensor([p.delta, p.kappa, p.epsb], dtype=torch.float64, requires_grad=True)
    xa = torch.tensor(x, requires_grad=True)
    s = xa
    for k in range(n):
        s = R.kob_step(s, p, pv[0], pv[1], pv[2], k)
    (0.5 * ((s[0] - tgt) ** 2).sum()).backward()
    gp, gx, _ = _grads(p, x, tgt.to(DEV), n)
    np.testing.assert_allclose(gp.numpy(), pv.grad.numpy(), rtol=1e-9)
    ref = xa.grad.numpy()
    assert np.abs(gx.cpu().numpy() - ref).max() <= 1e-9 * np.abs(ref).max()


def test_checkpoint_spacing_and_graphs_invariant():
    """Checkpoint spacing (keep-all, 5, sqrt N, one segment) and graph vs
    direct launches change nothing but the parameter sums' atomic order."""
    n = 24
    p, x, tgt = _misfit_setup(nsteps=n)
    ref_p, ref_x, ref_l = _grads(p, x, tgt, n, segment=n)
    for seg, graphs in ((1, True), (5, True), (0, True), (0, False), (7, False)):
        gp_, gx_, l_ = _grads(p, x, tgt, n, segment=seg, graphs=graphs)
        assert l_ == ref_l
        assert torch.equal(gx_, ref_x)
        assert torch.allclose(gp_, ref_p, rtol=1e-12, atol=0)


def test_rollout_handle_reuse_with_new_values():
    """One handle, two forward/backward rounds with different parameter values
    and step origins: the captured graphs read the new values."""
    n = 12
    p, x, tgt = _misfit_setup(nsteps=n)
    run = adjoint.Rollout(p, n)
    res = []
    for vals, s0 in (([p.delta, p.kappa, p.epsb], 0), ([0.03, 1.7, 0.011], 40)):
        pv = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
        x0 = dev(x).requires_grad_(True)
        out = adjoint.rollout(x0, p, n, param_values=pv, step0=s0, runner=run)
        (0.5 * ((out[0] - tgt) ** 2).sum()).backward()
        fresh = adjoint.rollout(dev(x), p.replace(delta=vals[0], kappa=vals[1], epsb=vals[2]), n, step0=s0,
                                graphs=False)
        assert torch.equal(out.detach(), fresh)
        res.append(pv.grad.clone())
    assert not torch.equal(res[0], res[1])
    run.close()


def test_fp32_adjoint_tracks_fp64():
    n = 24
    p, x, tgt = _misfit_setup(nsteps=n)
    gp64, gx64, _ = _grads(p, x, tgt, n)
    gp32, gx32, _ = _grads(p, x, tgt.float(), n, dtype=torch.float32)
    rel = ((gp32 - gp64).abs() / gp64.abs()).max().item()
    assert rel <= 2e-3, rel
    relx = float((gx32.double() - gx64).norm() / gx64.norm())
    assert relx <= 2e-3, relx


def test_graingrowth_rollout_gradients():
    n = 16
    p = gg_params()
    x = gg_state(p)
    tgt = adjoint.rollout(dev(x), p.replace(mobil=1.3), n).detach()
    base = [p.mobil, p.grcoef, p.gamma]

    def loss(pv, x0):
        out = adjoint.rollout(x0, p, n, param_values=pv)
        return 0.5 * ((out - tgt) ** 2).sum()

    pv = torch.tensor(base, dtype=torch.float64, requires_grad=True)
    x0 = dev(x).requires_grad_(True)
    loss(pv, x0).backward()
    for k in range(3):
        h = 1e-4 * abs(base[k])
        vp = torch.tensor([b + (h if i == k else 0) for i, b in enumerate(base)], dtype=torch.float64)
        vm = torch.tensor([b - (h if i == k else 0) for i, b in enumerate(base)], dtype=torch.float64)
        fd = (float(loss(vp, dev(x))) - float(loss(vm, dev(x)))) / (2 * h)
        assert abs(float(pv.grad[k]) - fd) <= 1e-5 * abs(fd), (k, float(pv.grad[k]), fd)
    d = dev(np.random.default_rng(5).standard_normal(x.shape))
    h = 1e-6
    b64 = torch.tensor(base, dtype=torch.float64)
    fd = (float(loss(b64, dev(x) + h * d)) - float(loss(b64, dev(x) - h * d))) / (2 * h)
    ad = float((x0.grad * d).sum())
    assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)


def test_invalid_arguments():
    import ctypes
    p = kob_params()
    st = adjoint.Stepper(p)
    x = dev(kob_state(p))
    lib = amps.lib()
    # in-place forward and adjoint are refused
    assert lib.amps_step_forward(ctypes.byref(st.params), amps.F64, ctypes.c_void_p(x.data_ptr()),
                                 ctypes.c_void_p(x.data_ptr()), 0, None) == 1
    gp = torch.zeros(3, dtype=torch.float64, device=DEV)
    assert lib.amps_step_adjoint(ctypes.byref(st.params), amps.F64, ctypes.c_void_p(x.data_ptr()),
                                 ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                 ctypes.c_void_p(gp.data_ptr()), 0, None) == 1
    # backward before forward
    run = adjoint.Rollout(p, 4)
    with pytest.raises(amps.AmpsError):
        run.backward(torch.zeros_like(x))
    with pytest.raises(ValueError):
        run.forward(x.float())
    run.close()
