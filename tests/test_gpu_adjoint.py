"""Adjoint (rmn_adjoint) against finite differences, through the C ABI.

The checked quantity is the vector-Jacobian product phi(theta) = <g, I(theta)>
for a fixed image adjoint g (the L2-loss gradient I - T against a target T
rendered at parameters perturbed by up to +-10%), I the linear composed image
(Photo::shade(Full)) of the 16-material Cornell variant.

* Base colour and emission: the estimator's random decisions do not depend
  on them, so with common random numbers (same seed) a central difference
  differentiates the same realisation the adjoint replays: agreement within
  2% (h = 1e-3), on the GPU renderer and on the CPU oracle (which draws the
  same counter-based streams).
* Roughness: the GGX sample directions, the branch choice and Russian
  roulette move with it, so a difference of one realisation is dominated by
  jumps; the adjoint uses the score function and is unbiased, not
  realisation-exact. Checked as means over independent seeds against the
  finite-difference means, within their standard errors.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from raym0nade_gb300 import api, scenes  # noqa: E402

MAXD = 8


def _cam(w, spp):
    return scenes.cornell_camera(w, w, spp, max_depth=MAXD)


def _forward(params, seed, w, spp):
    m = api.Model(scenes.cornell16(params))
    a = api.RenderArgs.from_camera(_cam(w, spp), seed=seed)
    ph = api.render(m, a)
    return m, a, ph, ph.shade(api.Full)


def _target_adjoint(p0, w, spp=64):
    """g = I(p0) - T, T rendered at perturbed parameters with another seed."""
    rng = np.random.default_rng(5)
    pt = p0.copy()
    pt[:, 0:4] *= rng.uniform(0.9, 1.1, (16, 4))
    pt[:, 4] *= 1.1
    _, _, _, t = _forward(pt, 99, w, spp)
    _, _, _, i0 = _forward(p0, 98, w, spp)
    return (i0 - t).reshape(-1, 3).contiguous()


def _phi(params, seed, w, spp, g):
    _, _, _, img = _forward(params, seed, w, spp)
    return float((img.reshape(-1, 3).double() * g.double()).sum())


def _fd(params, i, k, h, phi):
    pp, pm = params.copy(), params.copy()
    pp[i, k] += h
    pm[i, k] -= h
    return (phi(pp) - phi(pm)) / (2.0 * h)


def _check_rel(adj, fd, rel=0.02):
    scale = np.abs(fd).max()
    big = np.abs(fd) >= 1e-2 * scale
    assert big.sum() > 0
    err = np.abs(adj - fd)
    assert (err[big] <= rel * np.abs(fd[big])).all(), np.c_[adj, fd][big][err[big] > rel * np.abs(fd[big])]
    assert (err[~big] <= 2e-3 * scale).all()


def test_base_and_emission_match_crn_differences():
    p0 = scenes.cornell16_params()
    w, spp, seed = 40, 32, 3
    g = _target_adjoint(p0, w)
    m, a, ph, _ = _forward(p0, seed, w, spp)
    grad = api.adjoint(m, a, ph, g).cpu().numpy().astype(np.float64)
    phi = lambda p: _phi(p, seed, w, spp, g)
    adj, fd = [], []
    for i in range(16):
        for k in range(3):
            adj.append(grad[i, k])
            fd.append(_fd(p0, i, k, 1e-3, phi))
    adj.append(grad[scenes.CORNELL16_LIGHT, 4])
    fd.append(_fd(p0, scenes.CORNELL16_LIGHT, 4, 1e-3, phi))
    _check_rel(np.array(adj), np.array(fd))
    # emission of the non-emitters and base/roughness of the emitter: exactly 0
    others = [i for i in range(16) if i != scenes.CORNELL16_LIGHT]
    assert np.all(grad[others, 4] == 0.0)
    assert np.all(grad[scenes.CORNELL16_LIGHT, 0:4] == 0.0)


def test_base_matches_cpu_oracle_differences(port):
    """The oracle (CPU restatement, same random streams) differentiated by
    central differences against the GPU adjoint."""
    p0 = scenes.cornell16_params()
    w, spp, seed = 32, 16, 7
    cam = _cam(w, spp)
    g = _target_adjoint(p0, w)
    m, a, ph, _ = _forward(p0, seed, w, spp)
    grad = api.adjoint(m, a, ph, g).cpu().numpy().astype(np.float64)
    gn = g.cpu().numpy().astype(np.float64).reshape(w, w, 3)

    def phi(p):
        rec = port.scene(scenes.cornell16(p)).render(cam, seed=seed, mode=1)
        lin = rec[..., 16:19] * (rec[..., 0:3] + rec[..., 8:11]) + rec[..., 4:7] + rec[..., 12:15] + rec[..., 19:22]
        return float((np.nan_to_num(lin.astype(np.float64)) * gn).sum())

    mats = [0, 2, 3, 4, 6, 11]
    adj, fd = [], []
    for i in mats:
        for k in range(3):
            adj.append(grad[i, k])
            fd.append(_fd(p0, i, k, 1e-3, phi))
    adj.append(grad[scenes.CORNELL16_LIGHT, 4])
    fd.append(_fd(p0, scenes.CORNELL16_LIGHT, 4, 1e-3, phi))
    # a few pixels' paths branch differently on the two sides (CUDA's and
    # glibc's sinf/cosf differ in the last bit), hence 5% here
    _check_rel(np.array(adj), np.array(fd), rel=0.05)


def test_roughness_matches_differences_in_expectation():
    p0 = scenes.cornell16_params()
    w, spp, h, seeds = 32, 512, 0.02, [10, 11, 12, 13]
    g = _target_adjoint(p0, w)
    mats = [i for i in range(16) if i != scenes.CORNELL16_LIGHT]
    A, F = [], []
    for s in seeds:
        m, a, ph, _ = _forward(p0, s, w, spp)
        A.append(api.adjoint(m, a, ph, g).cpu().numpy().astype(np.float64)[mats, 3])
        F.append([_fd(p0, i, 3, h, lambda p: _phi(p, s, w, spp, g)) for i in mats])
    A, F = np.array(A), np.array(F)
    n = len(seeds)
    ma, mf = A.mean(0), F.mean(0)
    sa, sf = A.std(0, ddof=1) / np.sqrt(n), F.std(0, ddof=1) / np.sqrt(n)
    tol = 4.0 * np.sqrt(sa ** 2 + sf ** 2) + 0.02 * np.abs(mf) + 1e-3 * np.abs(mf).max()
    assert (np.abs(ma - mf) <= tol).all(), np.c_[ma, mf, sa, sf]
    # the score-function estimate is far less noisy than the differences
    assert np.median(sa) < np.median(sf)


class RenderFn(torch.autograd.Function):
    """I(params) for the 16-material Cornell box, with rmn_adjoint as the
    backward pass. params: (16, 5) base r, g, b, roughness, emission scale."""

    @staticmethod
    def forward(ctx, params, w, spp, seed):
        m, a, ph, img = _forward(params.detach().cpu().numpy().astype(np.float64), seed, w, spp)
        ctx.state = (m, a, ph)
        return img

    @staticmethod
    def backward(ctx, d_img):
        m, a, ph = ctx.state
        grad = api.adjoint(m, a, ph, d_img.reshape(-1, 3).contiguous().float())
        return grad.to(d_img.device, torch.float64), None, None, None


def test_autograd_function_and_descent():
    p0 = scenes.cornell16_params()
    w, spp, seed = 32, 32, 4
    target = _forward(np.where(np.arange(5) < 3, p0 * 0.8, p0), 50, w, 256)[3]
    params = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
    img = RenderFn.apply(params, w, spp, seed)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    m, a, ph, img2 = _forward(p0, seed, w, spp)
    direct = api.adjoint(m, a, ph, (2.0 * (img2 - target)).reshape(-1, 3).contiguous())
    np.testing.assert_allclose(params.grad.cpu().numpy(), direct.cpu().numpy(), rtol=1e-5, atol=1e-4)
    # a few steps of gradient descent on the base colours lower the loss
    losses = []
    with torch.no_grad():
        p = params.detach().clone()
    for _ in range(4):
        p.requires_grad_(True)
        lo = ((RenderFn.apply(p, w, spp, seed) - target) ** 2).sum()
        lo.backward()
        losses.append(float(lo.detach()))
        with torch.no_grad():
            step = torch.zeros_like(p)
            step[:, 0:3] = p.grad[:, 0:3]
            p = (p - 2e-3 * step / step.abs().max()).clamp(0.01, 1.0).detach()
    assert losses[-1] < losses[0]


def test_adjoint_argument_errors():
    m = api.Model(scenes.cornell16())
    a = api.RenderArgs.from_camera(_cam(16, 4), seed=1)
    ph = api.render(m, a)
    g = torch.zeros((16 * 16, 3), dtype=torch.float32, device="cuda")
    ph.dropped = None
    with pytest.raises(api.RmnError) as e:
        api.adjoint(m, a, ph, g)
    assert e.value.status == 1
    ph.dropped = torch.full((16 * 16,), -1, dtype=torch.int32, device="cuda")
    mg = api.Model(scenes.cornell_glass())
    pg = api.render(mg, a)
    with pytest.raises(api.RmnError) as e:
        api.adjoint(mg, a, pg, g)
    assert e.value.status == 4  # RMN_ERR_UNSUPPORTED


def test_c5_all_parameters_against_central_differences():
    """The differentiation configuration itself: the 16-material Cornell box
    at 512 x 512, depth 16, the L2 loss to a target rendered at parameters
    perturbed by up to +-10%, and all 16 x 5 parameters.

    The adjoint is checked at the sample count of its differences (1024 spp
    per seed; the timed configuration's 32 spp has another expectation,
    because the firefly clamp's bias depends on the sample count):
    * base colour and emission: central differences with common random
      numbers, h = 1e-3, differentiate the realisation the adjoint replays:
      within 2% (measured: 1e-4);
    * roughness: the difference of one realisation is dominated by jumps
      (branch flips, moved hits), so the means over 8 seeds (8192 spp in all)
      are compared, h = 1e-2 (at h = 1e-3 the jumps' variance, which grows
      as 1/h, is several times larger), within 2% plus four standard errors;
    * parameters that leave the scene unchanged (emission scale of the 15
      materials without emission) have an exactly zero difference: their
      adjoint must be exactly zero."""
    w, spp, maxd = 512, 1024, 16
    p0 = scenes.cornell16_params()
    cam = lambda n: scenes.cornell_camera(w, w, n, max_depth=maxd)

    def fwd(params, seed, n):
        m = api.Model(scenes.cornell16(params))
        a = api.RenderArgs.from_camera(cam(n), seed=seed)
        ph = api.render(m, a)
        return m, a, ph, ph.shade(api.Full)

    rng = np.random.default_rng(5)
    pt = p0.copy()
    pt[:, 0:4] *= rng.uniform(0.9, 1.1, (16, 4))
    pt[:, 4] *= 1.1
    g = (2.0 * (fwd(p0, 98, 256)[3] - fwd(pt, 99, 256)[3])).reshape(-1, 3).contiguous()
    gd = g.double()
    phi = lambda params, seed: float((fwd(params, seed, spp)[3].reshape(-1, 3).double() * gd).sum())
    base = scenes.cornell16(p0).materials

    def unchanged(params):
        return np.array_equal(scenes.cornell16(params).materials, base)

    def fd(i, k, h, seed):
        pp, pm = p0.copy(), p0.copy()
        pp[i, k] += h
        pm[i, k] -= h
        if unchanged(pp) and unchanged(pm):
            return None
        return (phi(pp, seed) - phi(pm, seed)) / (2.0 * h)

    seeds = list(range(1, 9))
    adj = []
    for s in seeds:
        m, a, ph, _ = fwd(p0, s, spp)
        adj.append(api.adjoint(m, a, ph, g).cpu().numpy().astype(np.float64))
    adj = np.array(adj)
    # base colour and emission, seed 1: the realisation's derivative
    a1, f1, zero = [], [], []
    for i in range(16):
        for k in (0, 1, 2, 4):
            d = fd(i, k, 1e-3, seeds[0])
            if d is None:
                zero.append(adj[0, i, k])
            else:
                a1.append(adj[0, i, k])
                f1.append(d)
    assert len(zero) == 15 and np.all(np.array(zero) == 0.0)
    _check_rel(np.array(a1), np.array(f1), rel=0.02)
    # roughness: means over the seeds
    F = np.array([[fd(i, 3, 1e-2, s) for i in range(16)] for s in seeds])
    A = adj[:, :, 3]
    n = len(seeds)
    ma, mf = A.mean(0), F.mean(0)
    se = np.sqrt(A.var(0, ddof=1) / n + F.var(0, ddof=1) / n)
    tol = 0.02 * np.abs(mf) + 4.0 * se + 1e-3 * np.abs(mf).max()
    print("roughness adjoint", np.round(ma, 1), "differences", np.round(mf, 1), "standard error", np.round(se, 1))
    assert (np.abs(ma - mf) <= tol).all(), np.c_[ma, mf, se]
