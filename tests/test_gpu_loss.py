"""EndtoEnd loss and fluence gradient on the GPU (ee_loss_and_grad).

The gradient of
    L = sum w0 (d - t0)^2 + sum w (d - t)_+^2 + eta sum_k ||D x_k||_1,
    d = sum_k A_k (G * x_k)
is checked (a) against central finite differences (step 1e-3) of the FP64
oracle's loss on 64 seeded pixels -- only the perturbed beam's dose is
recomputed, with its whole fluence map so that its crop box stays the one of
the unperturbed call -- and (b) against the oracle's own adjoint.
Tolerance: 2e-3 of max |dL/dx|.
"""
import numpy as np
import pytest
from scipy.ndimage import convolve

from endtoend_gb300 import engine, inputs
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

SIGMA = 1.5
ETA = 1e-3


def _gauss(sigma):
    R = int(np.ceil(3 * sigma))
    k = np.exp(-0.5 * (np.arange(-R, R + 1) / sigma) ** 2)
    k /= k.sum()
    return np.outer(k, k)


def _spread(x, K):
    return convolve(x.astype(np.float64), K, mode="constant", cval=0.0)


def _smooth(x):
    dx = np.diff(x, axis=1)
    dy = np.diff(x, axis=0)
    g = np.zeros_like(x)
    g[:, :-1] -= np.sign(dx)
    g[:, 1:] += np.sign(dx)
    g[:-1, :] -= np.sign(dy)
    g[1:, :] += np.sign(dy)
    return np.abs(dx).sum() + np.abs(dy).sum(), g


@pytest.fixture(scope="module")
def problem():
    vol = inputs.slab_phantom(32, 0.25)
    phys = inputs.make_physics(seed=5, spacing_cm=0.25)
    nz, ny, nx = vol.density.shape
    zz, yy, xx = np.meshgrid(*[(np.arange(n) - (n - 1) / 2) * 0.25 for n in (nz, ny, nx)], indexing="ij")
    ptv = (xx ** 2 + yy ** 2 + zz ** 2) <= 1.5 ** 2
    oar = ((xx - 1.8) ** 2 / 1.0 + (yy + 0.5) ** 2 / 2.0 + zz ** 2 / 1.5) <= 1.0
    oar &= ~ptv
    w0 = ptv.astype(np.float32)
    t0 = ptv.astype(np.float32) * 1.0
    w = oar.astype(np.float32) * 0.3
    t = oar.astype(np.float32) * 0.4
    rng = np.random.default_rng(9)
    beams = []
    for g, c in [(15.0, 0.0), (140.0, 25.0), (260.0, -30.0)]:
        b = inputs.single_beam(fmap=(24, 24), beamlet_cm=0.15, gantry_deg=g, couch_deg=c)
        b.fluence = rng.uniform(0.2, 1.0, (24, 24)).astype(np.float32)
        beams.append(b)
    return vol, phys, beams, (w0, t0, w, t)


def _engine_grad(vol, phys, beams, arrays):
    import torch
    w0, t0, w, t = (torch.from_numpy(a.ravel()).cuda() for a in arrays)
    x = torch.from_numpy(engine.concat_fluence(beams)).cuda()
    dose = torch.zeros(vol.nvoxels, dtype=torch.float32, device="cuda")
    xg = torch.zeros_like(x)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        terms = e.loss_and_grad_device(beams, x.data_ptr(), dose.data_ptr(), xg.data_ptr(),
                                       ptv=(w0.data_ptr(), t0.data_ptr()), oar=(w.data_ptr(), t.data_ptr()),
                                       eta=ETA, spread_sigma=SIGMA)
        torch.cuda.synchronize()
    return terms, dose.cpu().numpy().reshape(vol.density.shape), xg.cpu().numpy()


def _oracle_pieces(vol, phys, beams, arrays):
    """Per-beam oracle doses of the spread fluence and the oracle gradient."""
    w0, t0, w, t = (a.astype(np.float64) for a in arrays)
    K = _gauss(SIGMA)
    o = Oracle(vol, phys, kernel_mode=2)
    dose = np.zeros(vol.density.shape)
    for b in beams:
        bs = inputs.Beam(**{**b.__dict__, "fluence": _spread(b.fluence, K).astype(np.float32)})
        dose += o.beam_dose(bs)[0]
    gd = 2 * w0 * (dose - t0) + 2 * w * np.maximum(dose - t, 0)
    grads = []
    for b in beams:
        bs = inputs.Beam(**{**b.__dict__, "fluence": _spread(b.fluence, K).astype(np.float32)})
        fg = o.beam_dose_adjoint(bs, gd)[0]
        _, sg = _smooth(b.fluence.astype(np.float64))
        grads.append(_spread(fg, K) + ETA * sg)
    return o, K, dose, grads


def _loss(dose, arrays, beams):
    w0, t0, w, t = (a.astype(np.float64) for a in arrays)
    ld = np.sum(w0 * (dose - t0) ** 2) + np.sum(w * np.maximum(dose - t, 0) ** 2)
    ls = sum(_smooth(b.fluence.astype(np.float64))[0] for b in beams)
    return ld + ETA * ls


def test_loss_terms_and_gradient_vs_oracle(problem):
    vol, phys, beams, arrays = problem
    terms, dose, xg = _engine_grad(vol, phys, beams, arrays)
    _, _, odose, ograds = _oracle_pieces(vol, phys, beams, arrays)
    assert np.abs(dose - odose).max() <= 1e-3 * odose.max()
    ref = _loss(odose, arrays, beams)
    assert abs(sum(terms) - ref) <= 1e-3 * abs(ref), (terms, ref)
    og = np.concatenate([g.ravel() for g in ograds])
    assert np.abs(xg - og).max() <= 2e-3 * np.abs(og).max()


def test_gradient_central_differences_64_pixels(problem):
    vol, phys, beams, arrays = problem
    _, _, xg = _engine_grad(vol, phys, beams, arrays)
    o, K, dose, _ = _oracle_pieces(vol, phys, beams, arrays)
    rng = np.random.default_rng(17)
    sizes = [b.fluence.size for b in beams]
    offs = np.cumsum([0] + sizes)
    h = 1e-3
    # the L1 smoothness term has kinks where neighbouring pixels are equal:
    # pixels with a neighbour within 2h are excluded (a central difference
    # across a kink is not the derivative at either side)
    smooth_ok = []
    for b in beams:
        f = b.fluence.astype(np.float64)
        ok = np.ones(f.shape, bool)
        dx = np.abs(np.diff(f, axis=1)) < 2 * h
        dy = np.abs(np.diff(f, axis=0)) < 2 * h
        ok[:, :-1] &= ~dx
        ok[:, 1:] &= ~dx
        ok[:-1, :] &= ~dy
        ok[1:, :] &= ~dy
        smooth_ok.append(ok.ravel())
    cand = np.nonzero(np.concatenate(smooth_ok))[0]
    picks = rng.choice(cand, size=64, replace=False)
    fd, eg = [], []
    for p in picks:
        k = int(np.searchsorted(offs, p, side="right") - 1)
        q = int(p - offs[k])
        # beam k's dose at x_k +- h e_p, full fluence map (the crop box is
        # set by the whole map, so it is the same as in the unperturbed call)
        dk = {}
        for sgn in (+1, -1):
            f = beams[k].fluence.astype(np.float64).copy()
            f.ravel()[q] += sgn * h
            bk = inputs.Beam(**{**beams[k].__dict__, "fluence": _spread(f, K).astype(np.float64)})
            dk[sgn] = o.beam_dose(bk)[0]
        b0 = inputs.Beam(**{**beams[k].__dict__, "fluence": _spread(beams[k].fluence, K)})
        d0 = o.beam_dose(b0)[0]
        lp = _loss(dose - d0 + dk[+1], arrays, _perturbed(beams, k, q, +h))
        lm = _loss(dose - d0 + dk[-1], arrays, _perturbed(beams, k, q, -h))
        fd.append((lp - lm) / (2 * h))
        eg.append(xg[p])
    fd, eg = np.array(fd), np.array(eg)
    scale = np.abs(fd).max()
    assert scale > 0
    assert np.abs(fd - eg).max() <= 2e-3 * scale + 1e-6, np.abs(fd - eg).max() / scale


def _perturbed(beams, k, q, h):
    out = []
    for i, b in enumerate(beams):
        f = b.fluence.astype(np.float64).copy()
        if i == k:
            f.ravel()[q] += h
        out.append(inputs.Beam(**{**b.__dict__, "fluence": f}))
    return out
