"""Parity at the stated sizes of the batched-candidate (200x200x160 phantom,
1024-beam grid), annealing-loss and beamlet-coefficient workloads.

* Candidate beams: three beams spread over the 1024-beam 4-pi grid on the
  200x200x160 head-and-neck phantom at 2 mm, computed in one batched call
  (per-beam outputs).  Exp fast path against the FP64 oracle of the same
  operator <= 1e-3 of Dmax, and against the reference discretisation (24-radius
  table, texture-unit 8-bit weights) <= 5e-3 of Dmax with a 1 %/1 mm gamma
  pass rate >= 99.5 %; the table mode against the FP64 oracle of the table
  <= 1e-3 and against the reference discretisation <= 1.5e-3.
* Annealing loss: 20 beams of 128x128 fluence pixels of 0.78 mm on the same
  phantom with a PTV and three OARs, Gaussian spread sigma 1.5 px, eta 1e-3.
  The gradient of ee_loss_and_grad against central differences (step 1e-3)
  of the loss on 64 seeded pixels.  The loss is evaluated in FP64 from the
  engine's doses: the dose is linear in the fluence, so the dose change of a
  pixel is taken from one extra beam call with that pixel's spread delta
  added (x 10) to the beam's whole map, which keeps the beam's crop box.
  Tolerance 2e-3 of max |dL/dx|.  A batch of proposals (angles moved by
  N(0, 5 deg)) is checked against independent loss evaluations (rel 1e-4).
The beamlet-coefficient workload is in test_gpu_beamlet_cfg4.py.
"""
import numpy as np
import pytest
from scipy.ndimage import convolve

from endtoend_gb300 import engine, inputs, metrics
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _rel(a, ref):
    return float(np.abs(a.astype(np.float64) - ref).max() / np.abs(ref).max())


# ------------------------------------------------------- candidate beams ----
@pytest.fixture(scope="module")
def cand():
    vol, phys, beams = inputs.config1(1024)
    beams = [beams[i] for i in (0, 511, 1023)]
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        d_exp = e.beam_dose(beams, per_beam=True)
        e.set_mode("table")
        d_tab = e.beam_dose(beams, per_beam=True)
    return vol, phys, beams, d_exp, d_tab


@pytest.mark.parametrize("k", [0, 1, 2])
def test_candidate_beams_full_phantom(cand, k):
    vol, phys, beams, d_exp, d_tab = cand
    b = beams[k]
    ref = Oracle(vol, phys, kernel_mode=0, tex_emulate=True).beam_dose(b)[0]
    e64 = Oracle(vol, phys, kernel_mode=2).beam_dose(b)[0]
    t64 = Oracle(vol, phys, kernel_mode=0).beam_dose(b)[0]
    err = {"exp_vs_fp64": _rel(d_exp[k], e64), "exp_vs_reference": _rel(d_exp[k], ref),
           "table_vs_fp64": _rel(d_tab[k], t64), "table_vs_reference": _rel(d_tab[k], ref)}
    gamma = metrics.gamma_pass_rate(d_exp[k], ref, voxel_mm=2.0)
    print(f"candidate beam {k} (fluence {b.fluence.shape}): {err}, gamma 1%/1mm {gamma:.4f}")
    assert err["exp_vs_fp64"] <= 1e-3
    assert err["exp_vs_reference"] <= 5e-3
    assert gamma >= 0.995
    assert err["table_vs_fp64"] <= 1e-3
    assert err["table_vs_reference"] <= 1.5e-3


# --------------------------------------------------------- annealing loss ----
SIGMA, ETA, H = 1.5, 1e-3, 1e-3


def _gauss(sigma):
    R = int(np.ceil(3 * sigma))
    k = np.exp(-0.5 * (np.arange(-R, R + 1) / sigma) ** 2)
    k /= k.sum()
    return np.outer(k, k)


def _spread(x, K):
    return convolve(x.astype(np.float64), K, mode="constant", cval=0.0)


def _smooth(x):
    return np.abs(np.diff(x, axis=1)).sum() + np.abs(np.diff(x, axis=0)).sum()


@pytest.fixture(scope="module")
def anneal():
    vol = inputs.head_neck_phantom(shape=(200, 200, 160), voxel_cm=0.2, with_oars=True)
    phys = inputs.make_physics(seed=0, spacing_cm=0.2)
    rng = np.random.default_rng(21)
    ptv = vol.masks["PTV"].astype(np.float32)
    ow = np.zeros_like(ptv)
    ot = np.zeros_like(ptv)
    for k in range(3):
        m = vol.masks[f"OAR{k}"]
        ow[m] += rng.uniform(0.1, 0.5)
        ot[m] = rng.uniform(0.3, 0.6)
    beams = []
    for g, c in inputs.four_pi_angles(20, step_deg=18.0, seed=8):
        b = inputs.single_beam(fmap=(128, 128), beamlet_cm=0.078, gantry_deg=float(g), couch_deg=float(c))
        b.fluence = rng.uniform(0.0, 1.0, (128, 128)).astype(np.float32)
        beams.append(b)
    return vol, phys, beams, (ptv, ptv.copy(), ow, ot), rng


def _loss_d(dose, arrays):
    w0, t0, w, t = arrays
    return float(np.sum(w0 * (dose - t0) ** 2) + np.sum(w * np.maximum(dose - t, 0.0) ** 2))


def test_annealing_loss_gradient_central_differences(anneal):
    import torch

    vol, phys, beams, arrays, _ = anneal
    arr64 = [a.astype(np.float64) for a in arrays]
    dv = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32).ravel()).cuda()
    w0, t0, w, t = (dv(a) for a in arrays)
    x = dv(engine.concat_fluence(beams))
    dose = torch.zeros(vol.nvoxels, device="cuda")
    xg = torch.zeros_like(x)
    K = _gauss(SIGMA)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        terms = e.loss_and_grad_device(beams, x.data_ptr(), dose.data_ptr(), xg.data_ptr(),
                                       ptv=(w0.data_ptr(), t0.data_ptr()), oar=(w.data_ptr(), t.data_ptr()),
                                       eta=ETA, spread_sigma=SIGMA)
        torch.cuda.synchronize()
        xg = xg.cpu().numpy().astype(np.float64)
        # per-beam doses of the spread maps, and the loss from them in FP64
        spread = [_spread(b.fluence, K) for b in beams]
        dk = []
        for b, s in zip(beams, spread):
            bs = inputs.Beam(**{**b.__dict__, "fluence": s.astype(np.float32)})
            dk.append(e.beam_dose([bs]).astype(np.float64))
        d = np.sum(dk, axis=0)
        ref_terms = _loss_d(d, arr64) + ETA * sum(_smooth(b.fluence.astype(np.float64)) for b in beams)
        assert abs(sum(terms) - ref_terms) <= 1e-4 * abs(ref_terms), (terms, ref_terms)
        # 64 seeded pixels away from the smoothness term's kinks (a neighbour
        # within 2h makes the central difference straddle |.|'s corner)
        rng = np.random.default_rng(17)
        sizes = [b.fluence.size for b in beams]
        offs = np.cumsum([0] + sizes)
        cand = []
        for k, b in enumerate(beams):
            f = b.fluence.astype(np.float64)
            ok = np.ones(f.shape, bool)
            dx = np.abs(np.diff(f, axis=1)) < 2 * H
            dy = np.abs(np.diff(f, axis=0)) < 2 * H
            ok[:, :-1] &= ~dx
            ok[:, 1:] &= ~dx
            ok[:-1, :] &= ~dy
            ok[1:, :] &= ~dy
            cand.append(np.nonzero(ok.ravel())[0] + offs[k])
        picks = rng.choice(np.concatenate(cand), size=64, replace=False)
        C = 10.0
        fd, eg = [], []
        for p in picks:
            k = int(np.searchsorted(offs, p, side="right") - 1)
            q = int(p - offs[k])
            delta = np.zeros_like(beams[k].fluence, dtype=np.float64)
            delta.ravel()[q] = 1.0
            stamp = _spread(delta, K)
            bp = inputs.Beam(**{**beams[k].__dict__, "fluence": (spread[k] + C * stamp).astype(np.float32)})
            dd = (e.beam_dose([bp]).astype(np.float64) - dk[k]) / C
            f = beams[k].fluence.astype(np.float64)
            fp, fm = f.copy(), f.copy()
            fp.ravel()[q] += H
            fm.ravel()[q] -= H
            g = (_loss_d(d + H * dd, arr64) - _loss_d(d - H * dd, arr64)) / (2 * H)
            g += ETA * (_smooth(fp) - _smooth(fm)) / (2 * H)
            fd.append(g)
            eg.append(xg[p])
    fd, eg = np.array(fd), np.array(eg)
    scale = np.abs(fd).max()
    err = np.abs(fd - eg).max() / scale
    print(f"annealing loss: 64 central differences vs gradient, max |diff| / max |FD| = {err:.2e} (scale {scale:.3e})")
    assert scale > 0
    assert err <= 2e-3


def test_annealing_proposals_full_size(anneal):
    import torch

    vol, phys, beams, arrays, _ = anneal
    rng = np.random.default_rng(33)
    dv = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32).ravel()).cuda()
    w0, t0, w, t = (dv(a) for a in arrays)
    x = dv(engine.concat_fluence(beams))
    props = []
    for _ in range(4):
        prop = []
        for b in beams:
            c = inputs.Beam(**{**b.__dict__})
            c.azimuth = b.azimuth + float(rng.normal(0, np.radians(5)))
            c.zenith = b.zenith + float(rng.normal(0, np.radians(5)))
            prop.append(c)
        props.append(prop)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        L = e.make_loss(ptv=(w0.data_ptr(), t0.data_ptr()), oar=(w.data_ptr(), t.data_ptr()), eta=ETA,
                        spread_sigma=SIGMA)
        got = e.evaluate_proposals(props, x.data_ptr(), L)
        dose = torch.zeros(vol.nvoxels, device="cuda")
        xg = torch.zeros_like(x)
        for i, prop in enumerate(props):
            terms = e.loss_and_grad_device(prop, x.data_ptr(), dose.data_ptr(), xg.data_ptr(),
                                           ptv=(w0.data_ptr(), t0.data_ptr()), oar=(w.data_ptr(), t.data_ptr()),
                                           eta=ETA, spread_sigma=SIGMA)
            ref = terms[0] + terms[1]
            assert abs(got[i] - ref) <= 1e-4 * abs(ref), (i, got[i], ref)
