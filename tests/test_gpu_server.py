"""Request server (ee_server_*): every request's dose and fluence gradient
are the same whether it is computed alone on an engine context or batched
with other requests on the server, across volumes, request kinds and
concurrent submitters; admission refuses a request over the HBM budget."""
import threading

import numpy as np
import pytest

from endtoend_gb300 import engine, inputs

pytestmark = pytest.mark.gpu


def _volumes():
    a = inputs.slab_phantom(40, 0.25)
    b = inputs.head_neck_phantom(shape=(44, 40, 36), voxel_cm=0.25, seed=4)
    return [a, b]


def _requests(vols, n, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(n):
        v = int(rng.integers(0, len(vols)))
        nb = int(rng.integers(1, 4))
        beams = []
        for _ in range(nb):
            m = int(rng.integers(5, 12))
            b = inputs.single_beam(fmap=(m, m), beamlet_cm=0.4, gantry_deg=float(rng.uniform(0, 360)),
                                   couch_deg=float(rng.choice([0.0, 20.0, -30.0])))
            b.fluence = rng.uniform(0.1, 1.0, (m, m)).astype(np.float32)
            beams.append(b)
        grad = None
        if k % 2 == 1:
            grad = rng.standard_normal(vols[v].density.shape).astype(np.float32)
        reqs.append((v, beams, grad))
    return reqs


def _alone(vols, phys, reqs):
    import torch
    out = []
    engs = []
    for vol in vols:
        e = engine.Engine(0)
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        engs.append(e)
    for v, beams, grad in reqs:
        e = engs[v]
        nvox = vols[v].nvoxels
        fl = torch.from_numpy(engine.concat_fluence(beams)).cuda()
        dose = torch.zeros(nvox, device="cuda")
        if grad is None:
            e.beam_dose_device(beams, fl.data_ptr(), dose.data_ptr())
            e.synchronize()
            out.append((dose.cpu().numpy().reshape(vols[v].density.shape), None))
        else:
            g = torch.from_numpy(grad.ravel()).cuda()
            fg = torch.zeros_like(fl)
            e.dose_and_adjoint_device(beams, fl.data_ptr(), dose.data_ptr(), g.data_ptr(), fg.data_ptr())
            e.synchronize()
            out.append((dose.cpu().numpy().reshape(vols[v].density.shape), fg.cpu().numpy()))
    for e in engs:
        e.close()
    return out


def _check(reqs, ref, got):
    for k, ((v, beams, grad), (d0, f0), (d1, f1)) in enumerate(zip(reqs, ref, got)):
        scale = float(d0.max())
        assert scale > 0, k
        assert np.allclose(d1, d0, rtol=1e-5, atol=1e-6 * scale), (k, float(np.abs(d1 - d0).max() / scale))
        if grad is not None:
            f1 = np.concatenate([x.ravel() for x in f1])
            fs = float(np.abs(f0).max())
            assert np.allclose(f1, f0, rtol=1e-4, atol=1e-5 * fs), (k, float(np.abs(f1 - f0).max() / fs))
        else:
            assert f1 is None


def test_server_same_alone_and_in_the_mix():
    vols = _volumes()
    phys = inputs.make_physics(seed=7, spacing_cm=0.25)
    reqs = _requests(vols, 10, seed=21)
    ref = _alone(vols, phys, reqs)
    with engine.Server(0, slots=2, max_batch_beams=8) as srv:
        srv.set_physics(phys, mode="exp")
        ids = [srv.add_volume(v) for v in vols]
        assert ids == [0, 1]
        tickets = [srv.submit(v, beams, grad) for v, beams, grad in reqs]
        got = [srv.wait(t) for t in tickets]
        _check(reqs, ref, got)
        st = srv.stats()
        assert st["completed"] == len(reqs)
        assert st["p99_ms"] >= st["p50_ms"] > 0
        # one request at a time on the same server: the same numbers again
        got1 = [srv.wait(srv.submit(v, beams, grad)) for v, beams, grad in reqs]
        _check(reqs, ref, got1)


def test_server_concurrent_submitters():
    vols = _volumes()
    phys = inputs.make_physics(seed=7, spacing_cm=0.25)
    reqs = _requests(vols, 12, seed=5)
    ref = _alone(vols, phys, reqs)
    got = [None] * len(reqs)
    with engine.Server(0, slots=3, max_batch_beams=6) as srv:
        srv.set_physics(phys, mode="exp")
        for v in vols:
            srv.add_volume(v)

        def client(idx):
            tickets = [(k, srv.submit(*reqs[k])) for k in idx]
            for k, t in tickets:
                got[k] = srv.wait(t)

        ths = [threading.Thread(target=client, args=(list(range(j, len(reqs), 3)),)) for j in range(3)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
    _check(reqs, ref, got)


def test_server_admission_and_errors():
    vols = _volumes()
    phys = inputs.make_physics(seed=7, spacing_cm=0.25)
    v, beams, _ = _requests(vols, 1, seed=3)[0]
    with engine.Server(0, slots=1, hbm_budget=1 << 20) as srv:  # 1 MiB: nothing fits
        srv.set_physics(phys, mode="exp")
        srv.add_volume(vols[0])
        srv.add_volume(vols[1])
        t = srv.submit(v, beams)
        with pytest.raises(engine.EEError) as ei:
            srv.wait(t)
        assert ei.value.code == engine.EE_ERR_NOMEM
        with pytest.raises(engine.EEError):
            srv.submit(7, beams)  # unknown volume


def test_server_serving_workload_sizes():
    """The serving workload at its stated sizes: head-and-neck phantoms of
    96^3, 128^3, 160^3 and 256x256x192 voxels at 2 mm, requests of 1-40 beams
    with fluence grids 16^2-64^2, dose or dose + gradient (the first 12
    requests of the seeded 50/s stream, all queued at once on 2 slots): every
    request equals its result alone (rtol 1e-5 dose, 1e-4 gradient)."""
    vols, raw = inputs.serving_workload(12, 50.0, seed=9)
    rng = np.random.default_rng(13)
    grads = [rng.standard_normal(v.density.shape).astype(np.float32) for v in vols]
    reqs = [(r["volume"], r["beams"], grads[r["volume"]] if r["grad"] else None) for r in raw]
    assert {len(b) for _, b, _ in reqs} and max(len(b) for _, b, _ in reqs) > 20
    phys = inputs.make_physics(seed=0, spacing_cm=0.2)
    ref = _alone(vols, phys, reqs)
    with engine.Server(0, slots=2, max_batch_beams=256) as srv:
        srv.set_physics(phys, mode="exp")
        for v in vols:
            srv.add_volume(v)
        tickets = [srv.submit(v, beams, grad) for v, beams, grad in reqs]
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
    _check(reqs, ref, got)
    assert st["completed"] == len(reqs)
