"""Beam sharding over ranks (endtoend_gb300/distributed.py) on the CPU:
world_size 2 over gloo, the per-rank compute done by the FP64 oracle.  The
sharded dose and the sharded loss gradient equal the single-process results;
the beam assignment is the reference's (dosecalc-beam/main.cu:241-261)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from endtoend_gb300 import distributed, inputs


def test_beam_shards_follow_the_reference_assignment():
    assert distributed.beam_shards(10, 3) == [(0, 4), (4, 3), (7, 3)]
    assert distributed.beam_shards(2, 4) == [(0, 1), (1, 1), (2, 0), (2, 0)]
    assert distributed.beam_shards(0, 2) == [(0, 0), (0, 0)]
    shards = distributed.beam_shards(1024, 8)
    assert sum(n for _, n in shards) == 1024 and all(n == 128 for _, n in shards)
    with pytest.raises(ValueError):
        distributed.beam_shards(4, 0)


def _case():
    vol = inputs.slab_phantom(20, 0.5)
    phys = inputs.make_physics(seed=1, spacing_cm=0.5)
    rng = np.random.default_rng(3)
    beams = []
    for g, c in [(0.0, 0.0), (90.0, 10.0), (200.0, -20.0)]:
        b = inputs.single_beam(fmap=(4, 4), beamlet_cm=1.0, gantry_deg=g, couch_deg=c)
        b.fluence = rng.uniform(0.2, 1.0, (4, 4)).astype(np.float32)
        beams.append(b)
    target = np.full(vol.density.shape, 0.01)
    return vol, phys, beams, target


def _funcs(vol, phys, target):
    from oracle.oracle import Oracle
    o = Oracle(vol, phys, kernel_mode=2, nthreads=2)

    def local_dose(shard):
        d = np.zeros(vol.density.shape)
        for b in shard:
            d += o.beam_dose(b)[0]
        return torch.from_numpy(d)

    def local_adjoint(shard, gdose):
        g = gdose.numpy()
        parts = [o.beam_dose_adjoint(b, g)[0].ravel() for b in shard]
        return torch.from_numpy(np.concatenate(parts) if parts else np.zeros(0))

    def dose_loss(dose):
        r = dose - torch.from_numpy(target)
        return float((r * r).sum()), 2.0 * r

    return local_dose, local_adjoint, dose_loss


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        vol, phys, beams, target = _case()
        local_dose, local_adjoint, dose_loss = _funcs(vol, phys, target)
        sizes = [int(b.fluence.size) for b in beams]
        loss, grad, dose = distributed.sharded_loss_and_grad(local_dose, local_adjoint, dose_loss, beams, sizes)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), loss=loss, grad=grad.numpy(), dose=dose.numpy())
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_dose_and_gradient_over_gloo(tmp_path):
    vol, phys, beams, target = _case()
    local_dose, local_adjoint, dose_loss = _funcs(vol, phys, target)
    dose1 = local_dose(beams)
    loss1, gd = dose_loss(dose1)
    grad1 = local_adjoint(beams, gd).numpy()
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        z = np.load(os.path.join(str(tmp_path), f"rank{r}.npz"))
        np.testing.assert_allclose(z["dose"], dose1.numpy(), rtol=1e-12, atol=1e-15 * float(dose1.max()))
        assert abs(float(z["loss"]) - loss1) <= 1e-10 * abs(loss1)
        np.testing.assert_allclose(z["grad"], grad1, rtol=1e-10, atol=1e-14 * float(np.abs(grad1).max()))
        assert z["grad"].shape == (sum(int(b.fluence.size) for b in beams),)
