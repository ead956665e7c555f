"""Benchmark of the CCCS beam-dose engine (forward + adjoint beam-doses/s).

Workload (one step): the batched candidate-beam set -- 200x200x160 voxel
head-and-neck-like phantom at 2 mm, 1024 non-coplanar beams on a ~6 degree
4-pi grid, per-beam fluence maps of 8^2..40^2 beamlets of 2.5 mm with U(0,1)
weights, 8x6 = 48 double-exponential collapsed cones, FP32.  One step is the
forward dose of every beam plus the adjoint (fluence gradient) of every beam.
Inputs are seeded synthetic data (no public dataset exists for this path).

value : beam-doses/s with inputs resident in HBM (CUDA events on the engine
        stream, L2 flushed between steps).
e2e   : the same through the host-pointer C-ABI calls (pinned host fluence and
        dose gradient in, dose and fluence gradient out).
plain : one beam per call (the plain per-beam path), for the batched/plain ratio.

``--impl reference`` times the CPU restatement of the reference algorithm
(24-radius cumulative-kernel walk, FP32, OpenMP on all host cores) on a
bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "beam-doses/s fwd+adjoint batched vs plain, 1 GB300, <=0.5% Dmax err; p50/p99 ms"
UNIT = "beam-doses/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--beams", type=int, default=1024)
    ap.add_argument("--plain-beams", type=int, default=32)
    ap.add_argument("--scratch-gb", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-slots", type=int, default=2)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--beamlet-beams", type=int, default=64)
    ap.add_argument("--table-beams", type=int, default=64)
    ap.add_argument("--no-table", action="store_true")
    ap.add_argument("--no-beamlet", action="store_true")
    ap.add_argument("--no-anneal", action="store_true")
    ap.add_argument("--clocks-csv", default=None, help="keep the nvidia-smi samples of the timed region here")
    ap.add_argument("--profile-case", default=None, choices=["exp", "table", "walk"],
                    help="small case for ncu captures: forward + adjoint of --profile-beams beams of the workload, "
                         "twice, in this kernel mode; prints one line and exits")
    ap.add_argument("--profile-beams", type=int, default=2)
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl"
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, path=None):
        """path: keep the raw samples there (CSV); by default a temporary file
        that is removed once the summary is read."""
        self.index = index
        self.proc = None
        self.keep = path is not None
        self.path = path

    def start(self):
        try:
            if self.keep:
                os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
            else:
                fd, self.path = tempfile.mkstemp(prefix=f"ee_clocks_rank{self.index}_", suffix=".csv")
                os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            if not self.keep and self.path:
                try:
                    os.remove(self.path)
                except OSError:
                    pass
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not self.keep:
            try:
                os.remove(self.path)
            except OSError:
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(n_beams, seed_offset=0):
    from endtoend_gb300 import inputs
    vol = inputs.head_neck_phantom(shape=(200, 200, 160), voxel_cm=0.2)
    phys = inputs.make_physics(seed=0, spacing_cm=0.2)
    beams = inputs.candidate_beams(n_beams, seed=3 + seed_offset)
    return vol, phys, beams


def annealing_leg(args, eng, phys):
    """Annealing loss (config 2): the head-and-neck phantom with PTV weight 1 /
    target 1 and three OAR ellipsoids (weights 0.1-0.5, thresholds 0.3-0.6),
    20 beams of 128x128 fluence pixels of 0.78 mm, Gaussian spread sigma 1.5
    px, eta 1e-3.  Times ee_loss_and_grad (forward + adjoint of the 20 beams),
    a batch of 64 proposals (every angle moved by N(0, 5 deg), one grouped
    call over 1280 beams) and one annealing iteration (20 per-beam proposals,
    sequential acceptance, one fluence step)."""
    import torch
    from endtoend_gb300 import inputs
    vol = inputs.head_neck_phantom(shape=(200, 200, 160), voxel_cm=0.2, with_oars=True)
    eng.set_volume(vol)
    rng = np.random.default_rng(21)
    ptv = vol.masks["PTV"].astype(np.float32)
    ow = np.zeros_like(ptv)
    ot = np.zeros_like(ptv)
    for k in range(3):
        m = vol.masks[f"OAR{k}"]
        ow[m] += rng.uniform(0.1, 0.5)
        ot[m] = rng.uniform(0.3, 0.6)
    dv = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32).ravel()).cuda()
    t = {"pw": dv(ptv), "pt": dv(ptv), "ow": dv(ow), "ot": dv(ot)}
    L = eng.make_loss(ptv=(t["pw"].data_ptr(), t["pt"].data_ptr()), oar=(t["ow"].data_ptr(), t["ot"].data_ptr()),
                      eta=1e-3, spread_sigma=1.5)
    beams = []
    for g, c in inputs.four_pi_angles(20, step_deg=18.0, seed=8):
        b = inputs.single_beam(fmap=(128, 128), beamlet_cm=0.078, gantry_deg=float(g), couch_deg=float(c))
        b.fluence = rng.uniform(0.0, 1.0, (128, 128)).astype(np.float32)
        beams.append(b)
    x = dv(engine_concat(beams))
    dose = torch.zeros(vol.nvoxels, device="cuda")
    grad = torch.zeros_like(x)

    def lg():
        return eng.loss_and_grad_device(beams, x.data_ptr(), dose.data_ptr(), grad.data_ptr(),
                                        ptv=(t["pw"].data_ptr(), t["pt"].data_ptr()),
                                        oar=(t["ow"].data_ptr(), t["ot"].data_ptr()), eta=1e-3, spread_sigma=1.5)

    lg()
    t0 = time.perf_counter()
    for _ in range(3):
        lg()
    t_lg = (time.perf_counter() - t0) / 3
    props = []
    for q in range(64):
        prop = []
        for b in beams:
            c = inputs.Beam(**{**b.__dict__})
            c.azimuth = b.azimuth + float(rng.normal(0, np.radians(5)))
            c.zenith = b.zenith + float(rng.normal(0, np.radians(5)))
            prop.append(c)
        props.append(prop)
    eng.evaluate_proposals(props[:2], x.data_ptr(), L)
    t0 = time.perf_counter()
    eng.evaluate_proposals(props, x.data_ptr(), L)
    t_prop = time.perf_counter() - t0
    t0 = time.perf_counter()
    eng.optimize_annealing(beams, x.data_ptr(), L, iterations=1, step_size=1e-3, sigma_deg=5.0, temperature=1e-3,
                           fluence_steps=1, seed=3)
    t_it = time.perf_counter() - t0
    return {"workload": "200x200x160 @2mm head-neck phantom, PTV + 3 OARs, 20 beams x 128^2 fluence @0.78 mm, "
                        "spread sigma 1.5 px, eta 1e-3; 64 proposals of N(0,5 deg) angle moves",
            "loss_and_grad_ms": t_lg * 1e3, "loss_and_grad_beam_doses_per_s": 20 / t_lg,
            "proposals_per_s": 64 / t_prop, "proposal_beam_doses_per_s": 64 * 20 / t_prop,
            "anneal_iteration_s": t_it}


def engine_concat(beams):
    from endtoend_gb300 import engine
    return engine.concat_fluence(beams)


def measured_6x_physics(spacing_cm):
    """The reference's cumulative kernel for its measured 6 MV spectrum and
    dsa point kernels, 8 x 6 cones (the output of the reference's own
    spectra.cpp / kernel.cpp build, stored in tests/golden/kernel)."""
    from endtoend_gb300 import engine, inputs
    z = np.load(os.path.join(ROOT, "tests", "golden", "kernel", "spec_6X_measured.npz"))
    g = lambda k: z["nt8_np6_" + k]
    params, _ = engine.fit_exp_kernel(g("radii"), g("cum_total"))
    return inputs.Physics(energy=g("energy"), fluence=g("fluence"), mu=g("mu"), mu_en=g("mu_en"), ntheta=8, nphi=6,
                          radii=g("radii").astype(np.float64), exp_params=params.astype(np.float64),
                          cumkern=g("cum_total").astype(np.float64), theta_deg=g("conv_theta").astype(np.float64),
                          phi_deg=g("conv_phi").astype(np.float64), rev_latspacing=spacing_cm,
                          rev_longspacing=spacing_cm, penumbra=1.0)


def table_leg(args, eng, vol, beams, d_fl, d_dose, d_grad, d_fgrad, offs):
    """The reference's own discretisation at speed: the 24-radius cumulative
    table walk evaluated exactly in O(L * nradii) (EE_KERNEL_TABLE), forward +
    adjoint, with the measured 6 MV kernel, on beams spread over the batch;
    beside it the reference's step-by-step O(L^2) walk (EE_KERNEL_TABLE_WALK)
    on the same beams.  CUDA events on the engine stream, direct call."""
    import torch
    n = min(args.table_beams, len(beams))
    pick = np.linspace(0, len(beams) - 1, n).round().astype(int)
    sub = [beams[i] for i in pick]
    from endtoend_gb300 import engine
    fl = torch.from_numpy(engine.concat_fluence(sub)).cuda()
    fg = torch.zeros_like(fl)
    stream = torch.cuda.ExternalStream(eng.stream)
    eng.set_physics(measured_6x_physics(float(vol.voxel[0])), mode="table")
    out = {"workload": f"{n} beams spread over the batch, measured 6 MV cumulative kernel (24 radii), 8x6 cones",
           "unit": UNIT}
    try:
        for mode in ("table", "walk"):
            eng.set_mode(mode)
            f = lambda: eng.dose_and_adjoint_device(sub, fl.data_ptr(), d_dose.data_ptr(), d_grad.data_ptr(),
                                                    fg.data_ptr())
            f()
            eng.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            f()
            b.record(stream)
            b.synchronize()
            out[mode] = n / (a.elapsed_time(b) / 1e3)
    finally:
        eng.set_physics(args.phys, mode="exp")
    out["table_over_walk"] = out["table"] / out["walk"]
    return out


def beamlet_leg(args, eng):
    """Beamlet dose columns (ee_beamlet_columns_device): beams of the 4-pi
    candidate grid with 40x40 unit-weight beamlets of 2.5 mm, each column
    thresholded at 1e-4 of its maximum into FP32 CSR with int32 row indices
    (device-resident).  Host clock around each call (the call synchronises)."""
    from endtoend_gb300 import inputs
    angs = inputs.four_pi_angles(1162, seed=5)
    pick = np.linspace(0, len(angs) - 1, max(1, args.beamlet_beams)).round().astype(int)
    beams = []
    for g, c in angs[pick]:
        b = inputs.single_beam(fmap=(40, 40), beamlet_cm=0.25, gantry_deg=float(g), couch_deg=float(c))
        b.fluence = np.ones((40, 40), np.float32)
        beams.append(b)
    eng.beamlet_columns_device(beams[0], 1e-4)  # warm-up (workspace growth)
    nbl, nnz, t = 0, 0, 0.0
    for b in beams:
        t0 = time.perf_counter()
        d = eng.beamlet_columns_device(b, 1e-4)
        t += time.perf_counter() - t0
        nbl += d.nbeamlets
        nnz += d.nnz
    out_bytes = nnz * 8 + (nbl + len(beams)) * 8
    return {"workload": f"{len(beams)} beams of the 1162-beam 4-pi grid, 200x200x160 @2mm head-neck phantom, "
                        "40x40 beamlets of 2.5 mm, threshold 1e-4 of each column max, FP32 CSR + int32 rows",
            "beamlets": nbl, "seconds": t, "beamlets_per_s": nbl / t, "nnz_per_beamlet": nnz / max(nbl, 1),
            "output_gb_per_s": out_bytes / t / 1e9}


def serving_leg(args, device, phys):
    """Request loop (ee_server_*) under Poisson arrivals versus the plain path
    (one request at a time through the host-pointer calls, FIFO-queued against
    the same arrival times)."""
    import ctypes as C
    import threading
    from endtoend_gb300 import engine, inputs

    vols, reqs = inputs.serving_workload(args.serve_requests, args.serve_rate, seed=9)
    rng = np.random.default_rng(13)
    grads = [rng.standard_normal(v.density.shape).astype(np.float32) for v in vols]
    nbeams = sum(len(r["beams"]) for r in reqs)

    # plain: one engine context per phantom, one request per call
    engs = []
    for v in vols:
        e = engine.Engine(device)
        e.set_volume(v)
        e.set_physics(phys, mode="exp")
        engs.append(e)

    def plain_call(r):
        e = engs[r["volume"]]
        if not r["grad"]:
            e.beam_dose(r["beams"])
            return
        eb = engine.to_ee_beams(r["beams"])
        fl = engine.concat_fluence(r["beams"])
        dose = np.empty(vols[r["volume"]].density.shape, np.float32)
        fg = np.empty_like(fl)
        g = grads[r["volume"]]
        e._check(e.lib.ee_dose_and_adjoint(e.h, eb, len(r["beams"]), C.c_void_p(fl.ctypes.data),
                                           C.c_void_p(dose.ctypes.data), engine.DOSE_SUM, C.c_void_p(g.ctypes.data),
                                           C.c_void_p(fg.ctypes.data)))

    for k in range(len(vols)):  # warm contexts
        plain_call({"volume": k, "beams": reqs[0]["beams"][:1], "grad": True})
    service = []
    for r in reqs:
        t0 = time.perf_counter()
        plain_call(r)
        service.append(time.perf_counter() - t0)
    for e in engs:
        e.close()
    end, lat = 0.0, []
    for r, sv in zip(reqs, service):
        end = max(end, r["t"]) + sv
        lat.append(end - r["t"])
    lat_plain = np.array(lat) * 1e3
    # both forms on the same basis: beams over the makespan (first arrival
    # to last completion); the plain path's busy-time rate beside it
    plain = {"beams_per_s": nbeams / end, "busy_beams_per_s": nbeams / sum(service),
             "p50_ms": float(np.percentile(lat_plain, 50)), "p99_ms": float(np.percentile(lat_plain, 99)),
             "makespan_s": end}

    srv = engine.Server(device, slots=args.serve_slots, max_batch_beams=256)
    srv.set_physics(phys, mode="exp")
    for v in vols:
        srv.add_volume(v)
    for k in range(len(vols)):  # every slot builds its contexts
        ts = [srv.submit(k, reqs[0]["beams"][:1], grads[k]) for _ in range(args.serve_slots)]
        for t in ts:
            srv.wait(t)
    srv.reset_stats()
    tickets = []
    done = threading.Event()

    failed = []

    def waiter():
        i = 0
        while not (done.is_set() and i >= len(tickets)):
            if i < len(tickets):
                try:
                    srv.wait(tickets[i])
                except engine.EEError as e:
                    failed.append(str(e))
                i += 1
            else:
                time.sleep(0.001)

    th = threading.Thread(target=waiter)
    th.start()
    t_start = time.perf_counter()
    for r in reqs:
        dt = t_start + r["t"] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        tickets.append(srv.submit(r["volume"], r["beams"], grads[r["volume"]] if r["grad"] else None))
    done.set()
    th.join()
    makespan = time.perf_counter() - t_start
    st = srv.stats()
    srv.close()
    return {
        "workload": f"{len(reqs)} requests, Poisson {args.serve_rate:g}/s, phantoms "
                    + ", ".join("x".join(str(n) for n in s) for s in inputs.SERVING_SHAPES)
                    + " @2mm, 1-40 beams, fluence 16^2-64^2 @2.5mm, dose or dose+gradient",
        "beams": nbeams, "slots": args.serve_slots,
        "served": {"beams_per_s": nbeams / makespan, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                   "completed": st["completed"], "failed": len(failed), "makespan_s": makespan},
        "plain": plain,
        "served_over_plain": (nbeams / makespan) / plain["beams_per_s"],
    }


def cpu_reference_sample(vol, phys, beams, steps=1, warmup=0, nthreads=None):
    """FP32 OpenMP restatement of the reference chain (table kernel) on one
    beam: forward dose + adjoint.  Returns seconds per beam-dose."""
    from oracle.oracle import Oracle
    o = Oracle(vol, phys, kernel_mode=0, precision=32, nthreads=nthreads)
    g = np.random.default_rng(7).standard_normal(vol.density.shape).astype(np.float32)
    times = []
    for i in range(warmup + steps):
        b = beams[i % len(beams)]
        t0 = time.perf_counter()
        o.beam_dose(b)
        o.beam_dose_adjoint(b, g)
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
    return float(np.mean(times)), o.setup.nthreads


def run_reference(args, ws, rank):
    if rank != 0:
        return
    vol, phys, beams = make_workload(8)
    # bounded sample: one beam forward + adjoint per step
    t_step, cores = cpu_reference_sample(vol, phys, beams, steps=args.steps, warmup=min(args.warmup, 1))
    v = 1.0 / t_step
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": "batched candidate beams: 200x200x160 @2mm head-neck phantom, 48 cones, "
                                   "fluence 8^2-40^2 beamlets @2.5mm; sample = 1 beam fwd+adjoint per step",
                       "kernel": "reference 24-radius cumulative table walk (O(L^2) per line)",
                       "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "1 beam forward + adjoint of the batched candidate workload per step"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# DRAM bytes (read + write) per crop-box voxel of each stage, from ncu
# captures of the chain kernels on eight beams of this workload (dram__bytes
# of one call's launches / sum of V_beam = 12.37 M; k_gather_T and
# k_cone_T_lane captured again with their current forms); roofline.traffic
# scales the dominant stage's figure to the profiled step.
DRAM_BYTES_PER_VBEAM = {"terma": 1.0, "cone": 251.9, "gather": 51.7, "gather_T": 102.3, "cone_T": 230.3,
                        "terma_T": 3.5, "geometry": 0.0}


def algorithmic_bytes(infos):
    """Per-solve algorithmic bytes: 392 * V_beam per beam (TERMA 8 B/voxel,
    each of 24 cone directions 8 B/voxel read + 8 B/voxel dose RMW)."""
    vb = sum(i["v_beam"] for i in infos)
    return 392.0 * vb, vb


def profile_case(args):
    """Two forward + adjoint calls on a few beams spread over the workload
    (the launches an ncu capture selects with -k / -s / -c)."""
    import torch
    from endtoend_gb300 import engine
    vol, phys, beams = make_workload(args.beams)
    nb = max(1, args.profile_beams)
    beams = beams[::max(1, len(beams) // nb)][:nb]
    eng = engine.Engine(0)
    eng.set_volume(vol)
    eng.set_physics(phys, mode=args.profile_case)
    fl = torch.from_numpy(engine.concat_fluence(beams)).cuda()
    dose = torch.zeros(vol.nvoxels, device="cuda")
    g = torch.from_numpy(np.random.default_rng(11).standard_normal(vol.nvoxels).astype(np.float32)).cuda()
    fg = torch.zeros_like(fl)
    for _ in range(2):
        eng.dose_and_adjoint_device(beams, fl.data_ptr(), dose.data_ptr(), g.data_ptr(), fg.data_ptr())
    eng.synchronize()
    infos = [eng.beam_info(i) for i in range(nb)]
    print(json.dumps({"profile_case": args.profile_case, "beams": nb, "v_beam": sum(i["v_beam"] for i in infos),
                      "max_line": [i["max_line"] for i in infos]}))
    eng.close()


def main():
    args = parse()
    if args.profile_case:
        profile_case(args)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import torch
    from endtoend_gb300 import engine, metrics

    torch.cuda.set_device(local)
    vol, phys, beams = make_workload(args.beams, seed_offset=rank)
    args.phys = phys
    eng = engine.Engine(local)
    eng.set_volume(vol)
    eng.set_physics(phys, mode="exp")
    eng.set_scratch_limit(args.scratch_gb << 30)
    stream = torch.cuda.ExternalStream(eng.stream)
    nfull = vol.nvoxels
    fl_host = engine.concat_fluence(beams)
    d_fl = torch.from_numpy(fl_host).cuda()
    d_dose = torch.zeros(nfull, dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(11)
    grad_host = rng.standard_normal(nfull).astype(np.float32)
    d_grad = torch.from_numpy(grad_host).cuda()
    d_fgrad = torch.zeros_like(d_fl)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def step_device():
        eng.dose_and_adjoint_device(beams, d_fl.data_ptr(), d_dose.data_ptr(), d_grad.data_ptr(), d_fgrad.data_ptr())

    # planned batch: the whole forward + adjoint captured into one CUDA graph
    plan = eng.plan(beams, d_fl.data_ptr(), d_dose.data_ptr(), d_grad.data_ptr(), d_fgrad.data_ptr())
    plan_info = plan.info()

    def step_plan():
        plan.launch()

    for _ in range(args.warmup):
        step_device()
        step_plan()
    eng.synchronize()
    plan.status()
    # one profiled step (untimed): per-stage device time + launches
    eng.set_profiling(True)
    eng.read_profile()
    step_device()
    eng.synchronize()
    prof = eng.read_profile()
    eng.set_profiling(False)
    infos = [eng.beam_info(i) for i in range(len(beams))]

    def timed(fn):
        ms = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        return ms

    clocks = ClockSampler(local, args.clocks_csv)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    step_ms = timed(step_plan)
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    plan.status()
    t_dev = max_over_ranks(sum(step_ms) / 1e3, ws)
    value = ws * len(beams) * args.steps / t_dev
    # the same batch through the direct pipeline call (one geometry read-back per chunk)
    pipe_ms = timed(step_device)
    pipeline_value = len(beams) * args.steps / (sum(pipe_ms) / 1e3)

    # e2e through host pointers (pinned host memory)
    pin_fl = torch.from_numpy(fl_host).pin_memory().numpy()
    pin_grad = torch.from_numpy(grad_host).pin_memory().numpy()
    pin_dose = torch.zeros(nfull, dtype=torch.float32).pin_memory().numpy()
    pin_fgrad = torch.zeros(fl_host.size, dtype=torch.float32).pin_memory().numpy()
    import ctypes as C
    eb = engine.to_ee_beams(beams)

    def step_host():
        eng._check(eng.lib.ee_dose_and_adjoint(eng.h, eb, len(beams), C.c_void_p(pin_fl.ctypes.data),
                                               C.c_void_p(pin_dose.ctypes.data), engine.DOSE_SUM,
                                               C.c_void_p(pin_grad.ctypes.data), C.c_void_p(pin_fgrad.ctypes.data)))

    step_host()
    barrier(ws)
    torch.cuda.synchronize()
    e2e_lat = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step_host()
        e2e_lat.append(time.perf_counter() - t0)
    barrier(ws)
    t_e2e = max_over_ranks(sum(e2e_lat), ws)
    e2e = ws * len(beams) * args.steps / t_e2e
    h2d = pin_fl.nbytes + pin_grad.nbytes
    d2h = pin_dose.nbytes + pin_fgrad.nbytes

    # plain per-beam path: one beam per call
    # plain path on beams spread evenly through the batch (same size mix)
    npl = min(args.plain_beams, len(beams))
    allofs = np.cumsum([0] + [b.fluence.size for b in beams])
    pick = np.linspace(0, len(beams) - 1, npl).round().astype(int)
    pb = [beams[i] for i in pick]
    offs = allofs[pick]
    torch.cuda.synchronize()
    lat = []
    t0 = time.perf_counter()
    for i, b in enumerate(pb):
        s0 = time.perf_counter()
        eng.dose_and_adjoint_device([b], d_fl.data_ptr() + 4 * int(offs[i]), d_dose.data_ptr(), d_grad.data_ptr(),
                                    d_fgrad.data_ptr() + 4 * int(offs[i]))
        eng.synchronize()
        lat.append(time.perf_counter() - s0)
    plain = npl / (time.perf_counter() - t0)

    # the reference's discretisation with the measured 6 MV kernel
    table = None
    if not args.no_table and rank == 0:
        table = table_leg(args, eng, vol, beams, d_fl, d_dose, d_grad, d_fgrad, allofs)

    # roofline of the dominant stage (CUDA-event stage times of the profiled step)
    dom = max(prof, key=lambda k: prof[k][0])
    alg_bytes, vb = algorithmic_bytes(infos)
    stage_bytes = {
        "terma": 8.0 * vb, "cone": 24 * 12.0 * vb, "gather": 24 * 4.0 * vb + 4.0 * vb,
        "gather_T": 24 * 4.0 * vb + 4.0 * vb, "cone_T": 24 * 12.0 * vb, "terma_T": 8.0 * vb, "geometry": 0.0,
    }
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    dom_ms, dom_launches = prof[dom]
    achieved = stage_bytes.get(dom, 0.0) / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    # traffic and achieved refer to the same unit of work: the dominant
    # stage over all beams of one step
    traffic = DRAM_BYTES_PER_VBEAM.get(dom, 0.0) * vb
    roof = {"bound": "hbm", "kernel": f"k_{dom}", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic,
            "traffic_unit": "bytes per step of the dominant stage (ncu dram bytes per V_beam voxel x sum V_beam)",
            "algorithmic_bytes": stage_bytes.get(dom, 0.0),
            "peak_source": "measured" if peaks else "fallback",
            "stage_ms": {k: round(v[0], 3) for k, v in prof.items()},
            "chain_frac": (2 * alg_bytes / (sum(step_ms) / len(step_ms) / 1e3) / 1e9) / peak}
    # kernels per graph replay: per chunk geom_init, terma, geometry, cone, gather,
    # rev_zero, gather_T, cone_T, terma_T
    gpu_launches = int(plan_info["chunks"]) * 9 * args.steps

    # accuracy vs the reference discretisation on one beam (FP64 oracle,
    # 24-radius table, texture 8-bit weights)
    acc = None
    if not args.no_accuracy and rank == 0:
        from oracle.oracle import Oracle
        o_ref = Oracle(vol, phys, kernel_mode=0, tex_emulate=True)
        o_64 = Oracle(vol, phys, kernel_mode=2)
        acc = {"beams": [], "max_abs_diff_over_dmax_vs_reference_discretisation": 0.0,
               "max_abs_diff_over_dmax_vs_fp64_oracle_same_kernel": 0.0, "gamma_1pct_1mm_vs_reference": 1.0}
        for bi in sorted({0, len(beams) // 2}):
            b = beams[bi]
            d = eng.beam_dose([b])
            ref, _ = o_ref.beam_dose(b)
            ref64, _ = o_64.beam_dose(b)
            acc["beams"].append(bi)
            acc["max_abs_diff_over_dmax_vs_reference_discretisation"] = max(
                acc["max_abs_diff_over_dmax_vs_reference_discretisation"], metrics.max_rel_diff(d, ref))
            acc["max_abs_diff_over_dmax_vs_fp64_oracle_same_kernel"] = max(
                acc["max_abs_diff_over_dmax_vs_fp64_oracle_same_kernel"], metrics.max_rel_diff(d, ref64))
            acc["gamma_1pct_1mm_vs_reference"] = min(acc["gamma_1pct_1mm_vs_reference"],
                                                     metrics.gamma_pass_rate(d, ref, voxel_mm=2.0))

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        t_cpu, cores = cpu_reference_sample(vol, phys, beams, steps=1, warmup=0)
        cpu = {"value": 1.0 / t_cpu, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "1 beam forward + adjoint (FP32 OpenMP restatement, 24-radius table walk)"}

    beamlet = None
    if not args.no_beamlet and rank == 0:
        eng.synchronize()
        beamlet = beamlet_leg(args, eng)

    annealing = None
    if not args.no_anneal and rank == 0:
        eng.synchronize()
        plan.close()
        annealing = annealing_leg(args, eng, phys)

    # the request server runs on its own contexts: release the batch's
    # buffers first
    eng.synchronize()
    plan.close()
    eng.close()
    serving = None
    if not args.no_serve and rank == 0:
        serving = serving_leg(args, local, phys)

    lat_ms = np.array(lat) * 1e3
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "batched candidate beams: 200x200x160 @2mm head-neck phantom, "
                                   f"{len(beams)} beams/GPU, 48 cones (8x6), fluence 8^2-40^2 @2.5mm; "
                                   "step = forward + adjoint of every beam",
                       "kernel": "double exponential, O(L) recurrence, one lane per cone line",
                       "path": "planned batch replayed from one captured CUDA graph",
                       "parallelism": f"beams sharded x{ws}",
                       "l2": "flushed (256 MB write) between timed steps"},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "plain": {"value": plain, "unit": UNIT, "beams": npl, "p50_ms": float(np.percentile(lat_ms, 50)),
                      "p99_ms": float(np.percentile(lat_ms, 99))},
            "batched_over_plain": value / plain,
            "pipeline": {"value": pipeline_value, "unit": UNIT, "note": "same batch, direct call (host geometry read-back per chunk)"},
            "table_measured_6x": table,
            "plan": plan_info,
            "serving": serving,
            "beamlet": beamlet,
            "annealing": annealing,
            "gpu_launches": gpu_launches,
            "roofline": roof,
            "clocks": clk,
            "accuracy": acc,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
