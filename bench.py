#!/usr/bin/env python
"""Benchmark of the DEM hot path on the 1M-sphere rotating Hertz drum.

One step = one pass of [Leapfrog(reset=True), InsertionSortCollider, ContactLoop] over the
whole scene (1 000 000 lognormal spheres, 20 000 facets, 2 rotating wall caps,
Cp2_FrictMat_HertzPhys + Law2_L6Geom_HertzPhys_DMT). ``value`` is particle-steps/s with the
state resident in HBM; ``e2e`` drives the same step through the C ABI from host buffers
(wg_run_host: page-locked host state copied in, one step, copied out, every step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--precision fp32|fp64]

N>1 (launched by torch.distributed.run) runs independent replicas, one scene per GPU
(the single-scene path has no exchange step); ``value`` is the sum over ranks.
``--impl reference`` times the CPU restatement of the reference (OpenMP, all host cores) on
a bounded sample of the same workload and prints the same JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "particle-steps/s at 1M spheres (FP32 vs FP64 plain); batched jobs/s, p50/p99"
UNIT = "particle-steps/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_scene(args, seed, n=None, precision=None):
    """The drum, filled by seeded random insertion and compacted into a resting bed on the GPU."""
    from woodem_gb300 import scenes
    n = n or args.spheres
    scale = (n / 1e6) ** (1 / 3.0)
    t = time.time()
    S = scenes.hertz_drum(n=n, seed=seed, diameter=1.2 * scale, length=0.6 * scale, div=201, axDiv=50,
                          precision=precision or args.precision, settle_steps=args.settle, settle_g=args.settle_g)
    log("scene of %d spheres built and settled (%d steps at %g g) in %.1fs" % (n, args.settle, args.settle_g, time.time() - t))
    return S


def bed_stats(S, radius):
    """Where the settled bed sits: the 99.5th percentile and the mean of the sphere heights, in drum
    radii from the axis (a bed filling 40% of the drum has its free surface at z = -0.16 R)."""
    from woodem_gb300 import _plan
    A = _plan.compile_scene(S)
    nd = S.dem._nodes.soa
    sph = A.particles["shape"] == 0
    z = nd.col("pos")[A.particles["nodes"][sph, 0], 2]
    return {"top_z_over_R": round(float(np.percentile(z, 99.5)) / radius, 4), "mean_z_over_R": round(float(z.mean()) / radius, 4)}


def snapshot(S):
    nd = S.dem._nodes.soa
    return {k: nd.col(k).copy() for k in ("pos", "ori", "vel", "angVel", "force", "torque")}


def restore(S, st):
    S.close()
    nd = S.dem._nodes.soa
    for k, v in st.items():
        nd.col(k)[:] = v
    S.step = 0
    S.time = 0.0


# Algorithmic bytes per unit of work: the compulsory DRAM traffic of an ideal one-pass step,
# counted from stored widths (the per-unit figures of the reference path's cost model):
#   particle-step (Leapfrog)          b_p = 156 read + 104 written = 260 B
#   real contact (contact kernel)     b_r = 192 B FP64 Hertz, 124 B FP32-force mode
#   potential, not real contact       b_v = 16 B
#   facet-step (vertices + fakeVel)   96 B
#   collider full run                 104 B per particle + 8 B per potential contact
BYTES = {"b_p": 260, "b_r": {"fp64": 192, "fp32": 124}, "b_v": 16, "b_f": 96, "coll_p": 104, "coll_c": 8}


def measure_gpu(args, rank, world, S=None, prec=None, e2e=True):
    from woodem_gb300 import _native
    if S is None:
        S = build_scene(args, seed=args.seed + rank)
    if prec:
        S.gpu.precision = prec
    t0 = time.time()
    S.run(args.warmup)
    sim = S._sim
    L, h = sim.H.L, sim.H.h
    from woodem_gb300 import tune
    tune.set_launch(sim, args.contact_block if (prec or args.precision) == "fp32" else 0, args.chunk_steps, False,
                    not args.serial_contacts)
    S.run(3)
    st0 = sim.stats()
    log("[rank %d] warmup %d steps done in %.1fs: %d contacts (%d real), %d full runs" %
        (rank, args.warmup, time.time() - t0, st0.n_contacts, st0.n_real, st0.n_full_runs))
    if rank == 0:
        from woodem_gb300 import scenes
        S.sync()
        sp = np.linalg.norm(scenes._sphere_nodes(S, "vel"), axis=1)
        log("sphere speed after warmup: median %.3g, p99 %.3g, p99.99 %.3g, max %.3g m/s; %d above 1 m/s" %
            (np.median(sp), np.percentile(sp, 99), np.percentile(sp, 99.99), sp.max(), int(np.count_nonzero(sp > 1.0))))
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0))) if rank == 0 else None
    if clocks:
        clocks.start()
    barrier(world)
    if args.profile:
        L.wg_profiler(1)
    t1 = time.perf_counter()
    S.run(args.steps)
    t2 = time.perf_counter()
    if args.profile:
        L.wg_profiler(0)
    ck = clocks.stop() if clocks else None
    tot, ph, nl = sim.timing()
    st1 = sim.stats()
    n_spheres = args.spheres
    A = S._sim.A
    res = dict(ms=tot, wall=(t2 - t1) * 1e3, phases=ph.tolist(), launches=nl, st0=st0, st1=st1, clocks=ck,
               n_nodes=A.n_nodes, n_par=A.n_particles, n_spheres=n_spheres,
               n_facets=int(np.count_nonzero(A.particles["shape"] == 2)))
    # e2e through wg_run_host with page-locked host buffers
    if e2e and not args.no_e2e:
        na = S._sim.A.n_nodes
        nbytes = 19 * 8 * na
        p = L.wg_host_alloc(nbytes)
        if not p:
            raise MemoryError("wg_host_alloc")
        import ctypes
        buf = np.ctypeslib.as_array((ctypes.c_double * (19 * na)).from_address(p))
        parts = [buf[0:3 * na], buf[3 * na:7 * na], buf[7 * na:10 * na], buf[10 * na:13 * na], buf[13 * na:16 * na],
                 buf[16 * na:19 * na]]
        sim.H.check(L.wg_get_nodes(h, *[_native.ptr(x) for x in parts]), "get_nodes")
        ne = args.e2e_steps
        sim.H.check(L.wg_run_host(h, 1, *[_native.ptr(x) for x in parts]), "run_host")  # warm
        barrier(world)
        te = time.perf_counter()
        for _ in range(ne):
            sim.H.check(L.wg_run_host(h, 1, *[_native.ptr(x) for x in parts]), "run_host")
        te = time.perf_counter() - te
        L.wg_host_free(p)
        res["e2e"] = dict(seconds=te, steps=ne, h2d=(3 + 4 + 3 + 3 + 3 + 3) * 8 * na, d2h=(3 + 4 + 3 + 3 + 3 + 3) * 8 * na)
    return res


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    """The maximum of x over the ranks (a CUDA tensor under NCCL, a CPU tensor under gloo)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, ms_local, world):
    """Whole-job rate of `world` replicas that each processed units_per_rank units in ms_local ms:
    the units of all ranks over the slowest rank's time (weak scaling). Every rank must call it."""
    ms = allreduce_max(ms_local, world)
    return world * units_per_rank / (ms / 1e3), ms


def cpu_sample(args, seconds, threads):
    """Oracle (CPU restatement, OpenMP, reference structure) on a 100k-sphere drum of the same
    construction; returns (particle-steps/s, steps, spheres)."""
    from woodem_gb300 import _plan
    from oracle.oracle import Oracle
    n = args.cpu_spheres
    S = build_scene(args, seed=args.seed, n=n, precision="fp64")
    S.close()
    A = _plan.compile_scene(S)
    O = Oracle(A, threads=threads, deterministic=False)
    O.run(2)  # initial sort and first contacts outside the timed sample
    steps = 0
    t = time.perf_counter()
    while True:
        O.run(5)
        steps += 5
        el = time.perf_counter() - t
        if el > seconds or steps >= 2000:
            break
    O.close()
    return n * steps / el, steps, n, el


# the kernels behind each roofline entry (the contact loop of the FP32-force mode is the facet/wall
# kernel followed by the sphere-sphere kernel, timed together by the phase events)
KERNELS = {"contact_loop": "k_contact_fp32 (facets, walls) + k_contact_ss32p (sphere-sphere)", "k_contact_fp64": "k_contact_fp64",
           "k_leapfrog32": "k_leapfrog32", "k_leapfrog": "k_leapfrog"}


def traffic_per_launch(kern, R, P, nF, n):
    """DRAM bytes (read + write) per launch of the kernel (or per contact loop), from the committed
    ncu capture summary: bytes per unit of that capture scaled to this launch's units, or None."""
    try:
        with open(os.path.join(HERE, "profiles", "dram_per_unit.json")) as f:
            d = json.load(f)[kern]
    except Exception:
        return None
    return (d.get("per_real", 0.0) * R + d.get("per_potential", 0.0) * P + d.get("per_sphere", 0.0) * n +
            d.get("per_facet", 0.0) * nF)


def measure_batch(args):
    """Parametric batch of independent box settles (sphere counts log-uniform in [1k, 50k], per-scene
    radius, tanPhi, young, damping): scene-steps/s of the one-scene-at-a-time GPU path (each scene
    its own simulation, run in turn) against the batch in one simulation, with the default launch
    shape and with the autotuned one (CUDA-graph chunks among the candidates), both precisions."""
    from woodem_gb300 import scenes, tune
    from woodem_gb300.batch import Batch
    K, W, T = args.batch_scenes, 20, args.batch_steps
    out = {"scenes": K, "steps": T, "warmup": W, "scene_kind": "box settle (lattice, 6 walls, FrictPhys+IdealElPl)"}

    def build(prec):
        ss, tab = scenes.batch_study(n_scenes=K, seed=args.seed + 1, precision=prec)
        out["spheres"] = int(tab["n"].sum())
        return ss

    # one scene at a time
    ss = build("fp64")
    tot_ms = 0.0
    for S in ss:
        S.run(W)
        S.run(T)
        tot_ms += S._sim.timing()[0]
        S.close()
    out["one_at_a_time_fp64"] = {"scene_steps_per_s": K * T / (tot_ms / 1e3), "ms": tot_ms}
    log("batch: one at a time %.1f ms for %d scene-steps" % (tot_ms, K * T))
    for prec in ("fp64", "fp32"):
        for tuned in (False, True):
            ss = build(prec)
            B = Batch(ss)
            B.run(W)
            best = None
            if tuned:
                best, med = tune.autotune(B, trial_steps=16, rounds=1)
            B.run(T)
            ms = B.timing()[0]
            key = "batched_%s_%s" % (prec, "tuned" if tuned else "default")
            out[key] = {"scene_steps_per_s": K * T / (ms / 1e3), "ms": ms}
            if best:
                out[key]["launch"] = {"contact_block": best[0], "chunk_steps": best[1], "cuda_graph": bool(best[2]),
                                      "concurrent_contacts": bool(best[3])}
            log("batch: %s %.1f ms" % (key, ms))
            B.close()
    base = out["one_at_a_time_fp64"]["scene_steps_per_s"]
    out["speedup_fp64_tuned"] = out["batched_fp64_tuned"]["scene_steps_per_s"] / base
    out["speedup_fp32_tuned"] = out["batched_fp32_tuned"]["scene_steps_per_s"] / base
    out["jobs_per_s_fp32_tuned"] = out["batched_fp32_tuned"]["scene_steps_per_s"] / 10000.0
    return out


def measure_serving(args):
    """Serving loop on a seeded Poisson stream of jobs (box settles and periodic shears with
    probability 0.5, sizes log-uniform, step counts uniform; sizes and step counts scaled down from
    the 10-minute stream so that the run stays within the benchmark's time): continuous batching
    (SlotPool + periodic jobs on their own streams) against the same stream served one job at a
    time, each with the same arrival times; p50/p99 latency (queueing included), jobs/s,
    particle-steps/s."""
    from woodem_gb300 import scenes, _plan, serve
    prec = "fp32"
    rate, horizon = args.serve_rate, args.serve_seconds
    nmin, nmax, smin, smax = 2000, 30000, 2000, 5000

    def make_box(n, seed):
        r = 3e-3 + 3e-3 * ((seed % 1000) / 1000.0)
        return scenes.box_settle_scaled(n, r, seed=seed % 100000, precision=prec)

    def make_peri(n, seed):
        S = scenes.periodic_shear(n=n, seed=seed % 100000, fill_fraction=0.4, shear_rate=1.0, precision=prec)
        return S

    def stream():
        return serve.poisson_jobs(rate, horizon, args.seed + 5, make_box, make_peri, nmin, nmax, smin, smax)

    out = {"arrival_rate_jobs_per_s": rate, "arrivals_seconds": horizon, "sizes": [nmin, nmax], "steps": [smin, smax],
           "precision": prec, "stream": "seeded Poisson, p(periodic shear)=0.5, p(box settle)=0.5"}
    template = _plan.compile_scene(make_box(2000, 1))
    caps = [32000] * 4 + [12000] * 8 + [4000] * 8
    pool = serve.SlotPool(caps, precision=prec, template=template)
    srv = serve.Server(pool, hbm_budget=150e9, tick=250, max_periodic=4, clock="wall")
    jobs = stream()
    done = srv.run(jobs, horizon=horizon * 3)
    pool.close()
    el = srv.elapsed
    out["continuous_batching"] = dict(serve.latency_stats(done), jobs=len(jobs), finished=len(done), seconds=el,
                                      jobs_per_s=len(done) / el, particle_steps_per_s=srv.particle_steps / el,
                                      slots=len(caps), slot_capacities=sorted(set(caps)))
    log("serving: batched %d/%d jobs in %.1fs" % (len(done), len(jobs), el))
    # one job at a time, same arrivals, FIFO
    jobs = stream()
    t0 = time.perf_counter()
    fin, psteps = [], 0.0
    for j in jobs:
        now = time.perf_counter() - t0
        if now < j.arrival:
            time.sleep(j.arrival - now)
        if time.perf_counter() - t0 > horizon * 3:
            break
        S = j.build()
        S.run(j.steps)
        S.sync()
        S.close()
        j.end = time.perf_counter() - t0
        fin.append(j)
        psteps += j.n * j.steps
    el = time.perf_counter() - t0
    out["one_at_a_time"] = dict(serve.latency_stats(fin), jobs=len(jobs), finished=len(fin), seconds=el, jobs_per_s=len(fin) / el,
                                particle_steps_per_s=psteps / el)
    log("serving: one at a time %d/%d jobs in %.1fs" % (len(fin), len(jobs), el))
    return out


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=100)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp64", "fp32"])
    ap.add_argument("--settle", type=int, default=16000, help="steps compacting the random fill into a resting bed "
                    "(followed by 3/4 as many steps easing gravity back to 1 g)")
    ap.add_argument("--settle-g", type=float, default=40.0, help="gravity multiplier while compacting")
    ap.add_argument("--no-other", action="store_true", help="skip timing the other precision mode")
    ap.add_argument("--profile", action="store_true", help="bracket the timed steps with cudaProfilerStart/Stop")
    ap.add_argument("--spheres", type=int, default=1_000_000)
    ap.add_argument("--cpu-spheres", type=int, default=100_000)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=200)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--serve-rate", type=float, default=8.0, help="serving: job arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=15.0, help="serving: arrivals over this many seconds")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--contact-block", type=int, default=0,
                    help="launch shape of the contact kernels (wg_set_launch): 128/256 one contact per thread, "
                         "-256 the resident-grid FP32 sphere-sphere kernel with prefetch")
    ap.add_argument("--chunk-steps", type=int, default=32, help="steps queued per host check of the collider request")
    ap.add_argument("--serial-contacts", action="store_true",
                    help="facet/wall contacts before the sphere-sphere ones (default: beside them on a second stream)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = env_rank()
    cfg = {"workload": "hertz-drum-1M", "spheres": args.spheres, "facets": 20000, "walls": 2, "settle_steps": args.settle,
           "settle_g": args.settle_g, "sphere_order": "Morton curve of the settled positions",
           "law": "Cp2_FrictMat_HertzPhys+Law2_L6Geom_HertzPhys_DMT", "precision": args.precision,
           "l2": "inputs larger than L2 (device state > 1 GB)", "replicas": world}
    if args.impl == "reference":
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        v, steps, n, el = cpu_sample(args, args.cpu_seconds, threads)
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": cfg, "impl": "reference",
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": "%d steps of a %d-sphere drum of the same construction (20k facets, Hertz), "
                                           "OpenMP restatement of the reference CPU path" % (steps, n)},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    import __graft_entry__
    if rank == 0:
        __graft_entry__.build()
    barrier(world)
    __graft_entry__.build()
    from woodem_gb300 import _native
    _native.lib()
    # each rank drives its own GPU (replicas)
    if world > 1:
        from woodem_gb300 import core  # noqa
    S = build_scene(args, seed=args.seed + rank)
    bed = bed_stats(S, 0.6 * (args.spheres / 1e6) ** (1 / 3.0))
    log("bed: %s" % bed)
    st0 = snapshot(S)
    res = measure_gpu(args, rank, world, S=S, prec=args.precision)
    res["bed"] = bed
    other = None
    if not args.no_other:
        restore(S, st0)
        oprec = "fp64" if args.precision == "fp32" else "fp32"
        other = measure_gpu(args, rank, world, S=S, prec=oprec, e2e=False)
        other["prec"] = oprec
    S.close()
    n_sph = res["n_spheres"]
    value, ms = replica_rate(n_sph * args.steps, res["ms"], world)
    st0, st1 = res["st0"], res["st1"]
    hbm, src = peaks()
    R = 0.5 * (st0.n_real + st1.n_real)
    P = 0.5 * (st0.n_contacts + st1.n_contacts)
    nF = res["n_facets"]
    nfull = st1.n_full_runs - st0.n_full_runs
    # per-launch algorithmic bytes of the two per-step kernels, and of the whole step
    contact_bytes = R * BYTES["b_r"][args.precision] + (P - R) * BYTES["b_v"] + nF * BYTES["b_f"]
    leapfrog_bytes = res["n_spheres"] * BYTES["b_p"]
    coll_bytes = (BYTES["coll_p"] * res["n_par"] + BYTES["coll_c"] * P) * nfull / args.steps
    step_bytes = leapfrog_bytes + contact_bytes + coll_bytes
    ph = [x / args.steps for x in res["phases"]]
    if ph[1] >= ph[0]:
        kern, kbytes, kern_ms = ("contact_loop" if args.precision == "fp32" else "k_contact_fp64"), contact_bytes, ph[1]
    else:
        kern, kbytes, kern_ms = "k_leapfrog%s" % ("32" if args.precision == "fp32" else ""), leapfrog_bytes, ph[0]
    achieved = kbytes / (kern_ms / 1e3) / 1e9 if kern_ms > 0 else 0.0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic", "config": cfg,
            "roofline": {"bound": "hbm", "kernel": kern, "kernels": KERNELS.get(kern, kern), "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic_per_launch(kern, R, P, nF, res["n_spheres"]),
                         "peak_source": src, "bytes_per_launch": kbytes, "launch_ms": kern_ms},
            "step": {"contacts": P, "real": R, "real_per_sphere": R / n_sph, "full_runs": nfull,
                     "phase_ms": {"leapfrog": ph[0], "contact": ph[1], "collider": ph[3]},
                     "algorithmic_bytes": step_bytes, "achieved_gbs": step_bytes / (ms / args.steps / 1e3) / 1e9,
                     "frac": step_bytes / (ms / args.steps / 1e3) / 1e9 / hbm},
            "gpu_launches": int(res["launches"]), "clocks": res["clocks"]}
    if "bed" in res:
        cfg["bed"] = res["bed"]
    if other is not None:
        ovalue, oms = replica_rate(n_sph * args.steps, other["ms"], world)
        ost0, ost1 = other["st0"], other["st1"]
        oph = [x / args.steps for x in other["phases"]]
        line["other_precision"] = {"precision": other["prec"], "value": ovalue,
                                   "ms_per_step": oms / args.steps,
                                   "phase_ms": {"leapfrog": oph[0], "contact": oph[1], "collider": oph[3]},
                                   "real": 0.5 * (ost0.n_real + ost1.n_real), "contacts": 0.5 * (ost0.n_contacts + ost1.n_contacts)}
    if "e2e" in res:
        e = res["e2e"]
        evalue, _ = replica_rate(n_sph * e["steps"], e["seconds"] * 1e3, world)
        line["e2e"] = {"value": evalue, "unit": UNIT, "h2d_bytes_per_step": e["h2d"],
                       "d2h_bytes_per_step": e["d2h"], "steps": e["steps"],
                       "call": "wg_run_host(1 step) with page-locked host state"}
    if rank == 0 and not args.no_batch:
        line["batch"] = measure_batch(args)
    if rank == 0 and not args.no_serve:
        line["serving"] = measure_serving(args)
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, steps, n, el = cpu_sample(args, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d steps of a %d-sphere drum of the same construction (20k facets, Hertz), "
                                          "OpenMP restatement of the reference CPU path" % (steps, n)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
