#!/usr/bin/env python
"""Benchmark of the DEM hot path on the 1M-sphere rotating Hertz drum, plus the other workloads.

One step = one pass of [Leapfrog(reset=True), InsertionSortCollider, ContactLoop] over the
whole scene (1 000 000 lognormal spheres, 20 000 facets, 2 rotating wall caps,
Cp2_FrictMat_HertzPhys + Law2_L6Geom_HertzPhys_DMT). ``value`` is particle-steps/s with the
state resident in HBM; the collider's full runs are counted at their natural rate (the per-step
collider time over a calibration run plus the timed steps replaces the full runs that happened to
fall inside the timed steps). ``e2e`` drives the same step through the C ABI from host buffers
(wg_run_host: page-locked host state copied in, one step, copied out, every step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--precision fp32|fp64]
                    [--legs other,e2e,c0,c1,batch,serve,cpu]

Further legs in the same JSON line: ``box_settle_10k`` (10 000 spheres in a walled box, 20 000
steps, both precisions), ``periodic_shear_200k`` (200 000 spheres in a periodic cell, compressed
then sheared, both precisions with the FP32-force error against FP64), ``batch`` (256 box settles
in one simulation against one at a time, same precision), ``serving`` (a Poisson stream of box
settles and periodic shears, continuous batching against one job at a time) and ``cpu_baseline``.

N>1 (launched by torch.distributed.run) runs independent replicas, one scene per GPU
(the single-scene path has no exchange step); ``value`` is the sum over ranks.
``--impl reference`` times the CPU restatement of the reference (OpenMP, all host cores, the
reference's parallel structure) on the same settled 1M-sphere drum and prints the same JSON line;
the settled state is prepared by a separate process (``--write-state``), so the timed process
loads no GPU code.
"""
import argparse
import json
import math
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
ALL_LEGS = ("other", "e2e", "c0", "c1", "batch", "serve", "cpu")


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
                                       "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
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


def drum_geometry(n):
    """Drum dimensions for n spheres: the 1M-sphere drum (1.2 m x 0.6 m) scaled with n^(1/3)."""
    scale = (n / 1e6) ** (1 / 3.0)
    return dict(diameter=1.2 * scale, length=0.6 * scale, div=201, axDiv=50)


def build_scene(args, seed, n=None, precision=None):
    """The drum, filled by seeded random insertion and compacted into a resting bed on the GPU."""
    from woodem_gb300 import scenes
    n = n or args.spheres
    t = time.time()
    S = scenes.hertz_drum(n=n, seed=seed, precision=precision or args.precision, settle_steps=args.settle, settle_g=args.settle_g,
                          **drum_geometry(n))
    log("scene of %d spheres built and settled (%d steps at %g g) in %.1fs" % (n, args.settle, args.settle_g, time.time() - t))
    return S


def bed_stats(S, radius):
    """Where the settled bed sits: the 99.5th percentile and the mean of the sphere heights, in drum
    radii from the axis (a bed filling 40% of the drum has its free surface at z = -0.16 R)."""
    from woodem_gb300 import scenes
    z = scenes._sphere_nodes(S, "pos")[:, 2]
    return {"top_z_over_R": round(float(np.percentile(z, 99.5)) / radius, 4), "mean_z_over_R": round(float(z.mean()) / radius, 4)}


def snapshot(S):
    S.sync()
    nd = S.dem._nodes.soa
    st = {k: nd.col(k).copy() for k in ("pos", "ori", "vel", "angVel", "force", "torque")}
    if S.isPeriodic:
        st["_cell"] = (np.array(S.cell.hSize, float), np.array(S.cell.trsf, float), np.array(S.cell._gradV, float),
                       np.array(S.cell.nextGradV, float))
    return st


def restore(S, st):
    """Put a snapshot back (the device simulation is released: contacts restart from the positions)."""
    S.close()
    nd = S.dem._nodes.soa
    for k, v in st.items():
        if k != "_cell":
            nd.col(k)[:] = v
    if "_cell" in st:
        hs, tr, gv, ngv = st["_cell"]
        S.cell.hSize, S.cell.trsf, S.cell._gradV, S.cell.nextGradV = hs.copy(), tr.copy(), gv.copy(), ngv.copy()
    S.step = 0
    S.time = 0.0


# Algorithmic bytes per unit of work: the compulsory DRAM traffic of an ideal one-pass step,
# counted from stored widths (the per-unit figures of the reference path's cost model):
#   particle-step (Leapfrog)          b_p = 156 read + 104 written = 260 B
#   real contact (contact kernel)     b_r = 192 B FP64 Hertz / 208 B FP64 IdealElPl, 124 B FP32-force mode
#   potential, not real contact       b_v = 16 B
#   facet-step (vertices + fakeVel)   96 B
#   collider full run                 104 B per particle + 8 B per potential contact
BYTES = {"b_p": 260, "b_r": {("fp64", "hertz"): 192, ("fp64", "elpl"): 208, ("fp32", "hertz"): 124, ("fp32", "elpl"): 124},
         "b_v": 16, "b_f": 96, "coll_p": 104, "coll_c": 8}


def step_bytes(prec, law, n_sph, n_par, R, P, nF, full_per_step):
    """Algorithmic bytes of one step: Leapfrog, contact loop and the collider at its full-run rate."""
    contact = R * BYTES["b_r"][(prec, law)] + (P - R) * BYTES["b_v"] + nF * BYTES["b_f"]
    leapfrog = n_sph * BYTES["b_p"]
    coll = (BYTES["coll_p"] * n_par + BYTES["coll_c"] * P) * full_per_step
    return leapfrog, contact, coll


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measure_gpu(args, rank, world, S, prec, e2e=True):
    """Warm-up, calibration of the collider's full-run rate and cost, the K timed steps, and e2e."""
    from woodem_gb300 import _native, tune
    S.gpu.precision = prec
    t0 = time.time()
    S.run(args.warmup)
    sim = S._sim
    L, h = sim.H.L, sim.H.h
    tune.set_launch(sim, args.contact_block if prec == "fp32" else 0, args.chunk_steps, False, not args.serial_contacts)
    S.run(3)
    st0 = sim.stats()
    log("[rank %d] %s warmup %d steps done in %.1fs: %d contacts (%d real), %d full runs" %
        (rank, prec, args.warmup, time.time() - t0, st0.n_contacts, st0.n_real, st0.n_full_runs))
    # clocks sampled from the calibration steps on, so that the samples are taken under load
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0))) if rank == 0 else None
    if clocks:
        clocks.start()
    # calibration: the collider's full runs at their natural rate over calib_steps steps
    cal = None
    if args.calib_steps > 0:
        S.run(args.calib_steps)
        ctot, cph, _ = sim.timing()
        st_c = sim.stats()
        cal = dict(steps=args.calib_steps, full_runs=st_c.n_full_runs - st0.n_full_runs, collider_ms=float(cph[3]), ms=ctot)
        st0 = st_c
    barrier(world)
    if args.profile:
        L.wg_profiler(1)
    t1 = time.perf_counter()
    S.run(args.steps)
    t2 = time.perf_counter()
    if args.profile:
        L.wg_profiler(0)
    ck = clocks.stop() if clocks else None
    if ck is not None:
        ck["window"] = "sampled every 100 ms over the calibration and timed steps"
    tot, ph, nl = sim.timing()
    st1 = sim.stats()
    A = sim.A
    K = args.steps
    full_win = st1.n_full_runs - st0.n_full_runs
    cal_steps = cal["steps"] if cal else 0
    cal_coll = cal["collider_ms"] if cal else 0.0
    cal_full = cal["full_runs"] if cal else 0
    coll_per_step = (cal_coll + float(ph[3])) / (cal_steps + K)
    full_per_step = (cal_full + full_win) / (cal_steps + K)
    ms_amort = (tot - float(ph[3])) + K * coll_per_step
    res = dict(ms=ms_amort, ms_window=tot, wall=(t2 - t1) * 1e3, phases=ph.tolist(), launches=nl, st0=st0, st1=st1, clocks=ck,
               n_nodes=A.n_nodes, n_par=A.n_particles, n_spheres=int(np.count_nonzero(A.particles["shape"] == 0)),
               n_facets=int(np.count_nonzero(A.particles["shape"] == 2)), calibration=cal, full_window=full_win,
               coll_per_step=coll_per_step, full_per_step=full_per_step)
    if e2e:
        na = A.n_nodes
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


def oracle_sample(S, seconds, threads, min_steps=20, warm_steps=2):
    """The CPU restatement of the reference path (timing build, OpenMP, the reference's parallel
    structure: guided contact loop with atomic force adds) on the scene's current state; returns
    (particle-steps/s, timed steps, spheres, seconds, warm-up seconds)."""
    from woodem_gb300 import _plan
    from oracle.oracle import Oracle
    A = _plan.compile_scene(S)
    n = int(np.count_nonzero(A.particles["shape"] == 0))
    O = Oracle(A, threads=threads, deterministic=False, fast=True)
    tw = time.perf_counter()
    O.run(warm_steps)  # initial sort and first contacts outside the timed sample
    tw = time.perf_counter() - tw
    steps = 0
    t = time.perf_counter()
    while True:
        O.run(1)
        steps += 1
        el = time.perf_counter() - t
        if steps >= min_steps and el > seconds:
            break
    O.close()
    return n * steps / el, steps, n, el, tw


def write_state(args, path):
    """--write-state: build and settle the benchmark drum (GPU) and store the sphere state."""
    import __graft_entry__
    __graft_entry__.build()
    from woodem_gb300 import scenes
    S = build_scene(args, seed=args.seed, precision="fp64")
    S.close()
    np.savez(path, pos=scenes._sphere_nodes(S, "pos"), vel=scenes._sphere_nodes(S, "vel"), angVel=scenes._sphere_nodes(S, "angVel"),
             radius=scenes.sphere_radii(S))


def reference_arm(args, cfg):
    """The CPU restatement of the reference path on the settled drum of the GPU arm."""
    from woodem_gb300 import scenes
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "drum_state.npz")
        t = time.time()
        cmd = [sys.executable, os.path.abspath(__file__), "--write-state", path, "--spheres", str(args.spheres), "--settle",
               str(args.settle), "--settle-g", str(args.settle_g), "--seed", str(args.seed)]
        subprocess.run(cmd, check=True, stdout=sys.stderr)
        log("settled state prepared by a separate process in %.1fs" % (time.time() - t))
        st = np.load(path)
        S = scenes.hertz_drum_from_state(st["pos"], st["radius"], st["vel"], st["angVel"], precision="fp64",
                                         **drum_geometry(args.spheres))
    v, steps, n, el, tw = oracle_sample(S, args.cpu_seconds, threads, warm_steps=args.warmup)
    sample = ("%d steps (after %d warm-up steps with the initial sort, %.1fs) of the settled %d-sphere drum (20k facets, Hertz), "
              "the same state as the GPU arm; oracle timing build (-O3, OpenMP), reference parallel structure" %
              (steps, args.warmup, tw, n))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": dict(cfg, spheres_timed=n, steps_timed=steps), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------- other workloads
def kinetic(S):
    """Translational + rotational kinetic energy of the spheres (host copy of the state)."""
    from woodem_gb300 import _plan
    S.sync()
    A = _plan.compile_scene(S)
    sph = A.particles["nodes"][A.particles["shape"] == 0, 0]
    nd = A.nodes
    m, I = nd["mass"][sph], nd["inertia"][sph]
    v, w = nd["vel"][sph], nd["angVel"][sph]
    return float(0.5 * np.sum(m * np.sum(v * v, axis=1)) + 0.5 * np.sum(I * w * w))


def contact_force_error(S64, S32):
    """Per-contact global force of two simulations of the same state after one step: the largest
    and the median difference over the real contacts both have, relative to the contact's force
    (or to 1e-4 of the largest force for weaker contacts), and the largest difference of a
    particle's net force relative to its largest contact force."""
    c64, c32 = S64._sim.contacts(), S32._sim.contacts()
    k64 = c64["id_lo"].astype(np.int64) << 32 | c64["id_hi"].astype(np.int64)
    k32 = c32["id_lo"].astype(np.int64) << 32 | c32["id_hi"].astype(np.int64)
    both = np.intersect1d(k64[c64["real"] != 0], k32[c32["real"] != 0])
    i64 = np.searchsorted(k64, both)
    i32 = np.searchsorted(k32, both)
    f64, f32 = c64["fglob"][i64], c32["fglob"][i32]
    mag = np.linalg.norm(f64, axis=1)
    # relative to the contact's force, or to 1e-4 of the largest force for the weaker contacts (the
    # tests' definition: the FP32-force overlap is exact to ~2^-46 of the centre distance, a growing
    # fraction of an ever smaller overlap)
    rel = np.linalg.norm(f32 - f64, axis=1) / np.maximum(mag, 1e-4 * (mag.max() if len(mag) else 0.0) + 1e-300)
    ok = mag > 0
    S64.sync()
    S32.sync()
    F64, F32 = S64.dem._nodes.soa.col("force"), S32.dem._nodes.soa.col("force")
    # largest contact force per particle
    n = len(F64)
    big = np.zeros(n)
    np.maximum.at(big, c64["id_lo"][c64["real"] != 0], np.linalg.norm(c64["fglob"][c64["real"] != 0], axis=1))
    np.maximum.at(big, c64["id_hi"][c64["real"] != 0], np.linalg.norm(c64["fglob"][c64["real"] != 0], axis=1))
    sel = big > 1e-6 * (big.max() if len(big) else 0.0)
    pr = np.linalg.norm(F32[sel] - F64[sel], axis=1) / big[sel]
    return {"contacts_compared": int(ok.sum()), "contact_force_rel_max": float(rel[ok].max()) if ok.any() else None,
            "contact_force_rel_median": float(np.median(rel[ok])) if ok.any() else None,
            "net_force_rel_max": float(pr.max()) if sel.any() else None,
            "real_contacts_fp64": int(np.count_nonzero(c64["real"])), "real_contacts_fp32": int(np.count_nonzero(c32["real"]))}


def run_timed(S, steps):
    S.run(steps)
    tot, ph, nl = S._sim.timing()
    st = S._sim.stats()
    return tot, ph, nl, st


def measure_c0(args):
    """Box settle: 10 000 spheres (r 5 mm) on a jittered 22x22x21 lattice in a 0.3x0.3x0.6 m box of 6
    walls, IdealElPl, damping 0.2, dt = 0.3 pWaveDt, 20 000 steps from the lattice, FP64 plain and
    FP32-force; then the one-step force error of FP32 against FP64 from the settled FP64 state."""
    from woodem_gb300 import scenes
    T = args.c0_steps
    out = {"workload": "box-settle-10k", "spheres": 10000, "walls": 6, "steps": T, "law": "Law2_L6Geom_FrictPhys_IdealElPl",
           "start": "jittered lattice (seed %d)" % args.seed}
    hbm, _ = peaks()
    fin = {}
    for prec in ("fp64", "fp32"):
        S = scenes.box_settle(n=10000, seed=args.seed, precision=prec)
        tot, ph, nl, st = run_timed(S, T)
        n = 10000
        ke = kinetic(S)
        z = scenes._sphere_nodes(S, "pos")[:, 2]
        lf, ct, co = step_bytes(prec, "elpl", n, n + 6, st.n_real, st.n_contacts, 0, st.n_full_runs / T)
        ms = tot / T
        out[prec] = {"particle_steps_per_s": n * T / (tot / 1e3), "ms_per_step": ms, "full_runs": int(st.n_full_runs),
                     "launches": int(nl), "real_contacts_end": int(st.n_real), "coordination_end": 2.0 * st.n_real / n,
                     "kinetic_energy_end": ke, "mean_z_end": float(z.mean()), "top_z_end": float(np.percentile(z, 99.5)),
                     "step_bytes": lf + ct + co, "achieved_gbs": (lf + ct + co) / (ms / 1e3) / 1e9,
                     "frac": (lf + ct + co) / (ms / 1e3) / 1e9 / hbm}
        fin[prec] = S
        log("c0 %s: %.3f ms/step, %d real contacts at the end" % (prec, ms, st.n_real))
    a, b = out["fp64"], out["fp32"]
    out["fp32_vs_fp64_end"] = {k: abs(b[k] - a[k]) / abs(a[k]) for k in ("coordination_end", "mean_z_end", "top_z_end")}
    out["fp32_vs_fp64_end"]["kinetic_energy_abs_j"] = abs(b["kinetic_energy_end"] - a["kinetic_energy_end"])
    # one step of each precision from the settled FP64 state
    snap = snapshot(fin["fp64"])
    pair = {}
    for prec in ("fp64", "fp32"):
        S = scenes.box_settle(n=10000, seed=args.seed, precision=prec)
        restore(S, snap)
        S.run(1)
        pair[prec] = S
    out["one_step_error"] = contact_force_error(pair["fp64"], pair["fp32"])
    for S in list(pair.values()) + list(fin.values()):
        S.close()
    return out


def measure_c1(args):
    """Periodic shear: 200 000 spheres (r uniform in [2, 4] mm) placed by seeded random insertion at
    solid fraction 0.35 in a periodic cube (random insertion jams below the configuration's 0.55),
    compressed isotropically to 0.55 and on to ``c1_phi`` (a packing with contacts), then sheared
    (xz rate 1/s); the same compressed state is run in FP64 plain and FP32-force mode: the
    one-step contact-force and stress error, then ``c1_steps`` steps of each with the stress
    tensor and the coordination number at the end."""
    from woodem_gb300 import scenes
    from woodem_gb300.dem import ContactLoop
    n, T = args.c1_spheres, args.c1_steps
    t = time.time()
    S = scenes.periodic_shear(n=n, seed=args.seed, fill_fraction=0.35, shear_rate=1.0, precision="fp32",
                              compress_steps=args.c1_compress, compress_to=args.c1_phi)
    loop = [e for e in S.engines if isinstance(e, ContactLoop)][0]
    loop.evalStress = True
    snap = snapshot(S)
    side = float(np.linalg.det(np.asarray(S.cell.hSize))) ** (1 / 3.0)
    r = scenes.sphere_radii(S)
    phi = float(np.sum(4 / 3.0 * math.pi * r ** 3)) / side ** 3
    log("c1: %d spheres placed and compressed (%d steps) in %.1fs, solid fraction %.3f" % (n, args.c1_compress, time.time() - t, phi))
    out = {"workload": "periodic-shear-200k", "spheres": n, "steps": T, "compress_steps": args.c1_compress,
           "compressed_to": args.c1_phi,
           "solid_fraction_start": phi, "cell_side_m": side, "shear": "nextGradV[0,2] = 1/s, HomoGradV2",
           "law": "Law2_L6Geom_FrictPhys_IdealElPl"}
    hbm, _ = peaks()
    # one step of each precision from the compressed state (a second scene object holds the FP32 run)
    S32 = scenes.periodic_shear(n=n, seed=args.seed, fill_fraction=0.35, shear_rate=1.0, precision="fp32",
                                centers=snap["pos"])
    loop32 = [e for e in S32.engines if isinstance(e, ContactLoop)][0]
    loop32.evalStress = True
    for X, prec in ((S, "fp64"), (S32, "fp32")):
        restore(X, snap)
        X.gpu.precision = prec
        X.run(1)
    err = contact_force_error(S, S32)
    s64, s32 = np.array(loop.stress), np.array(loop32.stress)
    err["stress_rel"] = float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64))
    out["one_step_error"] = err
    S32.close()
    for prec in ("fp64", "fp32"):
        restore(S, snap)
        S.gpu.precision = prec
        tot, ph, nl, st = run_timed(S, T)
        sig = np.array(loop.stress)
        lf, ct, co = step_bytes(prec, "elpl", n, n, st.n_real, st.n_contacts, 0, st.n_full_runs / T)
        ms = tot / T
        out[prec] = {"particle_steps_per_s": n * T / (tot / 1e3), "ms_per_step": ms, "full_runs": int(st.n_full_runs),
                     "real_contacts_end": int(st.n_real), "coordination_end": 2.0 * st.n_real / n,
                     "stress_end": sig.tolist(), "kinetic_energy_end": kinetic(S), "step_bytes": lf + ct + co,
                     "achieved_gbs": (lf + ct + co) / (ms / 1e3) / 1e9, "frac": (lf + ct + co) / (ms / 1e3) / 1e9 / hbm}
        log("c1 %s: %.3f ms/step, %d real contacts at the end" % (prec, ms, st.n_real))
    a, b = out["fp64"], out["fp32"]
    s64, s32 = np.array(a["stress_end"]), np.array(b["stress_end"])
    out["fp32_vs_fp64_end"] = {"stress_rel": float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64)),
                               "coordination_rel": abs(b["coordination_end"] - a["coordination_end"]) / a["coordination_end"]}
    S.close()
    return out


def measure_batch(args):
    """Parametric batch (C3): 256 independent box settles (sphere counts log-uniform in [1k, 50k],
    per-scene radius, tanPhi, young, damping) run together for batch_steps - batch_window steps,
    then, from that settled state, a window of batch_window steps timed one scene at a time (each
    scene its own simulation, in turn), batched with the default launch shape and batched with the
    autotuned one, in each precision."""
    from woodem_gb300 import scenes, tune
    from woodem_gb300.batch import Batch
    K, T, Wn = args.batch_scenes, args.batch_steps, args.batch_window
    warm = max(0, T - Wn)
    out = {"scenes": K, "steps": T, "window": Wn, "window_start": warm,
           "scene_kind": "box settle (lattice, 6 walls, FrictPhys+IdealElPl)"}
    ss, tab = scenes.batch_study(n_scenes=K, seed=args.seed + 1, precision="fp32")
    nsph = int(tab["n"].sum())
    out["spheres"] = nsph
    t = time.time()
    B = Batch(ss)
    B.run(warm)
    B.close()
    log("batch: %d scenes advanced %d steps together in %.1fs" % (K, warm, time.time() - t))
    snaps = [snapshot(S) for S in ss]

    def reset(prec):
        for S, sn in zip(ss, snaps):
            restore(S, sn)
            S.gpu.precision = prec

    for prec in ("fp64", "fp32"):
        reset(prec)
        tot_ms, real = 0.0, 0
        for S in ss:
            S.run(Wn)
            tot_ms += S._sim.timing()[0]
            real += S._sim.stats().n_real
            S.close()
        one = {"scene_steps_per_s": K * Wn / (tot_ms / 1e3), "particle_steps_per_s": nsph * Wn / (tot_ms / 1e3), "ms": tot_ms,
               "real_contacts_per_scene_end": real / K}
        out["one_at_a_time_%s" % prec] = one
        log("batch: one at a time %s %.1f ms for %d scene-steps" % (prec, tot_ms, K * Wn))
        # autotune on the same state (its trial steps are not part of the timed window)
        reset(prec)
        B = Batch(ss)
        # FP64 batch steps are ~6x longer and the shapes differ less: half as many trial steps
        best, med = tune.autotune(B, trial_steps=args.tune_steps if prec == "fp32" else max(32, args.tune_steps // 2),
                                  rounds=args.tune_rounds)
        B.H.close()
        B.H = None
        runs = {}
        for tuned in (False, True):
            reset(prec)
            B = Batch(ss)
            if tuned:
                tune.set_launch(B, *best)
            B.run(Wn)
            ms = B.timing()[0]
            st_real = sum(B.scene_stats(k).n_real for k in range(K))
            B.H.close()
            B.H = None
            key = "batched_%s_%s" % (prec, "tuned" if tuned else "default")
            runs[key] = {"scene_steps_per_s": K * Wn / (ms / 1e3), "particle_steps_per_s": nsph * Wn / (ms / 1e3), "ms": ms,
                         "real_contacts_per_scene_end": st_real / K}
            if tuned:
                runs[key]["launch"] = {"contact_block": best[0], "chunk_steps": best[1], "cuda_graph": bool(best[2]),
                                       "concurrent_contacts": bool(best[3])}
                runs[key]["trial_ms_per_step"] = {str(c): v for c, v in med.items()}
            log("batch: %s %.1f ms" % (key, ms))
        out.update(runs)
        out["speedup_%s_tuned" % prec] = runs["batched_%s_tuned" % prec]["scene_steps_per_s"] / one["scene_steps_per_s"]
        out["speedup_%s_default" % prec] = runs["batched_%s_default" % prec]["scene_steps_per_s"] / one["scene_steps_per_s"]
    out["jobs_per_s_fp32_tuned"] = out["batched_fp32_tuned"]["scene_steps_per_s"] / float(T)
    out["speedup_basis"] = "batched and one-at-a-time at the same precision, same state, same window"
    return out


def measure_serving(args):
    """Serving (C4): a seeded Poisson stream of jobs, each a box settle or a periodic shear with
    probability 0.5, sizes log-uniform in [2 000, 300 000] spheres, step counts uniform in
    [5 000, 50 000], materials as in the batch study, HBM budget 150 GB. Overload: the stream's
    arrivals over serve_seconds at serve_rate jobs/s, served for serve_wall seconds by continuous
    batching and by one job at a time (FIFO), each from the same arrivals; capacity is the
    particle-steps done in that time (finished jobs plus the progress of unfinished ones). A
    sub-capacity stream (serve_low_rate) is served to completion by continuous batching for its
    latencies."""
    from woodem_gb300 import scenes, _plan, serve
    prec = args.serve_precision
    nmin, nmax, smin, smax = 2000, 300000, 5000, 50000

    def materials(seed):
        rng = np.random.default_rng(seed)
        return dict(radius=float(rng.uniform(3e-3, 6e-3)), tanPhi=float(math.exp(rng.uniform(math.log(0.2), math.log(0.8)))),
                    young=float(math.exp(rng.uniform(math.log(1e6), math.log(1e8)))), damping=float(rng.uniform(0.0, 0.4)))

    def make_box(n, seed):
        m = materials(seed)
        return scenes.box_settle_scaled(n, m["radius"], seed=seed % 100000, young=m["young"], tanPhi=m["tanPhi"],
                                        damping=m["damping"], precision=prec)

    def make_peri(n, seed):
        m = materials(seed)
        return scenes.periodic_shear(n=n, seed=seed % 100000, rmin=m["radius"] / 2, rmax=m["radius"], young=m["young"],
                                     tanPhi=m["tanPhi"], damping=m["damping"], fill_fraction=0.3, shear_rate=1.0, precision=prec,
                                     pack_device=True)

    def peri_phases(n, steps, seed):
        # the first 30 % of the steps compress the cell isotropically from 0.30 to 0.55 solid
        # fraction, the rest shear it (the periodic-shear configuration's sequence)
        m = materials(seed)
        dt = 0.3 * (m["radius"] / 2) / math.sqrt(m["young"] / 2600.0)
        rate = math.log((0.55 / 0.3) ** (1 / 3.0)) / (0.3 * steps * dt)
        g = np.zeros((3, 3))
        g[0, 2] = 1.0
        return [(0.3, -rate * np.eye(3)), (0.7, g)]

    def stream(rate, horizon, seed):
        return serve.poisson_jobs(rate, horizon, seed, make_box, make_peri, nmin, nmax, smin, smax, peri_phases=peri_phases)

    out = {"precision": prec, "sizes": [nmin, nmax], "steps": [smin, smax], "hbm_budget_gb": 150,
           "stream": "seeded Poisson, p(periodic shear)=0.5, p(box settle)=0.5, materials as the batch study"}
    template = _plan.compile_scene(make_box(2000, 1))
    # slot capacities (spheres + 6 walls of a box job)
    caps = [300016] * 2 + [100016] * 6 + [30016] * 12 + [10016] * 16

    def pool():
        return serve.SlotPool(caps, precision=prec, template=template)

    def continuous(jobs, horizon):
        p = pool()
        srv = serve.Server(p, hbm_budget=150e9, tick=500, max_periodic=4, clock="wall")
        done = srv.run(jobs, horizon=horizon)
        p.close()
        el = srv.elapsed
        return dict(serve.latency_stats(done), jobs=len(jobs), finished=len(done), seconds=el, jobs_per_s=len(done) / el,
                    particle_steps_per_s=(srv.particle_steps + srv.partial_particle_steps) / el,
                    finished_particle_steps_per_s=srv.particle_steps / el)

    def one_at_a_time(jobs, wall):
        t0 = time.perf_counter()
        fin, psteps = [], 0.0
        for j in jobs:
            now = time.perf_counter() - t0
            if now >= wall:
                break
            if now < j.arrival:
                time.sleep(j.arrival - now)
            S = j.build()
            j.start = time.perf_counter() - t0
            for n, g in j.phase_steps():
                if g is not None:
                    S.cell.nextGradV = np.asarray(g, float)
                while n > 0 and time.perf_counter() - t0 < wall:
                    k = min(n, 2000)
                    S.run(k)
                    n -= k
                    j.done_steps += k
            S.sync()
            S.close()
            psteps += j.n * j.done_steps
            if j.done_steps >= j.steps:
                j.end = time.perf_counter() - t0
                fin.append(j)
        el = time.perf_counter() - t0
        return dict(serve.latency_stats(fin), jobs=len(jobs), finished=len(fin), seconds=el, jobs_per_s=len(fin) / el,
                    particle_steps_per_s=psteps / el)

    rate, H, wall = args.serve_rate, args.serve_seconds, args.serve_wall
    out["overload"] = {"arrival_rate_jobs_per_s": rate, "arrivals_seconds": H, "served_seconds": wall}
    out["overload"]["continuous_batching"] = continuous(stream(rate, H, args.seed + 5), wall)
    log("serving: overload, continuous batching: %s" % out["overload"]["continuous_batching"])
    out["overload"]["one_at_a_time"] = one_at_a_time(stream(rate, H, args.seed + 5), wall)
    log("serving: overload, one at a time: %s" % out["overload"]["one_at_a_time"])
    cb, oa = out["overload"]["continuous_batching"], out["overload"]["one_at_a_time"]
    out["capacity_ratio"] = cb["particle_steps_per_s"] / oa["particle_steps_per_s"] if oa["particle_steps_per_s"] else None
    out["capacity_definition"] = ("particle-steps per second of wall time over all jobs, finished ones and the progress of "
                                  "unfinished ones (the stream's jobs hold up to 1.5e10 particle-steps each, so few finish "
                                  "within the overload run; finished-job counts and latencies come from the sub-capacity run)")
    lr, lh = args.serve_low_rate, args.serve_low_seconds
    out["sub_capacity"] = {"arrival_rate_jobs_per_s": lr, "arrivals_seconds": lh}
    out["sub_capacity"]["continuous_batching"] = continuous(stream(lr, lh, args.seed + 6), lh * 4)
    log("serving: sub-capacity, continuous batching: %s" % out["sub_capacity"]["continuous_batching"])
    return out


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
    ap.add_argument("--calib-steps", type=int, default=1000, help="steps before the timed ones that measure the collider's "
                    "full-run rate and cost")
    ap.add_argument("--legs", default=",".join(ALL_LEGS), help="further measurements: " + ",".join(ALL_LEGS))
    ap.add_argument("--no-other", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--profile", action="store_true", help="bracket the timed steps with cudaProfilerStart/Stop")
    ap.add_argument("--spheres", type=int, default=1_000_000)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--c0-steps", type=int, default=20000)
    ap.add_argument("--c1-spheres", type=int, default=200000)
    ap.add_argument("--c1-steps", type=int, default=5000)
    ap.add_argument("--c1-compress", type=int, default=30000)
    ap.add_argument("--c1-phi", type=float, default=0.62, help="solid fraction the periodic cell is compressed to")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=10000)
    ap.add_argument("--batch-window", type=int, default=1000)
    ap.add_argument("--tune-steps", type=int, default=200, help="autotuner: steps per trial (several collider full runs)")
    ap.add_argument("--tune-rounds", type=int, default=2)
    ap.add_argument("--serve-precision", default="fp32", choices=["fp64", "fp32"])
    ap.add_argument("--serve-rate", type=float, default=20.0, help="serving: job arrivals per second (overload run)")
    ap.add_argument("--serve-seconds", type=float, default=20.0, help="serving: arrivals over this many seconds")
    ap.add_argument("--serve-wall", type=float, default=30.0, help="serving: seconds each overload run serves")
    ap.add_argument("--serve-low-rate", type=float, default=0.1, help="serving: sub-capacity arrivals per second "
                    "(the capacity is ~0.2 jobs/s: a mean job is ~1.6e9 particle-steps)")
    ap.add_argument("--serve-low-seconds", type=float, default=60.0)
    ap.add_argument("--contact-block", type=int, default=0,
                    help="launch shape of the contact kernels (wg_set_launch): 128/256 one contact per thread, "
                         "-256 the resident-grid FP32 sphere-sphere kernel with prefetch")
    ap.add_argument("--chunk-steps", type=int, default=32, help="steps queued per host check of the collider request")
    ap.add_argument("--serial-contacts", action="store_true",
                    help="facet/wall contacts before the sphere-sphere ones (default: beside them on a second stream)")
    ap.add_argument("--write-state", default=None, help=argparse.SUPPRESS)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    legs = set(x for x in args.legs.split(",") if x)
    for flag, leg in (("no_other", "other"), ("no_e2e", "e2e"), ("no_cpu", "cpu"), ("no_batch", "batch"), ("no_serve", "serve")):
        if getattr(args, flag):
            legs.discard(leg)
    if args.write_state:
        write_state(args, args.write_state)
        return
    rank, world, local = env_rank()
    cfg = {"workload": "hertz-drum-1M", "spheres": args.spheres, "facets": 20000, "walls": 2, "settle_steps": args.settle,
           "settle_g": args.settle_g, "sphere_order": "Morton curve of the settled positions",
           "law": "Cp2_FrictMat_HertzPhys+Law2_L6Geom_HertzPhys_DMT", "precision": args.precision,
           "l2": "inputs larger than L2 (device state > 1 GB)", "replicas": world}
    if args.impl == "reference":
        if rank != 0:
            return
        reference_arm(args, cfg)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    import __graft_entry__
    if rank == 0:
        __graft_entry__.build()
    barrier(world)
    __graft_entry__.build()
    from woodem_gb300 import _native
    _native.lib()
    S = build_scene(args, seed=args.seed + rank)
    bed = bed_stats(S, 0.6 * (args.spheres / 1e6) ** (1 / 3.0))
    log("bed: %s" % bed)
    st0 = snapshot(S)
    res = measure_gpu(args, rank, world, S, args.precision, e2e="e2e" in legs)
    other = None
    if "other" in legs:
        restore(S, st0)
        oprec = "fp64" if args.precision == "fp32" else "fp32"
        other = measure_gpu(args, rank, world, S, oprec, e2e=False)
        other["prec"] = oprec
    S.close()
    n_sph = res["n_spheres"]
    value, ms = replica_rate(n_sph * args.steps, res["ms"], world)
    st0r, st1 = res["st0"], res["st1"]
    hbm, src = peaks()
    R = 0.5 * (st0r.n_real + st1.n_real)
    P = 0.5 * (st0r.n_contacts + st1.n_contacts)
    nF = res["n_facets"]
    lf_b, ct_b, co_b = step_bytes(args.precision, "hertz", n_sph, res["n_par"], R, P, nF, res["full_per_step"])
    step_b = lf_b + ct_b + co_b
    ph = [x / args.steps for x in res["phases"]]
    if ph[1] >= ph[0]:
        kern, kbytes, kern_ms = ("contact_loop" if args.precision == "fp32" else "k_contact_fp64"), ct_b, ph[1]
    else:
        kern, kbytes, kern_ms = "k_leapfrog%s" % ("32" if args.precision == "fp32" else ""), lf_b, ph[0]
    achieved = kbytes / (kern_ms / 1e3) / 1e9 if kern_ms > 0 else 0.0
    ms_step = ms / args.steps
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic", "config": cfg,
            "roofline": {"bound": "hbm", "kernel": kern, "kernels": KERNELS.get(kern, kern), "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic_per_launch(kern, R, P, nF, n_sph),
                         "peak_source": src, "bytes_per_launch": kbytes, "launch_ms": kern_ms},
            "step": {"contacts": P, "real": R, "real_per_sphere": R / n_sph, "full_runs_in_window": res["full_window"],
                     "full_runs_per_step": res["full_per_step"], "collider_ms_per_step": res["coll_per_step"],
                     "ms_per_step_window": res["ms_window"] / args.steps,
                     "collider_accounting": "collider time per step over the calibration run and the timed steps "
                                            "(%s calibration steps) in place of the full runs inside the timed steps" %
                                            (res["calibration"]["steps"] if res["calibration"] else 0),
                     "phase_ms": {"leapfrog": ph[0], "contact": ph[1], "collider": res["coll_per_step"]},
                     "algorithmic_bytes": step_b, "achieved_gbs": step_b / (ms_step / 1e3) / 1e9,
                     "frac": step_b / (ms_step / 1e3) / 1e9 / hbm},
            "gpu_launches": int(res["launches"]), "clocks": res["clocks"]}
    cfg["bed"] = bed
    if other is not None:
        ovalue, oms = replica_rate(n_sph * args.steps, other["ms"], world)
        ost0, ost1 = other["st0"], other["st1"]
        oph = [x / args.steps for x in other["phases"]]
        oR = 0.5 * (ost0.n_real + ost1.n_real)
        oP = 0.5 * (ost0.n_contacts + ost1.n_contacts)
        olf, oct_, oco = step_bytes(other["prec"], "hertz", n_sph, other["n_par"], oR, oP, nF, other["full_per_step"])
        line["other_precision"] = {"precision": other["prec"], "value": ovalue, "ms_per_step": oms / args.steps,
                                   "phase_ms": {"leapfrog": oph[0], "contact": oph[1], "collider": other["coll_per_step"]},
                                   "real": oR, "contacts": oP,
                                   "contact_loop_frac": oct_ / (oph[1] / 1e3) / 1e9 / hbm if oph[1] > 0 else None,
                                   "leapfrog_frac": olf / (oph[0] / 1e3) / 1e9 / hbm if oph[0] > 0 else None,
                                   "step_frac": (olf + oct_ + oco) / (oms / args.steps / 1e3) / 1e9 / hbm}
    if "e2e" in res:
        e = res["e2e"]
        evalue, _ = replica_rate(n_sph * e["steps"], e["seconds"] * 1e3, world)
        line["e2e"] = {"value": evalue, "unit": UNIT, "h2d_bytes_per_step": e["h2d"],
                       "d2h_bytes_per_step": e["d2h"], "steps": e["steps"],
                       "call": "wg_run_host(1 step) with page-locked host state"}
    if rank == 0 and "c0" in legs:
        line["box_settle_10k"] = measure_c0(args)
    if rank == 0 and "c1" in legs:
        line["periodic_shear_200k"] = measure_c1(args)
    if rank == 0 and "batch" in legs:
        line["batch"] = measure_batch(args)
    if rank == 0 and "serve" in legs:
        line["serving"] = measure_serving(args)
    if rank == 0 and "cpu" in legs:
        # the oracle on the state the timed GPU steps started from
        restore(S, st0)
        threads = os.cpu_count() or 1
        v, steps, n, el, tw = oracle_sample(S, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d steps of the settled %d-sphere drum (the state the timed GPU steps start from), "
                                          "oracle timing build (-O3, OpenMP), reference parallel structure" % (steps, n)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# the kernels behind each roofline entry (the contact loop of the FP32-force mode is the facet/wall
# kernel beside the sphere-sphere kernel, timed together by the phase events)
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


if __name__ == "__main__":
    main()
