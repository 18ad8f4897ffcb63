#!/usr/bin/env python
"""Throughput of main_portal.x's node loop on GB300.

One step = one pass of the hot path over the whole cloud: the radiation field
of every node (line table + fused Voronoi walk / channel integration) and the
polarized statistical-equilibrium solve of every node, i.e. the OpenMP loop
main_para.f90:210-257 of the reference.  Workload: the power-law sphere with
262,144 points (seed 1), a 10-level linear rotor (9 lines), 24x24 directions
(388 rays per node), 129 velocity channels, kmax = 6 (34 x 34 SE systems).

  value    ray-segments/s over all ranks, cloud resident in HBM, kernel work
           timed with CUDA events on the library's stream, L2 flushed between
           steps;
  e2e      the same metric through the C ABI from pinned host buffers: every
           step uploads the cloud (portal_set_cloud), runs the node loop and
           reads pol_pops back;
  cpu_baseline  the FP64 oracle port (OpenMP over nodes like the reference)
           on this host's cores, on a bounded sample of the same nodes;
  stages   the SE's node-solves/s (34 x 34, and 74 x 74 for a 20-level rotor
           at kmax 6) and the Stokes image's pixel-channels/s;
  cube1m   one pass over the 1,048,576-point turbulent cube (20 levels,
           32x32 directions, 129 channels) with its roofline and CPU sample;
  batch64  64 uneven clouds in one persistent launch under a CUDA graph
           (autotuned) against the same models one after another;
  convergence   time to converged populations (within 3e-5 of a reference
           fixed point, rho^0_0 and rho^2_0, the tightest distance every
           method reaches with the FP32 field; the runs that stop by the 1e-6
           change per pass are reported beside) on a held-out 16,384-point
           turbulent cube: plain, Ng, accelerated (local operator + Ng),
           warm-started by the MLP the run trains on eight other cubes, and
           warm-started + accelerated.

--impl reference times that CPU port alone on the same workload.
Multi-GPU: every rank runs its own replica of the workload (weak scaling);
the ranks only meet for a barrier and the max of the step times.
"""
from __future__ import annotations

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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-to-converged SE (1e-6 rel) warm-start vs plain; ray-segments/s; HBM GB/s"
UNIT = "ray-segments/s"


def workload_config(cloud, mol, rc, n_points):
    return {
        "workload": "power-law sphere, %d points (seed 1), %d-level linear rotor (%d lines), "
                    "%dx%d directions, %d channels, kmax %d" % (n_points, mol.nlev, mol.r_num, rc.nth,
                                                                 rc.nph, 2 * rc.nvel + 1, rc.kmax),
        "points": int(n_points), "levels": int(mol.nlev), "lines": int(mol.r_num),
        "directions": rc.nth, "channels": 2 * rc.nvel + 1, "kmax": rc.kmax,
        "step": "radiation field + polarized SE solve of every node (main_portal.x node loop)",
        "l2": "flushed between timed steps (256 MiB write)",
    }


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_constant(key):
    """A per-segment figure of the radiation-field kernel from the ncu summary
    committed under profiles/ (a line "key: value"), None when absent."""
    p = os.path.join(ROOT, "profiles", "radiation_field_sphere262k.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def traffic_per_segment():
    """DRAM bytes per ray segment of the radiation-field kernel (ncu)."""
    return profile_constant("dram_bytes_per_segment")


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1])); smax = max(smax, float(r[2]))
                for i, n in enumerate(names):
                    if r[5 + i].strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def sample_nodes_for(seconds, per_node_s, n_total):
    return int(max(16, min(n_total, seconds / max(per_node_s, 1e-6))))


def cpu_port_rate(cloud, mol, rc, target_s, repeats=1):
    """Oracle port on this host's cores over a contiguous node range (node
    order is random in radius, so a range is a random sample)."""
    import oracle
    P = oracle.OracleProblem(cloud, mol)
    nthreads = os.cpu_count() or 1
    # calibration: 2 nodes per thread; per_node = wall time per node at full
    # thread count
    t = time.perf_counter()
    _, _, _, nseg, _ = P.radiation_field(rc, 1, 2 * nthreads, nthreads)
    per_node = (time.perf_counter() - t) / (2 * nthreads)
    n = sample_nodes_for(target_s, per_node, cloud.bulk_node_num)
    rates = []
    for r in range(repeats):
        lo = 1 + (r * n) % max(1, cloud.bulk_node_num - n)
        t = time.perf_counter()
        J0, J2, _, nseg, _ = P.radiation_field(rc, lo, lo + n - 1, nthreads)
        P.solve_se(rc.kmax, J0, J2, lo, lo + n - 1, nthreads)
        dt = time.perf_counter() - t
        rates.append((nseg / dt, dt, n, nseg))
    return rates, nthreads


def build_workload(n_points, n_depth=10000):
    from portal_gb300 import synth
    cloud, mol, rc = synth.config_cloud("sphere262k", n_points=n_points)
    rc.n_depth = n_depth
    return cloud, mol, rc


def reference_arm(args, rank, world):
    if rank != 0:
        return 0
    cloud, mol, rc = build_workload(args.points, args.n_depth)
    cfg = workload_config(cloud, mol, rc, cloud.node_num)
    for _ in range(args.warmup):
        pass  # the CPU port has no warm-up state; each step is cold by construction
    rates, cores = cpu_port_rate(cloud, mol, rc, args.cpu_seconds, repeats=args.steps)
    vals = [r[0] for r in rates]
    value = statistics.median(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.median([r[1] for r in rates]) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d consecutive nodes of %d per step, all their rays + SE" %
                                       (rates[0][2], cloud.bulk_node_num)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _qi_errors(cube, ref_cube):
    """Largest |Q/I| and |U/I| difference of an image against a reference
    image of the same cloud (pixels and channels where the reference I is
    above 1e-3 of its peak; the denominators of the image parity tests)."""
    I, Q, U = ref_cube[0], ref_cube[1], ref_cube[2]
    ok = np.isfinite(I) & np.isfinite(Q) & np.isfinite(U)
    Ipk = np.abs(I[ok]).max()
    den = np.maximum(np.abs(I), 1e-3 * Ipk)
    dq = np.where(ok, np.abs(cube[1] - Q) / den, 0.0)
    du = np.where(ok, np.abs(cube[2] - U) / den, 0.0)
    return float(max(dq.max(), du.max()))


def convergence_leg(device, n_points=16384, n_train=8, epochs=60, target=3e-5):
    """Time to converged populations on a held-out turbulent cube: plain,
    Ng, accelerated (local operator + Ng every 4 passes), warm-started by the
    MLP the run trains on n_train other cubes, and warm-started +
    accelerated.  Two measures per method (portal_gb300.convergence): the
    run that stops by the change per pass (tol 1e-6, the relative residual)
    and the true distance of its result to a reference fixed point (the
    accelerated iteration run far past its floor); and the time of a run of
    exactly the passes the method needs to bring rho^0_0 (relative) and
    rho^2_0 / rho^0_0 within `target` of that reference -- 3e-5, the
    tightest distance every method reaches: with J in FP32 (~5e-7) the plain
    map's own limit lies ~2e-5 from the accelerated one (its fixed point is
    ill-conditioned by 1/(1 - q), q ~ 0.97).  Each method's Stokes image
    (65 x 65 pixels x 33 channels, line 1-0 at 45 degrees) is compared with
    the reference's."""
    import torch
    import portal_gb300 as pg
    from portal_gb300 import convergence as conv
    from portal_gb300 import synth
    from portal_gb300.warmstart import WarmStart

    mol = synth.linear_rotor(20)
    rc = synth.RunConfig(nth=16, nph=16, nvel=32, kmax=2, gvec=synth.gauge_vector(4))
    out = {"workload": "turbulent cube (lognormal density sigma_ln 1.5, mean 1e4 cm^-3; k^-11/3 velocity, "
                       "1 km/s rms; field along x + equal turbulent part), %d points, 20-level rotor, 16x16 "
                       "directions, 65 channels, kmax 2; held-out seed 300" % n_points,
           "target": target, "criterion": "max relative error of rho^0_0 and max |d rho^2_0|/rho^0_0 "
                                          "against the reference fixed point, levels above 1e-12 of each "
                                          "node's largest",
           "residual_tol": 1e-6}
    im = dict(l1=[1], l2=[2], th_inc=0.78539816339, ph_az=0.0, nvel=16, dvel=100.0, v0=0.0, im_pix=32,
              im_size=0.7)

    def image(ctx, pp):
        cube, _ = ctx.image(im["l1"], im["l2"], im["th_inc"], im["ph_az"], im["nvel"], im["dvel"], im["v0"],
                            im["im_pix"], im["im_size"], pol_pops=pp, quantities=3)
        return cube[:3, 0].astype(np.float64)

    with WarmStart(mol.j_lev, seed=1, device=device) as ws, pg.Context(device) as ctx:
        ctx.set_molecule(mol)
        t0 = time.perf_counter()
        Xs, Ys = [], []
        for i in range(n_train):
            cl = synth.turbulent_cube(n_points, 200 + i, mol, grid=32)
            ctx.set_cloud(cl)
            X, Y, _ = ws.collect(ctx, rc, cl.ab_all, cl.bulk_node_num)
            Xs.append(X)
            Ys.append(Y)
        t1 = time.perf_counter()
        losses = ws.fit(np.concatenate(Xs), np.concatenate(Ys), epochs=epochs)
        t2 = time.perf_counter()
        out["training"] = {"clouds": n_train, "rows": int(sum(len(x) for x in Xs)), "epochs": epochs,
                           "data_seconds": t1 - t0, "fit_seconds": t2 - t1,
                           "loss_first_last": [float(losses[0]), float(losses[-1])]}
        cl = synth.turbulent_cube(n_points, 300, mol, grid=32)
        live = np.zeros(cl.node_num, dtype=bool)
        live[:cl.bulk_node_num] = cl.ab_all[:cl.bulk_node_num] > 0

        def set_cloud():
            ctx.set_cloud(cl)

        set_cloud()
        t0 = time.perf_counter()
        ref, rec = conv.reference_solution(ctx, rc)
        rec["seconds"] = time.perf_counter() - t0
        out["reference"] = rec
        ref_img = image(ctx, ref)
        for name, warm, ng, lo in (("plain", False, 0, False), ("ng", False, 4, False),
                                   ("accelerated", False, 4, True), ("warm", True, 0, False),
                                   ("warm_accelerated", True, 4, True)):
            r = conv.time_to_error(ctx, set_cloud, rc, ref, live, target=target, ng_period=ng, local_operator=lo,
                                   warm=ws if warm else None, sync=torch.cuda.synchronize)
            r["qi_abs_err"] = _qi_errors(image(ctx, r.pop("pol_pops")), ref_img)
            out[name] = r
        # where the change-per-pass rule (the relative residual, tol 1e-6)
        # stops each method, how long that takes and how far it is from the
        # reference fixed point
        for name, warm, ng, lo in (("plain", False, 0, False), ("ng", False, 4, False),
                                   ("accelerated", False, 4, True), ("warm", True, 0, False),
                                   ("warm_accelerated", True, 4, True)):
            set_cloud()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if warm:
                pp, _, n, res, _ = ws.solve(ctx, rc, tol=1e-6, max_iter=3000, ng_period=ng, local_operator=lo)
            else:
                pp, _, n, res, _ = ctx.lambda_iterate(rc, tol=1e-6, max_iter=3000, ng_period=ng, local_operator=lo)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            e0, e2 = conv.rho_errors(pp, ref, live)
            out[name]["residual_rule"] = {"passes": int(n) + (1 if warm else 0), "seconds": dt,
                                          "last_change": float(res[-1]), "err_rho00": e0, "err_rho20": e2,
                                          "qi_abs_err": _qi_errors(image(ctx, pp), ref_img)}
    out["speedup_vs_plain"] = {k: out["plain"]["seconds"] / out[k]["seconds"]
                               for k in ("ng", "accelerated", "warm", "warm_accelerated")}
    out["speedup_vs_plain_residual_rule"] = {
        k: out["plain"]["residual_rule"]["seconds"] / out[k]["residual_rule"]["seconds"]
        for k in ("ng", "accelerated", "warm", "warm_accelerated")}
    out["warm_gain"] = {"passes_plain_over_warm": out["plain"]["passes"] / out["warm"]["passes"],
                        "seconds_accelerated_over_warm_accelerated":
                            out["accelerated"]["seconds"] / out["warm_accelerated"]["seconds"],
                        "training_seconds": out["training"]["data_seconds"] + out["training"]["fit_seconds"]}
    out["note"] = ("seconds: host wall time of one call of exactly the passes the method needs to reach the "
                   "target (feature pass and network inference included for warm runs); passes of warm runs "
                   "include the feature pass; qi_abs_err against the reference fixed point's image")
    return out


def se_large_stage(device, cloud, nlev=20, kmax=6, reps=2):
    """SE throughput at the largest system the named workloads pose: a
    20-level rotor at kmax 6 (74 x 74 systems) on the benchmark cloud's node
    conditions, the radiation field set to the local Planck intensity with a
    1e-3 anisotropy (the SE's cost does not depend on J's values).  Returns
    node-solves/s and the FP32 factorisation's flop rate against the FP32
    peak at the sampled clock."""
    import dataclasses
    import torch
    import portal_gb300 as pg
    from portal_gb300 import synth
    mol = synth.linear_rotor(nlev)
    frac = synth.lte_fractions(mol, np.maximum(cloud.t_kin, 1.0))
    cl = dataclasses.replace(cloud, lev_p=np.ascontiguousarray(frac * (cloud.ab_all * cloud.h2_dens)[:, None]))
    nu = np.asarray(mol.nu)
    T = np.maximum(cloud.t_kin, 1.0)[:, None]
    J0 = 1.4744995e-50 * nu ** 3 / np.expm1(4.79924e-11 * nu / T)
    J2 = 1e-3 * J0 * np.cos(np.arange(cloud.node_num))[:, None]
    with pg.Context(device) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(cl)
        best = 1e30
        for _ in range(reps + 1):
            pops, st = ctx.solve_se(kmax, J0, J2)
            best = min(best, ctx.kernel_times()["solve_se"][0])
    n = ctx_cdim(mol, kmax)
    nodes = cl.bulk_node_num
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    return {"system": "%d x %d (%d levels, kmax %d)" % (n, n, nlev, kmax), "launch_ms": best,
            "node_solves_per_s": nodes / (best * 1e-3), **lu_rates(nodes, n, best), "sms": sms,
            "refined_to_fp64": int(((st & pg.NODE_REFINE) != 0).sum()),
            "singular": int(((st & pg.NODE_SINGULAR) != 0).sum())}


def warmstart_1m_leg(device, n_train=8, train_points=16384, epochs=60):
    """The learned warm start on a held-out cube of the 1M-point recipe
    (1,048,576 points, seed 301): the network is trained as in the
    convergence leg (eight 16,384-point cubes of the same recipe), then the
    1M cube is converged by the accelerated iteration (local operator + Ng,
    plain pass deciding at tol 1e-6) from LTE and from the network's start;
    the 1025 x 1025 x 257 Stokes cube of the converged state follows.  16x16
    directions and 65 channels (at 32x32 / 129 one pass takes ~53 s; the
    plain iteration, ~370 passes, is not run at this size)."""
    import torch
    import portal_gb300 as pg
    from portal_gb300 import synth
    from portal_gb300.warmstart import WarmStart
    mol = synth.linear_rotor(20)
    rc = synth.RunConfig(nth=16, nph=16, nvel=32, kmax=2, gvec=synth.gauge_vector(4))
    out = {"workload": "turbulent cube, 1,048,576 points (seed 301, 128^3 fields), 20-level rotor, 16x16 "
                       "directions, 65 channels, kmax 2; network trained on %d cubes of %d points" %
                       (n_train, train_points)}
    with WarmStart(mol.j_lev, seed=1, device=device) as ws, pg.Context(device) as ctx:
        ctx.set_molecule(mol)
        t0 = time.perf_counter()
        Xs, Ys = [], []
        for i in range(n_train):
            cl = synth.turbulent_cube(train_points, 200 + i, mol, grid=32)
            ctx.set_cloud(cl)
            X, Y, _ = ws.collect(ctx, rc, cl.ab_all, cl.bulk_node_num)
            Xs.append(X)
            Ys.append(Y)
        t1 = time.perf_counter()
        ws.fit(np.concatenate(Xs), np.concatenate(Ys), epochs=epochs)
        out["training_seconds"] = {"data": t1 - t0, "fit": time.perf_counter() - t1}
        t0 = time.perf_counter()
        big = synth.turbulent_cube(1048576, 301, mol, grid=128)
        out["cloud_generation_s"] = time.perf_counter() - t0
        res = {}
        for name, warm in (("accelerated", False), ("warm_accelerated", True)):
            ctx.set_cloud(big)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if warm:
                pp, _, n, r, nseg = ws.solve(ctx, rc, tol=1e-6, max_iter=400, ng_period=4, local_operator=True)
            else:
                pp, _, n, r, nseg = ctx.lambda_iterate(rc, tol=1e-6, max_iter=400, ng_period=4, local_operator=True)
            torch.cuda.synchronize()
            res[name] = pp
            out[name] = {"passes": int(n) + (1 if warm else 0), "seconds": time.perf_counter() - t0,
                         "last_change": float(r[-1]), "segments": int(nseg)}
        a, w = res["accelerated"][:, 0::2], res["warm_accelerated"][:, 0::2]
        sig = np.abs(a) >= 1e-12 * np.abs(a).max(axis=1, keepdims=True)
        out["max_rel_diff_rho00"] = float((np.abs(w - a) / np.where(sig, np.abs(a), 1.0))[sig].max())
        out["speedup_warm"] = out["accelerated"]["seconds"] / out["warm_accelerated"]["seconds"]
        # the 1025 x 1025 x 257 Stokes cube of the converged state
        ctx.image([1], [2], 0.78539816339, 0.0, 128, 50.0, 0.0, 512, 0.7, pol_pops=res["warm_accelerated"],
                  quantities=4)
        kt = ctx.kernel_times()
        im_ms = kt["emcoefs"][0] + kt["image_walk"][0] + kt["image_rt"][0]
        out["image"] = {"cube": "1025 x 1025 pixels x 257 channels, line 1-0, 45 degrees", "kernel_ms": im_ms,
                        "pixel_channels_per_s": 1025 * 1025 * 257 / (im_ms * 1e-3)}
    return out


def _batch_cloud_worker(i):
    from portal_gb300 import synth
    return synth.batch_cloud(i)


def cube1m_leg(device, clk=None, cpu_seconds=10.0):
    """The 1,048,576-point turbulent cube (20-level rotor, 19 lines, 32x32
    directions = 678 rays per node, 129 channels, kmax 2): one node-loop pass
    (radiation field + SE) of the whole cloud, after a 16,384-point pass of
    the same shape has loaded the kernel variant; ray-segments/s, the HBM
    roofline of the radiation-field kernel, and the oracle port on a node
    sample of the same cloud."""
    import portal_gb300 as pg
    from portal_gb300 import synth
    t0 = time.perf_counter()
    cloud, mol, rc = synth.config_cloud("cube1m")
    gen_s = time.perf_counter() - t0
    small, _, _ = synth.config_cloud("cube1m", n_points=16384)
    with pg.Context(device) as ctx:
        ctx.set_molecule(mol)
        ctx.set_cloud(small)
        ctx.radiation_field(rc, fetch=False)
        ctx.set_cloud(cloud)
        t0 = time.perf_counter()
        _, _, _, nseg = ctx.radiation_field(rc, fetch=False)
        kt = ctx.kernel_times()
        ctx.solve_se(rc.kmax, fetch=False)
        kse = ctx.kernel_times()
        wall = time.perf_counter() - t0
    rf_ms = kt["radiation_field"][0]
    se_ms = kse["solve_se"][0]
    deg = float(np.diff(cloud.nb_off).mean())
    b_seg = 4 + deg * (4 + 12) + 12 + 4 + 4 + 4 + 4 * mol.nlev
    peak, kind = peaks()
    ach = b_seg * nseg / (rf_ms * 1e-3) / 1e9
    out = {"workload": "turbulent cube, 1,048,576 points (seed 4), 20-level rotor (19 lines), 32x32 directions, "
                       "129 channels, kmax 2", "cloud_generation_s": gen_s,
           "segments": int(nseg), "radiation_field_ms": rf_ms, "se_ms": se_ms, "pass_wall_s": wall,
           "ray_segments_per_s": nseg / ((rf_ms + kt["line_table"][0] + se_ms) * 1e-3),
           "node_solves_per_s": cloud.bulk_node_num / (se_ms * 1e-3),
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "algorithmic_bytes_per_segment": b_seg, "peak_source": kind}}
    rates, cores = cpu_port_rate(cloud, mol, rc, cpu_seconds, repeats=1)
    out["cpu_baseline"] = {"value": rates[0][0], "unit": UNIT, "cores": cores, "kind": "port",
                           "sample": "%d consecutive nodes of %d (all their rays + SE), %.1f s" %
                                     (rates[0][2], cloud.bulk_node_num, rates[0][1])}
    return out


def batch_leg(device, n_clouds=64):
    """64 uneven clouds (10k-300k points, 5-20 levels; 16x16 directions, 65
    channels, kmax 2) through one persistent radiation-field launch and one
    SE launch (portal_batch_*), launch shapes chosen by the autotuner:
    one pass replayed from the CUDA graph, one issued directly, and the same
    models one after another through the single-model calls."""
    import multiprocessing as mp
    import portal_gb300 as pg
    from portal_gb300 import synth
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        models = pool.map(_batch_cloud_worker, range(n_clouds))
    gen_s = time.perf_counter() - t0
    rc = synth.RunConfig(gvec=synth.gauge_vector(3), **synth.BATCH_RUN_CONFIG)
    ctxs = []
    try:
        for cl, mol in models:
            c = pg.Context(device)
            c.set_molecule(mol)
            c.set_cloud(cl)
            ctxs.append(c)
        with pg.Batch(device) as b:
            for c in ctxs:
                b.add(c)
            t0 = time.perf_counter()
            b.prepare(rc, autotune=True)
            prep_s = time.perf_counter() - t0
            cfg, tune = b.config()
            nseg_g, ms_g = b.run(use_graph=True)
            nseg_d, ms_d = b.run(use_graph=False)
    finally:
        for c in ctxs:
            c.close()
    # the same models one after another through one context (each model's
    # upload is outside the timed calls)
    import torch
    seq_s, nseg_s = 0.0, 0
    with pg.Context(device) as c:
        for cl, mol in models:
            c.set_molecule(mol)
            c.set_cloud(cl)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, _, _, n = c.radiation_field(rc, fetch=False)
            c.solve_se(rc.kmax, fetch=False)
            torch.cuda.synchronize()
            seq_s += time.perf_counter() - t0
            nseg_s += n
    pts = int(sum(cl.node_num for cl, _ in models))
    return {"workload": "%d power-law clouds (seeds 100-%d), %d points in all, 5-20 levels, 16x16 directions, "
                        "65 channels, kmax 2" % (n_clouds, 99 + n_clouds, pts),
            "cloud_generation_s": gen_s, "prepare_s": prep_s,
            "launch_shapes": {"line_group": int(cfg[0]), "rf_blocks_per_sm": int(cfg[1]),
                              "se_warps_per_block": int(cfg[2]), "se_blocks_per_sm": int(cfg[3])},
            "graph_pass_ms": ms_g, "direct_pass_ms": ms_d, "sequential_pass_s": seq_s,
            "segments": int(nseg_g), "graph_ray_segments_per_s": nseg_g / (ms_g * 1e-3),
            "sequential_ray_segments_per_s": nseg_s / seq_s,
            "note": "graph and direct: device time of the pass; sequential: host wall time of the single-model "
                    "calls (radiation field + SE), one model after another through one context"}


def profile_case(name):
    """Small fixed workloads for capturing one kernel with ncu; each is seeded
    and ends in seconds, so a capture of a few launches ends by itself.
      mlp_forward   k_gemm_tc: 3 predicts of 65,536 rows through 8 -> 256 x 3 -> 40;
      image         k_image: 2 images, 257 x 257 pixels x 129 channels of a
                    32,768-point sphere of the benchmark recipe (seed 1, 10 levels),
                    line 1-0 at 45 degrees, from the cloud's own populations;
      se            k_solve_se: 2 solves of a 32,768-point sphere at 20 levels,
                    kmax 6 (74 x 74 systems)."""
    import portal_gb300 as pg
    from portal_gb300 import build as pbuild
    from portal_gb300 import synth
    pbuild.build()
    if name == "mlp_forward":
        X = np.random.default_rng(0).normal(size=(65536, 8)).astype(np.float32)
        with pg.MLP(8, 256, 3, 40, seed=1) as m:
            for _ in range(3):
                Y = m.predict(X)
        print("mlp_forward ok", float(np.abs(Y).mean()))
    elif name == "image":
        cloud, mol, rc = synth.config_cloud("sphere262k", n_points=32768)
        g = np.sqrt(2.0 * mol.j_lev + 1.0)
        pp = np.zeros((cloud.node_num, 2 * mol.nlev))
        pp[:, 0::2] = cloud.lev_p / np.maximum(cloud.lev_p.sum(axis=1, keepdims=True), 1e-300) / g
        pp[:, 1::2] = 1e-3 * pp[:, 0::2]
        with pg.Context(0) as ctx:
            ctx.set_molecule(mol)
            ctx.set_cloud(cloud)
            for _ in range(2):
                # n_depth_rt 1024: 0.6 GB of march scratch instead of 6 GB
                cube, st = ctx.image([1], [2], 0.78539816339, 0.0, 64, 50.0, 0.0, 128, 0.7, pol_pops=pp,
                                     quantities=4, n_depth_rt=1024)
            kt = ctx.kernel_times()
        print("image ok", int(st.sum()), float(np.nanmax(cube[0])), {k: v for k, v in kt.items() if v[1]})
    elif name == "se":
        cloud, mol, rc = synth.config_cloud("sphere262k", n_points=32768)
        r = se_large_stage(0, cloud, reps=1)
        print("se ok", r)
    else:
        raise SystemExit("unknown profile case %r" % name)
    return 0


def reduce_replicas(t, units, dist=None):
    """Whole-job figures of N independent replicas: the slowest rank's time
    (max over ranks) and the units all ranks processed (sum).  dist is
    torch.distributed (gloo here) or None for one rank."""
    if dist is None:
        return float(t), float(units)
    import torch
    tt = torch.tensor([float(t)], dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    uu = torch.tensor([float(units)], dtype=torch.float64)
    dist.all_reduce(uu, op=dist.ReduceOp.SUM)
    return float(tt.item()), float(uu.item())


def lu_rates(nodes, n, launch_ms, sms=None, sm_mhz=None):
    """FP32 factorisation flop rate of an SE launch (2/3 n^3 per node of n
    unknowns) and, given the SM count and the sampled clock, its fraction of
    the FP32 FMA peak (SMs x 128 lanes x 2 flop x clock)."""
    r = {"fp32_lu_flop_per_s": nodes * (2.0 / 3.0) * n ** 3 / (launch_ms * 1e-3)}
    if sms and sm_mhz:
        peak = sms * 128 * 2 * float(sm_mhz) * 1e6
        r["fp32_peak_flop_per_s"] = peak
        r["fp32_lu_frac"] = r["fp32_lu_flop_per_s"] / peak
    return r


def ctx_cdim(mol, kmax):
    """Order of the SE system: components K = 0, 2, .. min(2J, kmax) per level."""
    return int(sum(min(2 * int(j), kmax) // 2 + 1 for j in mol.j_lev))


def gpu_arm(args, rank, world, local_rank):
    import torch
    import portal_gb300 as pg
    from portal_gb300 import build as pbuild

    pbuild.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    cloud, mol, rc = build_workload(args.points, args.n_depth)
    N, nlev = cloud.node_num, mol.nlev
    stream = torch.cuda.Stream()
    ctx = pg.Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_molecule(mol)

    # reference-layout host arrays in pinned memory (what a Fortran caller passes)
    def pinned(a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        t = torch.empty(a.shape, dtype=torch.float64 if dtype == np.float64 else torch.int32, pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()
    temp = np.stack([cloud.t_kin, cloud.t_dust], axis=1)
    host = dict(xyz=pinned(cloud.xyz, np.float64), vel=pinned(cloud.vel, np.float64),
                b_all=pinned(cloud.b_all, np.float64), temp_all=pinned(temp, np.float64),
                dust_p=pinned(cloud.dust_p, np.float64), h2_dens=pinned(cloud.h2_dens, np.float64),
                ab_all=pinned(cloud.ab_all, np.float64), lev_p=pinned(cloud.lev_p, np.float64),
                bvec=pinned(cloud.bvec, np.float64), del_ne=pinned(cloud.del_ne(), np.int32),
                del_num_ne=pinned(cloud.del_num_ne(), np.int32))
    h2d = sum(int(v.nbytes) for v in host.values())
    pops_host = pinned(np.zeros((2 * nlev, N)), np.float64)
    d2h = int(pops_host.nbytes) + 4 * N

    def upload():
        ctx.set_cloud_arrays(N, cloud.bulk_node_num, nlev, host["xyz"], host["vel"], host["b_all"],
                             host["temp_all"], host["dust_p"], host["h2_dens"], host["ab_all"], host["lev_p"],
                             host["bvec"], host["del_ne"], host["del_num_ne"], cloud.tx)

    upload()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def step():
        _, _, _, nseg = ctx.radiation_field(rc, fetch=False)
        kt_rf = ctx.kernel_times()
        ctx.solve_se(rc.kmax, fetch=False)
        kt_se = ctx.kernel_times()
        return nseg, kt_rf, kt_se

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    clocks.start()
    times, rf_ms, se_ms, launches, nseg_tot = [], [], [], 0, 0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        nseg, kt_rf, kt_se = step()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        rf_ms.append(kt_rf["radiation_field"][0])
        se_ms.append(kt_se["solve_se"][0])
        launches += kt_rf["line_table"][1] + kt_rf["radiation_field"][1] + kt_se["solve_se"][1]
        nseg_tot += nseg
    torch.cuda.synchronize()
    clk = clocks.stop()
    t_total_ms = sum(times)
    t_total_ms, nseg_all = reduce_replicas(t_total_ms, nseg_tot, dist)
    value = nseg_all / (t_total_ms * 1e-3)
    nseg_step = nseg_tot / args.steps

    # ---- end to end through the C ABI from pinned host memory ----
    e2e_times = []
    for _ in range(max(1, args.e2e_steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        upload()
        ctx.radiation_field(rc, fetch=False)
        ctx.solve_se(rc.kmax, out=pops_host)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    t_e2e = statistics.median(e2e_times)
    t_e2e, _ = reduce_replicas(t_e2e, 0, dist)
    e2e_val = nseg_step * world / t_e2e

    # ---- the other two stages' throughput: SE node solves, Stokes image ----
    se_launch_ms = statistics.median(se_ms)
    n_se = ctx_cdim(mol, rc.kmax)
    sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
    stages = {"se": {"node_solves_per_s": cloud.bulk_node_num / (se_launch_ms * 1e-3), "launch_ms": se_launch_ms,
                     "system": "%d x %d (kmax %d)" % (n_se, n_se, rc.kmax),
                     **lu_rates(cloud.bulk_node_num, n_se, se_launch_ms, sms, clk.get("sm_mhz") if clk else None)}}
    if not args.no_image:
        im_pix, im_nvel = 256, 64
        ctx.image([1], [2], 0.78539816339, 0.0, im_nvel, 50.0, 0.0, im_pix, 0.7, quantities=4)   # warm-up
        ctx.image([1], [2], 0.78539816339, 0.0, im_nvel, 50.0, 0.0, im_pix, 0.7, quantities=4)
        kt = ctx.kernel_times()
        im_ms = kt["emcoefs"][0] + kt["image_walk"][0] + kt["image_rt"][0]
        npx = 2 * im_pix + 1
        stages["image"] = {"pixel_channels_per_s": npx * npx * (2 * im_nvel + 1) / (im_ms * 1e-3),
                           "kernel_ms": im_ms, "cube": "%dx%d pixels x %d channels, line 1-0, inclination 45 deg"
                                                       % (npx, npx, 2 * im_nvel + 1)}

    if not args.no_se_large:
        sl = se_large_stage(local_rank, cloud)
        n_l = int(sl["system"].split(" x ")[0])
        sl.update(lu_rates(cloud.bulk_node_num, n_l, sl["launch_ms"], sl["sms"], clk.get("sm_mhz") if clk else None))
        stages["se_large"] = sl

    # ---- roofline of the dominant kernel (radiation field) ----
    deg = float(np.diff(cloud.nb_off).mean())
    b_seg = 4 + deg * (4 + 12) + 12 + 4 + 4 + 4 + 4 * nlev
    rf_launch_ms = statistics.median(rf_ms)
    achieved = b_seg * nseg_step / (rf_launch_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    tps = traffic_per_segment()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": (tps * nseg_step) if tps else None,
            "kernel": "k_radiation_field", "algorithmic_bytes_per_segment": b_seg,
            "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
            "launch_ms": rf_launch_ms, "segments_per_launch": nseg_step}
    # the kernel's actual bound is instruction issue (its data is L2-resident):
    # warp instructions per segment (ncu, profiles/) x segments / launch time
    # against one warp instruction per SMSP per cycle at the sampled SM clock
    wips = profile_constant("warp_instructions_per_segment")
    if wips and clk and clk.get("sm_mhz"):
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        ipeak = sms * 4 * float(clk["sm_mhz"]) * 1e6
        iach = wips * nseg_step / (rf_launch_ms * 1e-3)
        roof["issue"] = {"achieved": iach, "peak": ipeak, "unit": "warp instructions/s", "frac": iach / ipeak,
                         "warp_instructions_per_segment": wips,
                         "peak_source": "%d SMs x 4 schedulers x 1 instruction/cycle at %.0f MHz" %
                                        (sms, float(clk["sm_mhz"]))}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 ray integration, f32 LU + f64 refinement",
            "data": "synthetic", "config": workload_config(cloud, mol, rc, N),
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "roofline": roof, "clocks": clk, "stages": stages}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rates, cores = cpu_port_rate(cloud, mol, rc, args.cpu_seconds, repeats=1)
        line["cpu_baseline"] = {"value": rates[0][0], "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": "%d consecutive nodes of %d (all their rays + SE), %.1f s" %
                                          (rates[0][2], cloud.bulk_node_num, rates[0][1])}
    ctx.close()
    if rank == 0 and world == 1 and not args.no_cube1m:
        line["cube1m"] = cube1m_leg(local_rank, clk)
    if rank == 0 and world == 1 and not args.no_batch:
        line["batch64"] = batch_leg(local_rank)
    if rank == 0 and world == 1 and not args.no_convergence:
        line["convergence"] = convergence_leg(local_rank)
    if rank == 0 and world == 1 and args.warmstart_1m:
        line["warmstart_1m"] = warmstart_1m_leg(local_rank)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--points", type=int, default=262144)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-image", action="store_true", help="skip the Stokes-image throughput leg")
    ap.add_argument("--no-cube1m", action="store_true",
                    help="skip the 1,048,576-point turbulent-cube pass")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 64-cloud batch (persistent launch under a CUDA graph)")
    ap.add_argument("--warmstart-1m", action="store_true",
                    help="also run the learned warm start on a held-out 1,048,576-point cube (~10 min)")
    ap.add_argument("--no-se-large", action="store_true",
                    help="skip the 74 x 74 SE throughput stage (20-level rotor, kmax 6)")
    ap.add_argument("--no-convergence", action="store_true",
                    help="skip the time-to-converged comparison (plain / accelerated / warm-started)")
    ap.add_argument("--n-depth", type=int, default=10000,
                    help="walk length limit (main_portal.x's n_depth); smaller values shrink the walk scratch")
    ap.add_argument("--profile-case", choices=["mlp_forward", "image", "se"],
                    help="run one small fixed workload for an ncu capture instead of the benchmark")
    args = ap.parse_args()
    if args.profile_case:
        return profile_case(args.profile_case)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.gpus == 1 else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank, world)
    return gpu_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
