#!/usr/bin/env python3
"""Benchmark of the GB300 sphere mobility solve (one JSON line on rank 0).

Workload (one "step"): one mobility solve of configuration 2 — 64 rigid spheres of radius 1
placed by seeded random sequential addition in a box of side 20 (min surface gap 0.1),
SH order 16 (36,992 grid points), N(0,1) forces and torques — to 1e-8 relative residual with
GMRES(50). The headline arm is the mixed-precision solve (FP32 operator inside FP64 iterative
refinement); the plain FP64 GPU solve of the same problem is timed beside it.

  value : solves/s with the forces already resident in HBM (smob_solve_mob_device), each step timed
          with CUDA events on the library's stream, L2 evicted (256 MB write) between steps
  e2e   : the same through smob_solve_mob with host buffers (pinned when torch is importable):
          host->device copy of the 6N forces and device->host copy of the 6N velocities inside
  roofline : the dominant kernel (FP32 traction far field): algorithmic FLOPs (30 per pair) per launch
          / average launch time, against the FP32 FMA issue rate measured in the same run
  roofline_far_df : the same for the fused float-float pass (the largest share of a mixed solve):
          59 flop per evaluated pair (traction + single layer) over its average time
  cpu_baseline : one full FP64 solve of the workload by the C++/OpenMP restatement of the reference
          path, on this host's cores
  rel_err_vs_oracle : velocities against the restatement's solve of this workload at relative
          residual 1e-12 (a committed fixture)

--impl reference times that CPU restatement alone (the reference itself cannot be built: its
SCTL/STKFMM/Trilinos dependencies are absent), one full solve per step, on the same workload and
metric.
Multi-GPU: replicas only (each rank solves its own copy of the workload on its own GPU).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "mobility solves/s & p50/p99 latency at 1e-8 resid, mixed vs plain FP64 GPU"
TOL = 1e-8
RESTART = 50
L2_FLUSH_BYTES = 256 << 20
WORKLOAD = ("cfg2: 64 spheres a=1, seeded RSA in box 20 (min gap 0.1), p=16 (36992 points), "
            "N(0,1) force/torque, GMRES(50) to 1e-8 relative residual")
# DRAM bytes (read + write) of one FP32 traction far-field launch on this workload, from an ncu capture
# (GB300, k_far32_ct<1>, the entry kernel with coarse sources and targets: 4,364,032 read, 0 written)
CFG2_FAR32_DRAM_BYTES = 4364032


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def far_pairs(mob):
    """Pairs per far-field launch: all target-source pairs of different spheres minus the near pairs'
    sphere blocks (those are evaluated spectrally)."""
    ng = np.array([(p + 1) * (2 * p + 2) for p in mob.orders], dtype=np.int64)
    M = ng.sum()
    pairs = M * M - (ng * ng).sum()
    t, s = mob.near_pairs()
    pairs -= (ng[t] * ng[s]).sum()
    return int(pairs)


def run_native(args, world, rank, local, dist):
    import ctypes

    from spheresimulator_gb300 import PREC_FP64, PREC_MIXED, SphereSTKMobMat, configs, solve_opts
    from spheresimulator_gb300 import _native as N

    L = N.lib()
    cfg = configs.cfg2()
    mob = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], device=local)
    h = mob.handle
    n6 = 6 * mob.n_spheres
    force = np.ascontiguousarray(cfg["force"])
    d_force, d_vel = ctypes.c_void_p(), ctypes.c_void_p()
    N.check(L.smob_device_alloc(h, 8 * n6, ctypes.byref(d_force)))
    N.check(L.smob_device_alloc(h, 8 * n6, ctypes.byref(d_vel)))
    N.check(L.smob_memcpy_h2d(h, d_force, force.ctypes.data_as(ctypes.c_void_p), 8 * n6))
    stats = (N.ProblemStats * 1)()

    def solve_dev(prec, pc=0):
        o = solve_opts(TOL, RESTART, 1000, prec, precond=pc)
        code = L.smob_solve_mob_device(h, d_force, d_vel, None, ctypes.byref(o), stats)
        N.check(code)
        return stats[0].as_dict()

    def timed(prec, steps, pc=0):
        ms = []
        st = None
        for _ in range(steps):
            N.check(L.smob_flush_l2(h, L2_FLUSH_BYTES))
            N.check(L.smob_timer_mark(h))
            st = solve_dev(prec, pc)
            t = ctypes.c_double()
            N.check(L.smob_timer_elapsed(h, ctypes.byref(t)))
            ms.append(t.value)
        return np.array(ms), st

    for _ in range(args.warmup):
        solve_dev(PREC_MIXED)
    solve_dev(PREC_FP64)

    # ---- headline: mixed precision, inputs resident
    barrier(dist)
    l0, hc0 = mob.launch_stats()
    with ClockSampler(local) as clk:
        ms_mixed, st_mixed = timed(PREC_MIXED, args.steps)
    l1, hc1 = mob.launch_stats()
    launches = (l1 - l0) / max(args.steps, 1)
    host_calls = (hc1 - hc0) / max(args.steps, 1)
    total_s = allmax(dist, ms_mixed.sum() / 1e3)
    # the same solves with the host-driven restart loop (captured 4-step blocks, host checks between them)
    mob.set_loop_graph(False)
    timed(PREC_MIXED, 2)
    l0, hc0 = mob.launch_stats()
    k_host = max(3, min(args.steps, 10))
    ms_hostloop, _ = timed(PREC_MIXED, k_host)
    l1, hc1 = mob.launch_stats()
    mob.set_loop_graph(True)
    loop_graph = {"on": mob.loop_graph_info()[0], "kernels_per_solve": round(launches, 1),
                  "host_launch_calls_per_solve": round(host_calls, 1),
                  "host_loop": {"solves_per_s": round(1e3 / float(ms_hostloop.mean()), 3),
                                "p50_ms": round(float(np.percentile(ms_hostloop, 50)), 3), "steps": k_host,
                                "kernels_per_solve": round((l1 - l0) / k_host, 1),
                                "host_launch_calls_per_solve": round((hc1 - hc0) / k_host, 1)}}
    vel_mixed = np.zeros(n6)
    N.check(L.smob_memcpy_d2h(h, vel_mixed.ctypes.data_as(ctypes.c_void_p), d_vel, 8 * n6))

    # ---- plain FP64 GPU solve of the same problem
    fp64_steps = max(1, min(args.steps, args.fp64_steps))
    ms_fp64, st_fp64 = timed(PREC_FP64, fp64_steps)
    vel_fp64 = np.zeros(n6)
    N.check(L.smob_memcpy_d2h(h, vel_fp64.ctypes.data_as(ctypes.c_void_p), d_vel, 8 * n6))

    # ---- the same mixed solve with the block-diagonal right preconditioner (smob_solve_opts.precond = 1)
    solve_dev(PREC_MIXED, 1)
    ms_pc, st_pc = timed(PREC_MIXED, args.steps, 1)
    vel_pc = np.zeros(n6)
    N.check(L.smob_memcpy_d2h(h, vel_pc.ctypes.data_as(ctypes.c_void_p), d_vel, 8 * n6))
    pc_total = allmax(dist, ms_pc.sum() / 1e3)

    # ---- the same mixed solve with every FP32 far-field pair summed directly (no coarse equivalent sources)
    eps_default = mob.far_compression_info()[0]
    eps_hp_default = mob.far_compression_info(hp=True)[0]
    mob.set_far_compression(0, 0)
    for _ in range(args.warmup):
        solve_dev(PREC_MIXED)
    ms_dir, st_dir = timed(PREC_MIXED, args.steps)
    vel_dir = np.zeros(n6)
    N.check(L.smob_memcpy_d2h(h, vel_dir.ctypes.data_as(ctypes.c_void_p), d_vel, 8 * n6))
    dir_total = allmax(dist, ms_dir.sum() / 1e3)
    mob.set_far_compression(eps_default, eps_hp_default)
    solve_dev(PREC_MIXED)

    # ---- end to end through the host-pointer API
    try:
        import torch
        hf = torch.from_numpy(force).pin_memory()
        hv = torch.zeros(n6, dtype=torch.float64).pin_memory()
        fptr = ctypes.cast(hf.data_ptr(), N._DP)
        vptr = ctypes.cast(hv.data_ptr(), N._DP)
        pinned = True
    except Exception:
        hv_np = np.zeros(n6)
        fptr, vptr = N.dptr(force), N.dptr(hv_np)
        pinned = False
    e2e_ms = []
    for _ in range(args.steps):
        N.check(L.smob_flush_l2(h, L2_FLUSH_BYTES))
        o = solve_opts(TOL, RESTART, 1000, PREC_MIXED)
        N.check(L.smob_timer_mark(h))
        N.check(L.smob_solve_mob(h, fptr, vptr, None, ctypes.byref(o), stats))
        t = ctypes.c_double()
        N.check(L.smob_timer_elapsed(h, ctypes.byref(t)))
        e2e_ms.append(t.value)
    e2e_total = allmax(dist, sum(e2e_ms) / 1e3)

    # ---- instrumented pass: per-kernel CUDA-event times on the library stream
    mob.profile(True)
    mob.profile_reset()
    solve_dev(PREC_MIXED)
    prof = mob.profile_table()
    # the same solve with the other FP32 near-field kernel, then the other FP32 sphere-operator kernel
    # (tensor cores vs SIMT pipes), each against the defaults
    near_tc0, sph_tc0 = mob.near_tc(), mob.sphere_tc()
    mob.set_near_tc(not near_tc0)
    mob.profile_reset()
    solve_dev(PREC_MIXED)
    prof_near_alt = mob.profile_table()
    mob.set_near_tc(near_tc0)
    mob.set_sphere_tc(not sph_tc0)
    mob.profile_reset()
    solve_dev(PREC_MIXED)
    prof_sph_alt = mob.profile_table()
    mob.set_sphere_tc(sph_tc0)
    coarse_tc0 = mob.coarse_tc()
    mob.set_coarse_tc(not coarse_tc0)
    mob.profile_reset()
    solve_dev(PREC_MIXED)
    prof_coarse_alt = mob.profile_table()
    mob.profile(False)
    # and timed solves with the other coarse kernels: both SIMT, then only one of the two on the
    # tensor cores
    timed(PREC_MIXED, 2)
    ms_coarse_alt, _ = timed(PREC_MIXED, max(3, min(args.steps, 10)))
    coarse_modes = {}
    for mode in (2, 3):
        mob.set_coarse_tc(mode)
        timed(PREC_MIXED, 2)
        coarse_modes[mode] = round(1e3 / float(timed(PREC_MIXED, max(3, min(args.steps, 10)))[0].mean()), 3)
    mob.set_coarse_tc(coarse_tc0)
    f32, f64 = ctypes.c_double(), ctypes.c_double()
    N.check(L.smob_measure_fma_peaks(local, ctypes.byref(f32), ctypes.byref(f64)))
    tpt, tms, tcache = ctypes.c_int(), (ctypes.c_double * 3)(), ctypes.c_int()
    N.check(L.smob_tuning(h, ctypes.byref(tpt), tms, ctypes.byref(tcache)))

    if rank != 0:
        return None
    pairs = far_pairs(mob)
    direct, evaluated, coarse_macs = mob.far_pairs()
    assert direct == pairs, (direct, pairs)
    k_l, k_ms = prof.get("far_trac_fp32", (0, 0.0))
    avg_s = (k_ms / max(k_l, 1)) / 1e3
    achieved = 30.0 * evaluated / avg_s / 1e12 if avg_s > 0 else None
    c_l, c_ms = prof.get("far_coarse", (0, 0.0))
    eps, cpts, cent = mob.far_compression_info()
    eps_hp, cpts_hp, cent_hp = mob.far_compression_info(hp=True)
    tot_prof = sum(v[1] for v in prof.values())

    # ---- CPU baseline: one full FP64 oracle solve of the same workload, timed
    cpu = cpu_sample(cfg, args.cpu_threads)
    # ---- error against the oracle's solve of this workload at relative residual 1e-12 (committed fixture)
    gold = np.load(os.path.join(ROOT, "tests", "golden", "golden_cfg2_solve.npz"))
    assert np.array_equal(gold["force"], force) and np.array_equal(gold["centers"], cfg["centers"])
    v_orc = gold["vel"]
    dh, eh, mh = mob.far_pairs(hp=True)
    d_l, d_ms = prof.get("far_both_df", (0, 0.0))
    avg_df = (d_ms / max(d_l, 1)) / 1e3
    achieved_df = 59.0 * eh / avg_df / 1e12 if avg_df > 0 else None
    # evaluated pair interactions of the profiled solve: FP32 passes (one kernel per pair) and the fused
    # float-float pass (both kernels per pair)
    n_fp32_passes = prof.get("far_trac_fp32", (0, 0))[0] + prof.get("far_sl_fp32", (0, 0))[0]
    evaluated_per_solve = n_fp32_passes * evaluated + 2 * d_l * eh

    value = world * args.steps / total_s
    line = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(float(ms_mixed.mean()), 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 operator + f64 refinement (mixed)",
        "data": "synthetic (seeded RSA packing, N(0,1) forces)",
        "config": {"workload": WORKLOAD, "tol": TOL, "restart": RESTART, "precision": "mixed",
                   "l2": "flushed between steps (256 MB device write)", "parallelism": "replicas only"},
        "latency_ms": {"p50": round(float(np.percentile(ms_mixed, 50)), 4),
                       "p99": round(float(np.percentile(ms_mixed, 99)), 4)},
        "mixed": {"iterations": st_mixed["iterations"], "refinements": st_mixed["refinements"],
                  "passes_fp32": st_mixed["operator_passes_fp32"], "passes_fp64": st_mixed["operator_passes_fp64"],
                  "relres": st_mixed["relres"]},
        "fp64": {"solves_per_s": round(world * len(ms_fp64) / allmax(None, ms_fp64.sum() / 1e3), 4),
                 "p50_ms": round(float(np.percentile(ms_fp64, 50)), 3),
                 "p99_ms": round(float(np.percentile(ms_fp64, 99)), 3),
                 "iterations": st_fp64["iterations"], "passes_fp64": st_fp64["operator_passes_fp64"],
                 "relres": st_fp64["relres"], "steps": len(ms_fp64)},
        "mixed_vs_fp64_speedup": round(float(ms_fp64.mean() / ms_mixed.mean()), 3),
        "mixed_block_diagonal_precond": {
            "solves_per_s": round(world * args.steps / pc_total, 4),
            "p50_ms": round(float(np.percentile(ms_pc, 50)), 4), "p99_ms": round(float(np.percentile(ms_pc, 99)), 4),
            "iterations": st_pc["iterations"], "passes_fp32": st_pc["operator_passes_fp32"],
            "passes_fp64": st_pc["operator_passes_fp64"], "relres": st_pc["relres"],
            "rel_err_vs_fp64": float(np.linalg.norm(vel_pc - vel_fp64) / np.linalg.norm(vel_fp64)),
            "note": "optional (not the reference's Krylov path): GMRES on A P, P = each sphere's own operator inverted"},
        "mixed_direct_far_field": {
            "solves_per_s": round(world * args.steps / dir_total, 4),
            "p50_ms": round(float(np.percentile(ms_dir, 50)), 4), "p99_ms": round(float(np.percentile(ms_dir, 99)), 4),
            "iterations": st_dir["iterations"], "passes_fp32": st_dir["operator_passes_fp32"],
            "relres": st_dir["relres"],
            "rel_err_vs_fp64": float(np.linalg.norm(vel_dir - vel_fp64) / np.linalg.norm(vel_fp64)),
            "note": "the headline solve with the far field summed over every grid source pair in every pass "
                    "(smob_set_far_compression(ctx, 0, 0))"},
        "rel_err_mixed_vs_fp64": float(np.linalg.norm(vel_mixed - vel_fp64) / np.linalg.norm(vel_fp64)),
        "rel_err_vs_oracle": {"mixed": float(np.linalg.norm(vel_mixed - v_orc) / np.linalg.norm(v_orc)),
                              "fp64": float(np.linalg.norm(vel_fp64 - v_orc) / np.linalg.norm(v_orc)),
                              "oracle": "FP64 C++ restatement's solve of this workload to relres 1e-12 "
                                        "(tests/golden/golden_cfg2_solve.npz, %d iterations)" % int(gold["iters"])},
        "mixed_vs_fp64_like_for_like": {
            "speedup": round(float(ms_fp64.mean() / ms_dir.mean()), 3),
            "note": "mixed solve with the direct-sum far field (mixed_direct_far_field) against the plain FP64 "
                    "solve (direct sum): precision alone; mixed_vs_fp64_speedup adds the coarse far field"},
        "pair_interactions_per_s": round(pairs * (st_mixed["operator_passes_fp32"] + st_mixed["operator_passes_fp64"])
                                         / (ms_mixed.mean() / 1e3), 1),
        "pair_interactions_note": "direct-sum pairs per solve (every far target-source pair of every operator pass) "
                                  "/ solve time; the FP32 passes evaluate well-separated sphere pairs from coarse "
                                  "equivalent sources (far_compression)",
        "evaluated_pair_interactions_per_s": round(evaluated_per_solve / (ms_mixed.mean() / 1e3), 1),
        "evaluated_pair_interactions_note": "pair-kernel evaluations the far-field kernels actually perform per "
                                            "solve (FP32 passes x evaluated pairs + fused float-float pass x 2 "
                                            "kernels x its evaluated pairs) / solve time",
        "far_compression": {"eps": eps, "coarse_points": cpts, "entries": cent, "direct_pairs_per_pass": direct,
                            "evaluated_pairs_per_pass": evaluated,
                            "evaluated_fraction": round(evaluated / direct, 4) if direct else None,
                            "coarse_strength_macs_per_pass": coarse_macs,
                            "coarse_strength_ms_per_pass": round(c_ms / max(c_l, 1), 5),
                            "eps_float_float": eps_hp, "coarse_points_float_float": cpts_hp,
                            "entries_float_float": cent_hp},
        "roofline": {"kernel": "far_trac_fp32", "bound": "fp32_simt", "achieved": round(achieved, 3) if achieved else None,
                     "peak": round(f32.value, 3), "unit": "TFLOP/s",
                     "frac": round(achieved / f32.value, 4) if achieved else None,
                     "traffic": CFG2_FAR32_DRAM_BYTES,
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one k_far32_ct launch (the "
                                       "FP32 entry kernel) on this workload (ncu --set full, bench.py --far-once); "
                                       "algorithmic bytes (grid positions, normals, sources 1.8 MB, coarse points, "
                                       "normals and strengths 3.3 MB, candidate table 0.1 MB, each once; partial "
                                       "sums stay in L2) = 5.2 MB upper bound",
                     "peak_source": "FP32 FMA issue rate measured in this run (MEASURED_PEAKS.json has no SIMT entry)",
                     "flops_per_launch": 30.0 * evaluated, "pairs_per_launch": evaluated,
                     "pairs_note": "pairs one FP32 far-field pass evaluates (grid targets or a target sphere's coarse "
                                   "nodes, against grid sources or coarse equivalent sources, for well-separated "
                                   "sphere pairs), 30 flop each; the time is the pass's entry kernel, chunk sums "
                                   "and interpolation together",
                     "avg_launch_ms": round(avg_s * 1e3, 5), "launches_in_profiled_solve": k_l,
                     "share_of_kernel_time": round(k_ms / tot_prof, 4) if tot_prof else None,
                     "fp64_fma_peak_tflops": round(f64.value, 4)},
        "roofline_far_df": {
            "kernel": "far_both_df (k_far_df_ct + its chunk sums and interpolation: the fused float-float "
                      "traction + single-layer pass of the refinement residual)",
            "bound": "fp32_simt", "achieved": round(achieved_df, 3) if achieved_df else None,
            "peak": round(f32.value, 3), "unit": "TFLOP/s",
            "frac": round(achieved_df / f32.value, 4) if achieved_df else None,
            "pairs_per_launch": eh, "direct_pairs_per_launch": dh, "flops_per_pair": 59,
            "flops_note": "algorithmic work: traction 30 + single layer 29 flop per pair (FP64-class results, "
                          "emulated in float-float on the FP32 pipes at several FP32 operations per flop)",
            "avg_launch_ms": round(avg_df * 1e3, 5), "launches_in_profiled_solve": d_l,
            "share_of_kernel_time": round(d_ms / tot_prof, 4) if tot_prof else None},
        "kernel_ms_profiled_solve": {k: [v[0], round(v[1], 4)] for k, v in sorted(prof.items())},
        "tensor_cores": {
            "near_eval_trac_ms_tc_simt": [round((prof if near_tc0 else prof_near_alt).get("near_eval_trac", (0, 0.0))[1], 4),
                                          round((prof_near_alt if near_tc0 else prof).get("near_eval_trac", (0, 0.0))[1], 4)],
            "sphere_self_ms_tc_simt": [round((prof if sph_tc0 else prof_sph_alt).get("sphere_self", (0, 0.0))[1], 4),
                                       round((prof_sph_alt if sph_tc0 else prof).get("sphere_self", (0, 0.0))[1], 4)],
            "far_coarse_ms_tc_simt": [round((prof if coarse_tc0 else prof_coarse_alt).get("far_coarse", (0, 0.0))[1], 4),
                                      round((prof_coarse_alt if coarse_tc0 else prof).get("far_coarse", (0, 0.0))[1], 4)],
            "solves_per_s_other_coarse_kernel": round(1e3 / float(ms_coarse_alt.mean()), 3),
            "solves_per_s_coarse_tc_strengths_only": coarse_modes[2],
            "solves_per_s_coarse_tc_interpolation_only": coarse_modes[3],
            "default_near_tc": near_tc0, "default_sphere_tc": sph_tc0, "default_coarse_tc": coarse_tc0,
            "note": "per profiled mixed solve (serialised CUDA-event times), tcgen05 kernels vs SIMT kernels: the "
                    "FP32 near-field contraction as a TF32 GEMM (k_near_eval_tc), the FP32 sphere operator "
                    "with its Legendre stage as TF32 GEMMs (k_legendre_tc) and the FP32 coarse strengths as "
                    "TF32 GEMMs (k_coarse_src_tc), 3xTF32 split"},
        "autotune": {"fp32_targets_per_thread": tpt.value, "variant_ms_tpt_1_2_4": [round(v, 4) for v in tms],
                     "from_cache": bool(tcache.value),
                     "note": "tile of the FP32 grid kernels, tuned when a context first runs them (here the "
                             "direct-sum arm, coarse sources off); with coarse targets on (the default) the "
                             "FP32 passes run the entry kernel and do not use it"},
        "cpu_baseline": cpu,
        "e2e": {"value": round(world * args.steps / e2e_total, 4), "unit": "solves/s",
                "h2d_bytes_per_step": 8 * n6, "d2h_bytes_per_step": 8 * n6,
                "host_buffers": "pinned" if pinned else "pageable"},
        "gpu_launches": int(round(launches)),
        "host_launch_calls": int(round(host_calls)),
        "loop_graph": loop_graph,
        "clocks": clk.summary(),
    }
    return line


def run_config(args, world, rank, local, dist):
    """cfg3 (1024 spheres, near-singular gaps) and cfg4 (256 uneven independent problems, one
    batched solve) at 1e-8: mixed solves timed; one FP64-accurate reference solve of the same
    operator (float-float far field, FP64 elsewhere) gives the error; the CPU restatement's cost is
    extrapolated from its measured pair rate on cfg2."""
    import ctypes

    from spheresimulator_gb300 import PREC_FLOAT_FLOAT, PREC_FP64, PREC_MIXED, SphereSTKMobMat, configs, solve_opts
    from spheresimulator_gb300 import _native as N

    L = N.lib()
    cfg = getattr(configs, args.config)()
    mob = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg.get("quats"),
                          problem=cfg.get("problem"), device=local)
    h = mob.handle
    P = mob.n_problems
    n6 = 6 * mob.n_spheres
    force = np.ascontiguousarray(cfg["force"])
    d_force, d_vel = ctypes.c_void_p(), ctypes.c_void_p()
    N.check(L.smob_device_alloc(h, 8 * n6, ctypes.byref(d_force)))
    N.check(L.smob_device_alloc(h, 8 * n6, ctypes.byref(d_vel)))
    N.check(L.smob_memcpy_h2d(h, d_force, force.ctypes.data_as(ctypes.c_void_p), 8 * n6))
    stats = (N.ProblemStats * P)()

    def solve(prec):
        o = solve_opts(TOL, RESTART, 2000, prec)
        N.check(L.smob_flush_l2(h, L2_FLUSH_BYTES))
        N.check(L.smob_timer_mark(h))
        N.check(L.smob_solve_mob_device(h, d_force, d_vel, None, ctypes.byref(o), stats))
        t = ctypes.c_double()
        N.check(L.smob_timer_elapsed(h, ctypes.byref(t)))
        v = np.zeros(n6)
        N.check(L.smob_memcpy_d2h(h, v.ctypes.data_as(ctypes.c_void_p), d_vel, 8 * n6))
        return t.value, [s.as_dict() for s in stats], v

    for _ in range(args.warmup):
        solve(PREC_MIXED)
    barrier(dist)
    l0, hc0 = mob.launch_stats()
    ms, sts = [], None
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t, sts, vel = solve(PREC_MIXED)
            ms.append(t)
    l1, hc1 = mob.launch_stats()
    launches = (l1 - l0) / max(args.steps, 1)
    host_calls = (hc1 - hc0) / max(args.steps, 1)
    # one batched solve with the host-driven restart loop, for its launch counts and time
    mob.set_loop_graph(False)
    l0, hc0 = mob.launch_stats()
    t_host, _, _ = solve(PREC_MIXED)
    l1, hc1 = mob.launch_stats()
    mob.set_loop_graph(True)
    loop_graph = {"on": mob.loop_graph_info()[0], "kernels_per_step": round(launches, 1),
                  "host_launch_calls_per_step": round(host_calls, 1),
                  "host_loop": {"ms_per_step": round(t_host, 3), "kernels_per_step": l1 - l0,
                                "host_launch_calls_per_step": hc1 - hc0}}
    ms = np.array(ms)
    total_s = allmax(dist, ms.sum() / 1e3)
    ref_name = {"ff": PREC_FLOAT_FLOAT, "fp64": PREC_FP64}.get(args.ref)
    ref = None
    if ref_name is not None:
        # the reference solve sums every far-field pair directly (no coarse sources in any pass)
        eps32, eps_hp = mob.far_compression_info()[0], mob.far_compression_info(hp=True)[0]
        mob.set_far_compression(0, 0)
        tr, sts_ref, vref = solve(ref_name)
        mob.set_far_compression(eps32, eps_hp)
        err = float(np.linalg.norm(vel - vref) / np.linalg.norm(vref))
        ref = {"precision": args.ref, "far_field": "direct sum", "solve_ms": round(tr, 1),
               "rel_err_mixed_vs_ref": err,
               "iterations_total": int(sum(s["iterations"] for s in sts_ref)),
               "max_relres": max(s["relres"] for s in sts_ref),
               "speedup_mixed_vs_ref": round(tr / ms.mean(), 3)}
    mob.profile(True)
    mob.profile_reset()
    solve(PREC_MIXED)
    prof = mob.profile_table()
    mob.profile(False)
    f32, f64 = ctypes.c_double(), ctypes.c_double()
    N.check(L.smob_measure_fma_peaks(local, ctypes.byref(f32), ctypes.byref(f64)))
    tpt, tms, tcache = ctypes.c_int(), (ctypes.c_double * 3)(), ctypes.c_int()
    N.check(L.smob_tuning(h, ctypes.byref(tpt), tms, ctypes.byref(tcache)))
    if rank != 0:
        return None
    pairs = far_pairs_batched(mob)
    direct, evaluated, coarse_macs = mob.far_pairs()
    k_l, k_ms = prof.get("far_trac_fp32", (0, 0.0))
    avg_s = (k_ms / max(k_l, 1)) / 1e3
    achieved = 30.0 * evaluated / avg_s / 1e12 if avg_s > 0 else None
    c_l, c_ms = prof.get("far_coarse", (0, 0.0))
    eps, cpts, cent = mob.far_compression_info()
    eps_hp, cpts_hp, cent_hp = mob.far_compression_info(hp=True)
    its = [s["iterations"] for s in sts]
    # CPU restatement: pair rate measured on cfg2 (one FP64 operator pass), scaled to this workload
    c2 = configs.cfg2()
    from oracle import oracle as O
    nthreads = args.cpu_threads or os.cpu_count()
    O.set_threads(nthreads)
    op2 = O.Operator(c2["centers"], c2["radii"], c2["orders"])
    x2 = np.random.default_rng(0).standard_normal(3 * op2.m)
    op2.apply(x2)
    t0 = time.perf_counter()
    op2.apply(x2)
    dt2 = time.perf_counter() - t0
    rate = 1336336000 / dt2
    passes = sum(s["iterations"] for s in sts) / P + 4
    cpu_solve_s = passes * (pairs / P) / rate
    value = world * P * args.steps / total_s
    return {
        "metric": METRIC, "value": round(value, 4), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(float(ms.mean()), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 operator + f64 refinement (mixed)",
        "data": "synthetic (seeded RSA packing, N(0,1) forces)",
        "config": {"workload": args.config + ": " + CONFIG_TEXT[args.config], "tol": TOL, "restart": RESTART,
                   "problems_per_step": P, "points": mob.n_points, "near_pairs": mob.n_near_pairs,
                   "l2": "flushed between steps (256 MB device write)", "parallelism": "replicas only"},
        "latency_ms": {"p50": round(float(np.percentile(ms, 50)), 3), "p99": round(float(np.percentile(ms, 99)), 3),
                       "meaning": "time of one batched solve step (all problems of the step)"},
        "mixed": {"iterations_mean": float(np.mean(its)), "iterations_max": int(np.max(its)),
                  "all_converged": all(s["status"] == 0 for s in sts), "max_relres": max(s["relres"] for s in sts)},
        "reference_solve": ref,
        "pair_interactions_per_launch": pairs,
        "far_compression": {"eps": eps, "coarse_points": cpts, "entries": cent, "direct_pairs_per_pass": direct,
                            "evaluated_pairs_per_pass": evaluated,
                            "evaluated_fraction": round(evaluated / direct, 4) if direct else None,
                            "coarse_strength_macs_per_pass": coarse_macs,
                            "coarse_strength_ms_per_pass": round(c_ms / max(c_l, 1), 5),
                            "eps_float_float": eps_hp, "coarse_points_float_float": cpts_hp,
                            "entries_float_float": cent_hp},
        "roofline": {"kernel": "far_trac_fp32", "bound": "fp32_simt", "achieved": round(achieved, 3) if achieved else None,
                     "peak": round(f32.value, 3), "unit": "TFLOP/s",
                     "frac": round(achieved / f32.value, 4) if achieved else None, "traffic": None,
                     "pairs_per_launch": evaluated, "avg_launch_ms": round(avg_s * 1e3, 4)},
        "kernel_ms_profiled_solve": {k: [v[0], round(v[1], 3)] for k, v in sorted(prof.items())},
        "autotune": {"fp32_targets_per_thread": tpt.value, "variant_ms_tpt_1_2_4": [round(v, 4) for v in tms]},
        "cpu_baseline": {"value": round(P / (cpu_solve_s * P), 8) if cpu_solve_s > 0 else None, "unit": "solves/s",
                         "cores": nthreads, "kind": "port",
                         "sample": "extrapolated: FP64 restatement's pair rate on one cfg2 operator pass (%.3f s for "
                                   "1.336e9 pairs) x this workload's pairs per problem (%.3g) x %.1f passes per solve"
                                   % (dt2, pairs / P, passes)},
        "e2e": None,
        "gpu_launches": int(round(launches)),
        "host_launch_calls": int(round(host_calls)),
        "loop_graph": loop_graph,
        "clocks": clk.summary(),
    }


def run_serving(args, world, rank, local, dist):
    """cfg5: Poisson arrivals of independent mobility solves (N log-uniform in [4, nmax], p in
    {8,12,16,24}, a ~ U[0.9,1.1], gap 0.05, tol 1e-6 or 1e-8) submitted in real time to the
    continuous-batching server; latency = completion - submission on the server's clock."""
    import threading as th

    from spheresimulator_gb300 import PREC_FP64, PREC_MIXED, SolveServer, configs, warm_orders
    stream = configs.cfg5_stream(seed=5 + rank, n_requests=args.requests, rate=args.rate, nmax=args.nmax)
    # the server's start-up: the host tables of the orders the stream declares (p in {8, 12, 16, 24})
    warm = sorted({int(p) for r in stream for p in r["orders"]})
    t_warm = time.perf_counter()
    warm_orders(warm)
    t_warm = time.perf_counter() - t_warm

    def serve(reqs, precision, slots, small_sms=0, graphs=None):
        graphs = args.server_graphs if graphs is None else graphs
        srv = SolveServer(device=local, max_slots=slots, precision=precision, hbm_budget_bytes=args.hbm_budget,
                          small_sms=small_sms, graphs=graphs)
        part = srv.partition_info()
        ids = [None] * len(reqs)
        t_start = time.perf_counter()

        def feeder():
            for i, r in enumerate(reqs):
                dt = r["arrival"] - (time.perf_counter() - t_start)
                if dt > 0:
                    time.sleep(dt)
                ids[i] = srv.submit(r["centers"], r["radii"], r["orders"], r["force"], tol=r["tol"])

        f = th.Thread(target=feeder)
        f.start()
        f.join()
        infos = [srv.wait(i)[1] for i in ids]
        st = srv.stats()
        srv.close()
        lat = np.array([x["t_done"] - x["t_submit"] for x in infos])
        span = max(x["t_done"] for x in infos) - min(x["t_submit"] for x in infos)
        ok = all(x["status"] == 0 for x in infos)
        st["partition_sms"] = list(part)
        return lat, span, st, ok, infos

    sizes_all = np.array([len(r["radii"]) for r in stream])

    def buckets(lat):
        out = {}
        for name, lo, hi in (("n<=64", 0, 64), ("64<n<=512", 64, 512), ("n>512", 512, 1 << 30)):
            m = (sizes_all > lo) & (sizes_all <= hi)
            if m.any():
                out[name] = {"requests": int(m.sum()), "p50_ms": round(1e3 * float(np.percentile(lat[m], 50)), 2),
                             "p99_ms": round(1e3 * float(np.percentile(lat[m], 99)), 2)}
        return out

    barrier(dist)
    with ClockSampler(local) as clk:
        lat, span, st, ok, infos = serve(stream, PREC_MIXED, args.slots, args.small_sms)
    total = allmax(dist, span)
    if args.serve_log and rank == 0:
        with open(args.serve_log, "w") as fh:
            for r, x in zip(stream, infos):
                fh.write(json.dumps({"n": len(r["radii"]), "p": int(r["orders"][0]), "tol": r["tol"],
                                     "arrival": round(r["arrival"], 4), "queue_ms": round(1e3 * (x["t_admit"] - x["t_submit"]), 2),
                                     "ctx_ms": round(1e3 * (x["t_ctx"] - x["t_admit"]), 2),
                                     "solve_ms": round(1e3 * (x["t_done"] - x["t_ctx"]), 2),
                                     "iterations": x["stats"]["iterations"], "route": x["route"]}) + "\n")
    # the same stream with the other SM arrangement (a green-context partition, or none), for comparison
    other = None
    if args.compare_partition > 0:
        alt_sms = 0 if args.small_sms > 0 else args.compare_partition
        lat0, span0, st0, ok0, _ = serve(stream, PREC_MIXED, args.slots, alt_sms)
        other = {"small_sms": st0["partition_sms"][0], "big_sms": st0["partition_sms"][1],
                 "solves_per_s": round(len(stream) / span0, 4), "p50_ms": round(1e3 * float(np.percentile(lat0, 50)), 2),
                 "p99_ms": round(1e3 * float(np.percentile(lat0, 99)), 2), "by_size": buckets(lat0), "all_ok": ok0}
    # the small requests (n <= 64) solved one at a time on an idle server: their solo latency
    small = [dict(r, arrival=0.0) for r in stream if len(r["radii"]) <= 64][:8]
    solo = None
    if small:
        sl, sg = [], []
        for r in small:
            l1, _, _, _, _ = serve([r], PREC_MIXED, 1, 0)
            sl.append(float(l1[0]))
            l1, _, _, _, _ = serve([r], PREC_MIXED, 1, 0, graphs=True)
            sg.append(float(l1[0]))
        solo = {"requests": len(small), "p50_ms": round(1e3 * float(np.percentile(sl, 50)), 2),
                "max_ms": round(1e3 * max(sl), 2),
                "with_graphs": {"p50_ms": round(1e3 * float(np.percentile(sg, 50)), 2), "max_ms": round(1e3 * max(sg), 2),
                                "note": "request contexts capture CUDA graphs (each solves once)"}}
    sub = None
    if args.fp64_subset > 0:
        small = [dict(r, arrival=0.0) for r in stream if len(r["radii"]) <= args.fp64_subset]
        if small:
            lm, sm, _, okm, _ = serve(small, PREC_MIXED, args.slots)
            lf, sf, _, okf, _ = serve(small, PREC_FP64, args.slots)
            sub = {"requests": len(small), "max_spheres": args.fp64_subset, "submitted": "all at t=0",
                   "mixed": {"solves_per_s": round(len(small) / sm, 4), "p50_ms": round(1e3 * np.percentile(lm, 50), 2),
                             "p99_ms": round(1e3 * np.percentile(lm, 99), 2), "all_ok": okm},
                   "fp64": {"solves_per_s": round(len(small) / sf, 4), "p50_ms": round(1e3 * np.percentile(lf, 50), 2),
                            "p99_ms": round(1e3 * np.percentile(lf, 99), 2), "all_ok": okf},
                   "speedup_solves_per_s": round(sf / sm, 3)}
    if rank != 0:
        return None
    sizes = [len(r["radii"]) for r in stream]
    value = world * len(stream) / total
    return {
        "metric": METRIC, "value": round(value, 4), "unit": "solves/s", "n_gpus": world, "steps": len(stream),
        "warmup": 0, "ms_per_step": round(1e3 * total / len(stream), 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 operator + f64 refinement (mixed)",
        "data": "synthetic (seeded RSA packings, N(0,1) forces, Poisson arrivals)",
        "config": {"workload": "cfg5: served stream, %d requests, Poisson rate %.2f/s, N log-uniform [4,%d], "
                               "p in {8,12,16,24}, a~U[0.9,1.1], gap 0.05, tol 1e-6/1e-8" % (len(stream), args.rate, args.nmax),
                   "slots": args.slots, "parallelism": "replicas only",
                   "l2": "not flushed: requests arrive in real time, latency measured on the server clock",
                   "server_start": "per-order host tables of p in %s built before the stream (smob_warm_orders, "
                                   "%.2f s)" % (warm, t_warm)},
        "latency_ms": {"p50": round(1e3 * float(np.percentile(lat, 50)), 2),
                       "p99": round(1e3 * float(np.percentile(lat, 99)), 2)},
        "latency_by_size": buckets(lat),
        "small_requests_solo": solo,
        "sm_partition": {"small_sms": st["partition_sms"][0], "big_sms": st["partition_sms"][1],
                         "note": "0/0: no partition, stream priorities by size only; otherwise green contexts: "
                                 "requests with < 1e9 far-field pairs run on the small partition while a big "
                                 "request runs (on the whole device otherwise), big requests on the rest"},
        "other_sm_arrangement": other,
        "queue_wait_ms_p50": round(1e3 * float(np.percentile([x["t_admit"] - x["t_submit"] for x in infos], 50)), 2),
        "all_converged": ok, "span_s": round(total, 3),
        "requests": {"spheres_min": int(min(sizes)), "spheres_max": int(max(sizes)), "spheres_median": float(np.median(sizes))},
        "server": {"peak_running": st["peak_running"], "peak_bytes": st["peak_bytes"], "budget_bytes": st["budget_bytes"]},
        "small_request_subset_vs_fp64": sub,
        "e2e": None, "clocks": clk.summary(),
    }


CONFIG_TEXT = {
    "cfg3": "1024 spheres a~U[0.8,1.2], RSA in box 40 (min gap 0.05), p=16, mixed FP32/FP64 to 1e-8",
    "cfg4": "256 independent problems, N~U{2..128}, p~U{8,12,16}, a=1, box 4N^(1/3), gap 0.1, one batched solve",
}


def far_pairs_batched(mob):
    ng = np.array([(p + 1) * (2 * p + 2) for p in mob.orders], dtype=np.int64)
    prob = mob.problem if mob.problem is not None else np.zeros(len(ng), np.int64)
    pairs = 0
    for k in np.unique(prob):
        g = ng[prob == k]
        pairs += g.sum() ** 2 - (g * g).sum()
    t, s = mob.near_pairs()
    pairs -= (ng[t] * ng[s]).sum()
    return int(pairs)


def cpu_sample(cfg, threads):
    """One full FP64 mobility solve of the workload by the C++/OpenMP restatement (timed, host clock)."""
    from oracle import oracle as O
    nthreads = threads or os.cpu_count()
    O.set_threads(nthreads)
    op = O.Operator(cfg["centers"], cfg["radii"], cfg["orders"])
    t0 = time.perf_counter()
    r = op.solve_mob(cfg["force"], tol=TOL, restart=RESTART, maxit=1000)
    dt = time.perf_counter() - t0
    return {"value": round(1.0 / dt, 6), "unit": "solves/s", "cores": nthreads, "kind": "port",
            "sample": "one full FP64 mobility solve of the cfg2 workload to 1e-8 (%d GMRES iterations) timed = "
                      "%.3f s; direct-sum far field (the reference's STKFMM path is O(M))" % (r["iters"], dt)}


def run_reference(args, rank):
    """The reference path's CPU counterpart (the reference itself cannot be built: its SCTL, STKFMM and
    Trilinos dependencies are absent): each step is one full FP64 mobility solve of the cfg2 workload by
    the C++/OpenMP restatement on all host cores (direct-sum far field, spectral self and near
    corrections, restarted GMRES(50) to 1e-8), timed on the host clock."""
    if rank != 0:
        return None
    from oracle import oracle as O
    from spheresimulator_gb300 import configs
    nthreads = args.cpu_threads or os.cpu_count()
    O.set_threads(nthreads)
    cfg = configs.cfg2()
    op = O.Operator(cfg["centers"], cfg["radii"], cfg["orders"])
    r = None
    for _ in range(max(1, args.warmup)):
        r = op.solve_mob(cfg["force"], tol=TOL, restart=RESTART, maxit=1000)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = op.solve_mob(cfg["force"], tol=TOL, restart=RESTART, maxit=1000)
        ts.append(time.perf_counter() - t0)
    ts = np.array(ts)
    value = args.steps / ts.sum()
    sample = ("per step: one full FP64 mobility solve of the cfg2 workload (%d GMRES iterations to relres %.2e, "
              "direct-sum far field of 1.336e9 pairs per operator pass) by the C++/OpenMP restatement on %d "
              "threads; the reference evaluates that far field with STKFMM (O(M)), the restatement sums it "
              "directly (O(M^2))" % (r["iters"], r["relres"], nthreads))
    cpu = {"value": round(value, 6), "unit": "solves/s", "cores": nthreads, "kind": "port", "sample": sample}
    return {"metric": METRIC, "value": round(value, 6), "unit": "solves/s", "impl": "reference",
            "n_gpus": args.gpus, "cpu_threads": nthreads,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(float(ts.mean() * 1e3), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded RSA packing, N(0,1) forces)",
            "config": {"workload": WORKLOAD, "tol": TOL, "restart": RESTART, "precision": "fp64"},
            "latency_ms": {"p50": round(float(np.percentile(ts, 50) * 1e3), 3),
                           "p99": round(float(np.percentile(ts, 99) * 1e3), 3)},
            "cpu_baseline": cpu, "e2e": {"value": round(value, 6), "unit": "solves/s", "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0},
            "oracle_solve": {"iterations": r["iters"], "relres": r["relres"]}}


def run_multi(args, world, rank, local, dist):
    """Several right-hand sides on the cfg2 geometry (the columns SphereSTKMobMat::apply solves one
    by one): K columns in one smob_solve_mob_multi call against K smob_solve_mob calls, host buffers
    in and out (both timed end to end on the host clock; the calls are synchronous)."""
    from spheresimulator_gb300 import PREC_MIXED, SphereSTKMobMat, configs
    cfg = configs.cfg2()
    mob = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], device=local)
    k = args.multi
    F = np.random.default_rng(7).standard_normal((k, 6 * mob.n_spheres))
    kw = dict(tol=TOL, restart=RESTART, max_iters=1000, precision=PREC_MIXED)
    auto_tile = mob.tuning()[0]
    mob.set_multi_shared_pairs(False)

    def singles():
        return np.stack([mob.solveMob(F[j], **kw) for j in range(k)])

    for _ in range(max(1, args.warmup)):
        mob.solveMobMulti(F, **kw)
        singles()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vm = mob.solveMobMulti(F, **kw)
    t_multi = allmax(dist, time.perf_counter() - t0)
    its = [s["iterations"] for s in mob.last_stats]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vs = singles()
    t_single = allmax(dist, time.perf_counter() - t0)
    # the columns as a batch of copies (the default) are each their single solve, bit for bit
    bitwise = bool(np.array_equal(vm, vs))
    # the shared-pair kernels (each grid-point pair once for all columns) for comparison
    mob.set_multi_shared_pairs(True)
    mob.solveMobMulti(F, **kw)
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps // 2)):
        mob.solveMobMulti(F, **kw)
    t_shared = (time.perf_counter() - t0) / max(1, args.steps // 2)
    mob.set_multi_shared_pairs(False)
    err = float(np.linalg.norm(vm - vs) / np.linalg.norm(vs))
    if rank != 0:
        return None
    return {"metric": "mobility solves/s, K right-hand sides on one geometry (cfg2, mixed, 1e-8)",
            "value": round(world * k * args.steps / t_multi, 4), "unit": "columns/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "dtype": "f32 operator + f64 refinement (mixed)", "data": "synthetic (cfg2 geometry, N(0,1) columns)",
            "config": {"workload": WORKLOAD, "columns": k, "timing": "host clock around synchronous host-buffer calls"},
            "ms_per_step": round(1e3 * t_multi / args.steps, 3),
            "single_solves": {"columns_per_s": round(world * k * args.steps / t_single, 4),
                              "ms_per_k_columns": round(1e3 * t_single / args.steps, 3), "far_tile": auto_tile},
            "speedup_vs_single_solves": round(t_single / t_multi, 3),
            "iterations_per_column": its, "rel_diff_vs_single_solves": err,
            "bitwise_equal_to_single_solves": bitwise,
            "bitwise_note": "the columns are solved as a batch of copies of the problem with the single solves' "
                            "own settings and kernels",
            "shared_pair_kernels": {"columns_per_s": round(world * k / t_shared, 4),
                                    "note": "smob_set_multi_shared_pairs: each grid-point pair once for all "
                                            "columns (grid targets, every float-float pair)"}}


def contact_forces(centers, n_contacts, n_solves, seed):
    """Forces of a collision solver's iterations on one configuration: F = D gamma, the columns of D
    equal and opposite unit forces along the centre line of the n_contacts closest sphere pairs
    (the constraint directions of SphereSystem::resolveCollision), gamma >= 0 new every iteration."""
    c = np.asarray(centers)
    n = len(c)
    d = np.linalg.norm(c[:, None] - c[None], axis=-1) + np.eye(n) * 1e9
    pairs = sorted((d[i, j], i, j) for i in range(n) for j in range(i + 1, n))[:n_contacts]
    D = np.zeros((6 * n, len(pairs)))
    for k, (_, i, j) in enumerate(pairs):
        e = (c[j] - c[i]) / np.linalg.norm(c[j] - c[i])
        D[6 * i:6 * i + 3, k] = -e
        D[6 * j:6 * j + 3, k] = e
    g = np.random.default_rng(seed).uniform(0.0, 1.0, (n_solves, len(pairs)))
    return [D @ gk for gk in g]


def run_sequence(args, world, rank, local, dist):
    """A sequence of mobility solves on the cfg2 geometry, as the collision solver issues them: forces
    F = D gamma on --contacts contact directions with new gamma every solve (or, with --contacts 0,
    forces drifting by --drift per solve). Three initial guesses: zero; the reference's previous
    solution (xLast, BIE/SphereSTKMobMat.cpp:222); recycled solutions (warm_start "recycle"). Host
    buffers in and out, host clock around synchronous calls."""
    from spheresimulator_gb300 import PREC_MIXED, SphereSTKMobMat, configs
    cfg = configs.cfg2()
    k = args.sequence
    rng = np.random.default_rng(11)
    if args.contacts > 0:
        F = contact_forces(cfg["centers"], args.contacts, k, seed=11)
        model = "F = D gamma: %d contact directions (closest sphere pairs), gamma ~ U(0,1) new per solve" % \
            args.contacts
    else:
        F = [cfg["force"]]
        for _ in range(k - 1):
            f = F[-1]
            F.append(f + args.drift * np.linalg.norm(f) / np.sqrt(f.size) * rng.standard_normal(f.shape))
        model = "force k+1 = force k + %g |F|/sqrt(6N) N(0,1) per component" % args.drift
    kw = dict(tol=TOL, restart=RESTART, max_iters=1000, precision=PREC_MIXED)
    arms = {}
    for name in ("cold", "last", "recycle"):
        mob = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], device=local)
        for _ in range(max(1, args.warmup)):
            mob.solveMob(rng.standard_normal(F[0].shape), **kw)
        mob.recycle_clear()
        vel, its = [], []
        barrier(dist)
        t0 = time.perf_counter()
        for j in range(k):
            ws = {"cold": False, "last": j > 0, "recycle": "recycle"}[name]
            vel.append(mob.solveMob(F[j], warm_start=ws, **kw))
            its.append(mob.last_stats[0]["iterations"])
        t = allmax(dist, time.perf_counter() - t0)
        arms[name] = {"solves_per_s": round(world * k / t, 4), "ms_per_solve": round(1e3 * t / k, 3),
                      "iterations": its, "vel": vel}
    err = max(float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(arms["recycle"]["vel"],
                                                                                arms["cold"]["vel"]))
    for a in arms.values():
        a.pop("vel")
    if rank != 0:
        return None
    return {"metric": "mobility solves/s, a sequence of collision-solver forces on one geometry (cfg2, mixed, 1e-8)",
            "value": arms["recycle"]["solves_per_s"], "unit": "solves/s", "n_gpus": world, "steps": k,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "dtype": "f32 operator + f64 refinement (mixed)",
            "data": "synthetic (cfg2 geometry; %s)" % model,
            "config": {"workload": WORKLOAD, "solves": k, "forces": model,
                       "timing": "host clock around synchronous host-buffer calls"},
            "ms_per_step": arms["recycle"]["ms_per_solve"], "arms": arms,
            "speedup_vs_previous_solution_warm_start": round(arms["last"]["ms_per_solve"] /
                                                             arms["recycle"]["ms_per_solve"], 3),
            "speedup_vs_cold": round(arms["cold"]["ms_per_solve"] / arms["recycle"]["ms_per_solve"], 3),
            "max_rel_diff_recycle_vs_cold": err}


def far_once():
    """One far-field pass of each kernel family on the cfg2 workload, with few launches before them."""
    from spheresimulator_gb300 import PREC_FLOAT_FLOAT, PREC_FP64, PREC_MIXED, SphereSTKSHOperator, configs
    c = configs.cfg2()
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"])
    x = np.random.default_rng(0).standard_normal(3 * g.n_points)
    a = g.far_field(x, cTrac=1.0, precision=PREC_MIXED)
    b = g.far_field(x, cSL=1.0, cTrac=1.0, precision=PREC_FLOAT_FLOAT)
    d = g.far_field(x, cTrac=1.0, precision=PREC_FP64)
    print(json.dumps({"far_once": "cfg2", "points": int(g.n_points), "finite": bool(np.isfinite(a).all() and
                      np.isfinite(b).all() and np.isfinite(d).all())}))


def solve_once(host_loop=False):
    """Three mixed-precision cfg2 solves (the first captures the graphs), for a kernel launch list.
    host_loop: the host-driven restart loop (the same kernels; ncu lists no kernel that runs inside a
    conditional graph node's body, so a launch list of the loop's kernels needs this)."""
    from spheresimulator_gb300 import PREC_MIXED, SphereSTKMobMat, configs
    c = configs.cfg2()
    mob = SphereSTKMobMat(c["centers"], c["radii"], c["orders"])
    if host_loop:
        mob.set_loop_graph(False)
    for _ in range(3):
        v = mob.solveMob(c["force"], tol=TOL, restart=RESTART, max_iters=1000, precision=PREC_MIXED)
    print(json.dumps({"solve_once": "cfg2", "iterations": mob.last_stats[0]["iterations"],
                      "relres": mob.last_stats[0]["relres"], "finite": bool(np.isfinite(v).all())}))


def near_once():
    """One near-field pass (FP32 traction on the tensor cores, FP64 traction, FP32 traction on the SIMT
    pipes, then with the sphere operator's Legendre stage on the tensor cores) on the first 64 problems
    of cfg4: the batched shape, where every target point has near pairs."""
    from spheresimulator_gb300 import PREC_FP64, PREC_MIXED, SphereSTKSHOperator, configs
    c = configs.cfg4(n_problems=64)
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"], problem=c["problem"])
    x = np.random.default_rng(0).standard_normal(3 * g.n_points)
    a = g.near_field(x, cTrac=1.0, precision=PREC_MIXED)
    b = g.near_field(x, cTrac=1.0, precision=PREC_FP64)
    g.set_near_tc(False)
    g.set_sphere_tc(False)
    c = g.near_field(x, cTrac=1.0, precision=PREC_MIXED)  # the SIMT kernels, for the launch list
    g.set_sphere_tc(True)
    d = g.near_field(x, cTrac=1.0, precision=PREC_MIXED)  # the sphere operator with k_legendre_tc
    print(json.dumps({"near_once": "cfg4[:64]", "points": int(g.n_points), "near_pairs": int(g.n_near_pairs),
                      "rel_diff_fp32_fp64": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                      "rel_diff_simt_fp64": float(np.linalg.norm(c - b) / np.linalg.norm(b)),
                      "rel_diff_legendre_tc_fp64": float(np.linalg.norm(d - b) / np.linalg.norm(b))}))


def coarse_once():
    """One FP32 far-field pass with the coarse strengths on the tensor cores, then one with the SIMT
    GEMM, on the first 64 problems of cfg4 (the batched shape, many spheres per coarse map)."""
    from spheresimulator_gb300 import PREC_FP64, PREC_MIXED, SphereSTKSHOperator, configs
    c = configs.cfg4(n_problems=64)
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"], problem=c["problem"])
    x = np.random.default_rng(0).standard_normal(3 * g.n_points)
    g.set_coarse_tc(True)
    a = g.far_field(x, cSL=0.0, cTrac=1.0, precision=PREC_MIXED)
    g.set_coarse_tc(False)
    b = g.far_field(x, cSL=0.0, cTrac=1.0, precision=PREC_MIXED)
    print(json.dumps({"coarse_once": "cfg4[:64]", "points": int(g.n_points),
                      "coarse_points": int(g.far_compression_info()[1]),
                      "rel_diff_tc_simt": float(np.linalg.norm(a - b) / np.linalg.norm(b))}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=8)
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--config", default="cfg2", choices=["cfg2", "cfg3", "cfg4", "cfg5"])
    ap.add_argument("--ref", default="ff", choices=["ff", "fp64", "none"],
                    help="cfg3/cfg4: reference solve for the error (ff = FP64-accurate float-float far field)")
    ap.add_argument("--requests", type=int, default=32, help="cfg5: requests in the stream")
    ap.add_argument("--rate", type=float, default=2.0, help="cfg5: Poisson arrival rate (requests/s)")
    ap.add_argument("--nmax", type=int, default=2048, help="cfg5: largest sphere count of a request")
    ap.add_argument("--slots", type=int, default=8, help="cfg5: requests on the GPU at once")
    ap.add_argument("--hbm-budget", type=float, default=0.0, help="cfg5: admission budget in bytes (0: 64 GB)")
    ap.add_argument("--small-sms", type=int, default=0,
                    help="cfg5: SMs reserved (green context) for small requests while big ones run (0: none, "
                         "stream priorities by size only)")
    ap.add_argument("--serve-log", default="",
                    help="cfg5: write one JSON line per request (size, queue and run times) to this file")
    ap.add_argument("--server-graphs", type=int, default=0, choices=[0, 1, 2],
                    help="cfg5: CUDA graphs in request contexts: 0 none (eager launches, the default: "
                         "the lowest small-request latency), 1 all, 2 big requests")
    ap.add_argument("--compare-partition", type=int, default=0, metavar="SMS",
                    help="cfg5: also serve the stream with this many SMs reserved for small requests (without a "
                         "partition when --small-sms is set)")
    ap.add_argument("--fp64-subset", type=int, default=0,
                    help="cfg5: also serve the requests with at most this many spheres in mixed and plain FP64")
    ap.add_argument("--multi", type=int, default=0,
                    help="cfg2: solve this many right-hand sides together (smob_solve_mob_multi) against as "
                         "many single solves, and print that line instead of the headline")
    ap.add_argument("--sequence", type=int, default=0,
                    help="cfg2: a sequence of this many solves with drifting forces, zero / previous-solution / "
                         "recycled initial guesses; print that line instead of the headline")
    ap.add_argument("--contacts", type=int, default=12,
                    help="--sequence: contact directions spanning the forces (0: drifting forces instead)")
    ap.add_argument("--drift", type=float, default=0.05,
                    help="--sequence --contacts 0: relative force change per solve")
    ap.add_argument("--far-once", action="store_true",
                    help="cfg2: one far-field pass per kernel family (FP32 traction, fused float-float "
                         "traction + single layer, FP64 traction) and exit; a short program for ncu captures")
    ap.add_argument("--coarse-once", action="store_true",
                    help="one FP32 far-field pass with tensor-core and with SIMT coarse strengths (for ncu)")
    ap.add_argument("--host-loop", action="store_true",
                    help="with --solve-once: the host-driven restart loop instead of the loop graph")
    ap.add_argument("--solve-once", action="store_true",
                    help="three mixed cfg2 solves and exit; a short program for a kernel launch list")
    ap.add_argument("--near-once", action="store_true",
                    help="one near-field pass (FP32, FP64) on 64 problems of cfg4 and exit; a short program for ncu")
    args = ap.parse_args()
    if args.far_once:
        far_once()
        return
    if args.near_once:
        near_once()
        return
    if args.solve_once:
        solve_once(args.host_loop)
        return
    if args.coarse_once:
        coarse_once()
        return
    if args.warmup < 3 and args.impl == "native":
        args.warmup = 3
    world, rank, local, dist = dist_init()
    if args.impl == "reference":
        line = run_reference(args, rank)
    elif args.multi > 0:
        line = run_multi(args, world, rank, local, dist)
    elif args.sequence > 0:
        line = run_sequence(args, world, rank, local, dist)
    elif args.config == "cfg5":
        line = run_serving(args, world, rank, local, dist)
    elif args.config != "cfg2":
        line = run_config(args, world, rank, local, dist)
    else:
        line = run_native(args, world, rank, local, dist)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
