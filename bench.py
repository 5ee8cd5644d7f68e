"""Benchmark: converged DIVA velocity solves per second on the MISMIP+-shaped channel.

Workload (one step): a DIVA velocity solve from a cold start (u = 0) on the channel of
geometry.channel_case -- 640 km x 80 km, ~58k vertices, ~115k triangles, nz = 12, Schoof2005
friction, Picard to 1e-4 (calc_L2_norm_uv), BiCGStab/Jacobi to 1e-8 / 1e-5 (rtol / abstol).
Synthetic data: the geometry is generated from formulas, not read from files.

Arms
  ours (default)   the GB300 library.  `value` = solves/s of the headline path with inputs
                   resident in HBM, timed by CUDA events on the library's stream; `e2e` = the same
                   through ufe_solve_diva with host buffers (pinned), H2D and D2H inside the timed
                   region.  Three Krylov precisions are measured, each from the plain (zero)
                   start and from the learned Picard start: FP64; double-word (pairs of FP32
                   numbers, FP32 pipe); FP32 with FP64 refinement.  The headline is the fastest
                   learned-start path.  L2 is flushed (256 MB write) before every timed solve.
  reference        the CPU restatement of the reference's algorithm (oracle/, OpenMP on all host
                   cores) timed on a bounded sample of the same workload (the first Picard
                   iterations of the solve) and scaled to full solves by Krylov iteration count.

Multi-GPU (`--gpus N` under torchrun): replicas -- every rank solves its own copy; value is the
solves of all ranks over the slowest rank's time.

`--workload thermo` measures the batched column thermodynamics instead (200k vertices x 30 layers,
100 steps of 10 yr per run; column-steps/s), with the same arms.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402

METRIC = "converged SSA/DIVA velocity solves/s, learned+FP32 vs plain FP64, 1xGB300"
# channel variants the learned start trains on: (thickness [m], flow factor), each on its own mesh
CHANNEL_VARIANTS = [(210.0, 1.5e-17), (230.0, 2.5e-17), (270.0, 1.5e-17), (290.0, 2.5e-17),
                    (220.0, 3e-17), (240.0, 1.2e-17), (260.0, 3e-17), (280.0, 1.2e-17)]
LEARNED_SMOOTH = 8
LEARNED_VISC_PATHS = ("fp64", "fp32_pair", "fp32_pair_inexact")   # learned paths also run with the predicted viscosity
UNIT = "solves/s"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def pinned_like(torch, a):
    """A numpy view of pinned host memory holding a copy of `a` (same memory order)."""
    t = torch.empty(a.size, dtype=torch.float64 if a.dtype == np.float64 else torch.int32).pin_memory()
    v = t.numpy()
    if a.ndim == 2:
        v = v.reshape(a.shape[::-1]).T     # Fortran order view
    else:
        v = v.reshape(a.shape)
    v[...] = a
    return v, t


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkg = __graft_entry__.load_package()
    pkg.build()
    mesh, ice, params = pkg.geometry.channel_case(seed=0)
    params = _with(pkg, params, visc_it_nit=args.picard_nit)
    # the Krylov precisions, and the double-word mode with the two-phase inexact Picard iteration
    # (linear solves to krylov_forcing x their initial residual until the change norm first meets the
    # tolerance, then to the full tolerance until it meets it again)
    prec = {"fp64": _with(pkg, params, precision=pkg.abi.PREC_FP64),
            "fp32_pair": _with(pkg, params, precision=pkg.abi.PREC_FP32_PAIR),
            "fp32_refined": _with(pkg, params, precision=pkg.abi.PREC_FP32_REFINE),
            "fp32_pair_inexact": _with(pkg, params, precision=pkg.abi.PREC_FP32_PAIR, krylov_forcing=args.forcing)}
    steps_of = {"fp64": args.steps, "fp32_pair": args.steps, "fp32_refined": args.mixed_steps,
                "fp32_pair_inexact": args.steps}
    solver = pkg.VelocitySolver(mesh, device=local)
    solver.ice_upload(ice)
    stream = torch.cuda.ExternalStream(solver.stream_handle())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def l2_flush():
        with torch.cuda.stream(stream):
            flush.zero_()

    def slowest(t):
        if world > 1:
            tt = torch.tensor([t], device=f"cuda:{local}", dtype=torch.float64)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t = float(tt.item())
        return t

    def timed(fn, n, tag):
        """n solves, L2 flushed before each; the CUDA-event device time of every solve."""
        out = []
        barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            torch.cuda.nvtx.range_push(tag)
            for _ in range(n):
                l2_flush()
                out.append(fn())
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
            wall = time.perf_counter() - t0
        barrier()
        rate = world * len(out) / slowest(sum(st["device_ms"] for st in out) / 1000.0) if out else None
        return out, rate, clk, wall

    def solve(p):
        return solver.solve_resident(p, diva=True, cold_start=True)

    def kernels(sts, extra=0):
        # counted from the solve graph's kernel nodes; where a Picard iteration holds a Krylov loop
        # of three kernels per iteration the count follows that loop
        return sum((st["n_kernels"] + extra) if st["n_kernels"] >= 0 else 1 + 3 * st["n_visc_its"] + 3 * st["n_Axb_its"]
                   for st in sts)

    def summary(sts, rate, u_ref=None, u=None):
        d = {"value": round(rate, 4) if rate else None, "unit": UNIT,
             "picard_its": sts[0]["n_visc_its"] if sts else None, "krylov_its": sts[0]["n_Axb_its"] if sts else None,
             "fp64_its": sts[0]["n_fp64_its"] if sts else None, "pair_its": sts[0]["n_pair_its"] if sts else None,
             "ms_per_solve": round(sum(st["device_ms"] for st in sts) / len(sts), 3) if sts else None}
        if sts and sts[0]["n_refinements"]:
            d["refinements"] = sts[0]["n_refinements"]
        if u_ref is not None:
            d["rel_l2_vs_plain_fp64"] = round(float(np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)), 9)
        return d

    # warm-up: graph capture of every path
    for _ in range(args.warmup):
        solve(prec["fp64"])
    for name in prec:
        solve(prec[name])
    plain, plain_runs = {}, {}
    for name in prec:
        plain_runs[name] = timed(lambda: solve(prec[name]), steps_of[name], f"timed_plain_{name}")
    u_plain = {}
    for name in prec:
        solve(prec[name])
        u_plain[name] = np.r_[solver.velocity_download()]
    for name in prec:
        sts, rate, _, _ = plain_runs[name]
        plain[name] = summary(sts, rate, u_plain["fp64"] if name != "fp64" else None, u_plain[name])
        plain[name]["us_per_krylov_it_in_solve"] = round(1000.0 * plain[name]["ms_per_solve"]
                                                         / max(plain[name]["krylov_its"], 1), 2)
    value64 = plain_runs["fp64"][1]

    # ---- the FP64 reference solution for the velocity errors: the GPU FP64 path with Krylov to
    # rtol 1e-12, run to the tightest Picard tolerance that the reference's divergence control
    # (SSA_main.f90:196-213, DIVA_main.f90:211-228) lets finish on this channel
    F64 = pkg.abi.PREC_FP64
    ref_info, u_ref, tried = None, None, []
    for tol in args.ref_tols:
        p_ref = _with(pkg, params, precision=F64, stress_balance_PETSc_rtol=1e-12, stress_balance_PETSc_abstol=0.0,
                      visc_it_norm_dUV_tol=tol, visc_it_nit=1000)
        try:
            st = solver.solve_resident(p_ref, diva=True, cold_start=True)
        except pkg.UfeError as e:
            tried.append({"picard_tol": tol, "status": e.code})
            continue
        tried.append({"picard_tol": tol, "status": st["status"]})
        if st["status"] == 0:
            u_ref = np.r_[solver.velocity_download()]
            ref_info = {"picard_tol": tol, "krylov_rtol": 1e-12, "picard_its": st["n_visc_its"],
                        "krylov_its": st["n_Axb_its"], "relax_applied": round(st["visc_it_relax_applied"], 4),
                        "ms": round(st["device_ms"], 1), "tried": tried}
            break

    def err_ref(u):
        return None if u_ref is None else float("%.3g" % (np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)))

    # the persistent Krylov kernels of the FP64 and double-word solves, per iteration; the
    # three-kernel FP64 iteration beside them.  Algorithmic bytes of one iteration: two 2x2-block
    # SpMVs (blocks and columns, row pointers, the source vector and the result) and the vector
    # traffic of the recurrence, 15 streams of (u, v) pairs (r, r^, p, v, s, t, x, D^-1: reads and
    # writes); a double-word value takes the 8 bytes of an FP64 one.
    solve(prec["fp64"])
    us64, (nb, nnzb) = solver.profile_krylov_kernels(pkg.abi.PREC_FP64, repeats=50)
    bytes64 = nnzb * (32 + 4) + (nb + 1) * 4 + nb * 7 * 16
    bytes_it = 2 * (nnzb * 36 + (nb + 1) * 4 + 2 * 16 * nb) + 15 * 16 * nb
    us_it = {}
    for name in ("fp64", "fp32_pair"):
        solve(prec[name])
        try:
            us_it[name] = solver.profile_krylov_persistent(prec[name].precision, 200)
        except pkg.UfeError:
            us_it[name] = None
    peaks, peak_kind = measured_peaks()
    traffic = {}
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f)
    except OSError:
        pass

    # end to end through ufe_solve_diva with pinned host buffers (plain FP64)
    keep = []
    ice_h = {}
    for k, v in ice.items():
        if isinstance(v, np.ndarray) and k in ("Hi", "Hs", "A_flow", "fraction_gr_b", "mask_grounded_ice", "beta_sq",
                                               "alpha_sq", "effective_pressure"):
            ice_h[k], t = pinned_like(torch, v)
            keep.append(t)
    state0 = pkg.new_diva_state(mesh.nTri, mesh.nz)
    st_h = {}
    for k, v in state0.items():
        st_h[k], t = pinned_like(torch, v)
        keep.append(t)
    h2d = sum(v.nbytes for v in ice_h.values()) + sum(st_h[k].nbytes for k in st_h if not k.endswith("3D_b")
                                                      or k == "eta_3D_b")
    d2h = sum(v.nbytes for v in st_h.values())
    solver.solve_DIVA(ice_h, st_h, prec["fp64"])  # warm
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for k in st_h:
            st_h[k][...] = 0.0
        solver.solve_DIVA(ice_h, st_h, prec["fp64"])
    torch.cuda.synchronize()
    e2e_plain = world * args.steps / slowest(time.perf_counter() - t0)

    # ---- learned start: trained on channel variants (own meshes, thickness and flow factor
    # perturbed around the benchmark's), outside the timed region
    learned, learned_runs = None, {}
    if args.learned_variants > 0:
        net = pkg.LearnedStart(solver, seed=1)
        gen_ms, t_gen = 0.0, time.perf_counter()
        for sd, (h, a) in enumerate(CHANNEL_VARIANTS[:args.learned_variants], start=1):
            m_v, ice_v, p_v = pkg.geometry.channel_case(seed=sd, H=h, A=a)
            with pkg.VelocitySolver(m_v, device=local) as sv:
                sv.ice_upload(ice_v)
                x = net.features(sv)
                gen_ms += sv.solve_resident(p_v, diva=True, cold_start=True)["device_ms"]
                net.dataset_add(sv, x)
        gen_wall = time.perf_counter() - t_gen
        losses, train_ms = net.train(epochs=60, lr=2e-3)
        net.dataset_clear()
        solver.ice_upload(ice)
        predict_kernels = int(solver.lib.ufe_gnn_predict_kernels(LEARNED_SMOOTH))

        def learned_solve(p, visc=False):
            ms = net.predict(solver, smooth_passes=LEARNED_SMOOTH, viscosity=visc)
            st = dict(solver.solve_resident(p, diva=True, cold_start=False))
            st["device_ms"] += ms
            return st

        learned = {}
        for name in prec:
            learned_solve(prec[name])     # warm (graph capture of the warm-start path)
            learned_runs[name] = timed(lambda: learned_solve(prec[name]), steps_of[name], f"timed_learned_{name}")
            u = np.r_[solver.velocity_download()]
            sts, rate, _, _ = learned_runs[name]
            learned[name] = summary(sts, rate, u_plain["fp64"], u)
            learned[name]["rel_l2_vs_fp64_reference"] = err_ref(u)
            learned[name]["us_per_krylov_it_in_solve"] = round(1000.0 * learned[name]["ms_per_solve"]
                                                               / max(learned[name]["krylov_its"], 1), 2)
        # the same with the predicted viscosity in the first Picard iteration (every layer a
        # depth-uniform viscosity) in place of Glen's law on the predicted velocity
        for name in LEARNED_VISC_PATHS:
            key = f"visc_{name}"
            learned_solve(prec[name], True)
            learned_runs[key] = timed(lambda: learned_solve(prec[name], True), steps_of[name], f"timed_learned_{key}")
            u = np.r_[solver.velocity_download()]
            sts, rate, _, _ = learned_runs[key]
            learned[key] = summary(sts, rate, u_plain["fp64"], u)
            learned[key]["rel_l2_vs_fp64_reference"] = err_ref(u)
        # the headline's rule: the fastest learned path with FP32 Krylov arithmetic
        lkeys = [k for k in prec if k != "fp64"] + [f"visc_{k}" for k in LEARNED_VISC_PATHS if k != "fp64"]
        best_key = max(lkeys, key=lambda k: learned[k]["value"] or 0.0)
        best_visc = best_key.startswith("visc_")
        best = best_key[len("visc_"):] if best_visc else best_key
        # end to end through the public C ABI with pinned host buffers: ice upload, prediction,
        # resident solve, velocity download -- every step
        solver.ice_upload(ice_h)
        learned_solve(prec[best], best_visc)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            solver.ice_upload(ice_h)
            learned_solve(prec[best], best_visc)
            solver.velocity_download()
        torch.cuda.synchronize()
        t_e2e_l = slowest(time.perf_counter() - t0)
        # the accuracy target at the tight tolerance: plain FP64 (zero start) against learned start +
        # double-word Krylov, both run to the reference solution's Picard tolerance with the
        # benchmark's Krylov tolerance; one solve each after a warm-up
        if ref_info is not None:
            solver.ice_upload(ice)
            tight = {}
            for tag, pname, learned_start in (("plain_fp64", "fp64", False), ("learned_fp32_pair", "fp32_pair", True),
                                              ("learned_fp32_pair_inexact", "fp32_pair_inexact", True)):
                p_t = _with(pkg, prec[pname], visc_it_norm_dUV_tol=ref_info["picard_tol"], visc_it_nit=1000)
                run_t = (lambda: learned_solve(p_t)) if learned_start else (lambda: solve(p_t))
                try:
                    run_t()
                    sts_t, rate_t, _, _ = timed(run_t, 1, f"timed_tight_{tag}")
                    u_t = np.r_[solver.velocity_download()]
                    tight[tag] = {"value": round(rate_t, 4), "unit": UNIT, "picard_its": sts_t[0]["n_visc_its"],
                                  "krylov_its": sts_t[0]["n_Axb_its"], "status": sts_t[0]["status"],
                                  "rel_l2_vs_fp64_reference": err_ref(u_t), "_u": u_t}
                except pkg.UfeError as e:
                    tight[tag] = {"status": e.code}
            if "_u" in tight.get("plain_fp64", {}):
                a = tight["plain_fp64"]["_u"]
                for k in ("learned_fp32_pair", "learned_fp32_pair_inexact"):
                    if "_u" in tight.get(k, {}):
                        b = tight[k]["_u"]
                        tight[k]["rel_l2_vs_plain_fp64"] = float("%.3g" % (np.linalg.norm(b - a) / np.linalg.norm(a)))
                        tight[k]["speedup_vs_plain_fp64"] = round(tight[k]["value"] / tight["plain_fp64"]["value"], 3)
            for v in tight.values():
                if isinstance(v, dict):
                    v.pop("_u", None)
            learned["tight_tolerance_pair"] = tight
        net.close()
        learned["e2e"] = {"value": round(world * args.steps / t_e2e_l, 4), "unit": UNIT, "path": f"learned_{best_key}",
                          "h2d_bytes_per_step": int(sum(v.nbytes for v in ice_h.values())),
                          "d2h_bytes_per_step": int(2 * 8 * mesh.nTri)}
        learned["training"] = {"variants": args.learned_variants, "solves_device_s": round(gen_ms / 1000.0, 2),
                               "wall_s": round(gen_wall, 1), "train_ms": round(train_ms, 1),
                               "loss_first_last": [float(losses[0]), float(losses[-1])],
                               "smooth_passes": LEARNED_SMOOTH}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, u_oracle = cpu_baseline(pkg, mesh, ice, params)
        # the GPU FP64 path against the oracle's own full solve of the same inputs
        cpu["gpu_fp64_rel_l2_vs_oracle"] = float("%.3g" % (np.linalg.norm(u_plain["fp64"] - u_oracle)
                                                          / np.linalg.norm(u_oracle)))
        cpu["gpu_fp64_picard_krylov_its"] = [plain["fp64"]["picard_its"], plain["fp64"]["krylov_its"]]
    # the headline is the fastest measured path (zero or learned start, any Krylov precision); the
    # rates are already the slowest rank's, so every rank picks the same path
    cands = [(f"plain_{k}", plain_runs[k], k) for k in prec]
    if learned:
        cands += [(f"learned_{k}", learned_runs[k], k) for k in prec]
        cands += [(f"learned_visc_{k}", learned_runs[f"visc_{k}"], k) for k in LEARNED_VISC_PATHS]
    assert not learned or {c[0] for c in cands} >= {learned["e2e"]["path"]}
    fastest_any = max(cands, key=lambda c: c[1][1] or 0.0)
    # the metric is the learned start with FP32 Krylov arithmetic against plain FP64: the headline is
    # the fastest learned-start path with an FP32 Krylov mode (all paths are listed beside it)
    lcands = [c for c in cands if c[0].startswith("learned") and c[2] != "fp64"] or cands
    head_name, (head_sts, head_value, head_clk, head_wall), head_prec = max(lcands, key=lambda c: c[1][1] or 0.0)
    if head_name.startswith("learned"):
        launches = kernels(head_sts, predict_kernels)
    else:
        launches = kernels(head_sts)
    if learned and head_name == learned["e2e"]["path"]:
        head_e2e = learned["e2e"]
    else:
        # end to end through the public C ABI with pinned host buffers: ice upload, the solve
        # from the zero start (or the learned start), velocity download -- every step
        solver.ice_upload(ice_h)
        solve(prec[head_prec])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            solver.ice_upload(ice_h)
            solve(prec[head_prec])
            solver.velocity_download()
        torch.cuda.synchronize()
        head_e2e = {"value": round(world * args.steps / slowest(time.perf_counter() - t0), 4), "unit": UNIT,
                    "path": head_name, "h2d_bytes_per_step": int(sum(v.nbytes for v in ice_h.values())),
                    "d2h_bytes_per_step": int(2 * 8 * mesh.nTri)}
    if rank == 0:
        kname = {"fp64": "k_bicgstab_halo<double2,double4> (persistent FP64 BiCGStab)",
                 "fp32_pair": "k_bicgstab_halo<dw2,dwblk> (persistent double-word BiCGStab)"}
        kprec = {"fp32_pair_inexact": "fp32_pair"}.get(head_prec, head_prec)   # the persistent kernel it runs
        rk = kprec if kprec in us_it and us_it.get(kprec) else "fp64"

        def roof(name):
            us = us_it.get(name)
            if not us:
                return None
            ach = bytes_it / (us * 1e-6) / 1e9
            return {"bound": "hbm", "kernel": kname[name], "launch": "one BiCGStab iteration of the persistent kernel",
                    "achieved": round(ach, 1), "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                    "frac": round(ach / peaks.get("hbm_gbs"), 4), "peak_source": peak_kind,
                    "traffic": traffic.get(f"k_bicgstab_halo_{name}_bytes_per_iteration"),
                    "algorithmic_bytes_per_launch": int(bytes_it), "us_per_launch": round(us, 3)}

        roofline = roof(rk)
        ach3 = bytes64 / (us64[0] * 1e-6) / 1e9
        line = {
            "metric": METRIC, "value": round(head_value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000.0 / head_value, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "fp32_pair": "f64; Krylov in f32 pairs (double-word)",
                      "fp32_refined": "f64; Krylov in f32 with f64 refinement",
                      "fp32_pair_inexact": "f64; Krylov in f32 pairs (double-word), inexact Picard"}[head_prec],
            "data": "synthetic MISMIP+-shaped channel from formulas (no files)",
            "config": {"workload": "DIVA channel 640x80 km, cold start, Schoof2005, Picard 1e-4, BiCGStab/Jacobi",
                       "nV": mesh.nV, "nTri": mesh.nTri, "nz": mesh.nz, "unknowns": 2 * mesh.nTri,
                       "stiffness_blocks_2x2": int(nnzb), "l2": "flushed (256 MB write) before every solve",
                       "parallelism": f"replicas x{world}",
                       "path": head_name + (" (learned Picard start, inference inside the timed solves)"
                                            if head_name.startswith("learned") else " (zero start)")
                               + ", graph-resident solve"},
            "speedup_vs_plain_fp64": round(head_value / value64, 3),
            "fastest_any_path": {"path": fastest_any[0], "value": round(fastest_any[1][1], 4), "unit": UNIT,
                                 "speedup_vs_plain_fp64": round(fastest_any[1][1] / value64, 3)},
            "accuracy": accuracy_summary(plain, learned, ref_info, head_name, u_plain, err_ref),
            "plain": plain,
            "learned_start": learned,
            "e2e": head_e2e,
            "e2e_plain_fp64": {"value": round(e2e_plain, 4), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                               "d2h_bytes_per_step": int(d2h)},
            "roofline": roofline,
            "roofline_detail": {
                "persistent_fp64": roof("fp64"), "persistent_fp32_pair": roof("fp32_pair"),
                "three_kernel_fp64_p_spmv": {"kernel": "k_p_spmv<BsrMat<double,double,1>>",
                                             "achieved": round(ach3, 1), "frac": round(ach3 / peaks.get("hbm_gbs"), 4),
                                             "traffic": traffic.get("k_p_spmv_fp64_bytes_per_launch"),
                                             "algorithmic_bytes_per_launch": int(bytes64),
                                             "us_per_launch": round(float(us64[0]), 3)},
                "note": "the matrix and Krylov vectors (about 60 MB) stay in L2 across the iterations of a "
                        "linear solve; the FP64 kernel is bound by GB300's FP64 pipe, the double-word kernel "
                        "moves that arithmetic to the FP32 pipe"},
            "cpu_baseline": cpu,
            "clocks": head_clk.summary(),
            "gpu_launches": int(launches),
            "wall_s_timed": round(head_wall, 3),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


THERMO_METRIC = "column temperature solves (column-steps)/s, 200k columns x 30 layers, 1xGB300"
THERMO_UNIT = "column-steps/s"
THERMO_WORKLOAD = ("batched column thermodynamics: 200k vertices x 30 quadratic zeta layers, 100 steps of 10 yr, "
                   "15% ice-free columns, floating and grounding-line columns, upwind advection on the mesh")


def heat_bytes(nz, n_active, n_inactive):
    """Algorithmic bytes of one column pass (k_heat_columns on the mesh path): per column with ice
    the starting temperature, u, v, w, internal heating and the upwind triangle's u_b, v_b per
    layer (7 reads) and the result (1 write), 10 per-vertex scalars, the ti_up index and the
    upwind triangle's two operator rows (3 values each, 3 columns, 2 row pointers); per column
    without ice Hi_eff and T_surf in and the surface temperature out per layer."""
    active = 8 * nz * 8 + 10 * 8 + 4 + 2 * 3 * 8 + 3 * 4 + 2 * 4
    inactive = nz * 8 + 2 * 8
    return n_active * active + n_inactive * inactive


def run_thermo(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkg = __graft_entry__.load_package()
    pkg.build()
    mesh, fields, p = pkg.geometry.thermo_case(seed=0)
    nsteps = args.thermo_steps
    solver = pkg.VelocitySolver(mesh, device=local)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        solver.heat_upload(fields)
        solver.heat_step_resident(p, nsteps)
    times, unstable = [], []
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            solver.heat_upload(fields)            # back to the initial temperature, outside the events
            n, ms = solver.heat_step_resident(p, nsteps)
            times.append(ms)
            unstable.append(n)
        torch.cuda.synchronize()
        barrier()
        wall = time.perf_counter() - t0
    t_rank = sum(times) / 1000.0
    if world > 1:
        tt = torch.tensor([t_rank], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_rank = float(tt.item())
    value = world * args.steps * nsteps * mesh.nV / t_rank

    # roofline of the column pass
    solver.heat_upload(fields)
    us, (n_act, n_inact) = solver.profile_heat_kernels(p, repeats=20)
    nbytes = heat_bytes(mesh.nz, n_act, n_inact)
    peaks, peak_kind = measured_peaks()
    achieved = nbytes / (us[0] * 1e-6) / 1e9
    # DRAM bytes per launch from the ncu capture recorded in profiles/traffic.json; a capture on a
    # different column count is scaled by the columns with ice (the kernel's traffic grows with them)
    traffic, traffic_note = None, None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tj = json.load(f)
        t_cap, n_cap = tj.get("k_heat_columns_bytes_per_launch"), tj.get("k_heat_columns_active_columns")
        if t_cap and n_cap:
            traffic = int(round(t_cap * n_act / n_cap))
            traffic_note = (f"ncu capture of {n_cap} columns with ice scaled to this run's {n_act}"
                            if n_cap != n_act else "ncu capture of this workload")
    except OSError:
        pass

    # end to end: solve_3D_heat_equation with pinned host buffers, one thermodynamics step per call
    keep, fh = [], {}
    for k, v in fields.items():
        fh[k], t = pinned_like(torch, np.asfortranarray(v))
        keep.append(t)
    out, t_out = pinned_like(torch, np.zeros((mesh.nV, mesh.nz), order="F"))
    h2d = sum(v.nbytes for v in fh.values())
    d2h = out.nbytes
    solver.solve_3D_heat_equation(fh, p)
    barrier()
    torch.cuda.synchronize()
    n_e2e = max(3, args.steps)
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        T, _ = solver.solve_3D_heat_equation(fh, p)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    e2e_value = world * n_e2e * mesh.nV / t_e2e

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = thermo_cpu_baseline(pkg, mesh, fields, p, seconds=args.cpu_seconds)
    if rank == 0:
        line = {
            "metric": THERMO_METRIC, "value": round(value, 1), "unit": THERMO_UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sum(times) / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic fields from seeded smooth random fields on a generated mesh (no files)",
            "config": {"workload": THERMO_WORKLOAD, "nV": mesh.nV, "nTri": mesh.nTri, "nz": mesh.nz,
                       "time_steps_per_run": nsteps, "dt_yr": p.dt, "columns_with_ice": int(n_act),
                       "l2": "inputs larger than L2 (8 arrays of nV x nz doubles per step)",
                       "parallelism": f"replicas x{world}",
                       "path": "resident heat state, one column-pass + retry + Robin + bookkeeping launch per step"},
            "robin_columns_per_run": unstable[0],
            "e2e": {"value": round(e2e_value, 1), "unit": THERMO_UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "note": "ufe_solve_3D_heat_equation: one thermodynamics step per call, all fields uploaded"},
            "roofline": {"bound": "hbm", "kernel": "k_heat_columns<HeatMesh> (prelude + Thomas per column)",
                         "achieved": round(achieved, 1), "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                         "frac": round(achieved / peaks.get("hbm_gbs"), 4), "peak_source": peak_kind,
                         "traffic": traffic, "traffic_source": traffic_note, "algorithmic_bytes_per_launch": int(nbytes),
                         "us_per_launch": round(float(us[0]), 2),
                         "step_kernels_us": [round(float(x), 2) for x in us]},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "gpu_launches": int(4 * nsteps * args.steps),
            "wall_s_timed": round(wall, 3),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


THICKNESS_METRIC = "semi-implicit ice-thickness steps/s (calc_dHi_dt), 1xGB300"
THICKNESS_UNIT = "steps/s"


def thickness_bytes(nV, nTri, nnz, nconn, its):
    """Algorithmic bytes of one semi-implicit calc_dHi_dt step: each array a pass must read or
    write, once.  Matrix build: connections (C, triangle pair, Cw: 20 B), vertex geometry and
    fraction_margin (V, A, fm, ptr: 36 B), the velocities (16 B per triangle), M_divQ written (8 B
    per entry).  Explicit pass: M_divQ and columns read (12 B per entry), 14 vertex arrays.  System
    rows: M_divQ read and A written (20 B per entry), 9 vertex arrays.  Krylov: per iteration two
    SpMVs (12 B per entry + row pointers + source + result) and 15 vector streams.  Finish: 8
    vertex arrays."""
    build = nconn * 20 + nV * 36 + nTri * 16 + nnz * 8
    explicit = nnz * 12 + nV * 14 * 8
    system = nnz * 20 + nV * 9 * 8
    krylov = its * (2 * (nnz * 12 + nV * 4 + 2 * nV * 8) + 15 * nV * 8)
    return build + explicit + system + krylov + nV * 8 * 8


def run_thickness(args):
    """The semi-implicit ice-thickness step (calc_dHi_dt) on a large mesh: device time per step by
    CUDA events inside the call, end to end through ufe_calc_dHi_dt with pinned host buffers, and
    the oracle's step on the host cores."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pkg = __graft_entry__.load_package()
    pkg.build()
    t0 = time.perf_counter()
    mesh, fields, p = pkg.geometry.thickness_case(res=args.thick_res, seed=0)
    A, Cw = pkg.mesh.voronoi_geometry(mesh)
    build_s = time.perf_counter() - t0
    dt = 1.0
    keep, fh = [], {}
    for k, v in fields.items():
        fh[k], t = pinned_like(torch, np.ascontiguousarray(v))
        keep.append(t)
    with pkg.VelocitySolver(mesh, device=local) as s:
        s.voronoi_upload(A, Cw)
        for _ in range(args.warmup):
            s.calc_dHi_dt(p, fh, dt)
        torch.cuda.synchronize()
        dev_ms, its = [], []
        with ClockSampler(local) as clocks:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                g = s.calc_dHi_dt(p, fh, dt)
                dev_ms.append(g["stats"]["device_ms"])
                its.append(g["stats"]["n_Axb_its"])
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        nnz = int(mesh.nV + np.asarray(mesh.nC).sum())
        nconn = nnz - mesh.nV
        # the reference's Halfar_dome integrated test for this step: 500 years with Halfar's
        # velocity prescribed, RMSE of H against Halfar's solution per resolution
        halfar_rows = []
        for res in (40e3, 20e3, 10e3):
            hm, hf, hp = pkg.geometry.halfar_case(res=res)
            with pkg.VelocitySolver(hm, device=local) as hs:
                hs.voronoi_upload()
                _, rmse, nst = pkg.geometry.halfar_run(hs.calc_dHi_dt, hm, hf, hp)
            halfar_rows.append({"resolution_km": res / 1e3, "nV": hm.nV, "steps": nst, "rmse_m": round(rmse, 2)})
    value = args.steps / (sum(dev_ms) / 1000.0)
    e2e_value = args.steps / wall
    mean_its = float(np.mean(its))
    nbytes = thickness_bytes(mesh.nV, mesh.nTri, nnz, nconn, mean_its)
    peaks, peak_kind = measured_peaks()
    achieved = nbytes / (np.mean(dev_ms) * 1e-3) / 1e9
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        oracle = _oracle()
        orc = oracle.Oracle(mesh)
        q = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in fields.items()}
        for k in ("Hi_tplusdt", "divQ", "AMB"):
            q[k] = np.zeros(mesh.nV)
        n_cpu, tc = 0, time.perf_counter()
        while n_cpu < 3 and (n_cpu == 0 or time.perf_counter() - tc < args.cpu_seconds):
            q["dHi_dt"] = fields["dHi_dt"].copy()
            orc.calc_dHi_dt(A, Cw, p, q, dt)
            n_cpu += 1
        sec = (time.perf_counter() - tc) / n_cpu
        cpu = {"value": round(1.0 / sec, 4), "unit": THICKNESS_UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n_cpu} full steps of the same workload ({sec * 1000:.0f} ms each; the BiCGStab "
                         "loops use OpenMP, the matrix build and the border rule one core)"}
    if rank == 0:
        in_bytes = sum(v.nbytes for k, v in fh.items() if k in pkg.abi.THICKNESS_INPUTS or k == "dHi_dt")
        line = {
            "metric": THICKNESS_METRIC, "value": round(value, 2), "unit": THICKNESS_UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(float(np.mean(dev_ms)), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic dome, relief bed, radial outflow on a generated mesh (no files)",
            "config": {"workload": f"semi-implicit calc_dHi_dt (fs 1.5, BiCGStab/Jacobi rtol 1e-8, abstol 1e-6), "
                                   f"dome H0 3000 m R 330 km on an 800 km square, {args.thick_res / 1e3:g} km mesh",
                       "nV": mesh.nV, "nTri": mesh.nTri, "matrix_entries": nnz, "dt_yr": dt,
                       "krylov_its_mean": mean_its, "host_build_s": round(build_s, 1),
                       "l2": "every step uploads its inputs; the working set (matrix entries "
                             f"{nnz * 20 / 1e6:.0f} MB, vertex and triangle fields "
                             f"{(mesh.nV * 30 * 8 + mesh.nTri * 16) / 1e6:.0f} MB) exceeds the 129 MB L2"},
            "e2e": {"value": round(e2e_value, 2), "unit": THICKNESS_UNIT, "h2d_bytes_per_step": int(in_bytes),
                    "d2h_bytes_per_step": int(4 * 8 * mesh.nV),
                    "note": "ufe_calc_dHi_dt with pinned host arrays: upload, step, download of dHi_dt, "
                            "Hi_tplusdt, divQ, AMB"},
            "roofline": {"bound": "hbm", "kernel": "whole step (matrix build, explicit pass, system rows, "
                                                   "three-kernel CSR BiCGStab)",
                         "achieved": round(achieved, 1), "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                         "frac": round(achieved / peaks.get("hbm_gbs"), 4), "peak_source": peak_kind,
                         "traffic": None, "algorithmic_bytes_per_step": int(nbytes)},
            "halfar_dome": {"rows": halfar_rows,
                            "reference_scoreboard_rmse_m": {"10 km": 18.02},
                            "note": "500 yr of the semi-implicit step (f_s 1.5, dt 10 yr) with Halfar's (1983) "
                                    "shallow-ice velocity prescribed; the reference's integrated test couples its "
                                    "SIA solve instead"},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            # per step: 14 input gathers, matrix + neighbour counts (2), explicit pass and system
            # rows (10), the solve graph (Jacobi, init, 5 per Krylov iteration), 2 finishing
            # kernels, 4 output gathers
            "gpu_launches": int(round(args.steps * (34 + 5 * mean_its))),
            "wall_s_timed": round(wall, 3),
        }
        print(json.dumps(line))


LEARNED_WORKLOAD = ("learned Picard start, SSA ensemble: 30k-vertex mesh over 1500 km x 1500 km, bed -200 m + "
                    "GRF(400 m, 20 km), dome R = 600 km, floating below flotation, log-normal beta^2; 256 training "
                    "and 32 held-out geometries; Weertman m = 3, Picard 1e-4, BiCGStab/Jacobi 1e-8")


def run_learned(args):
    """The learned start on the 30k-vertex SSA ensemble: data from plain FP64 GPU solves, GPU training,
    held-out solves from the learned start."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pkg = __graft_entry__.load_package()
    pkg.build()
    mesh = pkg.geometry.ensemble_mesh(nV=args.learned_nv, seed=0)
    T = mesh.Tri - 1
    train_ids = range(args.learned_train)
    test_ids = range(100000, 100000 + args.learned_test)
    p32_of = lambda p: _with(pkg, p, precision=pkg.abi.PREC_FP32_REFINE)
    pair_of = lambda p: _with(pkg, p, precision=pkg.abi.PREC_FP32_PAIR)
    out = {}
    with pkg.VelocitySolver(mesh, device=local) as s:
        net = pkg.LearnedStart(s, seed=1)
        gen_ms, gen_its = 0.0, []
        t0 = time.perf_counter()
        for m in train_ids:
            ice, p = pkg.geometry.ensemble_member(mesh, m)
            s.ice_upload(ice)
            x = net.features(s)
            st = s.solve_resident(p, diva=False, cold_start=True)
            gen_ms += st["device_ms"]
            gen_its.append((st["n_visc_its"], st["n_Axb_its"]))
            net.dataset_add(s, x)
            if m % 16 == 0:
                print(f"training solve {m}: {st['n_visc_its']} Picard, {st['n_Axb_its']} Krylov, "
                      f"{st['device_ms']:.0f} ms", file=sys.stderr, flush=True)
        gen_wall = time.perf_counter() - t0
        losses, train_ms = net.train(epochs=args.learned_epochs, lr=args.learned_lr)
        net.dataset_clear()
        keys = ("cold_fp64", "cold_fp32_pair", "learned_fp64", "learned_fp32_pair", "learned_fp32",
                "learned_visc_fp64", "learned_visc_fp32_pair")
        rows = {k: [] for k in keys}
        errs = {k: [] for k in keys}
        pred_ms = []
        with ClockSampler(local) as clocks:
            for m in test_ids:
                ice, p = pkg.geometry.ensemble_member(mesh, m)
                on_ice = (ice["Hi"][T] > 0).all(axis=1)
                sel = np.r_[on_ice, on_ice]
                s.ice_upload(ice)
                st = s.solve_resident(p, diva=False, cold_start=True)
                rows["cold_fp64"].append(st)
                uc = np.r_[s.velocity_download()]
                ut = None
                if len(errs["cold_fp64"]) < args.learned_err_members:
                    # reference for the errors: the same solve continued to 1e-8
                    tight = _with(pkg, p, visc_it_norm_dUV_tol=1e-8, visc_it_nit=400)
                    try:
                        s.solve_resident(tight, diva=False, cold_start=False)
                    except pkg.UfeError:   # divergence control near round-off: settle for 1e-6
                        s.ice_upload(ice)
                        s.solve_resident(_with(pkg, p, visc_it_norm_dUV_tol=1e-6, visc_it_nit=400), diva=False)
                    ut = np.r_[s.velocity_download()]
                    errs["cold_fp64"].append(np.linalg.norm((uc - ut)[sel]) / np.linalg.norm(ut[sel]))
                st = s.solve_resident(pair_of(p), diva=False, cold_start=True)
                rows["cold_fp32_pair"].append(st)
                if ut is not None:
                    u = np.r_[s.velocity_download()]
                    errs["cold_fp32_pair"].append(np.linalg.norm((u - ut)[sel]) / np.linalg.norm(ut[sel]))
                for key, pp in (("learned_fp64", p), ("learned_fp32_pair", pair_of(p)), ("learned_fp32", p32_of(p)),
                                ("learned_visc_fp64", p), ("learned_visc_fp32_pair", pair_of(p))):
                    # learned_visc_*: the predicted viscosity also replaces Glen's law in the first iteration
                    pred_ms.append(net.predict(s, viscosity=key.startswith("learned_visc")))
                    st = s.solve_resident(pp, diva=False, cold_start=False)
                    rows[key].append(st)
                    if ut is not None:
                        u = np.r_[s.velocity_download()]
                        errs[key].append(np.linalg.norm((u - ut)[sel]) / np.linalg.norm(ut[sel]))
                print(f"held-out {m}: Picard iterations " +
                      " ".join(f"{k} {rows[k][-1]['n_visc_its']}" for k in keys), file=sys.stderr, flush=True)
        net.close()
    n = len(test_ids)
    mean_pred = float(np.mean(pred_ms))
    def rate(key, extra_ms=0.0):
        return n / ((sum(r["device_ms"] for r in rows[key]) + n * extra_ms) / 1000.0)
    vals = {k: rate(k, mean_pred if k.startswith("learned") else 0.0) for k in rows}
    best = max(vals, key=lambda k: vals[k])   # the fastest path, zero or learned start
    peaks, peak_kind = measured_peaks()
    line = {
        "metric": METRIC, "value": round(vals[best], 4), "unit": UNIT, "n_gpus": world, "steps": n, "warmup": 0,
        "ms_per_step": round(1000.0 / vals[best], 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (network bf16)",
        "data": "synthetic ensemble geometries from seeded random fields on a generated mesh (no files)",
        "config": {"workload": LEARNED_WORKLOAD, "nV": mesh.nV, "nTri": mesh.nTri,
                   "train": len(train_ids), "held_out": n, "epochs": args.learned_epochs, "path": best},
        "speedup_vs_plain_fp64": round(vals[best] / vals["cold_fp64"], 3),
        "paths": {k: {"value": round(vals[k], 4), "unit": UNIT,
                      "picard_its_mean": float(np.mean([r["n_visc_its"] for r in rows[k]])),
                      "krylov_its_mean": float(np.mean([r["n_Axb_its"] for r in rows[k]])),
                      "rel_l2_vs_tight_solve_mean": float(np.mean(errs[k])),
                      "rel_l2_vs_tight_solve_max": float(np.max(errs[k]))} for k in rows},
        "network": {"inference_ms_mean": round(mean_pred, 3), "train_ms": round(train_ms, 1),
                    "loss_first_last": [float(losses[0]), float(losses[-1])], "params": int(net.nparams)},
        "data_generation": {"solves": len(train_ids), "device_s": round(gen_ms / 1000.0, 2),
                            "wall_s": round(gen_wall, 1),
                            "picard_its_mean": float(np.mean([a for a, b in gen_its]))},
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))


DOME_WORKLOAD = ("SSA on the radially symmetric dome, 800 km square, ~8,500 vertices (10 km at the "
                 "margin, 40 km inside), Weertman m=3, BiCGStab/Jacobi 1e-8; Picard 1e-4 and a tight tolerance")
# dome variants the learned start trains on: (H0 [m], R [m], beta^2), each on its own mesh
DOME_VARIANTS = [(2600.0, 460e3, 7e3), (2800.0, 480e3, 1.3e4), (3200.0, 520e3, 8e3), (3400.0, 540e3, 1.2e4),
                 (2700.0, 530e3, 9e3), (3300.0, 470e3, 1.1e4), (2900.0, 510e3, 1.5e4), (3100.0, 490e3, 6e3)]


def run_dome(args):
    """The ~8,500-vertex SSA dome: the GPU FP64 path against the oracle's own solve (the parity check at
    size), and the accuracy target where the reference's Picard iteration converges tightly: plain
    FP64 against learned start + double-word Krylov, both at the benchmark tolerance and at a tight
    one, with every velocity error measured against a tightly converged FP64 solution."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pkg = __graft_entry__.load_package()
    pkg.build()
    mesh, ice, params = pkg.geometry.dome_case(seed=0)
    F64, PAIR = pkg.abi.PREC_FP64, pkg.abi.PREC_FP32_PAIR
    solver = pkg.VelocitySolver(mesh, device=local)
    solver.ice_upload(ice)
    stream = torch.cuda.ExternalStream(solver.stream_handle())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def solve(p, cold=True):
        with torch.cuda.stream(stream):
            flush.zero_()
        st = solver.solve_resident(p, diva=False, cold_start=cold)
        return st, np.r_[solver.velocity_download()]

    T_tight = args.dome_tight
    ref_p = _with(pkg, params, precision=F64, stress_balance_PETSc_rtol=1e-12, stress_balance_PETSc_abstol=0.0,
                  visc_it_norm_dUV_tol=args.dome_ref_tol, visc_it_nit=2000)
    st_ref, u_ref = solve(ref_p)

    def err(u):
        return float("%.3g" % (np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)))

    # the learned start, trained on tightly converged solutions of dome variants (outside the timed region)
    net = pkg.LearnedStart(solver, seed=1)
    t_gen, gen_ms = time.perf_counter(), 0.0
    for sd, (H0, R, b2) in enumerate(DOME_VARIANTS, start=1):
        m_v, ice_v, p_v = pkg.geometry.dome_case(seed=sd, H0=H0, R=R, beta_sq=b2)
        with pkg.VelocitySolver(m_v, device=local) as sv:
            sv.ice_upload(ice_v)
            x = net.features(sv)
            # the tightest tolerance the divergence control lets this variant finish
            for tol in (1e-12, 1e-10, 1e-8, 1e-6):
                try:
                    gen_ms += sv.solve_resident(_with(pkg, p_v, visc_it_norm_dUV_tol=tol, visc_it_nit=2000,
                                                      stress_balance_PETSc_rtol=1e-12,
                                                      stress_balance_PETSc_abstol=0.0),
                                                diva=False, cold_start=True)["device_ms"]
                    break
                except pkg.UfeError:
                    continue
            net.dataset_add(sv, x)
    gen_wall = time.perf_counter() - t_gen
    losses, train_ms = net.train(epochs=args.dome_epochs, lr=2e-3)
    net.dataset_clear()
    solver.ice_upload(ice)

    paths = {}
    for tol in (params.visc_it_norm_dUV_tol, T_tight):
        for name, prec, learned, forcing in (("plain_fp64", F64, False, 0.0), ("plain_fp32_pair", PAIR, False, 0.0),
                                             ("plain_fp32_pair_inexact", PAIR, False, args.forcing),
                                             ("learned_fp64", F64, True, 0.0), ("learned_fp32_pair", PAIR, True, 0.0),
                                             ("learned_fp32_pair_inexact", PAIR, True, args.forcing),
                                             ("learned_visc_fp64", F64, True, 0.0),
                                             ("learned_visc_fp32_pair", PAIR, True, 0.0),
                                             ("learned_visc_fp32_pair_inexact", PAIR, True, args.forcing)):
            p = _with(pkg, params, precision=prec, visc_it_norm_dUV_tol=tol, visc_it_nit=2000, krylov_forcing=forcing)
            ms, sts, u = [], None, None
            visc = name.startswith("learned_visc")   # the predicted viscosity in the first Picard iteration
            for i in range(args.warmup + args.steps):
                pred = net.predict(solver, smooth_passes=2, viscosity=visc) if learned else 0.0
                st, u = solve(p, cold=not learned)
                if i >= args.warmup:
                    ms.append(st["device_ms"] + pred)
                    sts = st
            paths[f"{name}@{tol:g}"] = {"value": round(1000.0 / float(np.mean(ms)), 3), "unit": UNIT,
                                        "ms_per_solve": round(float(np.mean(ms)), 2), "picard_its": sts["n_visc_its"],
                                        "krylov_its": sts["n_Axb_its"], "status": sts["status"],
                                        "relax_applied": round(sts["visc_it_relax_applied"], 4),
                                        "rel_l2_vs_fp64_reference": err(u)}
    # time to the accuracy target: every path at the loosest Picard tolerance (of a tightening list)
    # whose answer lands within 1e-6 of the FP64 reference solution
    to_target = {}
    for name, prec, learned, forcing in (("plain_fp64", F64, False, 0.0), ("plain_fp32_pair_inexact", PAIR, False, args.forcing),
                                         ("learned_fp32_pair", PAIR, True, 0.0),
                                         ("learned_fp32_pair_inexact", PAIR, True, args.forcing),
                                         ("learned_visc_fp32_pair", PAIR, True, 0.0),
                                         ("learned_visc_fp32_pair_inexact", PAIR, True, args.forcing)):
        tried = []
        for tol in (1e-12, 1e-13, 1e-14, 1e-15, 3e-16, 1e-16):
            p = _with(pkg, params, precision=prec, visc_it_norm_dUV_tol=tol, visc_it_nit=2000, krylov_forcing=forcing)
            ms, sts, u = [], None, None
            for i in range(args.warmup + args.steps):
                pred = net.predict(solver, smooth_passes=2, viscosity=name.startswith("learned_visc")) if learned else 0.0
                st, u = solve(p, cold=not learned)
                if i >= args.warmup:
                    ms.append(st["device_ms"] + pred)
                    sts = st
            e = err(u)
            tried.append({"picard_tol": tol, "rel_l2_vs_fp64_reference": e, "ms_per_solve": round(float(np.mean(ms)), 2),
                          "relax_applied": round(sts["visc_it_relax_applied"], 4)})
            if e <= 1e-6:
                to_target[name] = {"value": round(1000.0 / float(np.mean(ms)), 3), "unit": UNIT, "picard_tol": tol,
                                   "picard_its": sts["n_visc_its"], "krylov_its": sts["n_Axb_its"],
                                   "relax_applied": round(sts["visc_it_relax_applied"], 4),
                                   "rel_l2_vs_fp64_reference": e}
                break
        if name not in to_target:
            to_target[name] = {"value": None, "tried": tried}
    net.close()
    # the oracle on the same inputs: the benchmark solve timed on the host cores, and both paths at
    # Krylov rtol 1e-12 for the parity figure
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        oracle = _oracle()
        os.environ["OMP_NUM_THREADS"] = str(os.cpu_count())
        orc = oracle.Oracle(mesh)
        so = pkg.new_ssa_state(mesh.nTri)
        t0 = time.perf_counter()
        nvo, nao, sto = orc.solve_SSA(ice, so, _with(pkg, params))
        secs = time.perf_counter() - t0
        st_g, u_g = solve(_with(pkg, params, precision=F64))
        uo = np.r_[so["u_b"], so["v_b"]]
        pp = _with(pkg, params, precision=F64, stress_balance_PETSc_rtol=1e-12, stress_balance_PETSc_abstol=0.0)
        so12 = pkg.new_ssa_state(mesh.nTri)
        nv12, _, _ = orc.solve_SSA(ice, so12, pp)
        st12, u12 = solve(pp)
        uo12 = np.r_[so12["u_b"], so12["v_b"]]
        cpu = {"value": round(1.0 / secs, 4), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"full solve: {nvo} Picard / {nao} Krylov iterations in {secs:.2f} s",
               "gpu_fp64_rel_l2_vs_oracle": float("%.3g" % (np.linalg.norm(u_g - uo) / np.linalg.norm(uo))),
               "gpu_fp64_picard_its": st_g["n_visc_its"],
               "at_krylov_rtol_1e-12": {"gpu_vs_oracle_rel_l2": float("%.3g" % (np.linalg.norm(u12 - uo12)
                                                                                 / np.linalg.norm(uo12))),
                                        "picard_its_gpu_oracle": [st12["n_visc_its"], nv12]}}
    base = f"plain_fp64@{T_tight:g}"
    # the headline: the fastest learned-start path with FP32 Krylov arithmetic at the tight tolerance
    head = max((k for k in paths if k.startswith("learned") and "_fp32" in k and k.endswith(f"@{T_tight:g}")),
               key=lambda k: paths[k]["value"])
    met = paths[head]["rel_l2_vs_fp64_reference"] <= 1e-6
    lt = [k for k in to_target if k.startswith("learned") and to_target[k]["value"]]
    head_t = max(lt, key=lambda k: to_target[k]["value"]) if lt else None
    base_t = to_target.get("plain_fp64", {}).get("value")
    line = {"metric": METRIC, "value": paths[head]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": paths[head]["ms_per_solve"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64; Krylov in f32 pairs (double-word)",
            "data": "synthetic dome from formulas (no files)",
            "config": {"workload": DOME_WORKLOAD, "nV": mesh.nV, "nTri": mesh.nTri,
                       "l2": "flushed (256 MB write) before every solve", "path": head},
            "speedup_vs_plain_fp64": round(paths[head]["value"] / paths[base]["value"], 3),
            "reference_solution": {"picard_tol": args.dome_ref_tol, "krylov_rtol": 1e-12,
                                   "picard_its": st_ref["n_visc_its"], "krylov_its": st_ref["n_Axb_its"],
                                   "relax_applied": round(st_ref["visc_it_relax_applied"], 4)},
            "paths": paths,
            "to_1e-6": to_target,
            "to_1e-6_statement": (
                f"To land within 1e-6 of the FP64 reference solution, plain FP64 needs Picard tolerance "
                f"{to_target['plain_fp64'].get('picard_tol')} ({base_t} solves/s); the fastest learned-start FP32 path, "
                f"{head_t}, needs {to_target[head_t]['picard_tol']} ({to_target[head_t]['value']} solves/s, "
                f"{to_target[head_t]['value'] / base_t:.2f}x)" if head_t and base_t else
                "no learned-start FP32 path reached 1e-6 of the reference within Picard tolerance 1e-16"),
            "statement": (f"At Picard tolerance {T_tight:g} {head.split('@')[0].replace('_', ' ')} is "
                          f"{paths[head]['rel_l2_vs_fp64_reference']:.1e} from the FP64 reference solution "
                          f"(plain FP64 {paths[base]['rel_l2_vs_fp64_reference']:.1e}) at "
                          f"{paths[head]['value'] / paths[base]['value']:.2f}x the plain FP64 solves/s: the "
                          f"1e-6 target is {'met' if met else 'not met'}.  At the benchmark tolerance "
                          f"{params.visc_it_norm_dUV_tol:g} every path is about "
                          f"{paths[f'plain_fp64@{params.visc_it_norm_dUV_tol:g}']['rel_l2_vs_fp64_reference']:.1e} "
                          f"from it."),
            "learned_start": {"variants": len(DOME_VARIANTS), "solves_device_s": round(gen_ms / 1000.0, 2),
                              "wall_s": round(gen_wall, 1), "train_ms": round(train_ms, 1),
                              "loss_first_last": [float(losses[0]), float(losses[-1])]},
            "cpu_baseline": cpu}
    solver.close()
    if rank == 0:
        print(json.dumps(line))


def run_icestream(args):
    """The reference's SSA_icestream integrated test on the GPU: for each of its four resolutions a
    cold velocity solve and one warm-started from it (as its short transient run makes them), the
    RMSE of u on the south-north transect against Schoof's (2006) analytic ice stream, the
    reference scoreboard's figures beside it, and the GPU against the oracle on the 32 km run."""
    pkg = __graft_entry__.load_package()
    pkg.build()
    scoreboard = {32e3: 400.42, 4e3: 101.21}   # RMSE_32km, RMSE_4km (it_ideal_SSA_icestream_*.xml)
    rows = []
    for res in (32e3, 16e3, 8e3, 4e3):
        mesh, ice, p = pkg.geometry.icestream_case(res=res)
        with pkg.VelocitySolver(mesh) as g:
            s = pkg.new_ssa_state(mesh.nTri)
            its, ms = [], 0.0
            for _ in range(2):
                nv, na, st = g.solve_SSA(ice, s, p)
                its.append([nv, na])
                ms += st["device_ms"]
            ua = g.apply("MAP_B_A", s["u_b"])
        y, ut = pkg.geometry.transect_values(mesh, ua)
        an = pkg.geometry.schoof2006_u(y)
        rows.append({"resolution_km": res / 1e3, "nV": mesh.nV, "picard_krylov_its": its, "device_ms": round(ms, 1),
                     "rmse_m_per_yr": round(float(np.sqrt(np.nanmean((ut - an) ** 2))), 2),
                     "u_max_transect": round(float(np.nanmax(ut)), 1), "u_max_schoof": round(float(an.max()), 1),
                     "reference_scoreboard_rmse": scoreboard.get(res)})
    # GPU against the oracle, 32 km, Krylov to 1e-12
    mesh, ice, p = pkg.geometry.icestream_case(res=32e3)
    p = _with(pkg, p, stress_balance_PETSc_rtol=1e-12, stress_balance_PETSc_abstol=0.0)
    orc = _oracle().Oracle(mesh)
    a, b = pkg.new_ssa_state(mesh.nTri), pkg.new_ssa_state(mesh.nTri)
    with pkg.VelocitySolver(mesh) as g:
        nvg, _, _ = g.solve_SSA(ice, a, p)
    nvo, _, _ = orc.solve_SSA(ice, b, p)
    ug, uo = np.r_[a["u_b"], a["v_b"]], np.r_[b["u_b"], b["v_b"]]
    print(json.dumps({"workload": "SSA_icestream integrated test (Schoof 2006), 800 km square, 32/16/8/4 km",
                      "runs": rows, "gpu_vs_oracle_32km": {"rel_l2": float("%.3g" % (np.linalg.norm(ug - uo)
                                                                                       / np.linalg.norm(uo))),
                                                           "picard_its_gpu_oracle": [nvg, nvo]}}))


ENSEMBLE_WORKLOAD = ("ensemble of SSA solves on meshes of uneven size (log-uniform vertex counts), each its own "
                     "geometry of the learned-start ensemble family; autotuned rows per warp per mesh; members "
                     "solved one after another vs side by side (ufe_ensemble_solve)")


def run_ensemble(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    pkg = __graft_entry__.load_package()
    pkg.build()
    rng = np.random.default_rng(7)
    sizes = np.exp(rng.uniform(np.log(args.ens_min), np.log(args.ens_max), args.ens_members)).astype(int)
    # members shard over the ranks by size (no exchange on the data path); each rank builds and
    # solves its own share side by side
    mine = pkg.ensemble.shard(rank, world, sizes)
    members = []
    for k in mine:
        mesh = pkg.geometry.ensemble_mesh(nV=int(sizes[k]), seed=k)
        ice, p = pkg.geometry.ensemble_member(mesh, 500 + k)
        members.append((mesh, ice, p))
        print(f"rank {rank} member {k}: {mesh.nV} vertices", file=sys.stderr, flush=True)
    p = members[0][2] if members else pkg.abi.default_params()
    solvers = [pkg.VelocitySolver(m, device=local) for m, _, _ in members]
    tune = []
    for sv, (m, ice, _) in zip(solvers, members):
        sv.ice_upload(ice)
        sv.solve_resident(p, diva=False, cold_start=True)   # warm-up: graphs, and the system to tune on
        tune.append(sv.autotune(repeats=20)[0])
    # one after another (device time of each solve)
    seq_ms, its = 0.0, []
    for sv in solvers:
        st = sv.solve_resident(p, diva=False, cold_start=True)
        seq_ms += st["device_ms"]
        its.append((st["n_visc_its"], st["n_Axb_its"]))
    if solvers:
        pkg.ensemble_solve(solvers, p, diva=False, cold_start=True)   # warm-up of the concurrent launch
    walls = []
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            if solvers:
                stats, wall = pkg.ensemble_solve(solvers, p, diva=False, cold_start=True)
            else:
                wall = 0.0   # more ranks than members: this rank has none
            walls.append(wall)
    for sv in solvers:
        sv.close()
    # the only exchange: the per-member results, gathered on the host after the timed region
    results = pkg.ensemble.gather_results({k: {"nV": m.nV, "its": it, "tune": tu}
                                           for k, (m, _, _), it, tu in zip(mine, members, its, tune)})
    wall_max = pkg.ensemble.max_over_ranks(statistics.mean(walls), device=f"cuda:{local}")
    seq_total = pkg.ensemble.max_over_ranks(seq_ms, device=f"cuda:{local}")
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return
    n = len(results)
    order = sorted(results)
    value = n / (wall_max / 1000.0)
    line = {"metric": f"ensemble SSA velocity solves/s, members side by side, {world}xGB300", "value": round(value, 4),
            "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": 1,
            "ms_per_step": round(wall_max, 2), "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic ensemble geometries from seeded random fields on generated meshes (no files)",
            "config": {"workload": ENSEMBLE_WORKLOAD, "members": n, "vertices": [results[k]["nV"] for k in order],
                       "total_vertices": int(sum(results[k]["nV"] for k in order)),
                       "rows_per_warp": [results[k]["tune"] for k in order],
                       "parallelism": f"members partitioned over {world} rank(s) by size"},
            "one_after_another": {"value": round(n / (seq_total / 1000.0), 4), "unit": UNIT,
                                  "ms": round(seq_total, 1)},
            "speedup_side_by_side": round(seq_total / wall_max, 3),
            "picard_its": [results[k]["its"][0] for k in order], "krylov_its": [results[k]["its"][1] for k in order],
            "clocks": clocks.summary()}
    print(json.dumps(line))


MIXED_WORKLOAD = ("mixed-size DIVA ensemble: 64 members, vertex counts log-uniform in [20k, 400k] (8.1M in all), "
                  "6,000 km domain, fractal bed (slope -2, RMS 800 m, mean -300 m), dome R = 2,200 km, "
                  "H0 = 4,000 m, fine cells around the grounding zone; Weertman m = 3, Picard 1e-4, "
                  "BiCGStab/Jacobi 1e-8; members side by side (ufe_ensemble_solve)")


def _mixed_member(job):
    """Worker: build member k of the mixed-size ensemble (mesh and ice state) on the host."""
    k, nv = job
    pkg = __graft_entry__.load_package()
    mesh = pkg.geometry.mixed_ensemble_mesh(int(nv), seed=k)
    ice, _ = pkg.geometry.mixed_ensemble_member(mesh, k)
    return k, mesh, ice


def run_mixed(args):
    """The mixed-size DIVA ensemble: members partitioned over the ranks by size, each rank's share
    built on the host in parallel processes and solved side by side on its GPU."""
    import multiprocessing as mp
    import torch

    rank, world, local = dist_env()
    sizes = __graft_entry__.load_package().geometry.mixed_ensemble_sizes(n=args.mixed_members)
    pkg = __graft_entry__.load_package()
    mine = pkg.ensemble.shard(rank, world, sizes)
    t0 = time.perf_counter()
    # training geometries of the learned start: seeds apart from the members', 20k-60k vertices
    train_jobs = [(10_000 + i, int(20_000 * 3.0 ** (i / max(args.mixed_train - 1, 1))))
                  for i in range(args.mixed_train)] if args.mixed_mode == "sequential" else []
    with mp.get_context("spawn").Pool(processes=max(1, min(len(mine), os.cpu_count() or 1))) as pool:
        built = sorted(pool.map(_mixed_member, [(k, sizes[k]) for k in mine]), key=lambda t: t[0])
        train = pool.map(_mixed_member, train_jobs) if train_jobs else []
    gen_s = time.perf_counter() - t0
    print(f"rank {rank}: {len(built)} members built in {gen_s:.0f} s", file=sys.stderr, flush=True)
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    pkg.build()
    p = pkg.geometry.mixed_ensemble_params()
    if args.mixed_mode == "sequential":
        return run_mixed_sequential(args, pkg, built, p, gen_s, rank, world, local, train)
    solvers = []
    for k, mesh, ice in built:
        sv = pkg.VelocitySolver(mesh, device=local)
        sv.ice_upload(ice)
        sv.solve_resident(p, diva=True, cold_start=True)    # warm-up: graph capture
        solvers.append(sv)
    if solvers:
        pkg.ensemble_solve(solvers, p, diva=True, cold_start=True)   # warm-up of the concurrent launch
    if world > 1:
        torch.distributed.barrier()
    walls, stats = [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            if solvers:
                stats, wall = pkg.ensemble_solve(solvers, p, diva=True, cold_start=True)
            else:
                wall = 0.0
            walls.append(wall)
    results = pkg.ensemble.gather_results({k: {"nV": mesh.nV, "its": (st["n_visc_its"], st["n_Axb_its"]),
                                               "status": st["status"]}
                                           for (k, mesh, _), st in zip(built, stats)})
    wall_max = pkg.ensemble.max_over_ranks(statistics.mean(walls), device=f"cuda:{local}")
    for sv in solvers:
        sv.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return
    order = sorted(results)
    n = len(order)
    value = n / (wall_max / 1000.0)
    line = {"metric": f"mixed-size DIVA ensemble solves/s, members side by side, {world}xGB300",
            "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": 1,
            "ms_per_step": round(wall_max, 1), "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic ensemble geometries from seeded random fields on generated meshes (no files)",
            "config": {"workload": MIXED_WORKLOAD, "members": n,
                       "total_vertices": int(sum(results[k]["nV"] for k in order)),
                       "vertices": [results[k]["nV"] for k in order],
                       "parallelism": f"members partitioned over {world} rank(s) by size"},
            "picard_its": [results[k]["its"][0] for k in order],
            "krylov_its": [results[k]["its"][1] for k in order],
            "statuses": [results[k]["status"] for k in order],
            "host_build_s": round(gen_s, 1),
            "clocks": clocks.summary()}
    print(json.dumps(line))


def run_mixed_sequential(args, pkg, built, p, gen_s, rank, world, local, train=()):
    """The mixed-size DIVA ensemble member by member: each member's solve has the whole GPU, so it runs with the
    persistent Krylov kernels (members side by side cannot: a persistent kernel needs every SM).
    Three paths per member, each solved once (the device time of a solve excludes its graph
    capture): plain FP64 -- the reference's algorithm --, double-word Krylov inside the inexact
    Picard iteration, and the same from the learned start with its predicted viscosity (the
    network trained beforehand on the `train` geometries, outside the timed region); the
    per-member distances between the answers are reported."""
    import torch

    p64 = _with(pkg, p, precision=pkg.abi.PREC_FP64, visc_it_nit=args.picard_nit)
    pfast = _with(pkg, p, precision=pkg.abi.PREC_FP32_PAIR, krylov_forcing=args.forcing, visc_it_nit=args.picard_nit)
    net, host, train_info = None, None, None
    if train:
        host = pkg.ColumnSolver(device=local)
        net = pkg.LearnedStart(host, seed=1)
        gen_ms, t_tr = 0.0, time.perf_counter()
        for k, mesh, ice in train:
            with pkg.VelocitySolver(mesh, device=local) as sv:
                sv.ice_upload(ice)
                x = net.features(sv)
                gen_ms += sv.solve_resident(p64, diva=True, cold_start=True)["device_ms"]
                net.dataset_add(sv, x)
        losses, train_ms = net.train(epochs=args.mixed_epochs, lr=2e-3)
        net.dataset_clear()
        train_info = {"geometries": len(train), "vertices": [int(m.nV) for _, m, _ in train],
                      "solves_device_s": round(gen_ms / 1000.0, 2), "train_ms": round(train_ms, 1),
                      "wall_s": round(time.perf_counter() - t_tr, 1),
                      "loss_first_last": [float(losses[0]), float(losses[-1])]}
    paths = (("fp64", p64, False), ("fp32_pair_inexact", pfast, False)) + \
            ((("learned_visc_fp32_pair_inexact", pfast, True),) if net else ())
    rows = {}
    with ClockSampler(local) as clocks:
        for k, mesh, ice in built:
            with pkg.VelocitySolver(mesh, device=local) as sv:
                sv.ice_upload(ice)
                r = {"nV": mesh.nV}
                u = {}
                for name, pp, learned in paths:
                    try:
                        pred = net.predict(sv, smooth_passes=2, viscosity=True) if learned else 0.0
                        st = sv.solve_resident(pp, diva=True, cold_start=not learned)
                        r[name] = {"ms": st["device_ms"] + pred, "picard": st["n_visc_its"],
                                   "krylov": st["n_Axb_its"], "status": st["status"]}
                        u[name] = np.r_[sv.velocity_download()]
                    except pkg.UfeError as e:
                        r[name] = {"ms": None, "status": e.code}
                if "fp64" in u:
                    a = u["fp64"]
                    for name in u:
                        if name != "fp64":
                            key = "rel_l2_fast_vs_fp64" if name == "fp32_pair_inexact" else f"rel_l2_{name}_vs_fp64"
                            r[key] = float("%.3g" % (np.linalg.norm(u[name] - a) / np.linalg.norm(a)))
                rows[k] = r
            print(f"member {k}: {mesh.nV} vertices, " + ", ".join(f"{n} {r[n].get('ms')} ms" for n, _, _ in paths),
                  file=sys.stderr, flush=True)
    if net:
        net.close()
        host.close()
    results = pkg.ensemble.gather_results(rows)
    if rank != 0:
        return
    order = sorted(results)
    n = len(order)
    t64 = sum(results[k]["fp64"]["ms"] or 0.0 for k in order) / 1000.0
    tf = sum(results[k]["fp32_pair_inexact"]["ms"] or 0.0 for k in order) / 1000.0
    errs = [results[k].get("rel_l2_fast_vs_fp64") for k in order if results[k].get("rel_l2_fast_vs_fp64") is not None]
    learned = None
    if train:
        tl = sum(results[k]["learned_visc_fp32_pair_inexact"]["ms"] or 0.0 for k in order) / 1000.0
        el = [results[k].get("rel_l2_learned_visc_fp32_pair_inexact_vs_fp64") for k in order
              if results[k].get("rel_l2_learned_visc_fp32_pair_inexact_vs_fp64") is not None]
        learned = {"value": round(world * n / tl, 4) if tl > 0 else None, "unit": UNIT, "device_s": round(tl, 2),
                   "speedup_vs_plain_fp64": round(t64 / tl, 3) if tl > 0 else None,
                   "rel_l2_vs_fp64": {"median": float(np.median(el)), "max": float(np.max(el))} if el else None,
                   "training": train_info}
    line = {"metric": f"mixed-size DIVA ensemble solves/s, members one after another, {world}xGB300",
            "value": round(world * n / tf, 4), "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 0,
            "ms_per_step": round(1000.0 * tf, 1), "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
            "dtype": "f64; Krylov in f32 pairs (double-word), inexact Picard",
            "data": "synthetic ensemble geometries from seeded random fields on generated meshes (no files)",
            "config": {"workload": MIXED_WORKLOAD.replace("members side by side (ufe_ensemble_solve)",
                                                          "members one after another, persistent kernels"),
                       "members": n, "total_vertices": int(sum(results[k]["nV"] for k in order)),
                       "forcing": args.forcing},
            "plain_fp64": {"value": round(world * n / t64, 4), "unit": UNIT, "device_s": round(t64, 2)},
            "speedup_vs_plain_fp64": round(t64 / tf, 3),
            "rel_l2_fast_vs_fp64": {"median": float(np.median(errs)), "max": float(np.max(errs))} if errs else None,
            "learned_visc_fp32_pair_inexact": learned,
            "members": {str(k): results[k] for k in order},
            "host_build_s": round(gen_s, 1),
            "clocks": clocks.summary()}
    print(json.dumps(line))


def _with(pkg, p, **kw):
    q = pkg.abi.default_params(**{f: getattr(p, f) for f, _ in p._fields_ if f != "reserved"})
    for k, v in kw.items():
        setattr(q, k, v)
    return q


def thermo_cpu_baseline(pkg, mesh, fields, params, seconds=15.0, threads=None):
    """The oracle's solve_3D_heat_equation (OpenMP column loop on all host cores) stepped on the
    same workload until `seconds` have passed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    orc = oracle.Oracle(mesh)
    f = dict(fields)
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds and steps < 100:
        T, n, rc, _ = orc.solve_3D_heat_equation(f, params)
        f = dict(f, Ti=T)
        steps += 1
    elapsed = time.perf_counter() - t0
    return {"value": round(steps * mesh.nV / elapsed, 1), "unit": THERMO_UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} time steps of the same workload in {elapsed:.1f} s"}


def run_thermo_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    pkg = __graft_entry__.load_package()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    mesh, fields, p = pkg.geometry.thermo_case(seed=0)
    vals = []
    for i in range(args.warmup + args.steps):
        c = thermo_cpu_baseline(pkg, mesh, fields, p, seconds=args.cpu_seconds)
        if i >= args.warmup:
            vals.append(c)
    v = statistics.mean(c["value"] for c in vals)
    line = {"metric": THERMO_METRIC, "value": round(v, 1), "unit": THERMO_UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000.0 * mesh.nV / v, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic fields from seeded smooth random fields on a generated mesh (no files)",
            "config": {"workload": THERMO_WORKLOAD, "nV": mesh.nV, "nz": mesh.nz},
            "impl": "reference",
            "cpu_baseline": {"value": round(v, 1), "unit": THERMO_UNIT, "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": round(v, 1), "unit": THERMO_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference is Fortran; this arm times the project's C restatement of its algorithm"}
    print(json.dumps(line))


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle


def accuracy_summary(plain, learned, ref_info, head_name, u_plain, err_ref):
    """Every path's velocity error against the FP64 reference solution, and the target in words."""
    if ref_info is None:
        return {"reference": None, "statement": "no FP64 reference solution: every tolerance tried diverged"}
    out = {"reference": ref_info,
           "rel_l2_vs_fp64_reference": {f"plain_{k}": err_ref(u_plain[k]) for k in u_plain}}
    if learned:
        for k, v in learned.items():
            if isinstance(v, dict) and "rel_l2_vs_fp64_reference" in v:
                out["rel_l2_vs_fp64_reference"][f"learned_{k}"] = v["rel_l2_vs_fp64_reference"]
    tight = (learned or {}).get("tight_tolerance_pair", {})
    T = ref_info["picard_tol"]
    errs = out["rel_l2_vs_fp64_reference"]
    e0, eh = errs["plain_fp64"], errs.get(head_name)
    parts = [f"At the benchmark's Picard tolerance (1e-4 on the squared relative change) every path, plain FP64 "
             f"included, stops {min(errs.values()):.1e} to {max(errs.values()):.1e} from the FP64 reference "
             f"solution (plain FP64 {e0:.1e}, headline {eh:.1e}; reference: Picard tolerance {T:g}, Krylov rtol "
             f"1e-12), so the 1e-6 target is not met at that tolerance, by any path."]
    for k in ("learned_fp32_pair_inexact", "learned_fp32_pair"):
        lt = tight.get(k, {})
        if "speedup_vs_plain_fp64" in lt:
            met = lt["rel_l2_vs_fp64_reference"] <= 1e-6
            parts.append(f"Run to the reference's own tolerance {T:g}, {k.replace('_', ' ')} is "
                         f"{lt['rel_l2_vs_fp64_reference']:.1e} from the reference solution (plain FP64 "
                         f"{tight['plain_fp64']['rel_l2_vs_fp64_reference']:.1e}) at "
                         f"{lt['speedup_vs_plain_fp64']:.2f}x the plain FP64 solves/s: the 1e-6 target is "
                         f"{'met' if met else 'not met'}.")
    failed = ", ".join("%g" % t["picard_tol"] for t in ref_info["tried"][:-1]) or "none"
    parts.append(f"Tighter Picard tolerances ({failed}) end in the reference's divergence stop on this channel, "
                 f"and on the way its divergence control raises eps0^2 (relaxation {ref_info['relax_applied']} "
                 f"applied to reach {T:g}), which changes the viscosity law itself; so the solutions that different "
                 f"starts reach differ by ~1e-2 even at {T:g}.  The dome (--workload dome) converges "
                 f"without such steps and is where the 1e-6 target is measured.")
    out["statement"] = " ".join(parts)
    return out


def oracle_full_solve(pkg, mesh, ice, params, threads=None):
    """One complete DIVA solve by the oracle (OpenMP on all host cores): wall time, Picard and Krylov
    counts and the velocity (u, v) pairs."""
    oracle = _oracle()
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    orc = oracle.Oracle(mesh)
    p = _with(pkg, params)
    st = pkg.new_diva_state(mesh.nTri, mesh.nz, with_3d=False)
    t0 = time.perf_counter()
    nv, na, stats = orc.solve_DIVA(ice, st, p)
    secs = time.perf_counter() - t0
    return {"seconds": secs, "picard_its": nv, "krylov_its": na, "status": stats["status"], "cores": threads,
            "u": np.r_[st["u_vav_b"], st["v_vav_b"]]}


def cpu_baseline(pkg, mesh, ice, params, threads=None):
    """The oracle timed on one full solve of the benchmark channel (no extrapolation)."""
    full = oracle_full_solve(pkg, mesh, ice, params, threads)
    d = {"value": round(1.0 / full["seconds"], 6), "unit": UNIT, "cores": full["cores"], "kind": "port",
         "sample": f"full solve: {full['picard_its']} Picard / {full['krylov_its']} Krylov iterations in "
                   f"{full['seconds']:.1f} s (status {full['status']})",
         "picard_its": full["picard_its"], "krylov_its": full["krylov_its"], "seconds": round(full["seconds"], 2)}
    return d, full["u"]


def run_reference(args):
    """The reference arm: the oracle (the CPU restatement of the reference's algorithm) on the host
    cores.  One full solve is measured first; each timed step is then a bounded sample -- the first
    Picard iterations of the same solve -- whose rate is scaled by the Krylov iterations of that full
    solve, measured in this run."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    pkg = __graft_entry__.load_package()
    oracle = _oracle()
    oracle.build()
    mesh, ice, params = pkg.geometry.channel_case(seed=0)
    full = oracle_full_solve(pkg, mesh, ice, params)
    orc = oracle.Oracle(mesh)
    vals = []
    for i in range(args.warmup + args.steps):
        p = _with(pkg, params, visc_it_nit=args.ref_sample_picard - 1)
        st = pkg.new_diva_state(mesh.nTri, mesh.nz, with_3d=False)
        t0 = time.perf_counter()
        nv, na, _ = orc.solve_DIVA(ice, st, p)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            vals.append((na / full["krylov_its"]) / dt)
    v = statistics.mean(vals)
    sample = (f"first {args.ref_sample_picard} Picard iterations of the solve per step, scaled by the "
              f"{full['krylov_its']} Krylov iterations of a full solve measured in this run "
              f"({full['picard_its']} Picard iterations, {full['seconds']:.1f} s = "
              f"{1.0 / full['seconds']:.4f} solves/s)")
    line = {"metric": METRIC, "value": round(v, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000.0 / v, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic MISMIP+-shaped channel from formulas (no files)",
            "config": {"workload": "DIVA channel 640x80 km, cold start, Schoof2005, Picard 1e-4, BiCGStab/Jacobi",
                       "nV": mesh.nV, "nTri": mesh.nTri, "nz": mesh.nz},
            "impl": "reference",
            "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": full["cores"], "kind": "port",
                             "sample": sample},
            "full_solve": {"value": round(1.0 / full["seconds"], 6), "unit": UNIT, "seconds": round(full["seconds"], 2),
                           "picard_its": full["picard_its"], "krylov_its": full["krylov_its"]},
            "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference is Fortran with PETSc and has no compiler or PETSc here; this arm times the "
                    "project's C restatement of its algorithm"}
    print(json.dumps(line))


def run_probe(args):
    """Small fixed invocations of one kernel family, for profiler captures (no JSON line).

    krylov, krylov_pair: the DIVA channel (58k vertices), one Picard iteration of a cold-start
    solve (FP64, or double-word Krylov) with the Krylov solve capped at 200 iterations; host-loop
    mode, so the persistent BiCGStab runs as one plain cooperative launch.
    gnn: forward and gradient of the learned-start network on a 3-regular graph of 262,144 nodes."""
    os.environ["UFE_NO_GRAPH"] = "1"
    pkg = __graft_entry__.load_package()
    pkg.build()
    if args.probe == "solve":
        # one channel solve of the headline's kernel mix (double-word Krylov, inexact Picard) in
        # host-loop mode, after one warm-up solve: the launch list names every kernel of the path
        mesh, ice, params = pkg.geometry.channel_case(seed=0)
        p = _with(pkg, params, precision=pkg.abi.PREC_FP32_PAIR, krylov_forcing=args.forcing,
                  visc_it_nit=args.picard_nit)
        with pkg.VelocitySolver(mesh) as s:
            s.ice_upload(ice)
            for _ in range(2):
                st = s.solve_resident(p, diva=True, cold_start=True)
        print(json.dumps({"probe": "solve", "picard_its": st["n_visc_its"], "krylov_its": st["n_Axb_its"],
                          "device_ms": round(st["device_ms"], 1)}))
        return
    if args.probe == "big":
        # the largest member size of the mixed ensemble (400k vertices; the Krylov matrix, ~0.25 GB,
        # exceeds L2): one DIVA Picard iteration in host-loop mode with the Krylov solve capped at
        # 200 iterations, then the persistent kernels timed by CUDA events over 200 iterations
        mesh = pkg.geometry.mixed_ensemble_mesh(args.big_nv, seed=7)
        ice, p0 = pkg.geometry.mixed_ensemble_member(mesh, 7)
        out = {"nV": mesh.nV, "nTri": mesh.nTri}
        with pkg.VelocitySolver(mesh) as s:
            s.ice_upload(ice)
            for name, prec in (("fp64", pkg.abi.PREC_FP64), ("fp32_pair", pkg.abi.PREC_FP32_PAIR)):
                p = _with(pkg, p0, visc_it_nit=0, krylov_max_it=200, precision=prec)
                st = s.solve_resident(p, diva=True, cold_start=True)
                us_it = s.profile_krylov_persistent(prec, 200)
                us3, (nb, nnzb) = s.profile_krylov_kernels(pkg.abi.PREC_FP64, repeats=20)
                bytes_it = 2 * (nnzb * 36 + (nb + 1) * 4 + 2 * 16 * nb) + 15 * 16 * nb
                bytes_p = nnzb * (32 + 4) + (nb + 1) * 4 + nb * 7 * 16
                out[name] = {"krylov_its": st["n_Axb_its"], "us_per_iteration": round(us_it, 2),
                             "algorithmic_bytes_per_iteration": int(bytes_it),
                             "achieved_gbs": round(bytes_it / (us_it * 1e-6) / 1e9, 1)}
                out["three_kernel_fp64_us"] = [round(float(x), 2) for x in us3]
                out["k_p_spmv_fp64_gbs"] = round(bytes_p / (us3[0] * 1e-6) / 1e9, 1)
                out["blocks_2x2"] = int(nnzb)
        peaks, kind = measured_peaks()
        out["hbm_peak_gbs"] = peaks.get("hbm_gbs")
        print(json.dumps(out))
        return
    if args.probe in ("krylov", "krylov_pair"):
        mesh, ice, params = pkg.geometry.channel_case(seed=0)
        p = _with(pkg, params, visc_it_nit=0, krylov_max_it=200,
                  precision=pkg.abi.PREC_FP32_PAIR if args.probe == "krylov_pair" else pkg.abi.PREC_FP64)
        with pkg.VelocitySolver(mesh) as s:
            for _ in range(2):
                s.ice_upload(ice)
                st = s.solve_resident(p, diva=True, cold_start=True)
            print(f"probe krylov: {st['n_visc_its']} Picard, {st['n_Axb_its']} Krylov iterations", file=sys.stderr)
    else:
        n = 1 << 18
        i = np.arange(n)
        nbr = np.stack([i ^ 1, (i + 2) % n, (i - 2) % n], axis=1).astype(np.int32)
        rng = np.random.default_rng(0)
        x = rng.normal(size=(n, 16)).astype(np.float32)
        tgt = rng.normal(size=(n, 3)).astype(np.float32)
        w = np.full(n, 1.0 / n, np.float32)
        with pkg.ColumnSolver() as s:
            net = pkg.LearnedStart(s, seed=1)
            for _ in range(3):
                net.forward(nbr, x)
                loss, _ = net.loss_grad(nbr, x, tgt, w)
            net.close()
        print(f"probe gnn: loss {loss:.4f}", file=sys.stderr)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--forcing", type=float, default=0.1,
                    help="krylov_forcing of the inexact-Picard path (the early linear solves' residual reduction)")
    ap.add_argument("--picard-nit", type=int, default=200,
                    help="visc_it_nit of every channel path (a limit only: the tolerance ends the solves)")
    ap.add_argument("--mixed-train", type=int, default=12,
                    help="mixed-size ensemble: training geometries of the learned start (20k-60k vertices; 0: no learned path)")
    ap.add_argument("--mixed-epochs", type=int, default=60)
    ap.add_argument("--mixed-mode", choices=["sequential", "side_by_side"], default="sequential",
                    help="mixed-size ensemble: members one after another with the persistent kernels, or side by side")
    ap.add_argument("--ref-tols", type=float, nargs="+", default=[1e-10, 1e-9, 1e-8, 1e-7, 1e-6],
                    help="Picard tolerances tried, tightest first, for the FP64 reference solution")
    ap.add_argument("--ref-sample-picard", type=int, default=4,
                    help="Picard iterations per timed step of the reference arm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mixed-steps", type=int, default=1,
                    help="solves of the FP32+refinement path measured beside the headline")
    ap.add_argument("--dome-tight", type=float, default=1e-15, help="the tight Picard tolerance of --workload dome")
    ap.add_argument("--dome-ref-tol", type=float, default=1e-16, help="Picard tolerance of the dome's reference solution")
    ap.add_argument("--dome-epochs", type=int, default=200)
    ap.add_argument("--thick-res", type=float, default=1.25e3,
                    help="mesh spacing [m] of --workload thickness (1.25 km: about 410k vertices)")
    ap.add_argument("--workload", default="diva", choices=["diva", "thermo", "learned", "ensemble", "mixed", "dome", "icestream",
                                                         "thickness"],
                    help="diva: the headline velocity solve; thermo: the batched column thermodynamics; "
                         "learned: the learned Picard start on the SSA ensemble")
    ap.add_argument("--ens-members", type=int, default=12)
    ap.add_argument("--mixed-members", type=int, default=64,
                    help="members of the mixed-size DIVA ensemble (--workload mixed)")
    ap.add_argument("--ens-min", type=int, default=20000)
    ap.add_argument("--ens-max", type=int, default=120000)
    ap.add_argument("--learned-variants", type=int, default=8,
                    help="channel variants the learned start trains on before the timed region (0: skip)")
    ap.add_argument("--learned-nv", type=int, default=30000)
    ap.add_argument("--learned-train", type=int, default=256)
    ap.add_argument("--learned-test", type=int, default=32)
    ap.add_argument("--learned-epochs", type=int, default=40)
    ap.add_argument("--learned-lr", type=float, default=2e-3)
    ap.add_argument("--learned-err-members", type=int, default=8,
                    help="held-out members also solved to 1e-8 as the reference for the velocity errors")
    ap.add_argument("--thermo-steps", type=int, default=100, help="time steps per thermodynamics run")
    ap.add_argument("--big-nv", type=int, default=400_000, help="vertices of the --probe big mesh")
    ap.add_argument("--probe", choices=["krylov", "krylov_pair", "gnn", "big", "solve"], default=None,
                    help="run one small fixed case of a kernel family for a profiler capture and exit")
    args = ap.parse_args()
    if args.probe:
        run_probe(args)
    elif args.workload == "thermo":
        (run_thermo_reference if args.impl == "reference" else run_thermo)(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.workload == "dome":
        run_dome(args)
    elif args.workload == "icestream":
        run_icestream(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "mixed":
        run_mixed(args)
    elif args.workload == "thickness":
        run_thickness(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
