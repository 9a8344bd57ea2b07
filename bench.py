"""Benchmark of the per-step contact solve on GB300.

One bench "step" is one advance() of the solver: a full time step of the
Newton loop (LBVH rebuild and refits, contact detection and assembly,
block-Jacobi PCG, CCD and strain-limit line search) over the stacked-sheets
workload: 8 cloth sheets of 128 x 128 vertices (131,072 vertices, 254,016
triangles), seeded rotations and offsets, 2 cm apart above a fixed 0.6 m
cube, dt = 0.01 s, from t = 0.

Metric: Newton steps/s (Newton iterations completed / device time inside
advance()), with PCG ms-to-tolerance (relative L1 residual 1e-3) per solve.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* ours: W untimed steps, then the scene is re-initialized at t = 0 and K
  steps are timed with CUDA events on the library's stream, the L2 flushed
  (a 256 MiB write) before each step. `e2e` re-runs the same K steps from
  t = 0 through the C ABI the reference's driver calls per frame
  (update_constraint from host memory, advance, fetch to host memory), timed
  on the host clock. The CPU oracle (an OpenMP restatement of the same step,
  all host cores) is timed on the first steps of the same run as
  `cpu_baseline`.
* reference: the CPU restatement of the reference's step on the host cores,
  on the same workload and metric; each step is one advance() and the run
  stops after a bounded time.
* batched_pcg: the batched-scenes workload, 256 uneven cloth drops (sides
  16-96, sphere or box colliders). Their Newton systems are solved in one
  launch per autotuned team size, against one launch per system
  (ppf_gb300.batch).
* batched_steps: the same drops stepped whole for --batch-steps time steps
  from t = 0, one solver per scene, overlapped by host threads
  (ppf_gb300.multi), against one scene after another on the first steps.
* N > 1 (torchrun): replicas only. Each rank steps its own copy of the
  scene (seed = rank); value = Newton iterations of all ranks / max time.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
# hardware work queues for the batched scenes' streams, before CUDA starts
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
sys.path.insert(0, str(ROOT / "ppf-contact-solver_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "Newton steps/s (block-Jacobi PCG to rel. residual 1e-3)"
UNIT = "newton_iters/s"
WORKLOADS = {
    "stacked_sheets": ("stacked_sheets: 8 x 128x128 cloth sheets over a 0.6 m cube that is a "
                       "static collision mesh"),
    "sphere_field": ("sphere_field: one 1024x1024 cloth (1,048,576 vertices) dropped over 50 "
                     "fixed spheres of seeded radii 0.02-0.1 m"),
    "sphere_field_512": ("sphere_field_512: the same drop with a 512x512 cloth (262,144 "
                         "vertices), the small case for DRAM counters"),
    "twisted_tube": ("twisted_tube: a 256 x 512 tube (131,072 vertices), both end rings pinned "
                     "and turned at +-2 rad/s"),
    "cloth_sphere": ("cloth_sphere: one 64x64 cloth (4,096 vertices) dropped from 1 m onto a "
                     "fixed sphere of radius 0.3 m"),
}
WORKLOAD = WORKLOADS["stacked_sheets"]
L2_FLUSH_BYTES = 256 << 20
CPU_SAMPLE_SECONDS = 20.0
REF_BUDGET_SECONDS = 150.0


def _env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def _iteration_graph_stats(lib):
    import ctypes as C

    out = (C.c_ulonglong * 4)()
    lib.ppf_iteration_graph_stats(out)
    return [int(v) for v in out]


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _bytes_per_iter(fixed_blocks: int, dyn_blocks: int, n: int) -> int:
    """Algorithmic HBM bytes of one block-Jacobi PCG iteration: every unique
    upper-triangle block once (36 B value + 4 B column), 4 B of row pointer
    and 15 fp32 streams of 3 floats per vertex (SpMV: p in, Ap out; update:
    p, Ap, x, r, P^-1 (3 vectors) in, x, r, z out; direction: z, p in, p
    out), plus the scalar."""
    return 40 * fixed_blocks + 40 * dyn_blocks + 184 * n + 4


def aggregate(dist, device, seconds_or_ms: float, newton: int):
    """Whole-job numbers of a replicas run: the slowest rank's time and the
    Newton iterations of all ranks (one scene per rank, no data-path
    collective)."""
    import torch

    t = torch.tensor([seconds_or_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(newton)], dtype=torch.float64, device=device)
    dist.all_reduce(n)
    return float(t.item()), int(n.item())


def build_scene(seed: int = 0, workload: str = "stacked_sheets"):
    from ppf_gb300 import scenes

    if workload == "sphere_field":
        return scenes.sphere_field(1024, 50, seed=seed, dt=0.01)
    if workload == "sphere_field_512":
        return scenes.sphere_field(512, 50, seed=seed, dt=0.01)
    if workload == "twisted_tube":
        return scenes.twisted_tube(256, 512)
    if workload == "cloth_sphere":
        return scenes.cloth_sphere(64, dt=0.01)
    return scenes.stacked_sheets(128, 8, seed=seed, dt=0.01)


def run_ours(args, rank, local_rank, world):
    import ctypes as C

    import numpy as np
    import torch

    from ppf_gb300 import abi
    from ppf_gb300.session import Session

    os.environ.setdefault("PPF_RETURN_ON_FATAL", "1")
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    sc, motion = build_scene(seed=rank, workload=args.workload)
    curr0, prev0 = sc.positions()
    param0 = abi.ParamSet.from_buffer_copy(sc.param.contents)

    def restart():
        sc.set_positions(curr0, prev0)
        C.memmove(C.addressof(sc.param.contents), C.addressof(param0), C.sizeof(param0))
        return Session(sc, motion)

    s = restart()
    lib = s.lib
    for _ in range(args.warmup):
        r = s.step(fetch=False)
        if not r.success():
            raise RuntimeError(f"warm-up step failed: {r.as_dict()}")
    # the project's autotuner picks each traversal kernel's leaf-test form on
    # the warmed-up state (outside the timed region)
    tune_modes = (C.c_ubyte * 6)()
    if args.no_autotune:
        # the library's defaults (profiling runs: under a profiler the
        # autotuner's timings say nothing about the real choice)
        lib.ppf_get_tuning.argtypes = [C.POINTER(C.c_ubyte)]
        lib.ppf_get_tuning(tune_modes)
    else:
        lib.ppf_autotune.argtypes = [C.POINTER(C.c_ubyte)]
        if lib.ppf_autotune(tune_modes) != 0:
            raise RuntimeError("autotune failed")
    tuning = dict(zip(("detect_vertex", "detect_edge", "ccd_vertex", "ccd_mesh_vertex",
                       "ccd_edge", "isect"),
                      ("on the spot" if m else "warp rounds" for m in tune_modes)))

    # ---- device-timed region -------------------------------------------------
    s = restart()
    stream = torch.cuda.ExternalStream(lib.ppf_stream())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    newton = pcg_iters = 0
    pcg_ms_all, pcg_iters_all, pcg_bytes, solve_bytes, per_solve = [], [], 0, [], []
    max_contacts = 0
    sampler = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    launches0 = lib.ppf_kernel_launches()
    graph0 = _iteration_graph_stats(lib)
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[k][0].record(stream)
        r = s.step(fetch=False)
        ev[k][1].record(stream)
        if not r.success():
            raise RuntimeError(f"step {k} failed: {r.as_dict()}")
        st = s.stats()
        newton += st.newton_iters
        pcg_iters += st.pcg_iters_total
        max_contacts = max(max_contacts, st.max_contacts)
        for i in range(min(st.pcg_solves, abi.STATS_MAX_SOLVES)):
            b = _bytes_per_iter(st.fixed_blocks, st.dyn_blocks[i], st.vertices)
            pcg_ms_all.append(st.pcg_ms[i])
            pcg_iters_all.append(st.pcg_iters[i])
            pcg_bytes += b * st.pcg_iters[i]
            solve_bytes.append(b * st.pcg_iters[i])
            per_solve.append([k, int(st.pcg_iters[i]), round(float(st.pcg_ms[i]), 3),
                              int(st.dyn_blocks[i])])
    torch.cuda.synchronize()
    launches = int(lib.ppf_kernel_launches() - launches0)
    graph = {k: b - a for k, a, b in zip(("direct", "captures", "replays", "repeats"), graph0,
                                         _iteration_graph_stats(lib))}
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    # the flush runs between the events' predecessor and start: not timed
    if dist:
        total_ms, newton_all = aggregate(dist, "cuda", total_ms, newton)
    else:
        newton_all = newton
    value = newton_all / (total_ms / 1e3)

    # ---- end to end through the C ABI, host buffers --------------------------
    s = restart()
    n = sc.vertex_count
    # the bytes update_constraint, advance and fetch copy between host and
    # device, counted by the library itself (ppf_transfer_bytes)
    lib.ppf_transfer_bytes.argtypes = [C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]
    lib.ppf_transfer_bytes.restype = None
    h0, d0 = C.c_ulonglong(), C.c_ulonglong()
    h1, d1 = C.c_ulonglong(), C.c_ulonglong()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e2e_newton = 0
    first_step_x = None   # the GPU's positions after the first timed step
    contact_state = None  # the state after the first step with self-contact
    lib.ppf_transfer_bytes(C.byref(h0), C.byref(d0))
    t0 = time.perf_counter()
    for k in range(args.steps):
        lib.update_constraint(sc.constraint)
        r = s.step(fetch=True)
        if not r.success():
            raise RuntimeError(f"e2e step {k} failed: {r.as_dict()}")
        st = s.stats()
        e2e_newton += st.newton_iters
        if k == 0:
            first_step_x = sc.positions()[0]
        if contact_state is None and st.max_dyn_blocks > 0:
            contact_state = (k, *sc.positions(),
                             abi.ParamSet.from_buffer_copy(sc.param.contents))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    lib.ppf_transfer_bytes(C.byref(h1), C.byref(d1))
    h2d = (h1.value - h0.value) // args.steps
    d2h = (d1.value - d0.value) // args.steps
    e2e_value = e2e_newton / e2e_s
    if dist:
        e2e_s, e2e_all = aggregate(dist, "cuda", e2e_s, e2e_newton)
        e2e_value = e2e_all / e2e_s

    # ---- roofline of the dominant kernel (the persistent PCG) ----------------
    peak, peak_kind = _peaks()
    pcg_ms_total = sum(pcg_ms_all)
    achieved = pcg_bytes / (pcg_ms_total / 1e3) / 1e9 if pcg_ms_total > 0 else 0.0
    traffic = None
    tname = {"stacked_sheets": "pcg_stacked_sheets_traffic.json",
             "sphere_field": "pcg_sphere_field_traffic.json",
             "sphere_field_512": "pcg_sphere_field_traffic.json"}.get(args.workload, "")
    tfile = ROOT / "profiles" / tname
    if tname and tfile.is_file() and pcg_iters_all:
        # DRAM bytes per iteration from one ncu capture of this workload (the
        # sphere fields: of the 512 x 512 drop, scaled by vertices), times the
        # mean iterations per launch of this run
        t = json.loads(tfile.read_text())
        per_iter = t.get("dram_bytes_per_iteration")
        if per_iter:
            scale = n / t["vertices"] if "vertices" in t else 1.0
            traffic = int(per_iter * scale * (sum(pcg_iters_all) / len(pcg_iters_all)))
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                "kernel": "k_pcg (persistent block-Jacobi PCG, one launch per solve)",
                "peak_kind": peak_kind,
                "bytes_per_launch_mean": (sum(solve_bytes) / len(solve_bytes)
                                          if solve_bytes else 0)}
    ms_solve = sorted(pcg_ms_all)

    def pct(a, q):
        return a[min(len(a) - 1, int(q * len(a)))] if a else None

    out = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generator)",
        "config": {"workload": WORKLOADS[args.workload], "vertices": n, "dt": 0.01,
                   "time_steps": args.steps, "from": "t = 0 after a separate warm-up",
                   "l2": "256 MiB flush before every timed step",
                   "parallelism": "replicas" if world > 1 else "single"},
        "pcg": {"solves": len(pcg_ms_all), "ms_to_tol_median": pct(ms_solve, 0.5),
                "ms_to_tol_p90": pct(ms_solve, 0.9),
                "iters_median": pct(sorted(pcg_iters_all), 0.5),
                "iters_total": pcg_iters, "ms_total": round(pcg_ms_total, 3),
                "share_of_step": round(pcg_ms_total / total_ms, 4) if total_ms else None,
                "per_solve": {"fields": ["step", "iters", "ms", "contact_blocks"],
                              "rows": per_solve[:64]}},
        "newton_iters": newton_all, "max_contacts": max_contacts,
        "contact": {"solves": len(per_solve),
                    "solves_with_contact_blocks": sum(1 for r in per_solve if r[3] > 0),
                    "contact_blocks_max": max((r[3] for r in per_solve), default=0),
                    "max_active_contacts": max_contacts},
        "roofline": roofline,
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "bytes": "counted by the library at its host<->device copies "
                         "(ppf_transfer_bytes), mean per timed step",
                "path": "update_constraint + advance + fetch (C ABI, host DataSet)"},
        "gpu_launches": launches,
        # Newton iterations of the timed steps as one CUDA graph each: run
        # directly under a new capture key, captured, replayed, repeated
        # after a capacity overran
        "iteration_graph": graph,
        "clocks": clocks,
        "tuning": tuning,
    }
    if rank == 0 and args.precond_steps > 0:
        out["preconditioners"] = compare_preconditioners(restart, sc, lib, stream,
                                                         args.precond_steps)
    if rank == 0 and args.batch_count > 0:
        # the batched-scenes workload: many uneven drops' Newton systems
        # solved in one launch per team size (autotuned), against one launch
        # per system; outside the timed region of the headline
        from ppf_gb300 import batch

        out["batched_pcg"] = batch.run_bench(args.batch_count, seed=0, reps=3)
        # the same drops stepped whole (every stage), together: one solver
        # and iteration graph per scene, host threads overlapping them
        from ppf_gb300 import multi

        out["batched_steps"] = multi.run_bench(args.batch_count, steps=args.batch_steps, seed=0)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"], first_o = cpu_baseline(sc, curr0, prev0, param0,
                                                    CPU_SAMPLE_SECONDS)
        out["parity"] = parity_check(sc, lib, first_step_x, first_o, contact_state)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def compare_preconditioners(restart, sc, lib, stream, steps):
    """The same first `steps` time steps from t = 0 with each preconditioner:
    block-Jacobi (the reference's default and the headline's), the
    reference's aggregate additive Schwarz (ParamSet precond = 1) with its
    default two levels and with one, the
    first-order and FSAI factored preconditioners and, when the package holds
    trained weights, the learned one. Each solve runs to the same 1e-3
    relative residual. Device time per step from CUDA events on the
    library's stream."""
    import torch

    from ppf_gb300 import abi

    from ppf_gb300 import learned

    # (name, ParamSet precond, extension kind, ParamSet schwarz_levels)
    kinds = [("block_jacobi", 0, abi.PRECOND_BLOCK_JACOBI, 2),
             ("schwarz_two_level", 1, abi.PRECOND_BLOCK_JACOBI, 2),
             ("schwarz_one_level", 1, abi.PRECOND_BLOCK_JACOBI, 1),
             ("first_order_factor", 0, abi.PRECOND_FIRST_ORDER, 2),
             ("fsai", 0, abi.PRECOND_FSAI, 2)]
    out = {"steps": steps, "from": "t = 0", "tolerance": "1e-3 relative L1 residual"}
    if learned.WEIGHTS_FILE.exists():
        learned.use_weights()
        kinds.append(("learned", 0, abi.PRECOND_LEARNED, 2))
        out["learned_weights"] = learned.WEIGHTS_FILE.name
    for name, precond, kind, levels in kinds:
        sc.param.contents.precond = precond
        sc.param.contents.schwarz_levels = levels
        s = restart()
        sc.param.contents.precond = precond
        sc.param.contents.schwarz_levels = levels
        s.set_preconditioner(kind, 0.5)
        ev = []
        newton, fallbacks, ms, iters = 0, 0, [], []
        try:
            torch.cuda.synchronize()
            for k in range(steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                r = s.step(fetch=False)
                e1.record(stream)
                ev.append((e0, e1))
                if not r.success():
                    raise RuntimeError(f"{name} step {k} failed: {r.as_dict()}")
                st = s.stats()
                newton += st.newton_iters
                fallbacks += st.fallbacks
                for i in range(min(st.pcg_solves, abi.STATS_MAX_SOLVES)):
                    ms.append(float(st.pcg_ms[i]))
                    iters.append(int(st.pcg_iters[i]))
            torch.cuda.synchronize()
        finally:
            s.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
            sc.param.contents.precond = 0
            sc.param.contents.schwarz_levels = 2
        total = sum(a.elapsed_time(b) for a, b in ev)
        ms.sort()
        it = sorted(iters)
        out[name] = {"newton_iters_per_s": round(newton / (total / 1e3), 2),
                     "newton_iters": newton,
                     "pcg_ms_to_tol_median": round(ms[len(ms) // 2], 3),
                     "pcg_ms_to_tol_p90": round(ms[min(len(ms) - 1, int(0.9 * len(ms)))], 3),
                     "pcg_iters_median": it[len(it) // 2], "pcg_ms_total": round(sum(ms), 2),
                     "fallbacks_to_block_jacobi": fallbacks}
    if "learned" not in out:
        out["learned"] = "no trained weights in the package"
    return out


def parity_check(sc, lib, first_gpu, first_oracle, contact_state):
    """The oracle as checker of this run, outside every timed region.

    * first timed step: the oracle's first step of the CPU-baseline sample
      starts from the same state as the GPU's first timed step (t = 0); the
      positions after it must agree within 1e-5 relative.
    * first self-contact Newton system: the GPU state after the first timed
      step that assembled contact blocks is loaded into both the library and
      the oracle, each assembles and solves its first Newton system, and the
      pair sets are compared with the pairs within 1e-6 * ghat of the gap
      threshold listed (oracle/parity.py)."""
    import ctypes as C

    import numpy as np

    from oracle import binding, parity
    from ppf_gb300.session import Session

    out = {}
    if first_gpu is not None and first_oracle is not None:
        err = float(np.abs(first_gpu - first_oracle).max()) / float(np.abs(first_oracle).max())
        out["first_timed_step"] = {"rel_err": err, "tol": 1e-5, "pass": err <= 1e-5}
    if contact_state is None:
        out["first_contact_system"] = "no self-contact within the timed steps"
        return out
    k, curr, prev, prm = contact_state
    sc.set_positions(curr, prev)
    C.memmove(C.addressof(sc.param.contents), C.addressof(prm), C.sizeof(prm))
    Session(sc)
    n = sc.vertex_count
    dx = np.empty(3 * n, np.float32)
    it, rr = C.c_uint(), C.c_float()
    st_g = lib.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr))
    sg = binding.product_system(lib, n)
    o = binding.OracleSession(sc)
    st_o, _, _, _ = o.newton_system()
    so = o.system()
    res = parity.compare_systems(sg, so, curr, sc.array("face"), sc.array("edge"), 1e-3)
    b = so["force"].astype(np.float64).reshape(-1)
    rel = float(np.abs(b - parity.apply_system(so, dx)).sum() / np.abs(b).sum())
    pairs = res["pairs"]
    out["first_contact_system"] = {
        "state": f"after timed step {k}", "pairs": pairs["pairs"],
        "listed_within_1e-6_ghat": pairs["listed"],
        "pair_sets_equal_outside_listed": pairs["equal_outside_listed"],
        "contact_blocks": res["contact_blocks"],
        "fixed_blocks_max_rel_err": res.get("fixed_max_err"),
        "contact_blocks_max_rel_err": res.get("contact_max_err"),
        "force_max_rel_err": res["force_max_err"],
        "gpu_solution_true_rel_residual": rel, "pcg_states": [int(st_g), int(st_o)],
        "pass": bool(pairs["equal_outside_listed"] and res["fixed_max_err"] <= 1e-5
                     and res["force_max_err"] <= 1e-5 and rel < 2e-3)}
    return out


def _oracle_run(sc, curr0, prev0, param0, budget_s, max_steps=None, warmup=0,
                keep_first=False):
    """Steps the CPU oracle from t = 0 until the budget is spent (at least
    one step); returns (newton_iters, seconds, steps) and, with keep_first,
    the positions after the first step."""
    import ctypes as C

    from oracle.binding import OracleSession

    sc.set_positions(curr0, prev0)
    C.memmove(C.addressof(sc.param.contents), C.addressof(param0), C.sizeof(param0))
    o = OracleSession(sc)
    for _ in range(warmup):
        o.step()
    newton, secs, steps = 0, 0.0, 0
    first = None
    while True:
        t = time.perf_counter()
        r = o.step()
        secs += time.perf_counter() - t
        if not r.success():
            raise RuntimeError(f"oracle step failed: {r.as_dict()}")
        newton += o.stats()["newton_iters"]
        steps += 1
        if keep_first and steps == 1:
            first = o.positions()[0]
        if secs >= budget_s or (max_steps is not None and steps >= max_steps):
            break
    if keep_first:
        return newton, secs, steps, first
    return newton, secs, steps


def cpu_baseline(sc, curr0, prev0, param0, budget_s):
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    newton, secs, steps, first = _oracle_run(sc, curr0, prev0, param0, budget_s,
                                             keep_first=True)
    return ({"value": round(newton / secs, 3), "unit": UNIT, "cores": threads, "kind": "port",
             "sample": f"first {steps} time steps of the same workload from t = 0 "
                       f"({newton} Newton iterations, {secs:.1f} s), OpenMP oracle"}, first)


def run_reference(args, rank, local_rank, world):
    if rank != 0:
        return
    from ppf_gb300 import abi

    sc, _ = build_scene(seed=0)
    curr0, prev0 = sc.positions()
    param0 = abi.ParamSet.from_buffer_copy(sc.param.contents)
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    newton, secs, steps = _oracle_run(sc, curr0, prev0, param0, REF_BUDGET_SECONDS,
                                      max_steps=args.steps, warmup=min(args.warmup, 1))
    value = newton / secs
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT,
        "n_gpus": world, "steps": steps, "warmup": min(args.warmup, 1),
        "ms_per_step": round(1e3 * secs / steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generator)",
        "config": {"workload": WORKLOAD, "vertices": sc.vertex_count, "dt": 0.01,
                   "time_steps": steps, "from": "t = 0"},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads,
                         "kind": "port",
                         "sample": f"first {steps} time steps from t = 0 ({newton} Newton "
                                   f"iterations, {secs:.1f} s); the reference's GPU build "
                                   "needs CUDA 12.8 and cargo, neither present"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=120)  # the workload's run length
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the library's default traversal forms and PCG team")
    ap.add_argument("--precond-steps", type=int, default=24,
                    help="time steps of the preconditioner comparison (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=100,
                    help="time steps of the batched drops stepped together")
    ap.add_argument("--batch-count", type=int, default=256,
                    help="uneven drops of the batched-PCG comparison (0: skip)")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="stacked_sheets",
                    help="stacked_sheets (the headline), sphere_field (one 1M-vertex cloth), "
                         "twisted_tube or cloth_sphere (the 64x64 drop)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank, local_rank, world = _env_rank()
    if args.impl == "reference":
        run_reference(args, rank, local_rank, world)
    else:
        run_ours(args, rank, local_rank, world)


if __name__ == "__main__":
    main()
