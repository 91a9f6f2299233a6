"""Benchmark: Born forward + RTM adjoint throughput on one GB300.

One *step* is the hot path over one shot: the Born forward (rtmForward) plus
the RTM adjoint (sourceProp + rtmAdjoint) of configuration c2 (256^3 model,
368^3 compute grid, nt = 2000), i.e. 2 * N_interior * nt cell-updates.

  value  device-timed Gcell-updates/s with every input resident in HBM
  e2e    the same metric through the reference-facing C ABI
         (gpu_funcs_3d.h names) with pinned host buffers, host<->device
         copies inside the timed region, in the call order of
         rtm_zero_op_3d.cc (host_call_ms: each entry point's wall time)
  roofline  achieved GB/s of the dominant kernel (the fused RTM adjoint
         step) against the measured HBM copy bandwidth, and (stream_mix)
         against what plain streaming sustains for the step's own 7 read
         and 3 written arrays
  shot_steps_per_s  time steps of whole shots (Born forward + RTM adjoint)
         per second, over all ranks
  tile_ms_per_launch  per-tile time per launch of each step (with its
         best z segmentation) as the time loops measured them on their own
         steps (the chosen tile in tile_cfg, its z-segment depth in
         tile_zseg)
  fused_fma, exact_coupling  the same loops with fused multiply-add
         arithmetic, and with the Born coupling formed exactly as the
         reference's double expression (bit-identical traces)
  cpu_baseline  the oracle (C restatement of the reference cpuProp) on the
         host cores, on a bounded sample of the same workload

``--impl reference`` times the reference CPU implementation instead (the
compiled reference where it exists on this machine, else the oracle port).
Multi-GPU: shots are independent, so N ranks run N shots (weak scaling);
each step ends with the images summed over the ranks (one NCCL all-reduce,
the only exchange an RTM over shots needs).

``--adjoint exact`` times c2 as its configuration states it instead: the
exact linearised Born pair, the adjoint rebuilding the background from
checkpoints every 50 steps (per-phase times and bytes in the line).

Other configurations print their own line:
  --config c3  one 624^3 shot (512^3 model at 8 m, jt = 2, nt = 2999) per
               level storage (--storage f32,f32fma,bf16,f16; default
               f32,bf16,f16), results compared with the first storage's
  --config c4  48 shots of uneven aperture advanced together (one launch per
               step, time loops as CUDA graphs) against the same shots one
               after another (--storage for the level storage)
  --config c5  least-squares RTM: --steps CG iterations over --shots shots
               of the exact linearised pair (reduced model by default;
               --model-n 384 gives the full 384 x 384 x 256)
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "sc17-born_gb300")
L2_BYTES = 129 * 2 ** 20
FALLBACK_HBM_GBS = 6800.0
# algorithmic bytes per interior cell-update (fp32, compulsory traffic)
BYTES_PER_CELL = {"forward": 32, "source": 16, "adjoint": 40}


def package():
    if "born_gb300" in sys.modules:
        return sys.modules["born_gb300"]
    spec = importlib.util.spec_from_file_location(
        "born_gb300", os.path.join(PKG_DIR, "__init__.py"),
        submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["born_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def workload_module():
    spec = importlib.util.spec_from_file_location(
        "born_gb300_workload", os.path.join(PKG_DIR, "workload.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            d = json.load(open(path))
            for k in ("hbm_gbs", "hbm_GBps", "hbm"):
                if k in d:
                    v = d[k]
                    if isinstance(v, dict):
                        v = v.get("burst", v.get("value"))
                    return float(v), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def traffic_per_cell(kernel: str):
    """DRAM bytes per interior cell-update of a kernel from the committed
    ncu summary (profiles/<kernel>_dram.txt, line 'bytes_per_cell: X')."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_dram.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("bytes_per_cell:"):
            return float(line.split(":")[1])
    return None


class Clocks:
    """Samples SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", "-i", str(self.index),
                     f"--query-gpu={self.Q}", "--format=csv,noheader,nounits"],
                    capture_output=True, text=True, timeout=5).stdout
                self.rows.append([x.strip() for x in out.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for name, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_max(value: float, world: int) -> float:
    """Max of a per-rank value over all ranks (after a barrier)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shot_of_rank(rank: int, nshots: int) -> int:
    """Shots are independent: rank r runs shot r (modulo the shot count)."""
    return rank % max(1, nshots)


def aggregate_rate(cells_per_rank: float, steps: int, t_ms_max: float,
                   world: int) -> float:
    """Whole-job Gcell-updates/s: all ranks' cells over the slowest rank."""
    return world * cells_per_rank * steps / (t_ms_max / 1e3) / 1e9


# ---------------------------------------------------------------------------
def cpu_sample(case, threads: int, kind: str, budget_s: float = 20.0):
    """Gcell-updates/s of the CPU implementation on a truncated-nt sample of
    the same grid: Born forward + source propagation + RTM adjoint."""
    po = oracle_module()
    if kind == "reference" and po.ref_lib() is not None:
        os.environ["ORACLE_REF_THREADS"] = str(threads)
        mk = po.RefProp
    else:
        kind = "port"
        po.set_threads(threads)
        mk = po.PortProp
    n_int = (case["shape"][0] - 8) * (case["shape"][1] - 8) * (case["shape"][2] - 8)

    def run(nt):
        c = dict(case)
        c["nt"] = nt
        t0 = time.perf_counter()
        po.run_case(mk(), c, which="all")
        return time.perf_counter() - t0

    probe_nt = 2
    t = run(probe_nt)
    nt = probe_nt
    if budget_s > 0:
        per_step = t / probe_nt
        nt = int(max(2, min(200, budget_s / max(per_step, 1e-9))))
        t = run(nt)
    rate = 2.0 * n_int * nt / t / 1e9
    return {"value": round(rate, 4), "unit": "Gcell-updates/s", "nt": nt,
            "cores": threads, "kind": "reference" if kind == "reference" else "port",
            "sample": f"{case['name']} grid {case['shape'][2]}x{case['shape'][1]}x"
                      f"{case['shape'][0]}, Born forward + source propagation + "
                      f"RTM adjoint over nt={nt} of {case['nt']} steps "
                      f"({t:.1f} s)"}


def arm_config(case, storage: str, world: int) -> dict:
    """The ``config`` object of the c1/c2 line, printed identically by the
    GPU arm and the reference arm."""
    nz, ny, nx = case["shape"]
    n_int = (nx - 8) * (ny - 8) * (nz - 8)
    return {"workload": f"{case['name']}: 3D Born forward + RTM adjoint, "
            f"compute grid {nx}x{ny}x{nz}, nt={case['nt']}, "
            "random-boundary source reconstruction",
            "grid": [nz, ny, nx], "nt": case["nt"], "jt": case["jts"],
            "interior_cells": n_int, "storage": storage,
            "l2": "inputs larger than L2 (7 x %.0f MB fields)" %
                  (nx * ny * nz * 4 / 1e6),
            "parallelism": f"shots x{world} (one per GPU)" +
            (", image summed over the ranks every step (NCCL all-reduce)"
             if world > 1 else "")}


def oracle_module():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    return pyoracle


def run_reference_arm(args):
    """The reference's CPU path on the host cores: the compiled reference
    cpuProp where it exists on this machine, else the C restatement (the
    oracle port).  The shot's inputs come from the restatement's own
    geometry (pinned bit for bit to the reference's sources), so this arm
    loads no library of the product.  A full c2 step (nt = 2000) takes
    minutes on the CPU, so each timed step is a truncated-nt sample of the
    same shot and ms_per_step is extrapolated from it."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    po = oracle_module()
    wl = workload_module()
    case = wl.prepare_shot(po.Geometry(), args.config, nt=args.nt,
                           n=args.model_n)
    threads = os.cpu_count() or 1
    kind = "reference" if po.ref_lib() is not None else "port"
    # each timed sample gets an equal share of the CPU budget (at least a
    # few seconds); the warm-up samples are two-step runs
    per_sample = max(3.0, args.ref_budget / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_sample(case, threads, kind, budget_s=0.0)
    vals, last = [], None
    for _ in range(args.steps):
        last = cpu_sample(case, threads, kind, budget_s=per_sample)
        vals.append(last["value"])
    v = statistics.median(vals)
    n_int = wl.interior_cells(case["shape"])
    line = {
        "metric": "Gcell-updates/s Born fwd+adj", "value": v,
        "unit": "Gcell-updates/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(2.0 * n_int * case["nt"] / (v * 1e9) * 1e3, 1),
        "ms_per_step_extrapolated": True,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded, shapes of the config)",
        "config": arm_config(case, "f32", world),
        "sample_nt": last["nt"],
        "note": "each timed step is a sample of nt=%d of the %d FD steps of "
                "the shot (Born forward + source propagation + RTM adjoint);"
                " ms_per_step is extrapolated linearly to the full nt" %
                (last["nt"], case["nt"]),
        "cpu_baseline": dict(last, value=v),
        "e2e": {"value": v, "unit": "Gcell-updates/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def run_gpu_arm(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    born = package()
    born.lib()
    wl = workload_module()
    case = wl.prepare_shot(born, args.config, nt=args.nt, n=args.model_n,
                           shot=shot_of_rank(rank, 48))
    nz, ny, nx = case["shape"]
    nt, jt = case["nt"], case["jts"]
    n_int = wl.interior_cells(case["shape"])
    cells_per_step = 2 * n_int * nt

    prop = born.Gb300Prop(dev)
    if args.tile >= 0 or args.zseg > 0:
        prop.set_tiling(args.tile, args.zseg)
    prop.createSpace(case["d"], case["d"], case["d"], 50.0, 0.0005, 0.0005,
                     nx, ny, nz)
    prop.set_storage(args.storage or "f32")
    prop.transferSincTableS(8, jt, case["table_s"])
    prop.transferSincTableD(8, jt, case["table_d"])
    prop.transferSourceFunc(9, case["nt_big"], case["locs_s"], case["src"])
    prop.transferVelFunc1(nx, ny, nz, case["vel1"])
    prop.transferVelFunc2(nx, ny, nz, case["vel2"])
    rec = np.ascontiguousarray(case["rec_in"])
    prop.transferReceiverFunc(case["rec_nx"], case["rec_ny"], case["nt_big"],
                              case["locs_r"], rec)
    prop.check(prop.lib.born_set_reflectivity(prop.h, born.fptr(case["refl"])))
    stream = torch.cuda.ExternalStream(prop.stream, device=dev)

    def device_step(ev=None):
        if ev:
            ev[0].record(stream)
        prop.rtm_forward_device(jt, nt)
        if ev:
            ev[1].record(stream)
        prop.source_prop_device(jt, nt)
        if ev:
            ev[2].record(stream)
        prop.rtm_adjoint_device(jt, nt, swap=1)
        if ev:
            ev[3].record(stream)
        if world > 1:  # the shots' images summed over the ranks (NCCL)
            born.stack_image(prop)

    for _ in range(args.warmup):
        device_step()
    prop.synchronize()
    launches0 = prop.launches
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)]
           for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for k in range(args.steps):
            device_step(evs[k])
        stop.record(stream)
        prop.synchronize()
        torch.cuda.synchronize()
    launches = prop.launches - launches0
    tiles, tile_ms, zsegs = {}, {}, {}
    for mode, name in ((1, "forward"), (0, "source"), (2, "adjoint")):
        cfg, ms = prop.tuned_config(mode)
        tiles[name] = cfg
        zsegs[name] = prop.tuned_zseg(mode)
        # per-tile ms per launch (best z segmentation) as the loop's own
        # refinement measured them
        tile_ms[name] = [round(v, 4) for v in prop.loop_tile_ms(mode)]
    t_ms = start.elapsed_time(stop)
    t_ms = barrier_max(t_ms, world)
    fwd_ms = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps
    src_ms = sum(e[1].elapsed_time(e[2]) for e in evs) / args.steps
    adj_ms = sum(e[2].elapsed_time(e[3]) for e in evs) / args.steps
    value = aggregate_rate(cells_per_step, args.steps, t_ms, world)

    # the same loops with FP32 levels and fused multiply-add arithmetic
    # (within 1.4e-6 relative L2 of the reference order in the tests)
    fused = None
    if (args.storage or "f32") == "f32" and not args.no_fused:
        prop.set_storage("f32fma")
        for _ in range(2):  # warm-up, including the tuner for this storage
            device_step()
        prop.synchronize()
        fev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)]
               for _ in range(2)]
        for k in range(2):
            device_step(fev[k])
        prop.synchronize()
        f_ms = [sum(e[i].elapsed_time(e[i + 1]) for e in fev) / 2
                for i in range(3)]
        fused = {"value": round(cells_per_step / (sum(f_ms) / 1e3) / 1e9, 3),
                 "unit": "Gcell-updates/s", "steps": 2,
                 "forward_ms": round(f_ms[0], 2), "source_ms": round(f_ms[1], 2),
                 "adjoint_ms": round(f_ms[2], 2),
                 "arith": "FP32 levels, fused multiply-add stencil and "
                          "leapfrog (born_set_storage BORN_STORE_F32_FUSED)"}
        prop.set_storage("f32")

    # the same loops with the Born coupling formed exactly as the
    # reference's double expression (traces bit-identical to the reference)
    exact = None
    if (args.storage or "f32") == "f32" and not args.no_fused:
        prop.set_storage("f32exact")
        for _ in range(2):  # warm-up, including the tuner for this storage
            device_step()
        prop.synchronize()
        xev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)]
               for _ in range(2)]
        for k in range(2):
            device_step(xev[k])
        prop.synchronize()
        x_ms = [sum(e[i].elapsed_time(e[i + 1]) for e in xev) / 2
                for i in range(3)]
        exact = {"value": round(cells_per_step / (sum(x_ms) / 1e3) / 1e9, 3),
                 "unit": "Gcell-updates/s", "steps": 2,
                 "forward_ms": round(x_ms[0], 2), "source_ms": round(x_ms[1], 2),
                 "adjoint_ms": round(x_ms[2], 2),
                 "arith": "FP32 reference order, Born coupling as the "
                          "reference's double expression (born_set_storage "
                          "BORN_STORE_F32_EXACT; traces bit-identical)"}
        prop.set_storage("f32")

    # roofline of the dominant kernel: the fused RTM adjoint step
    peak, peak_kind = measured_peak()
    adj_launch_ms = adj_ms / nt
    achieved = BYTES_PER_CELL["adjoint"] * n_int / (adj_launch_ms / 1e3) / 1e9
    tpc = traffic_per_cell("adjoint_step")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": (round(tpc * n_int) if tpc else None),
                "kernel": "step_kernel<adjoint> (fused r+s step, image)",
                "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": BYTES_PER_CELL["adjoint"] * n_int,
                "avg_launch_ms": round(adj_launch_ms, 4)}
    # second denominator: what plain streaming sustains for the adjoint
    # step's own mix of arrays (7 read, 3 written, one grid field each)
    mix = born.stream_mix_gbs(7, 3, nx * ny * nz)
    roofline["stream_mix"] = {"reads": 7, "writes": 3, "gbs": round(mix, 1),
                              "frac": round(achieved / mix, 4)}
    phases = {"forward_ms": round(fwd_ms, 2), "source_ms": round(src_ms, 2),
              "adjoint_ms": round(adj_ms, 2),
              "forward_GBps": round(BYTES_PER_CELL["forward"] * n_int * nt /
                                    (fwd_ms / 1e3) / 1e9, 1),
              "source_GBps": round(BYTES_PER_CELL["source"] * n_int * (nt + 1) /
                                   (src_ms / 1e3) / 1e9, 1)}

    # e2e through the reference-facing C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = e2e_measure(born, case, args, dev, cells_per_step, world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_sample(case, os.cpu_count() or 1, "port",
                         budget_s=args.cpu_budget)

    if rank == 0:
        line = {
            "metric": "Gcell-updates/s Born fwd+adj", "value": round(value, 3),
            "unit": "Gcell-updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if (args.storage or "f32") == "f32" else
                     "f32 arithmetic; levels " + args.storage,
            "data": "synthetic (seeded, shapes of the config)",
            "config": arm_config(case, args.storage or "f32", world),
            # one shot-step: a time step of one shot's Born forward + RTM
            # adjoint (source propagation included), over all ranks
            "shot_steps_per_s": round(world * nt * args.steps / (t_ms / 1e3),
                                      1),
            "roofline": roofline, "phases": phases, "tile_cfg": tiles,
            "tile_zseg": zsegs,
            "tile_ms_per_launch": tile_ms,
            "clocks": clk.summary(), "gpu_launches": launches,
            "e2e": e2e, "cpu_baseline": cpu, "fused_fma": fused,
            "exact_coupling": exact,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def e2e_measure(born, case, args, dev, cells_per_step, world):
    """Steps through the gpu_funcs_3d.h entry points with pinned buffers."""
    import torch
    L = born.lib()
    nz, ny, nx = case["shape"]
    nt, jt = case["nt"], case["jts"]

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
        t.numpy()[...] = a
        return t

    vel1, vel2 = pinned(case["vel1"]), pinned(case["vel2"])
    src = pinned(case["src"])
    rec_in = pinned(case["rec_in"])
    rec_out = pinned(np.zeros_like(case["rec_in"]))
    refl = pinned(case["refl"])
    p0 = pinned(np.zeros(case["shape"], np.float32))
    p1 = pinned(np.zeros(case["shape"], np.float32))
    img = pinned(np.zeros(case["shape"], np.float32))
    zeros_rec = pinned(np.zeros_like(case["rec_in"]))
    locs_s = np.ascontiguousarray(case["locs_s"], np.int32)
    locs_r = np.ascontiguousarray(case["locs_r"], np.int32)
    ts = np.ascontiguousarray(case["table_s"], np.float32)
    fp = lambda t: C.cast(t.data_ptr(), born._fp)  # noqa: E731

    L.setup_cuda(1)
    L.create_gpu_space(case["d"], case["d"], case["d"], 50.0, .0005, .0005,
                       nx, ny, nz)
    L.transfer_sinc_table_s(8, jt, born.fptr(ts))
    L.set_ntblock(50)
    L.transfer_sinc_table_d(8, jt, born.fptr(ts))
    h = L.born_default_handle()
    if args.tile >= 0 or args.zseg > 0:
        L.born_set_tiling(h, args.tile, args.zseg)
    field = nx * ny * nz * 4

    calls = ("transfer_source_func", "transfer_vel_func1", "transfer_vel_func2",
             "transfer_receiver_func", "source_prop", "image_zero",
             "rtm_adjoint", "transfer_receiver_func(zeros)", "rtm_forward")
    call_s = dict.fromkeys(calls, 0.0)

    def step(timed=False):
        # every entry point below returns after its host copies completed,
        # so the wall time between two calls is that call's own time
        tk = [time.perf_counter()]

        def lap():
            if timed:
                tk.append(time.perf_counter())
        # rtm_zero_op::adjoint per shot (rtm_zero_op_3d.cc:249-282)
        L.transfer_source_func(9, case["nt_big"], born.iptr(locs_s), fp(src))
        lap()
        L.transfer_vel_func1(nx, ny, nz, fp(vel1))
        lap()
        L.transfer_vel_func2(nx, ny, nz, fp(vel2))
        lap()
        L.transfer_receiver_func(case["rec_nx"], case["rec_ny"],
                                 case["nt_big"], born.iptr(locs_r), fp(rec_in))
        lap()
        L.source_prop(nx, ny, nz, False, True, fp(p0), fp(p1), jt, 9, nt)
        lap()
        img.zero_()
        lap()
        L.rtm_adjoint(nx, ny, nz, jt, fp(p1), fp(p0), fp(img), 9, nt)
        lap()
        # rtm_zero_op::forward per shot (rtm_zero_op_3d.cc:147-185)
        L.transfer_receiver_func(case["rec_nx"], case["rec_ny"],
                                 case["nt_big"], born.iptr(locs_r),
                                 fp(zeros_rec))
        lap()
        L.rtm_forward(nx, ny, nz, jt, fp(refl), fp(rec_out), 9, nt,
                      case["nt_big"], case["rec_nx"], case["rec_ny"])
        lap()
        rc = L.born_default_status()
        if rc != 0:
            raise RuntimeError(L.born_default_error().decode())
        if timed:
            for k, name in enumerate(calls):
                call_s[name] += tk[k + 1] - tk[k]

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    steps = max(1, args.e2e_steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        step(timed=True)
    t = time.perf_counter() - t0
    t = barrier_max(t, world)
    copy_rates = pinned_copy_gbps(vel1, dev)
    rec_bytes = case["rec_in"].size * 4
    h2d = (2 * field + case["src"].size * 4 + 2 * rec_bytes + field + field)
    d2h = 2 * field + field + rec_bytes
    return {"value": round(world * cells_per_step * steps / t / 1e9, 3),
            "unit": "Gcell-updates/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "steps": steps,
            "api": "gpu_funcs_3d.h entry points, pinned host buffers",
            "host_call_ms": {k: round(v * 1e3 / steps, 2)
                             for k, v in call_s.items()},
            "pinned_copy_GBps": copy_rates}


def pinned_copy_gbps(host, dev, reps=3):
    """torch's own copies of one pinned field each way (CUDA events)."""
    import torch
    d = torch.empty(host.shape, dtype=host.dtype, device=dev)
    out = {}
    for name, dst, src in (("h2d", d, host), ("d2h", host, d)):
        dst.copy_(src, non_blocking=True)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        b.record()
        b.synchronize()
        out[name] = round(reps * host.numel() * 4 / (a.elapsed_time(b) / 1e3)
                          / 1e9, 1)
    return out


def run_exact(args):
    """c2 as its configuration states it: the exact linearised Born pair,
    born_lin_forward along the reflectivity and born_lin_adjoint of the
    traces it made (the source wavefield rebuilt from checkpoints every
    --ckpt steps), device-resident; one step = one forward + one adjoint of
    the shot, 2 * N_interior * nt cell-updates as in the headline line.

    Algorithmic bytes per interior cell and FD step: forward 32 (s and r:
    two levels each, velocity, reflectivity in; two levels out); adjoint 48
    = segment recompute storing A s 20 + adjoint step 28 (w: two levels,
    A s, velocity, image in; w and image out), plus 16 for a checkpointing
    sweep of the background when the forward's checkpoints cannot be reused
    (the line says which); plus 16 B per grid cell per segment for the
    checkpoint stores and 16 for their restores (two levels each) and 12 for
    the final division by v^2 dt^2."""
    import torch
    born = package()
    born.lib()
    wl = workload_module()
    case = wl.prepare_shot(born, args.config, nt=args.nt, n=args.model_n)
    nz, ny, nx = case["shape"]
    nt, jt = case["nt"], case["jts"]
    n_int = wl.interior_cells(case["shape"])
    n123 = nx * ny * nz
    interval = args.ckpt
    nseg = (nt + interval - 1) // interval
    prop = born.Gb300Prop(0)
    prop.createSpace(case["d"], case["d"], case["d"], 50.0, 0.0005, 0.0005,
                     nx, ny, nz)
    prop.transferSincTableS(8, jt, case["table_s"])
    prop.transferSincTableD(8, jt, case["table_d"])
    prop.transferSourceFunc(9, case["nt_big"], case["locs_s"], case["src"])
    prop.transferVelFunc1(nx, ny, nz, case["vel1"])
    prop.transferVelFunc2(nx, ny, nz, case["vel2"])
    rec = np.zeros_like(case["rec_in"])
    prop.transferReceiverFunc(case["rec_nx"], case["rec_ny"], case["nt_big"],
                              case["locs_r"], rec)
    prop.check(prop.lib.born_set_reflectivity(prop.h, born.fptr(case["refl"])))
    prop.check(prop.lib.born_set_checkpoint_interval(prop.h, interval))
    prop.set_checkpoint_storage(args.ckpt_storage)
    stream = torch.cuda.ExternalStream(prop.stream, device=0)

    def step(ev=None):
        prop.zero_traces()
        if ev:
            ev[0].record(stream)
        prop.lin_forward_device(jt, nt)
        if ev:
            ev[1].record(stream)
        prop.lin_adjoint_device(jt, nt, interval)
        if ev:
            ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    prop.synchronize()
    launches0 = prop.launches
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)]
           for _ in range(args.steps)]
    torch.cuda.synchronize()
    with Clocks(0) as clk:
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for k in range(args.steps):
            step(evs[k])
        stop.record(stream)
        prop.synchronize()
        torch.cuda.synchronize()
    launches = prop.launches - launches0
    t_ms = start.elapsed_time(stop)
    fwd_ms = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps
    adj_ms = sum(e[1].elapsed_time(e[2]) for e in evs) / args.steps
    # one more adjoint with its phases timed (events at phase boundaries)
    prop.time_phases(True)
    prop.zero_traces()
    prop.lin_forward_device(jt, nt)
    prop.lin_adjoint_device(jt, nt, interval)
    prop.synchronize()
    sweep_ms, recomp_ms, rev_ms, div_ms = prop.phase_times()
    reused = bool(prop.lib.born_checkpoints_reused(prop.h))
    prop.time_phases(False)
    # FP16 checkpoints: the gradient's distance from the FP32-checkpoint one
    ckpt_err = None
    if args.ckpt_storage != "f32":
        g16 = prop.get_image()
        prop.set_checkpoint_storage("f32")
        prop.zero_traces()
        prop.lin_forward_device(jt, nt)
        prop.lin_adjoint_device(jt, nt, interval)
        g32 = prop.get_image()
        ckpt_err = float(np.linalg.norm((g16 - g32).ravel()) /
                         max(np.linalg.norm(g32.ravel()), 1e-30))
    cells = 2 * n_int * nt
    value = cells * args.steps / (t_ms / 1e3) / 1e9
    algo = n_int * (32 + 48 + (0 if reused else 16)) * nt + \
        n123 * (32 * nseg + 12)
    peak, peak_kind = measured_peak()
    phases = {
        "lin_forward_ms": round(fwd_ms, 2), "lin_adjoint_ms": round(adj_ms, 2),
        "adjoint_sweep_ms": round(sweep_ms, 2),
        "adjoint_recompute_ms": round(recomp_ms, 2),
        "adjoint_reverse_ms": round(rev_ms, 2),
        "adjoint_division_ms": round(div_ms, 3),
        "lin_forward_GBps": round(32 * n_int * nt / (fwd_ms / 1e3) / 1e9, 1),
        "checkpoints_from_forward": reused,
        "sweep_GBps": (round(16 * n_int * nt / (sweep_ms / 1e3) / 1e9, 1)
                       if not reused else None),
        "recompute_GBps": round(20 * n_int * nt / (recomp_ms / 1e3) / 1e9, 1),
        "reverse_GBps": round(28 * n_int * nt / (rev_ms / 1e3) / 1e9, 1)}
    # roofline of the largest single kernel family by time
    fams = {"forward": (fwd_ms, 32, "step_kernel<born_lin> (s and r, "
                        "scattering source m A s)"),
            "reverse": (rev_ms, 28, "step_kernel<born_adj> (w step, image "
                        "+= (A s) w)"),
            "recompute": (recomp_ms, 20, "step_kernel<model> (background "
                          "step storing A s)"),
            "sweep": (sweep_ms, 16, "step_kernel<model> (background step)")}
    top = max(fams, key=lambda k: fams[k][0])
    ms_top, bpc, kname = fams[top]
    achieved = bpc * n_int / (ms_top / nt / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": None, "kernel": kname, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": bpc * n_int,
                "avg_launch_ms": round(ms_top / nt, 4),
                "whole_step_GBps": round(algo / (t_ms / args.steps / 1e3) /
                                         1e9, 1)}
    line = {"metric": "Gcell-updates/s Born fwd+adj (exact pair, "
                      "checkpointed adjoint)",
            "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t_ms / args.steps, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded, shapes of the config)",
            "config": {"workload": f"{case['name']}: exact linearised Born "
                       f"forward + adjoint, compute grid {nx}x{ny}x{nz}, "
                       f"nt={nt}, background checkpointed every {interval} "
                       "steps", "grid": [nz, ny, nx], "nt": nt,
                       "ckpt_interval": interval, "interior_cells": n_int,
                       "l2": "inputs larger than L2"},
            "algorithmic_bytes_per_step": int(algo),
            "roofline": roofline, "phases": phases,
            "checkpoint_storage": args.ckpt_storage,
            "gradient_rel_l2_vs_f32_checkpoints": ckpt_err,
            "checkpoint_bytes": int(2 * nseg * n123 *
                                    (2 if args.ckpt_storage == "f16" else 4)),
            "segment_bytes": int(interval * n123 * 4),
            "clocks": clk.summary(), "gpu_launches": launches}
    print(json.dumps(line), flush=True)
    return 0


def run_batched(args):
    """c4: batched multi-shot RTM (source propagation + adjoint of every
    shot, one launch per step for all shots, time loops as CUDA graphs)
    against the same shots run one after another."""
    import torch
    born = package()
    born.lib()
    wl = workload_module()
    nt = args.nt if args.nt else 2500
    t0 = time.perf_counter()
    shots, com = wl.prepare_batch_c4(born, nshots=args.shots, nt=nt)
    for h in shots:
        h.set_storage(args.storage)
    setup_s = time.perf_counter() - t0
    jt, ntf = com["jt"], com["nt"]
    cells = sum(wl.interior_cells(h.shape) for h in shots)
    batch = born.Batch(shots, graph=not args.no_graph)
    stream = torch.cuda.ExternalStream(batch.stream)

    def rtm_all():
        batch.source_prop(jt, ntf)
        batch.rtm_adjoint(jt, ntf)

    for _ in range(args.warmup):
        rtm_all()
    batch.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            rtm_all()
        e1.record(stream)
        batch.synchronize()
    t_b = e0.elapsed_time(e1) / args.steps
    # the same shots one after another through the single-shot loops
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    for h in shots:
        # tile autotuning of each shot's own grid happens outside the timing
        h.source_prop_device(jt, 1)
        h.rtm_adjoint_device(jt, 1, swap=1)
        h.synchronize()
    torch.cuda.synchronize()
    t_s = 0.0
    for h in shots:
        st = torch.cuda.ExternalStream(h.stream)
        e2.record(st)
        h.source_prop_device(jt, ntf)
        h.rtm_adjoint_device(jt, ntf, swap=1)
        e3.record(st)
        h.synchronize()
        t_s += e2.elapsed_time(e3)
    # RTM = source propagation + adjoint (two fields) per step
    cu = cells * ntf * 2
    line = {"metric": "Gcell-updates/s batched RTM (c4)",
            "value": round(cu / (t_b / 1e3) / 1e9, 3),
            "unit": "Gcell-updates/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_b, 2),
            "higher_is_better": True,
            "dtype": "f32 arithmetic; levels " + args.storage,
            "data": "synthetic (seeded, shapes of the config)",
            "config": {"workload": f"c4: {len(shots)} shots, apertures "
                       "192..320 x 192..320 x 256..400 on 800x800x400 at "
                       f"10 m, nt={ntf}", "graph": not args.no_graph},
            "shot_steps_per_s": round(len(shots) * ntf / (t_b / 1e3), 1),
            "sequential_ms": round(t_s, 2),
            "batched_over_sequential": round(t_s / t_b, 3),
            "setup_s": round(setup_s, 1), "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_storage(args):
    """c3: one shot of Born forward + RTM adjoint per level storage (FP32,
    BF16, FP16 with per-level power-of-two scales), each timed with CUDA
    events on the handle's stream; the 16-bit results are compared with the
    FP32 result of the same run (the FP64 comparison needs the CPU oracle and
    is made at test sizes)."""
    import torch
    born = package()
    born.lib()
    wl = workload_module()
    t0 = time.perf_counter()
    case = wl.prepare_shot(born, args.config, nt=args.nt, n=args.model_n)
    setup_s = time.perf_counter() - t0
    nz, ny, nx = case["shape"]
    nt, jt = case["nt"], case["jts"]
    n_int = wl.interior_cells(case["shape"])
    # compulsory bytes per interior cell of the three loops (fields 4 or 2 B)
    bpc = {"f32": (32, 16, 40), "f32fma": (32, 16, 40), "bf16": (20, 10, 28),
           "f16": (20, 10, 28)}
    res, ref = {}, None
    for st in args.storage.split(","):
        prop = born.Gb300Prop(0)
        prop.createSpace(case["d"], case["d"], case["d"], 50.0, 0.0005,
                         0.0005, nx, ny, nz)
        prop.transferSincTableS(8, jt, case["table_s"])
        prop.transferSincTableD(8, jt, case["table_d"])
        prop.transferSourceFunc(9, case["nt_big"], case["locs_s"],
                                case["src"])
        prop.transferVelFunc1(nx, ny, nz, case["vel1"])
        prop.transferVelFunc2(nx, ny, nz, case["vel2"])
        rec = np.ascontiguousarray(case["rec_in"])
        prop.transferReceiverFunc(case["rec_nx"], case["rec_ny"],
                                  case["nt_big"], case["locs_r"], rec)
        prop.check(prop.lib.born_set_reflectivity(prop.h,
                                                  born.fptr(case["refl"])))
        prop.set_storage(st)
        stream = torch.cuda.ExternalStream(prop.stream, device=0)

        def step(n_steps, ev=None):
            prop.zero_traces()
            if ev:
                ev[0].record(stream)
            prop.rtm_forward_device(jt, n_steps)
            if ev:
                ev[1].record(stream)
            prop.source_prop_device(jt, n_steps)
            if ev:
                ev[2].record(stream)
            prop.rtm_adjoint_device(jt, n_steps, swap=1)
            if ev:
                ev[3].record(stream)

        for _ in range(args.warmup):  # short loops: tuning and first touch
            step(8)
        prop.synchronize()
        ms = [0.0, 0.0, 0.0]
        with Clocks(0) as clk:
            for _ in range(args.steps):
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
                step(nt, ev)
                prop.synchronize()
                for k in range(3):
                    ms[k] += ev[k].elapsed_time(ev[k + 1]) / args.steps
        # the timed run leaves the image of the adjoint; the traces of the
        # forward loop were overwritten by nothing since
        img = prop.get_image()
        tr = prop.get_traces(rec)
        fwd, src, adj = ms
        b = bpc[st]
        r = {"ms": round(fwd + src + adj, 1),
             "value": round(2 * n_int * nt / ((fwd + src + adj) / 1e3) / 1e9,
                            3),
             "forward_ms": round(fwd, 1), "source_ms": round(src, 1),
             "adjoint_ms": round(adj, 1),
             "adjoint_GBps": round(b[2] * n_int * nt / (adj / 1e3) / 1e9, 1),
             "forward_GBps": round(b[0] * n_int * nt / (fwd / 1e3) / 1e9, 1),
             "clocks": clk.summary()}
        if ref is None:
            ref = (img, tr, r["ms"], st)
        else:
            def rel(a, b_):
                return float(np.linalg.norm((a - b_).ravel()) /
                             max(np.linalg.norm(b_.ravel()), 1e-30))
            r[f"image_rel_l2_vs_{ref[3]}"] = rel(img, ref[0])
            r[f"traces_rel_l2_vs_{ref[3]}"] = rel(tr, ref[1])
            r[f"speedup_vs_{ref[3]}"] = round(ref[2] / r["ms"], 3)
        res[st] = r
        del prop
        torch.cuda.synchronize()
    first = res[args.storage.split(",")[0]]
    line = {"metric": "Gcell-updates/s Born fwd+adj per storage (c3)",
            "value": first["value"], "unit": "Gcell-updates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": first["ms"], "higher_is_better": True,
            "dtype": "f32 arithmetic; levels " + args.storage,
            "data": "synthetic (seeded, shapes of the config)",
            "config": {"workload": f"{args.config}: Born forward + RTM adjoint,"
                       f" compute grid {nx}x{ny}x{nz}, nt={nt}, jt={jt}",
                       "grid": [nz, ny, nx], "nt": nt, "jt": jt,
                       "interior_cells": n_int},
            "storage": res, "setup_s": round(setup_s, 1)}
    print(json.dumps(line), flush=True)
    return 0


def run_lsrtm(args):
    """c5: least-squares RTM, Claerbout CG (cgstep) with FP64 dots and step
    lengths on the device, over the exact linearised Born pair of several
    shots (checkpointed background in the adjoint).  Observed data come from
    the same FP32 operator applied to a seeded sparse layered reflectivity;
    reported: rr.rr per iteration, model error, time per iteration."""
    import torch
    born = package()
    born.lib()
    wl = workload_module()
    kw, m_true = wl.c5_problem(model_n=args.model_n or 128,
                               nshots=args.shots, nt_data=args.nt or 400)
    n3, n2, n1 = m_true.shape
    d, nt_data = kw["d"][0], kw["nt_data"]
    shots = kw["shots"]
    t0 = time.perf_counter()
    op = born.BornOperator(exact=True, ckpt_interval=50, **kw)
    setup_s = time.perf_counter() - t0
    mt = torch.from_numpy(m_true).cuda()
    d_obs = torch.zeros(op.data_shape, device="cuda")
    op.forward(False, mt, d_obs)
    m = torch.zeros(op.model_shape, device="cuda")
    torch.cuda.synchronize()
    reused0 = op.checkpoints_reused
    t0 = time.perf_counter()
    with Clocks(0) as clk:
        res = op.cg(d_obs, m, args.steps)
        torch.cuda.synchronize()
    t_cg = time.perf_counter() - t0
    mm = m.cpu().numpy()
    err = float(np.linalg.norm(mm - m_true) / np.linalg.norm(m_true))
    nc = [int(op.lib.born_compute_size(k, 40, 4)) for k in (n1, n2, n3)]
    n_int = (nc[0] - 8) * (nc[1] - 8) * (nc[2] - 8)
    # field sweeps of nt steps: the solver's first forward (background +
    # scattered field), then per iteration one exact adjoint (background
    # sweep, segment recomputation, adjoint field) and one forward; a shot
    # adjoint that reuses kept checkpoints skips its background sweep
    skipped = op.checkpoints_reused - reused0
    sweeps = len(shots) * (2 + 5 * args.steps) - skipped
    line = {"metric": "CG iterations/s least-squares RTM (c5)",
            "value": round(args.steps / t_cg, 4), "unit": "iterations/s",
            "n_gpus": 1, "steps": args.steps, "warmup": 0,
            "ms_per_step": round(1e3 * t_cg / args.steps, 1),
            "higher_is_better": True, "dtype": "f32 (FP64 dots and steps)",
            "data": "synthetic (seeded layered velocity and sparse layered "
                    "reflectivity; data = the FP32 operator applied to it)",
            "config": {"workload": f"c5: {len(shots)} shots, model "
                       f"{n1}x{n2}x{n3} at {d:.0f} m, nt_data={nt_data} "
                       f"(FD nt={op.nt_fd}), exact linearised Born pair",
                       "full_config": "384x384x256, nt=2000 (--model-n 384)"},
            "rr_per_iteration": [float(r) for r in res],
            "rr_reduction": float(res[-1] / res[0]),
            "model_rel_error": err,
            "field_updates_per_s_G": round(
                n_int * op.nt_fd * sweeps / t_cg / 1e9, 2),
            "field_sweeps": sweeps, "background_sweeps_skipped": skipped,
            "setup_s": round(setup_s, 1), "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (c5: CG iterations; default 5, c5: 10)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c2",
                    choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--storage", default=None,
                    help="level storage: f32, bf16 or f16 (c3: a comma list,"
                         " default f32,bf16,f16; c4: one, default f32)")
    ap.add_argument("--shots", type=int, default=None,
                    help="c4: shots in the batch (48); c5: shots (16)")
    ap.add_argument("--no-graph", action="store_true",
                    help="c4: launch step by step instead of CUDA graphs")
    ap.add_argument("--model-n", type=int, default=None,
                    help="smaller model edge (profiling cases)")
    ap.add_argument("--nt", type=int, default=None,
                    help="fewer time steps (profiling cases)")
    ap.add_argument("--adjoint", default="reference",
                    choices=["reference", "exact"],
                    help="c1/c2: the reference's random-boundary RTM pair "
                         "(default) or the exact linearised pair with the "
                         "checkpointed adjoint")
    ap.add_argument("--ckpt", type=int, default=50,
                    help="--adjoint exact: checkpoint interval (steps)")
    ap.add_argument("--ckpt-storage", default="f32", choices=["f32", "f16"],
                    help="--adjoint exact: checkpoint storage")
    ap.add_argument("--tile", type=int, default=-1)
    ap.add_argument("--zseg", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds of CPU work for the cpu_baseline sample")
    ap.add_argument("--ref-budget", type=float, default=100.0,
                    help="--impl reference: seconds of CPU work over all "
                         "timed samples")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fused", action="store_true",
                    help="c2: skip the extra fused multiply-add and exact "
                         "coupling measurements")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 10 if args.config == "c5" else 5
    if args.shots is None:
        args.shots = 16 if args.config == "c5" else 48
    if args.warmup < 3 and args.impl == "gb300":
        print("note: warm-up raised to the minimum of 3", file=sys.stderr)
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.config == "c3":
        args.storage = args.storage or "f32,bf16,f16"
        return run_storage(args)
    if args.config == "c4":
        args.storage = args.storage or "f32"
        return run_batched(args)
    if args.config == "c5":
        return run_lsrtm(args)
    if args.adjoint == "exact":
        return run_exact(args)
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
