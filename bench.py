"""Throughput of the D3Q19 esoteric-pull (AA, in place) stream+collide step.

Workload (the 512^3 periodic box of the 3D plain-method configuration):
D3Q19, TRT (magic 1/4), tau 0.55, 512^3 cells, fully periodic, FP32 DDF,
seeded equilibrium start with u noise +-1e-4.  A step is one AA time step
over all cells (one launch of the fused step kernel).  The DDF is 10.2 GB,
far larger than the 129 MB L2, so no flush is needed between steps.

  value   MLUPs with the state resident in HBM (CUDA events around K steps)
  e2e     MLUPs through the public C ABI from host buffers: upload of the
          initial fields from pinned host memory, K calls of one time step,
          read-back of the velocity/density field to pinned host memory
  roofline  achieved HBM GB/s of the step kernel = 152 B/cell x cells /
          kernel time, against MEASURED_PEAKS.json hbm_gbs
  cpu_baseline  the CPU oracle (restatement of the reference's shader math)
          on a bounded sample, all host threads

--impl reference runs the reference arm: the reference's GL shaders cannot
run on these machines (no graphics stack), so the arm times the CPU
restatement of the same shader math on a bounded sample of the workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RES = (512, 512, 512)
TAU = 0.55
BYTES_PER_CELL = {0: 152, 2: 76, 3: 76}  # algorithmic: 19 reads + 19 writes (periodic box, no flag field)
METRIC = "D3Q19 MLUPs, % HBM peak: FP32 vs FP16-storage @ stated err; adjoint ms/grad"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons every 50 ms."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self._t = None

    def start(self):
        cmd = ["nvidia-smi", f"--id={self.index}",
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "50"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[4 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def seeded_velocity(n, seed=2):
    import numpy as np
    rng = np.random.default_rng(seed)
    return (1e-4 * rng.uniform(-1, 1, (n, 3))).astype(np.float32)


def make_solver(storage, res=RES, velocity=None):
    import boltzmannfluids_gb300 as bf
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.collision = bf.Collision.trt
    s.trt_magic = 0.25
    s.initialize_fields_from_arrays(res, TAU, velocity=velocity, periodic=(True, True, True),
                                    velocity_set=bf.VelocitySet.D3Q19, fp_accuracy=storage)
    return s


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline_sample(seconds_target=12.0):
    """The CPU oracle on a 128x128x64 slab of the workload (TRT, tau 0.55,
    periodic), all host threads; returns MLUPs and the sample description."""
    import numpy as np
    from oracle.oracle import Oracle
    res = (128, 128, 64)
    n = res[0] * res[1] * res[2]
    o = Oracle(res, TAU, velocity=seeded_velocity(n), velocity_set=4, esoteric=True, collision=1)
    o.iterate(1, False)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        o.iterate(1, False)
        steps += 1
        dt = time.perf_counter() - t0
        if dt >= seconds_target or steps >= 50:
            break
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return n * steps / dt / 1e6, threads, f"D3Q19 TRT AA FP32, {res[0]}x{res[1]}x{res[2]} periodic slab, {steps} steps"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    mlups, threads, sample = None, None, None
    per_step = []
    from oracle.oracle import Oracle
    import numpy as np
    res = (128, 128, 64)
    n = res[0] * res[1] * res[2]
    o = Oracle(res, TAU, velocity=seeded_velocity(n), velocity_set=4, esoteric=True, collision=1)
    for _ in range(args.warmup):
        o.iterate(1, False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t = time.perf_counter()
        o.iterate(1, False)
        per_step.append(time.perf_counter() - t)
    dt = time.perf_counter() - t0
    mlups = n * args.steps / dt / 1e6
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    sample = f"each step: one AA step of a {res[0]}x{res[1]}x{res[2]} periodic slab of the 512^3 workload"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(mlups, 3), "unit": "MLUPs", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "D3Q19 TRT esoteric-pull, tau 0.55, periodic box (CPU sample)",
                   "cells_per_step": n, "parallelism": "openmp"},
        "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPs", "cores": threads, "kind": "port",
                         "sample": sample + "; the reference's GL shaders are unavailable on this box, so the CPU "
                                            "restatement of the same shader math (oracle/) is timed"},
        "e2e": {"value": round(mlups, 3), "unit": "MLUPs", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_e2e(bf, res, vel, steps, world):
    """Public-API run from host memory: bf_initialize_fields from pinned host
    arrays, `steps` calls of one time step, read-back of the u/rho field."""
    import ctypes as C
    import numpy as np
    n = res[0] * res[1] * res[2]
    lib = bf.load_library()
    host_u = vel
    host_out = np.empty(n * 4, np.float32)
    try:
        import torch
        pin_u = torch.from_numpy(vel.reshape(-1)).pin_memory()
        pin_out = torch.empty(n * 4, dtype=torch.float32).pin_memory()
        host_u = pin_u.numpy().reshape(-1, 3)
        host_out = pin_out.numpy()
    except Exception:
        pass
    t0 = time.perf_counter()
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.collision = bf.Collision.trt
    s.initialize_fields_from_arrays(res, TAU, velocity=host_u, periodic=(True, True, True),
                                    velocity_set=bf.VelocitySet.D3Q19)
    for _ in range(steps - 1):
        s.iterate_time(steps=1, save=False)
    s.iterate_time(steps=1, save=True)
    rc = lib.bf_copy_field_to_host(s._h, 0, host_out.ctypes.data_as(C.c_void_p), host_out.nbytes)
    if rc != 0:
        raise RuntimeError(lib.bf_last_error().decode())
    dt = time.perf_counter() - t0
    del s
    return {"value": round(world * n * steps / dt / 1e6, 1), "unit": "MLUPs",
            "h2d_bytes_per_step": int(n * 3 * 4 / steps), "d2h_bytes_per_step": int(n * 4 * 4 / steps),
            "note": "timed: upload of the initial fields, the steps, read-back of the u/rho field; bytes amortised per step"}


def run_adjoint_leg(bf):
    """Differentiation configuration: D2Q9 BGK channel 512x256, tau 0.6,
    Poiseuille inlet u_max 0.05, partial-bounce-back obstacle in the central
    64x64 box, T = 2000 steps, checkpoints every 100 steps; ms per gradient
    (forward + backward) against the forward solve, device time by CUDA events."""
    from boltzmannfluids_gb300.adjoint import AdjointChannel, channel_setup
    res = (512, 256, 1)
    s, u_in, tgt = channel_setup(res)
    out = {"workload": "D2Q9 BGK channel 512x256, PSM obstacle, T=2000"}
    for K, key in ((100, "checkpoint_every_100"), (2000, "all_states_stored")):
        g = AdjointChannel(res, 0.6, bf.VelocitySet.D2Q9, 2000, K)
        g.set_parameters(s, u_in)
        g.set_target(tgt)
        g.forward()
        g.backward()
        f_ms, b_ms = g.time(5)
        out[key] = {"forward_ms": round(f_ms, 3), "backward_ms": round(b_ms, 3),
                    "ms_per_gradient": round(f_ms + b_ms, 3), "gradient_over_forward": round((f_ms + b_ms) / f_ms, 3)}
        del g
    return out


def run_gpu(args):
    rank, world, local = dist_env()
    if world > 1:
        # one process per GPU: the solver library uses the process's first
        # visible device, so each rank sees only its own
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import boltzmannfluids_gb300 as bf
    from boltzmannfluids_gb300 import build as _b
    _b.build()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl")
    res = (args.size, args.size, args.size)
    n = res[0] * res[1] * res[2]
    vel = seeded_velocity(n)
    main_st = {"fp32": bf.FloatingPointAccuracy.fp32, "fp16s": bf.FloatingPointAccuracy.fp16s,
               "fp16c": bf.FloatingPointAccuracy.fp16c}[args.storage]

    # ---- device-resident throughput (value) ----
    s = make_solver(main_st, res=res, velocity=vel)
    s.iterate_time(steps=max(args.warmup, 3), save=False)
    s.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms = s.benchmark_steps(args.steps)
    clock_info = clocks.stop()
    s.synchronize()
    t_step = ms / args.steps
    if dist:
        import torch
        t = torch.tensor([t_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())
    mlups = world * n / (t_step * 1e-3) / 1e6
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_CELL[int(main_st)] * n / (t_step * 1e-3) / 1e9
    # KE / mass after the timed run (FP64 reductions)
    red = s.reduce()
    del s

    # ---- 16-bit storage modes (same workload) ----
    sweep = {}
    for name, st in (() if args.no_sweep else (("fp16s", bf.FloatingPointAccuracy.fp16s),
                                                ("fp16c", bf.FloatingPointAccuracy.fp16c))):
        s2 = make_solver(st, res=res, velocity=vel)
        s2.iterate_time(steps=3, save=False)
        s2.synchronize()
        k = max(4, args.steps // 2)
        ms2 = s2.benchmark_steps(k)
        t2 = ms2 / k
        sweep[name] = {"mlups": round(n / (t2 * 1e-3) / 1e6, 1), "ms_per_step": round(t2, 4),
                       "achieved_gbs": round(BYTES_PER_CELL[st] * n / (t2 * 1e-3) / 1e9, 1),
                       "speedup_vs_fp32": round(t_step / t2, 3)}
        del s2

    # ---- end to end through the C ABI with host buffers (e2e) ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(bf, res, vel, args.steps, world)
    adj = None
    if not args.no_adjoint:
        adj = run_adjoint_leg(bf)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        mlups_cpu, threads, sample = cpu_baseline_sample()
        cpu = {"value": round(mlups_cpu, 3), "unit": "MLUPs", "cores": threads, "kind": "port", "sample": sample}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(mlups, 1), "unit": "MLUPs", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded equilibrium start, u noise 1e-4)",
            "config": {"workload": f"D3Q19 TRT (magic 1/4, tau 0.55) esoteric-pull, {args.size}^3 periodic box, "
                                   f"{args.storage} DDF",
                       "cells": n, "velocity_set": "D3Q19", "collision": "TRT", "storage": args.storage,
                       "l2": f"inputs larger than L2 ({n * 19 * (4 if args.storage == 'fp32' else 2) / 1e9:.2f} GB "
                             f"DDF vs 129 MB L2), no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None,
                         "peak_kind": peak_kind, "bytes_per_cell": BYTES_PER_CELL[int(main_st)]},
            "storage_sweep": sweep,
            "conservation_fp64": {"mass": red[0], "momentum": list(red[1:4]), "kinetic_energy": red[4]},
            "e2e": e2e,
            "adjoint": adj,
            "gpu_launches": args.steps,
            "clocks": clock_info,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--size", type=int, default=512, help="cube edge of the periodic box (512 = the workload)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-sweep", action="store_true", help="skip the 16-bit storage legs (profiling runs)")
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16s", "fp16c"], help="storage of the main leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
