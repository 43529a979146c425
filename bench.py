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
# DRAM bytes (read + write) per launch of fast_step_kernel<19, fp32, *, TRT> on
# the 512^3 box, from one single-pass ncu capture of dram__bytes_read.sum and
# dram__bytes_write.sum (odd 20.465e9, even 20.515e9; algorithmic 20.401e9):
# profiles/fast_step_kernel_d3q19_512_traffic.md
TRAFFIC_512_FP32 = 20.49e9
METRIC = "D3Q19 MLUPs, % HBM peak: FP32 vs FP16-storage @ stated err; adjoint ms/grad"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def slowest_rank_time(t_local, dist, device):
    """Max over ranks of a per-rank step time (the whole job runs at the
    slowest replica's pace); the local value without a process group."""
    if dist is None:
        return float(t_local)
    import torch
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_mlups(cells_per_rank, world, t_step_ms):
    """Whole-job throughput of `world` replicas: all ranks' cell updates over
    the slowest rank's step time."""
    return world * cells_per_rank / (t_step_ms * 1e-3) / 1e6


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
    arrays, `steps` calls of the drop-in LBM::iterate_time (one tick per call
    through the C ABI, fields saved on the first tick and then at most 60
    times a second, LBM.cpp:220-240), read-back of the u/rho field."""
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
        s.iterate_time()
    s.iterate_time(steps=1, save=True)  # the read-back's fields are the last tick's
    rc = lib.bf_copy_field_to_host(s._h, 0, host_out.ctypes.data_as(C.c_void_p), host_out.nbytes)
    if rc != 0:
        raise RuntimeError(lib.bf_last_error().decode())
    dt = time.perf_counter() - t0
    del s
    return {"value": round(world * n * steps / dt / 1e6, 1), "unit": "MLUPs",
            "h2d_bytes_per_step": int(n * 3 * 4 / steps), "d2h_bytes_per_step": int(n * 4 * 4 / steps),
            "note": "init upload + iterate_time() ticks (60 Hz saves) + u/rho read-back"}


def run_adjoint_leg(bf):
    """Differentiation configuration: D2Q9 BGK channel 512x256, tau 0.6,
    Poiseuille inlet u_max 0.05, partial-bounce-back obstacle in the central
    64x64 box, T = 2000 steps, checkpoints every 100 steps; ms per gradient
    (forward + backward) against the forward solve, device time by CUDA events."""
    from boltzmannfluids_gb300.adjoint import RESIDENT_AUTO, AdjointChannel, channel_setup

    def timed(res, vs, K, reps, resident=0):
        s, u_in, tgt = channel_setup(res)
        g = AdjointChannel(res, 0.6, vs, 2000, K, resident_states=resident)
        g.set_parameters(s, u_in)
        g.set_target(tgt)
        g.forward()
        g.backward()
        f_ms, b_ms = g.time(reps)
        r = g.resident_states
        del g
        return {"resident_states": r, "forward_ms": round(f_ms, 3), "backward_ms": round(b_ms, 3),
                "ms_per_gradient": round(f_ms + b_ms, 3), "gradient_over_forward": round((f_ms + b_ms) / f_ms, 3)}

    out = {"workload": "D2Q9 BGK channel 512x256, PSM obstacle, T=2000"}
    # checkpoints every 100 steps with the resident pool (a 512x256 D2Q9 state is 4.7 MB, so the
    # pool holds the whole trajectory and nothing is recomputed), with two segment buffers
    # (every state but the last segment's recomputed once), and with every state a checkpoint
    for K, R, key in ((100, RESIDENT_AUTO, "checkpoint_every_100"), (100, 0, "checkpoint_every_100_segments"),
                      (2000, 0, "all_states_stored")):
        out[key] = timed((512, 256, 1), bf.VelocitySet.D2Q9, K, 5, R)
    # the configuration's 3D case: D3Q19 channel 128^3 (periodic z), checkpoints every 100 steps;
    # the forward's last states kept in device memory (as many as fit), the rest recomputed
    w3 = "D3Q19 BGK channel 128x128x128 (periodic z), PSM obstacle, T=2000, K=100"
    out["d3q19_128"] = {"workload": w3 + ", resident pool (auto)",
                        **timed((128, 128, 128), bf.VelocitySet.D3Q19, 100, 2, RESIDENT_AUTO)}
    out["d3q19_128_segments"] = {"workload": w3 + ", two segment buffers",
                                 **timed((128, 128, 128), bf.VelocitySet.D3Q19, 100, 2)}
    return out


def run_precision_leg(bf, size, steps, every=100):
    """Precision configuration: D3Q19 BGK Taylor-Green vortex, u0 0.05,
    tau 0.52, periodic size^3, `steps` steps, in FP32, FP16S and FP16C
    storage against the FP64 reference stepper on the GPU.  Reports the
    kinetic-energy error curve (FP64 sums, every `every` steps), the final u
    field error and each storage's MLUPs on this workload (device time)."""
    import numpy as np
    from boltzmannfluids_gb300.workloads import taylor_green_3d
    res = (size, size, size)
    n = size ** 3
    rho, u = taylor_green_3d(res, 0.05)
    runs = {}
    for name in ("fp64", "fp32", "fp16s", "fp16c"):
        s = bf.LBM()
        s.is_collide_esoteric = True
        s.initialize_fields_from_arrays(res, 0.52, density=rho, velocity=u, velocity_set=bf.VelocitySet.D3Q19,
                                        fp_accuracy=getattr(bf.FloatingPointAccuracy, name))
        ke = [s.reduce()[4]]
        ms = 0.0
        for _ in range(steps // every):
            ms += s.benchmark_steps(every)
            ke.append(s.reduce()[4])
        s.reduce()  # also saves the fields of the current state
        vd = s.get_velocity_density_texture().reshape(-1, 4)[:, :3].astype(np.float64)
        runs[name] = (np.array(ke), vd, ms)
        del s
    ke64, u64, ms64 = runs["fp64"]
    scale = float(np.abs(u64).max())
    out = {"workload": f"D3Q19 BGK Taylor-Green vortex u0 0.05 tau 0.52, {size}^3 periodic, {steps} steps",
           "reference": "FP64 stepper on the GPU (storage fp64, bit-exact with the FP64 oracle)",
           "ke_fp64_final": float(ke64[-1]), "fp64_mlups": round(n * steps / (ms64 * 1e-3) / 1e6, 1)}
    for name in ("fp32", "fp16s", "fp16c"):
        ke, uu, ms = runs[name]
        err = np.abs(ke - ke64) / ke64
        du = uu - u64
        out[name] = {"ke_rel_err_max": float(err.max()), "ke_rel_err_final": float(err[-1]),
                     "u_err_max_over_umax": float(np.abs(du).max() / scale),
                     "u_err_rms_over_urms": float(np.sqrt((du ** 2).mean() / (u64 ** 2).mean())),
                     "mlups": round(n * steps / (ms * 1e-3) / 1e6, 1)}
    return out


def spinodal_solver(bf, res, storage, rho):
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.intermolecular_interaction_strength = -5.0
    s.initialize_fields_from_arrays(res, 1.0, density=rho, velocity_set=bf.VelocitySet.D3Q19, fp_accuracy=storage,
                                    is_flow_multiphase=True)
    return s


def run_multiphysics_leg(bf, sc_res=(256, 256, 256), sc_steps=20000, rb_res=(256, 256, 130), rb_steps=50000,
                         ref_sc_res=(64, 64, 64), ref_sc_steps=2000, ref_rb_res=(64, 64, 34), ref_rb_steps=50000):
    """Multiphysics configuration at its own sizes: Shan-Chen spinodal
    decomposition (D3Q19, psi = 1 - exp(-rho), G = -5, rho = 0.69 +
    0.01 U(-1,1) seeded) 256^3 x 20000 steps in FP32, FP16S and FP16C with the
    mass drift (FP64 sums); Rayleigh-Benard convection (D3Q19 flow + D3Q7
    temperature, hot bottom / cold top walls, Ra 1e5, Pr 0.71, T noise 1e-3
    seeded) 256x256x130 x 50000 steps with its Nusselt number and mass drift.
    Against the FP64 stepper (bit-exact with the FP64 oracle), at reduced sizes:
    the Shan-Chen mass drift and liquid fraction at 64^3 x 2000 steps and the
    Rayleigh-Benard Nusselt number at 64x64x34 x 50000 steps."""
    import numpy as np
    from boltzmannfluids_gb300.workloads import nusselt, rayleigh_benard, spinodal
    out = {}
    n = sc_res[0] * sc_res[1] * sc_res[2]
    sc = {"workload": f"Shan-Chen spinodal decomposition D3Q19, G -5, {sc_res[0]}^3 periodic, {sc_steps} steps"}
    rho = spinodal(sc_res, 0.69, 0.01, 4)
    for name in ("fp32", "fp16s", "fp16c"):
        s = spinodal_solver(bf, sc_res, getattr(bf.FloatingPointAccuracy, name), rho)
        m0 = s.reduce()[0]
        ms = s.benchmark_steps(sc_steps)
        m1 = s.reduce()[0]
        d = s.get_velocity_density_texture().reshape(-1, 4)[:, 3]
        sc[name] = {"mass_rel_drift": float((m1 - m0) / m0), "rho_min": float(d.min()), "rho_max": float(d.max()),
                    "liquid_fraction": float((d > 0.69).mean()), "mlups": round(n * sc_steps / (ms * 1e-3) / 1e6, 1)}
        del s
    # against FP64 at a reduced size: the mass FP64 arithmetic conserves and the phase split
    rn_ = ref_sc_res[0] * ref_sc_res[1] * ref_sc_res[2]
    rrho = spinodal(ref_sc_res, 0.69, 0.01, 4)
    ref = {}
    for name in ("fp64", "fp32", "fp16s", "fp16c"):
        s = spinodal_solver(bf, ref_sc_res, getattr(bf.FloatingPointAccuracy, name), rrho)
        m0 = s.reduce()[0]
        ms = s.benchmark_steps(ref_sc_steps)
        m1 = s.reduce()[0]
        d = s.get_velocity_density_texture().reshape(-1, 4)[:, 3]
        ref[name] = {"mass_rel_drift": float((m1 - m0) / m0), "liquid_fraction": float((d > 0.69).mean()),
                     "mlups": round(rn_ * ref_sc_steps / (ms * 1e-3) / 1e6, 1)}
        del s
    sc["vs_fp64"] = {"workload": f"{ref_sc_res[0]}^3 x {ref_sc_steps} steps", **ref}
    out["shan_chen"] = sc
    def rb_run(res, steps, kappa, storage, window, every):
        """Nusselt number at the last step and averaged over the last `window`
        steps (a sample every `every` steps: the convection at Ra 1e5 is
        unsteady, so single instants of two runs differ by the flow's own
        fluctuation); mass drift; MLUPs from the stepping time alone."""
        s, kappa, h = rayleigh_benard(res, kappa=kappa, storage=storage)
        m0 = s.reduce()[0]
        ms = s.benchmark_steps(steps - window)
        series = []
        for _ in range(window // every):
            ms += s.benchmark_steps(every)
            s.reduce()  # saves the current state's fields
            series.append(nusselt(s, kappa, h))
        m1 = s.reduce()[0]
        n = res[0] * res[1] * res[2]
        out = {"nusselt": float(series[-1]), "nusselt_mean": float(np.mean(series)),
               "nusselt_std": float(np.std(series)), "mass_rel_drift": float((m1 - m0) / m0),
               "mlups": round(n * steps / (ms * 1e-3) / 1e6, 1)}
        del s
        return out

    rb = {"workload": f"Rayleigh-Benard D3Q19+D3Q7 TRT, {rb_res[0]}x{rb_res[1]}x{rb_res[2]} (walls at z = 0, "
                      f"{rb_res[2] - 1}), Ra 1e5, Pr 0.71, {rb_steps} steps, FP32; Nusselt mean over the last "
                      f"{rb_steps // 5} steps, every {rb_steps // 100}",
          **rb_run(rb_res, rb_steps, 0.02, bf.FloatingPointAccuracy.fp32, rb_steps // 5, rb_steps // 100)}
    ref = {}
    for name in ("fp64", "fp32", "fp16s", "fp16c"):
        # the second half of the run: past the onset transient (~10,000 steps at this size) the
        # convection is statistically steady, and 100 samples average its 6-9 % fluctuation
        ref[name] = rb_run(ref_rb_res, ref_rb_steps, 0.008, getattr(bf.FloatingPointAccuracy, name),
                           ref_rb_steps // 2, ref_rb_steps // 200)
    ref["nusselt_rel_err_fp32"] = abs(ref["fp32"]["nusselt"] - ref["fp64"]["nusselt"]) / ref["fp64"]["nusselt"]
    for name in ("fp32", "fp16s", "fp16c"):
        ref[f"nusselt_mean_rel_err_{name}"] = (abs(ref[name]["nusselt_mean"] - ref["fp64"]["nusselt_mean"]) /
                                               ref["fp64"]["nusselt_mean"])
    rb["vs_fp64"] = {"workload": f"{ref_rb_res[0]}x{ref_rb_res[1]}x{ref_rb_res[2]} x {ref_rb_steps} steps, "
                                 f"Nusselt mean over the last {ref_rb_steps // 2} steps, every {ref_rb_steps // 200}",
                     **ref}
    out["rayleigh_benard"] = rb
    out["throughput_full_size"] = multiphysics_throughput(bf)
    return out


def run_fp64_error_leg(bf, cavity_steps=10000, sphere_res=(128, 64, 64), sphere_steps=2000):
    """Every storage's error against the FP64 stepper on the plain-method
    configurations: the D2Q9 BGK lid-driven cavity 256^2 (tau 0.6, lid u 0.1
    as a moving wall under halfway bounce-back, the other walls at rest) after
    10000 steps, and D3Q19 TRT flow past a sphere (velocity inlet 0.05,
    density outlet, periodic y/z) at half the configuration's size, 2000 steps.
    Error = max |u - u64| / max |u64| and max |rho - rho64| over fluid cells."""
    import numpy as np
    from boltzmannfluids_gb300.workloads import sphere_channel
    out = {}
    n = 256
    y, x = np.mgrid[0:n, 0:n]
    ids = np.zeros((n, n), np.uint32)
    ids[(x == 0) | (x == n - 1) | (y == 0)] = 1
    ids[y == n - 1] = 2
    fields = {}
    for name in ("fp64", "fp32", "fp16s", "fp16c"):
        s = bf.LBM()
        s.is_collide_esoteric = True
        s.boundary_mode = bf.BoundaryMode.bounce_back
        s.set_boundry_properties(1, velocity_translational=(0, 0, 0))
        s.set_boundry_properties(2, velocity_translational=(0.1, 0, 0))
        s.initialize_fields_from_arrays((n, n, 1), 0.6, boundry_id=ids.reshape(-1), periodic=(False, False, True),
                                        velocity_set=bf.VelocitySet.D2Q9,
                                        fp_accuracy=getattr(bf.FloatingPointAccuracy, name))
        s.iterate_time(steps=cavity_steps, save=True)
        fields[name] = s.get_velocity_density_texture().reshape(-1, 4).astype(np.float64)
        del s
    fluid = ids.reshape(-1) == 0
    ref = fields["fp64"][fluid]
    scale = np.abs(ref[:, :3]).max()
    out["cavity"] = {"workload": f"D2Q9 BGK lid-driven cavity 256^2, tau 0.6, lid 0.1, {cavity_steps} steps"}
    for name in ("fp32", "fp16s", "fp16c"):
        f = fields[name][fluid]
        out["cavity"][name] = {"u_err_max_over_umax": float(np.abs(f[:, :3] - ref[:, :3]).max() / scale),
                               "rho_err_max": float(np.abs(f[:, 3] - ref[:, 3]).max())}
    # r = ny/8 centred at (ny/2, ny/2, nz/2): r 8 at (32, 32, 32) in 128x64x64, r 16 at (64, 64, 64)
    # in the configuration's 256x128x128
    r_s = sphere_res[1] / 8.0
    rho, u, ids3, objs = sphere_channel(sphere_res, radius=r_s, center=(sphere_res[1] / 2.0, sphere_res[1] / 2.0,
                                                                       sphere_res[2] / 2.0))
    fields = {}
    for name in ("fp64", "fp32", "fp16s", "fp16c"):
        s = bf.LBM()
        s.is_collide_esoteric = True
        s.collision = bf.Collision.trt
        s.boundary_mode = bf.BoundaryMode.bounce_back
        for k, o in objs.items():
            s.set_boundry_properties(k, velocity_translational=(0, 0, 0), kind=o["kind"])
        s.initialize_fields_from_arrays(sphere_res, 0.55, density=rho, velocity=u, boundry_id=ids3,
                                        periodic=(False, True, True), velocity_set=bf.VelocitySet.D3Q19,
                                        fp_accuracy=getattr(bf.FloatingPointAccuracy, name))
        s.iterate_time(steps=sphere_steps, save=True)
        fields[name] = s.get_velocity_density_texture().reshape(-1, 4).astype(np.float64)
        del s
    fluid = ids3 == 0
    ref = fields["fp64"][fluid]
    scale = np.abs(ref[:, :3]).max()
    out["sphere"] = {"workload": f"D3Q19 TRT flow past a sphere r{r_s:g}, {sphere_res[0]}x{sphere_res[1]}x{sphere_res[2]}, "
                                 f"inlet 0.05, {sphere_steps} steps"}
    for name in ("fp32", "fp16s", "fp16c"):
        f = fields[name][fluid]
        out["sphere"][name] = {"u_err_max_over_umax": float(np.abs(f[:, :3] - ref[:, :3]).max() / scale),
                               "rho_err_max": float(np.abs(f[:, 3] - ref[:, 3]).max())}
    return out


def multiphysics_throughput(bf, steps=300):
    """MLUPs of the multiphysics configuration's step at its own sizes
    (Shan-Chen 256^3 in each storage -- the 16-bit ones also with the psi rows
    staged in shared memory and with cached stencil loads -- and
    Rayleigh-Benard 256x256x130), a few hundred timed steps each after the
    start-up steps."""
    from boltzmannfluids_gb300.workloads import rayleigh_benard, spinodal
    res = (256, 256, 256)
    n = res[0] * res[1] * res[2]
    out = {"steps_timed": steps}
    rho = spinodal(res, 0.69, 0.01, 4)
    # the library's default per storage, then each 16-bit storage with the psi rows staged in
    # shared memory by bulk copies (psi_tile) and with cached stencil loads (cached)
    for name, tile in (("fp32", None), ("fp16s", None), ("fp16c", None), ("fp16s", "1"), ("fp16c", "1"),
                       ("fp16s", "0"), ("fp16c", "0")):
        if tile is not None:
            os.environ["BF_PSI_TILE"] = tile
        s = spinodal_solver(bf, res, getattr(bf.FloatingPointAccuracy, name), rho)
        os.environ.pop("BF_PSI_TILE", None)
        s.iterate_time(steps=4, save=False)
        ms = s.benchmark_steps(steps)
        key = f"shan_chen_256^3_{name}" + {None: "", "1": "_psi_tile", "0": "_cached"}[tile] + "_mlups"
        out[key] = round(n * steps / (ms * 1e-3) / 1e6, 1)
        del s
    rres = (256, 256, 130)
    s, _, _ = rayleigh_benard(rres, kappa=0.02)
    s.iterate_time(steps=4, save=False)
    ms = s.benchmark_steps(steps)
    out["rayleigh_benard_256x256x130_fp32_mlups"] = round(rres[0] * rres[1] * rres[2] * steps / (ms * 1e-3) / 1e6, 1)
    del s
    return out


def run_sphere_leg(bf, steps=1000):
    """3D plain-method configuration: D3Q19 TRT (1/4, tau 0.55) flow past a
    sphere r 16 at (64, 64, 64), 256x128x128, velocity inlet 0.05, density
    outlet 1, periodic y/z, equilibrium start with u noise 1e-4; MLUPs of the
    generic step (objects, open boundaries, bounce-back) by CUDA events."""
    from boltzmannfluids_gb300.workloads import sphere_channel
    res = (256, 128, 128)
    n = res[0] * res[1] * res[2]
    rho, u, ids, objs = sphere_channel(res)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.collision = bf.Collision.trt
    s.boundary_mode = bf.BoundaryMode.bounce_back
    for k, o in objs.items():
        s.set_boundry_properties(k, velocity_translational=(0, 0, 0), kind=o["kind"])
    s.initialize_fields_from_arrays(res, 0.55, density=rho, velocity=u, boundry_id=ids, periodic=(False, True, True),
                                    velocity_set=bf.VelocitySet.D3Q19)
    s.iterate_time(steps=3, save=False)
    ms = s.benchmark_steps(steps)
    s.reduce()
    vd = s.get_velocity_density_texture().reshape(res[2], res[1], res[0], 4)
    out = {"workload": "D3Q19 TRT flow past a sphere r16, 256x128x128, inlet u 0.05, outlet rho 1, periodic y/z",
           "steps_timed": steps, "mlups": round(n * steps / (ms * 1e-3) / 1e6, 1),
           "achieved_gbs": round(153 * n * steps / (ms * 1e-3) / 1e9, 1),
           "wake_ux_behind_sphere": float(vd[64, 64, 88, 0])}
    del s
    return out


def compact_summary(sweep, adj, prec, multi, sphere, fp64err):
    """The headline figures of every leg in a few hundred characters (the
    end of the line, which short log tails keep)."""
    out = {}
    for name, v in (sweep or {}).items():
        out[name] = {"x_fp32": v["x_fp32"], "frac": v["frac"]}
    if adj:
        out["adjoint_grad_over_fwd"] = {"d2q9_512x256": adj["checkpoint_every_100"]["gradient_over_forward"],
                                        "d2q9_512x256_segments":
                                            adj["checkpoint_every_100_segments"]["gradient_over_forward"],
                                        "d3q19_128": adj["d3q19_128"]["gradient_over_forward"],
                                        "d3q19_128_segments": adj["d3q19_128_segments"]["gradient_over_forward"]}
    if prec:
        out["tg_ke_err_vs_fp64"] = {k: float(f"{prec[k]['ke_rel_err_max']:.2e}") for k in ("fp32", "fp16s", "fp16c")}
    if multi and "shan_chen" in multi:
        out["sc_mass_drift"] = {k: float(f"{multi['shan_chen'][k]['mass_rel_drift']:.2e}")
                                for k in ("fp32", "fp16s", "fp16c")}
    if multi and "rayleigh_benard" in multi:
        rb = multi["rayleigh_benard"]
        # at 256x256x130 the 50000 steps end inside the onset transient (the thermal diffusion
        # time h^2/kappa is 819,200 steps): the last step's value and the window's mean both stand
        out["rb_nusselt"] = {"last_step": round(rb["nusselt"], 4), "mean": round(rb["nusselt_mean"], 4),
                             "std": round(rb["nusselt_std"], 4)}
        if "vs_fp64" in rb:
            v = rb["vs_fp64"]
            out["rb_nusselt_err_vs_fp64"] = {**{f"mean_{k}": float(f"{v[f'nusselt_mean_rel_err_{k}']:.2e}")
                                                for k in ("fp32", "fp16s", "fp16c")},
                                             "last_step_fp32": float(f"{v['nusselt_rel_err_fp32']:.2e}"),
                                             "fp64_std_over_mean": float(f"{v['fp64']['nusselt_std'] / v['fp64']['nusselt_mean']:.2e}")}
    if fp64err:
        out["u_err_vs_fp64"] = {case: {k: float(f"{v[k]['u_err_max_over_umax']:.2e}") for k in ("fp32", "fp16s", "fp16c")}
                                for case, v in fp64err.items()}
    if sphere:
        out["sphere_mlups"] = sphere["mlups"]
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
    t_step = slowest_rank_time(ms / args.steps, dist, "cuda")
    mlups = job_mlups(n, world, t_step)
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
        gbs = BYTES_PER_CELL[st] * n / (t2 * 1e-3) / 1e9
        sweep[name] = {"mlups": round(n / (t2 * 1e-3) / 1e6, 1), "x_fp32": round(t_step / t2, 3),
                       "gbs": round(gbs, 1), "frac": round(gbs / peak, 3)}
        del s2

    # ---- end to end through the C ABI with host buffers (e2e) ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(bf, res, vel, args.steps, world)
    adj = None
    if not args.no_adjoint:
        adj = run_adjoint_leg(bf)
    prec = None
    if not args.no_precision:
        prec = run_precision_leg(bf, args.precision_size, args.precision_steps)
    multi = None
    if args.multiphysics_throughput_steps:
        multi = {"throughput_full_size": multiphysics_throughput(bf, args.multiphysics_throughput_steps)}
    elif not args.no_multiphysics:
        multi = run_multiphysics_leg(bf)
    fp64err = None
    if not args.no_fp64_errors:
        fp64err = (run_fp64_error_leg(bf, sphere_res=(256, 128, 128), sphere_steps=5000) if args.fp64_sphere_full
                   else run_fp64_error_leg(bf))
    sphere = None
    if not args.no_sphere:
        sphere = run_sphere_leg(bf, args.sphere_steps)
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
                         "frac": round(achieved / peak, 4),
                         "traffic": (TRAFFIC_512_FP32 if args.size == 512 and args.storage == "fp32" else None),
                         "traffic_unit": "DRAM bytes per launch (ncu capture of this workload)",
                         "peak_kind": peak_kind, "bytes_per_cell": BYTES_PER_CELL[int(main_st)]},
            # the detailed legs first; the compact summaries the records keep come last
            "conservation_fp64": {"mass": red[0], "momentum": list(red[1:4]), "kinetic_energy": red[4]},
            "precision": prec,
            "multiphysics": multi,
            "fp64_errors": fp64err,
            "sphere": sphere,
            "adjoint": adj,
            "e2e": e2e,
            "storage_sweep": sweep,
            "summary": compact_summary(sweep, adj, prec, multi, sphere, fp64err),
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
    ap.add_argument("--no-precision", action="store_true", help="skip the Taylor-Green precision leg")
    ap.add_argument("--precision-size", type=int, default=128, help="cube edge of the Taylor-Green precision leg")
    ap.add_argument("--precision-steps", type=int, default=2000)
    ap.add_argument("--no-multiphysics", action="store_true", help="skip the Shan-Chen / Rayleigh-Benard leg")
    ap.add_argument("--no-fp64-errors", action="store_true", help="skip the cavity / sphere errors against FP64")
    ap.add_argument("--fp64-sphere-full", action="store_true",
                    help="the sphere's FP64 comparison at the configuration's own size (256x128x128, r 16, 5000 steps)")
    ap.add_argument("--multiphysics-throughput-steps", type=int, default=0,
                    help="instead of the multiphysics leg, only its full-size throughput part with this many timed steps")
    ap.add_argument("--no-sphere", action="store_true", help="skip the flow-past-a-sphere leg")
    ap.add_argument("--sphere-steps", type=int, default=1000, help="timed steps of the flow-past-a-sphere leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
