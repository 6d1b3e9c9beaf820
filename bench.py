"""Benchmark of the Maxwell DG time step (DOF-stage updates per second).

Default workload: the periodic plane-wave box, 16^3 affine hex elements, N=7
(2,097,152 nodes x 6 field components), k=(1,1,1), dt = 0.5 x smallest GLL
spacing.  One benchmark step is one RK5 time step (5 stages) of the whole
mesh.  The headline form is the mixed-precision fused kernel; the all-FP64
fused form, the plain per-routine FP64 form and the CPU oracle are measured
beside it on the same workload, and the adjoint workload (8^3 el, N=7, random
eps, 2000 steps) gives the gradient/forward time ratio.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload planewave|cavity|dielectric|large]

--workload selects another configuration of the same contract: cavity (PEC
4^3 el, N=7, TM110 mode), dielectric (PEC 32^3 el, N=5, eps=4 sphere,
Gaussian E_z pulse; accuracy = L2 of mixed against the FP64 fused form) or
large (PEC 64^3 el, N=7, random eps in [1,4], 134M nodes; accuracy over
--accuracy-steps steps).

Prints one JSON line.  With --gpus N > 1 (under torchrun) every rank runs its
own replica of the workload on its GPU ("replicas only": the time step does
not shard inside one GPU's mesh), the timed region is bracketed by barriers
and the slowest rank's time is used.
"""
from __future__ import annotations

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

METRIC = "DOF-stage updates/s FP64 vs mixed at fixed L2 error; adjoint/forward time ratio"
UNIT = "DOF-stage updates/s"
BYTES_PER_NODE_STAGE = 208  # u r/w 96 + k r/w 96 + inverse-mass coefficients 16
CASE = "planewave"
WORKLOADS = {
    "planewave": "planewave 16^3 el N=7 periodic (2,097,152 nodes x 6), RK45",
    "cavity": "cavity 4^3 el N=7 PEC TM110 (32,768 nodes x 6), RK45",
    "dielectric": "dielectric 32^3 el N=5 PEC eps=4 sphere (7,077,888 nodes x 6), RK45",
    "large": "large 64^3 el N=7 PEC random eps (134,217,728 nodes x 6), RK45",
}
_EPS_CACHE = {}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-accuracy", action="store_true", help="skip the full-length L2 runs")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    p.add_argument("--no-adjoint", action="store_true", help="skip the adjoint/forward ratio run")
    p.add_argument("--workload", default="planewave", choices=sorted(WORKLOADS))
    p.add_argument("--adjoint-steps", type=int, default=0,
                   help="steps of the adjoint ratio run (default: the workload's 2000)")
    p.add_argument("--accuracy-steps", type=int, default=0,
                   help="steps of the accuracy runs (default: the configuration's own)")
    p.add_argument("--adjoint-only", action="store_true",
                   help="only the adjoint run (large: mixed forward, FP64 reverse, 180 GB)")
    return p.parse_args()


def host_snapshot_count(state_bytes, most=24):
    """Pinned host snapshots for the large gradient: at most half of the
    host's available memory, and at most `most`."""
    avail = 0
    try:
        with open("/proc/meminfo") as f:
            for ln in f:
                if ln.startswith("MemAvailable:"):
                    avail = int(ln.split()[1]) * 1024
    except OSError:
        pass
    return max(0, min(most, int(0.5 * avail // state_bytes))), avail


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """Per-launch DRAM bytes of a kernel at this workload, from the committed
    ncu summary (profiles/traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n):
    """One process per GPU under torchrun: NCCL where there are GPUs, gloo on
    a host without them (the host-side logic of the N > 1 path: replicas,
    barriers and the max over ranks)."""
    if n <= 1 or "RANK" not in os.environ:
        return None, 0, 1
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    world = int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist.init_process_group("gloo")
    return dist, rank, world


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def case_eps(c):
    """Per-node permittivity of the configuration (None when eps = 1)."""
    if c.eps is None:
        return None
    if c.name not in _EPS_CACHE:
        from nekcem_gb300 import MaxwellGPU
        g = MaxwellGPU.from_box(c.N, c.nel, c.lo, c.hi, c.bc, form="fused64")
        x, y, z = g.coords()
        g.close()
        _EPS_CACHE[c.name] = np.ascontiguousarray(c.eps(x, y, z), dtype=np.float64)
    return _EPS_CACHE[c.name]


def build_gpu_case(form, device_note=None):
    from nekcem_gb300 import MaxwellGPU, cases
    c = cases.make(CASE)
    g = MaxwellGPU.from_box(c.N, c.nel, c.lo, c.hi, c.bc, form=form, permittivity=case_eps(c))
    x, y, z = g.coords()
    dt = c.timestep(x, y, z)
    H, E = c.init_fields(x, y, z)
    return c, g, (x, y, z), dt, H, E


def time_form(form, steps, warmup, dist=None, clocks=None, min_sec=1.0, min_windows=3):
    """Windows of exactly `steps` steps, each bracketed by a barrier and a
    device sync and timed with CUDA events on the context's stream (max over
    ranks), repeated until they add up to `min_sec` (and at least
    `min_windows` of them); the median window is reported."""
    c, g, xyz, dt, H, E = build_gpu_case(form)
    g.set_state(H, E)
    t = 0.0
    if warmup:
        t, _ = g.time_steps(warmup, t, dt)
    barrier(dist)
    g.sync()
    if clocks is not None:
        clocks.__enter__()
        time.sleep(0.15)  # let the sampler start before the timed region
    win = []
    try:
        while len(win) < min_windows or sum(win) < 1e3 * min_sec:
            barrier(dist)
            g.sync()
            t, ms = g.time_steps(steps, t, dt)
            win.append(reduce_max(dist, ms))
    finally:
        if clocks is not None:
            clocks.__exit__(None, None, None)
    launches = g.last_launches()
    npts = g.npts
    g.close()
    return dict(ms=float(np.median(win)), steps=steps, windows=len(win), npts=npts,
                launches=launches, dt=dt, case=c)


def accuracy(form, nsteps=None):
    """L2 of the final state against the analytic solution, or (no analytic
    solution) the final state itself for a comparison between forms."""
    c, g, (x, y, z), dt, H, E = build_gpu_case(form)
    g.set_state(H, E)
    n = nsteps or c.nsteps
    t = g.run(n, 0.0, dt)
    if c.exact is not None:
        l2, li = g.cem_error(*c.exact(x, y, z, t))
        g.close()
        return float(np.sqrt(np.sum(l2 ** 2))), n, None
    Hn, En = g.get_state()
    bm1 = g.array("bmn")
    g.close()
    return None, n, (Hn, En, bm1)


def l2_between(a, b):
    """sqrt(sum_c sum_n bm1 (a - b)^2) / sqrt(sum_c sum_n bm1 b^2): the
    cem_error L2 of a against b, relative."""
    (Ha, Ea, bm1), (Hb, Eb, _) = a, b
    d = sum(float(np.sum(bm1 * (p - q) ** 2)) for p, q in ((Ha, Hb), (Ea, Eb)))
    r = sum(float(np.sum(bm1 * q ** 2)) for q in (Hb, Eb))
    return float(np.sqrt(d / r))


def e2e(steps, warmup, dist=None, min_sec=1.0, min_windows=3):
    """Through the C ABI with host buffers: every step copies the host fields
    in (H2D), runs the 5 stages and copies them back (D2H) -- the drop-in for
    one cem_maxwell_op_rk call (nekgpu_op_rk_host), pinned host memory.
    Windows of `steps` steps (wall clock, barrier on both sides) until they
    add up to `min_sec`; the median window is reported."""
    c, g, xyz, dt, H, E = build_gpu_case("mixed")
    H = np.ascontiguousarray(H); E = np.ascontiguousarray(E)
    g.register_host(H); g.register_host(E)
    t = 0.0
    for _ in range(warmup):
        g.op_rk_host(H, E, t, dt); t += dt
    win = []
    while len(win) < min_windows or sum(win) < min_sec:
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(steps):
            g.op_rk_host(H, E, t, dt); t += dt
        win.append(reduce_max(dist, time.perf_counter() - t0))
    # the host link alone: the whole state in (nekgpu_set_state) and out
    # (nekgpu_get_state) between the same page-locked arrays, best of five
    from nekcem_gb300 import _lib as L
    lib, dp = L.load(), (lambda a: a.ctypes.data_as(L.dp))

    def best_of(fn, reps=5):
        best = 1e30
        for _ in range(reps):
            g.sync()
            t0 = time.perf_counter()
            fn()
            g.sync()
            best = min(best, time.perf_counter() - t0)
        return best
    t_in = best_of(lambda: lib.nekgpu_set_state(g._h, dp(H), dp(E), g.npts))
    t_out = best_of(lambda: lib.nekgpu_get_state(g._h, dp(H), dp(E), g.npts))
    g.unregister_host(H); g.unregister_host(E)
    bytes_io = 6 * g.npts * 8
    npts = g.npts
    g.close()
    return dict(sec=float(np.median(win)), steps=steps, windows=len(win), npts=npts, h2d=bytes_io,
                d2h=bytes_io, link_h2d_gbs=bytes_io / t_in / 1e9, link_d2h_gbs=bytes_io / t_out / 1e9)


def adjoint_ratio(nsteps=0, case="adjoint", budget_mb=None, form="fused64", host_snapshots=0):
    """Gradient time over forward time.  Default: the adjoint workload (unit
    PEC box, 8^3 elements, N=7, eps = 1 + 3 sigmoid(smooth random field, seed
    4), Gaussian E_z source, 2000 steps, J = sum bm1 |E|^2 over [0.7,0.9]^3).
    case="large": the 64^3-element N=7 box with its own eps, under a device
    memory budget (NEKGPU_MEM_BUDGET_MB) that bounds the context and the
    gradient together.  Forward: nekgpu_time_steps of the context's form
    (CUDA events; over at most 50 steps, scaled to nsteps); gradient:
    nekgpu_adjoint_gradient (forward steps in the context's form, FP64
    reverse stages), its own CUDA-event times (forward part + reverse sweep,
    recomputation included), and its wall time."""
    from nekcem_gb300 import MaxwellGPU, cases
    c = cases.make(case)
    old = os.environ.get("NEKGPU_MEM_BUDGET_MB")
    if budget_mb:
        os.environ["NEKGPU_MEM_BUDGET_MB"] = str(int(budget_mb))
    try:
        eps = case_eps(c)
        g = MaxwellGPU.from_box(c.N, c.nel, c.lo, c.hi, c.bc, form=form, permittivity=eps)
        x, y, z = g.coords()
        bm1 = g.array("bmn")
        if c.source:
            g.set_source(**c.source)
        H0, E0 = c.init_fields(x, y, z)
        # probe box: the adjoint workload's; for the large box, around its pulse
        probe = ((0.4, 0.6),) * 3 if case == "large" else cases.make("adjoint").extra["probe"]
        (p0, p1), (q0, q1), (r0, r1) = probe
        inside = (x > p0) & (x < p1) & (y > q0) & (y < q1) & (z > r0) & (z < r1)
        jw = np.where(inside, bm1, 0.0)
        dt = c.timestep(x, y, z)
        n = nsteps or c.nsteps
        g.set_state(H0, E0)
        g.time_steps(3, 0.0, dt)  # warm-up
        g.set_state(H0, E0)
        nf = min(n, 50)
        _, fwd_ms = g.time_steps(nf, 0.0, dt)
        fwd_ms *= n / nf
        g.set_state(H0, E0)
        t_wall = time.perf_counter()
        J, dJ, fwd_part_ms, rev_ms = g.adjoint_gradient(n, 0.0, dt, jw,
                                                        host_snapshots=host_snapshots)
        t_wall = time.perf_counter() - t_wall
        hyb = None
        if form == "fused64" and case == "adjoint":
            # the same gradient with the segments recomputed in mixed stages
            g.set_state(H0, E0)
            Jh, dJh, fh, rh = g.adjoint_gradient(n, 0.0, dt, jw, recompute_mixed=True)
            hyb = {"gradient_ms": fh + rh, "reverse_sweep_ms": rh, "ratio": (fh + rh) / fwd_ms,
                   "J_equal": Jh == J,
                   "grad_max_rel_diff": float(np.abs(dJh - dJ).max() / np.abs(dJ).max())}
        g.close()
    finally:
        if budget_mb:
            if old is None:
                os.environ.pop("NEKGPU_MEM_BUDGET_MB", None)
            else:
                os.environ["NEKGPU_MEM_BUDGET_MB"] = old
    out = {"workload": WORKLOADS.get(case, "adjoint box 8^3 el N=7 PEC, random eps, E_z source"),
           "steps": n, "forward_ms": fwd_ms, "gradient_ms": fwd_part_ms + rev_ms,
           "gradient_forward_part_ms": fwd_part_ms, "reverse_sweep_ms": rev_ms,
           "ratio": (fwd_part_ms + rev_ms) / fwd_ms, "J": J,
           "grad_norm": float(np.linalg.norm(dJ)), "forward_form": form,
           "forward_timing": f"{nf} steps, scaled to {n}", "gradient_wall_s": t_wall,
           "host_snapshots": host_snapshots}
    if hyb:
        out["mixed_recompute"] = hyb
    if budget_mb:
        out["device_memory_budget_bytes"] = int(budget_mb) << 20
    return out


def cpu_model():
    """The host CPU as /proc/cpuinfo names it (model name, or implementer and
    part on Arm)."""
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read().splitlines()
    except OSError:
        return "unknown"
    fields = {}
    for ln in info:
        if ":" in ln:
            k, v = (p.strip() for p in ln.split(":", 1))
            fields.setdefault(k, v)
    if "model name" in fields:
        return fields["model name"]
    return f"implementer {fields.get('CPU implementer', '?')} part {fields.get('CPU part', '?')}"


def cpu_sample(min_sec=10.0, threads=None):
    """The CPU oracle (FP64 restatement of the reference's routines, all host
    threads unless `threads` is given) on the same mesh: RK steps until
    `min_sec` of wall time."""
    from nekcem_gb300 import cases
    from oracle import refcpu as R
    threads = threads or os.cpu_count() or 1
    R.set_threads(threads)
    c = cases.make(CASE)
    ref = R.RefBox(c.N, c.nel, c.lo, c.hi, c.bc)
    x, y, z = ref.coords()
    if c.eps is not None:
        ref.set_materials(c.eps(x, y, z), np.ones(ref.npts))
    dt = c.timestep(x, y, z)
    ref.set_state(*c.init_fields(x, y, z))
    t = ref.run(1, 0.0, dt)  # warm caches / threads
    steps, sec = 0, 0.0
    t0 = time.perf_counter()
    while sec < min_sec:
        t = ref.run(1, t, dt)
        steps += 1
        sec = time.perf_counter() - t0
    npts = ref.npts
    ref.close()
    return dict(value=6 * npts * 5 * steps / sec, sec=sec, steps=steps, threads=threads, npts=npts)


def run_reference(args):
    dist, rank, world = dist_setup(args.gpus)
    if rank != 0:
        return
    steps = max(1, min(args.steps, 60))
    warm = min(args.warmup, 2)
    from nekcem_gb300 import cases
    from oracle import refcpu as R
    threads = os.cpu_count() or 1
    R.set_threads(threads)
    c = cases.make(CASE)
    ref = R.RefBox(c.N, c.nel, c.lo, c.hi, c.bc)
    x, y, z = ref.coords()
    if c.eps is not None:
        ref.set_materials(c.eps(x, y, z), np.ones(ref.npts))
    dt = c.timestep(x, y, z)
    ref.set_state(*c.init_fields(x, y, z))
    t = ref.run(warm, 0.0, dt)
    t0 = time.perf_counter()
    ref.run(steps, t, dt)
    sec = time.perf_counter() - t0
    value = 6 * ref.npts * 5 * steps / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * sec / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[CASE],
                   "elements": c.nelt, "N": c.N, "form": "CPU oracle (FP64 restatement of the "
                   "reference's Fortran routines; the Fortran cannot be built here)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} RK steps of the full mesh after {warm} warm-up"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    global CASE
    args = parse()
    CASE = args.workload
    if args.impl == "reference":
        run_reference(args)
        return
    import nekcem_gb300
    nekcem_gb300.load()
    if args.adjoint_only:
        if CASE == "large":
            # 180 GB (171,661 MiB) of device memory for the context and the
            # gradient together; mixed forward steps, FP64 reverse stages,
            # binomial snapshots on the device and in pinned host memory
            nh, avail = host_snapshot_count(6 * 8 * 64 ** 3 * 8 ** 3)
            out = adjoint_ratio(args.adjoint_steps or 1000, case="large", budget_mb=171661,
                                form="mixed", host_snapshots=nh)
            out["host_mem_available_bytes"] = avail
        else:
            out = adjoint_ratio(args.adjoint_steps)
        print(json.dumps({"adjoint": out}), flush=True)
        return
    dist, rank, world = dist_setup(args.gpus)
    device = int(os.environ.get("LOCAL_RANK", 0))
    peak, peak_kind = measured_peaks()

    # headline: mixed form, device-resident inputs, CUDA-event timed windows
    # of exactly --steps steps (median window)
    clk = ClockSampler(device)
    mixed = time_form("mixed", args.steps, max(3, args.warmup), dist, clocks=clk)
    clocks = clk.summary()
    ms_step = mixed["ms"] / mixed["steps"]
    npts = mixed["npts"]
    dof_stage_per_step = 6 * npts * 5
    value = world * dof_stage_per_step * mixed["steps"] / (mixed["ms"] * 1e-3)
    launch_ms = mixed["ms"] / mixed["launches"]
    achieved = BYTES_PER_NODE_STAGE * npts / (launch_ms * 1e-3) / 1e9

    e = e2e(args.steps, 2, dist)
    e2e_value = world * dof_stage_per_step * e["steps"] / e["sec"]

    if rank != 0:
        return
    fp64 = time_form("fused64", max(5, args.steps // 4), 3)
    plain = time_form("plain", max(3, args.steps // 10), 2)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 contraction / f64 state+RK",
        "data": "synthetic",
        "config": {"workload": WORKLOADS[CASE],
                   "elements": mixed["case"].nelt, "N": mixed["case"].N, "form": "mixed",
                   "dt": mixed["dt"],
                   "timing": f"median of {mixed['windows']} CUDA-event windows of {args.steps} "
                             f"steps (>= 1 s in all)",
                   "l2_policy": f"inputs larger than L2: u in/out + k + inverse mass = "
                                f"{(6 * 8 * 3 + 16) * npts / 1e6:.0f} MB per stage",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": e["h2d"],
                "d2h_bytes_per_step": e["d2h"], "path": "nekgpu_op_rk_host, pinned host fields",
                "timing": f"median of {e['windows']} windows of {e['steps']} steps",
                "link_gbs": {"h2d": e["link_h2d_gbs"], "d2h": e["link_d2h_gbs"],
                             "how": "whole state through nekgpu_set_state / nekgpu_get_state, "
                                    "page-locked arrays, best of 5"}},
        "gpu_launches": mixed["launches"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": ncu_traffic(f"k_mixed_stage<{mixed['case'].N + 1}>"
                                            + ("" if CASE == "planewave" else f" {CASE}")),
                     "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": BYTES_PER_NODE_STAGE * npts},
        "clocks": clocks,
        "forms": {
            "fused64": {"value": dof_stage_per_step * fp64["steps"] / (fp64["ms"] * 1e-3),
                        "ms_per_step": fp64["ms"] / fp64["steps"],
                        "timing": f"median of {fp64['windows']} windows of {fp64['steps']} steps"},
            "plain64": {"value": dof_stage_per_step * plain["steps"] / (plain["ms"] * 1e-3),
                        "ms_per_step": plain["ms"] / plain["steps"],
                        "timing": f"median of {plain['windows']} windows of {plain['steps']} steps"},
        },
    }
    out["forms"]["mixed_over_fused64"] = value / world / out["forms"]["fused64"]["value"]
    out["forms"]["mixed_over_plain64"] = value / world / out["forms"]["plain64"]["value"]
    if not args.no_accuracy and world == 1:
        nacc = args.accuracy_steps or (100 if CASE == "large" else None)
        l2m, n, fin_m = accuracy("mixed", nacc)
        l2d, _, fin_d = accuracy("fused64", nacc)
        if l2m is not None:
            out["l2_vs_analytic"] = {"steps": n, "mixed": l2m, "fused64": l2d, "ratio": l2m / l2d}
        else:
            out["l2_mixed_vs_fused64"] = {"steps": n, "relative_l2": l2_between(fin_m, fin_d)}
    if not args.no_adjoint and world == 1 and CASE == "planewave":
        out["adjoint"] = adjoint_ratio(args.adjoint_steps)
    if not args.no_adjoint and world == 1 and CASE == "large":
        # 180 GB (171,661 MiB) for the context and the gradient together
        out["adjoint"] = adjoint_ratio(args.adjoint_steps or 10, case="large", budget_mb=171661)
    if not args.no_cpu and world == 1 and npts <= 10_000_000:
        cpu = cpu_sample()
        one = cpu_sample(threads=1)
        out["cpu_baseline"] = {"value": cpu["value"], "unit": UNIT, "cores": cpu["threads"],
                               "kind": "port", "sample": f"{cpu['steps']} RK steps of the full "
                               f"mesh, {cpu['sec']:.1f} s", "cpu": cpu_model(),
                               "single_thread": {"value": one["value"], "cores": 1,
                                                 "sample": f"{one['steps']} RK steps of the full "
                                                 f"mesh, {one['sec']:.1f} s"}}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
