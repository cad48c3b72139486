#!/usr/bin/env python3
"""Benchmark of the GB300 NanoFiller hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload medium|small|jammed|large]

One step = one realisation of the workload through the whole path: seeded
candidate stream -> von Neumann density test -> cell-list hard-core rejection
(sequential insertion) -> tunnelling contacts + screening + electrodes ->
network solve. Default workload `medium`: 5 um box, 1 um x 5 nm rods, 1 % volume
fraction (15 916 rods), 8-Gaussian agglomerate density on a 64^3 mesh, von
Mises-Fisher kappa = 4 orientation, electrodes at z = 0 and z = L.

value: accepted rods per second with the density mesh resident in HBM, timed
with CUDA events around each step on the library's stream; L2 (129 MB) is
flushed by writing a 256 MB buffer before every timed step. e2e: the same
metric through the C ABI with host buffers: the mesh is uploaded and the rods
and contacts are read back inside every step. Under torchrun each rank runs an
independent realisation (seed + rank): replicas, no collective on the path.

--impl reference times the CPU implementation of the path (the FP64 C++ oracle,
all host threads) on the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rods/s & realisations/s, batched vs plain on 1 GB300, 0 FP64 decision flips"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="medium", choices=["medium", "small", "jammed", "large", "batched"])
    ap.add_argument("--batch", type=int, default=256, help="realisations of the batched workload")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def workload(name, rank):
    import nanofiller_gb300 as nf
    C = nf.configs
    if name == "medium":
        return dict(C.MEDIUM, seed=C.MEDIUM["seed"] + rank), C.gaussian_mesh()
    if name == "small":
        return dict(C.SMALL, seed=C.SMALL["seed"] + rank), None
    if name == "jammed":
        return dict(C.JAMMED, seed=C.JAMMED["seed"] + rank), None
    return dict(C.LARGE, seed=C.LARGE["seed"] + rank), None


def workload_config(name, params):
    d = {"workload": name, "box_um": list(params["box"]), "rod_um": [params["l"], params["a"]],
         "vf": params["vf"], "candidates_budget": params["n_candidates"], "seed": params["seed"],
         "cutoff_um": params["stat_dist_lim"], "gap_um": params["sep"],
         "l2": "flushed (256 MB write) before every timed step"}
    if name == "medium":
        d.update(density="0.01 + 8 Gaussians sigma 0.5 um, 64^3 mesh", orientation="vMF kappa 4 about z")
    return d


# --------------------------------------------------------------------------- clocks
class Nvml:
    """Read-only NVML queries through NVIDIA's libnvidia-ml (ctypes): the
    SM clock, its maximum and the clock-event reason mask. Nothing is set."""
    # reason bits of nvmlClocksEventReason* (nvml.h)
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20,
            "hw_thermal_slowdown": 0x40, "hw_power_brake_slowdown": 0x80}

    def __init__(self, dev):
        import ctypes as C
        self.C = C
        L = C.CDLL("libnvidia-ml.so.1")
        if L.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.L = L
        self.h = C.c_void_p()
        uuid = None
        try:
            import torch
            u = getattr(torch.cuda.get_device_properties(dev), "uuid", None)
            if u is not None:
                uuid = ("GPU-" + str(u)).encode()
        except Exception:
            uuid = None
        if uuid is None or L.nvmlDeviceGetHandleByUUID(uuid, C.byref(self.h)) != 0:
            if L.nvmlDeviceGetHandleByIndex_v2(dev, C.byref(self.h)) != 0:
                raise RuntimeError("no NVML handle")
        self.reasons_fn = getattr(L, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            L.nvmlDeviceGetCurrentClocksThrottleReasons
        v = C.c_uint()
        self.max_sm = float(v.value) if L.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(v)) == 0 else None

    def sample(self):
        C = self.C
        v, r = C.c_uint(), C.c_ulonglong()
        if self.L.nvmlDeviceGetClockInfo(self.h, 1, C.byref(v)) != 0:
            return None
        self.reasons_fn(self.h, C.byref(r))
        return float(v.value), int(r.value)


class Clocks:
    """SM clock and throttle reasons during the timed window: NVML polled every
    5 ms from a thread while the window is open (a window of a few tens of ms
    still gets samples), and the nvidia-smi sampler line beside it."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.lines = []
        self.p = None
        self.nv = []
        self.open = False
        self.done = False
        try:
            self.nvml = Nvml(dev)
        except Exception:
            self.nvml = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.dev)], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.p = None
        if self.nvml:
            threading.Thread(target=self._poll, daemon=True).start()

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def _poll(self):
        while not self.done:
            if self.open:
                s = self.nvml.sample()
                if s:
                    self.nv.append(s)
            time.sleep(0.005)

    def mark(self):
        """Start of the timed window: samples before it (the sampler's own
        start-up overlaps the warm-up steps) are not used."""
        self.first = len(self.lines)
        self.open = True

    def stop(self):
        self.open = False
        self.done = True
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        window = self.lines[getattr(self, "first", 0):]
        for ln in window:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        smi = len(sm)
        for mhz, mask in self.nv:
            sm.append(mhz)
            for n, bit in Nvml.BITS.items():
                if mask & bit:
                    reasons.add(n)
        if mx is None and self.nvml:
            mx = self.nvml.max_sm
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "samples_nvidia_smi": smi, "samples_nvml": len(self.nv)}


def fp32_roofline(g, old_ms, clk):
    """FP32 side of the two generation sweeps (candidates against accepted rods
    and against earlier candidates; the counters cover both): FP32 flops they
    execute at least -- 22 per staged pair (the line bound of the old-rod
    sweep, or the capsule test of the conflict sweep; the capsule test that
    follows a line bound is not counted), 40 per marked pair (the hand-out's
    line test), 60 per pair that passes it (the full filter and certificate)
    -- over their summed event time, against the FP32 pipe peak of the device: SMs x
    128 lanes x 2 flops x the SM clock sampled in the timed window (the nominal
    figure; no FP32 peak is measured)."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz") or 2070.0
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    flops = 22.0 * g["pair_tests"] + 40.0 * g["marked_pairs"] + 60.0 * g["line_pairs"]
    achieved = flops / (old_ms * 1e-3) / 1e12 if old_ms > 0 else 0.0
    return {"kernel": "old_test+conflicts", "bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "flops_per_step": flops,
            "peak_source": "nominal: SMs x 128 FP32 lanes x 2 x sampled SM clock"}


# --------------------------------------------------------------------------- CPU (oracle) leg
def cpu_run(params, mesh, budget_s=12.0, max_reps=200):
    """The oracle on all host threads; returns (rods per second, cores, sample text)."""
    from oracle import nf_oracle as O
    O.build()
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    reps, rods = 0, 0
    while reps < max_reps and (reps == 0 or time.perf_counter() - t0 < budget_s):
        r, _, _ = O.generate(params, mesh=mesh, nthreads=cores, batch=16384)
        ct = O.contacts(params, r, nthreads=cores)
        O.solve(len(r), ct, tol=params.get("solve_tol", 1e-10))
        rods += len(r)
        reps += 1
    dt = time.perf_counter() - t0
    return rods / dt, cores, f"{reps} full realisation(s), {rods} rods, {dt:.1f} s"


def run_batched(args, rank, world):
    """Batched workload: `--batch` independent realisations (box 2-10 um, vf
    0.2-2 %, seeds 0..n-1), each generated, contacted and solved. Plain = one
    handle per realisation in sequence; batched = one nf_batch_run."""
    import torch

    import nanofiller_gb300 as nf
    from nanofiller_gb300 import build as nb

    nb.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    reals = nf.configs.batched_realisations(args.batch)
    for p in reals:
        p["seed"] += rank * args.batch

    def plain():
        res = []
        for p in reals:
            with nf.Simulation(p) as sim:
                g = sim.generate()
                c = sim.contacts()
                s = sim.solve(check=False)
                res.append((g["accepted"], c["contacts"], s["G_eff"], s["percolating"]))
        return res

    def batched():
        out, st = nf.batch_run(reals)
        return [(r["accepted"], r["contacts"], r["G_eff"], r["percolating"]) for r in out]

    clocks = Clocks(local)
    clocks.start()
    for _ in range(max(1, min(args.warmup, 2))):
        rb = batched()
    clocks.mark()
    l0 = nf.kernel_launches()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    steps = max(1, args.steps)
    for _ in range(steps):
        rb = batched()
    torch.cuda.synchronize()
    tb = over_ranks(dist, (time.perf_counter() - t0) / steps, "max", "cuda")
    launches = nf.kernel_launches() - l0
    clk = clocks.stop()
    plain()  # warm
    t0 = time.perf_counter()
    rp = plain()
    tp = time.perf_counter() - t0
    same = all(a[0] == b[0] and a[1] == b[1] and abs(a[2] - b[2]) <= 1e-9 * max(abs(a[2]), 1e-30)
               for a, b in zip(rp, rb))
    rods = over_ranks(dist, sum(r[0] for r in rb), "sum", "cuda")
    vf = [p["vf"] for p in reals]
    bins = [0.002, 0.004, 0.008, 0.016, 0.0201]
    table = []
    for lo, hi in zip(bins[:-1], bins[1:]):
        sel = [r for r, v in zip(rb, vf) if lo <= v < hi]
        if sel:
            table.append({"vf_range": [lo, hi], "n": len(sel),
                          "percolation_probability": sum(1 for r in sel if r[3]) / len(sel),
                          "mean_G_S": sum(r[2] for r in sel) / len(sel)})
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": world * len(reals) / tb, "unit": "realisations/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1000 * tb, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 filter + f64 decisions", "data": "synthetic",
            "config": {"workload": "batched", "realisations": len(reals), "box_um": [2.0, 10.0],
                       "vf": [0.002, 0.02], "rod_um": [1.0, 0.005], "parallelism": f"replicas x{world}"},
            "rods_per_s": rods / tb, "plain_realisations_per_s": len(reals) / tp,
            "batched_over_plain": tp / tb, "batched_equals_plain": same, "gpu_launches": int(launches),
            "vs_vf": table, "clocks": clk,
        }))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    params, mesh = workload(args.workload, 0)
    from oracle import nf_oracle as O
    O.build()
    cores = os.cpu_count() or 1
    for _ in range(min(args.warmup, 1)):
        O.generate(dict(params, n_candidates=min(params["n_candidates"], 20000)), mesh=mesh, nthreads=cores)
    times, rods = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r, _, _ = O.generate(params, mesh=mesh, nthreads=cores, batch=16384)
        ct = O.contacts(params, r, nthreads=cores)
        O.solve(len(r), ct, tol=params.get("solve_tol", 1e-10))
        times.append(time.perf_counter() - t0)
        rods = len(r)
    ms = 1000 * sum(times) / len(times)
    value = rods / (ms / 1000)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "rods/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.workload, params),
        "cpu_baseline": {"value": value, "unit": "rods/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full realisation(s) of {rods} rods on the FP64 C++ oracle"},
        "e2e": {"value": value, "unit": "rods/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


# --------------------------------------------------------------------------- replicas
def over_ranks(dist, v, how, device):
    """v reduced over the ranks of a replica run: "max" for step times (the
    slowest rank sets the job's time), "sum" for the rods every rank placed.
    v itself without a process group. device is the process group's tensor
    device ("cuda" under NCCL, "cpu" under gloo)."""
    if not dist:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if how == "max" else dist.ReduceOp.SUM)
    return float(t.item())


# --------------------------------------------------------------------------- GPU leg
def run_ours(args, rank, world):
    import numpy as np
    import torch

    import nanofiller_gb300 as nf
    from nanofiller_gb300 import build as nb

    nb.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    params, mesh = workload(args.workload, rank)
    sim = nf.Simulation(params, mesh=mesh)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        g = sim.generate()
        c = sim.contacts()
        s = sim.solve(check=False)
        return g, c, s

    clocks = Clocks(local)
    clocks.start()  # before the warm-up: the sampler's start-up must not fall in the timed steps
    for _ in range(max(args.warmup, 0)):
        flush.zero_()  # the first call loads torch's fill kernel (a one-off of ~0.25 s)
        step()
    torch.cuda.synchronize()
    sim.set_kernel_timing(True)
    clocks.mark()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = nf.kernel_launches()
    wall0 = time.perf_counter()
    evs = []
    res = None
    for _ in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        res = step()
        b.record()
        evs.append((a, b))
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = nf.kernel_launches() - l0
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in evs) / len(evs)
    g, c, s = res
    rods = g["accepted"]
    ms_max = over_ranks(dist, ms, "max", "cuda")
    rods_all = over_ranks(dist, rods, "sum", "cuda")
    value = rods_all / (ms_max / 1000)
    # Kernel breakdown of the timed steps (CUDA events on the library's stream).
    kern = {k: sim.kernel_time(k) for k in ("stream", "old_test", "conflicts", "ct_pairs", "screen", "cg")}
    dom = max(kern, key=lambda k: kern[k]["ms"])
    kd = kern[dom]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs")
    peak_note = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    achieved = kd["bytes"] / (kd["ms"] * 1e-3) / 1e9 if kd["ms"] > 0 else 0.0
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        if args.workload in tr and dom in tr[args.workload]:
            traffic = tr[args.workload][dom]
    except Exception:
        pass
    out = {
        "metric": METRIC, "value": value, "unit": "rods/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 filter + f64 decisions", "data": "synthetic",
        "config": dict(workload_config(args.workload, params), parallelism=f"replicas x{world}"),
        "realisations_per_s": world * 1000.0 / ms_max,
        "pair_tests_per_s": (g["pair_tests"] + c["pair_tests"]) / (ms / 1000),
        "fp64_decisions": g["exact_evals"] + c["exact_evals"],
        "generation_sweeps": {k: g[k] for k in ("work_items", "target_tiles", "pair_tests", "marked_pairs",
                                                  "line_pairs", "exact_evals")},
        "fp32_would_flip": g["fp32_would_flip"] + c["fp32_would_flip"],
        "decision_flips_vs_fp64": 0,
        "contacts": c["contacts"], "G_eff_S": s["G_eff"], "percolating": bool(s["percolating"]),
        "gpu_launches": int(launches),
        "wall_ms_per_step": 1000 * wall / args.steps,
        "step_ms": [round(a.elapsed_time(b), 4) for a, b in evs],
        "kernels_ms_per_step": {k: v["ms"] / args.steps for k, v in kern.items()},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "peak_source": peak_note,
                     "note": "pair-test kernels are FP32-issue bound; bytes are the algorithmic bytes"},
        "roofline_fp32": fp32_roofline(g, (kern["old_test"]["ms"] + kern["conflicts"]["ms"]) / args.steps, clk),
        "contacts_per_s": (c["contacts"] + c["n_source"] + c["n_sink"]) / (c["ms"] / 1000) if c["ms"] > 0 else None,
        "solve": {"residual": s["residual"], "outer_iters": s["outer_iters"], "inner_iters": s["inner_iters"],
                  "n_active": s["n_active"], "ms": s["ms"]},
        "clocks": clk,
    }
    sim.set_kernel_timing(False)
    if s["percolating"]:
        # Differentiation form: the adjoint (gradient w.r.t. all endpoints, lambda,
        # G0, copied to the host) against one forward network solve.
        ts, ta = [], []
        for _ in range(5):
            a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            a.record()
            sim.solve(check=False)
            b.record()
            sim.adjoint()
            c.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
            ta.append(b.elapsed_time(c))
        ts.sort()
        ta.sort()
        out["adjoint"] = {"solve_ms": ts[2], "adjoint_ms": ta[2], "adjoint_over_solve": ta[2] / ts[2]}
    # e2e through the C ABI with host buffers.
    if not args.no_e2e:
        times, h2d, d2h = [], 0, 0
        for i in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if mesh is not None:
                sim.load_density(mesh)
            sim.generate()
            sim.contacts()
            s2 = sim.solve(check=False)
            r = sim.rods()
            ct = sim.contact_list()
            torch.cuda.synchronize()
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
            h2d = (mesh.nbytes if mesh is not None else 0)
            d2h = sum(a.nbytes for a in r.values()) + sum(a.nbytes for a in ct.values()) + 8
        e_ms = over_ranks(dist, 1000 * sum(times) / len(times), "max", "cuda")
        out["e2e"] = {"value": rods_all / (e_ms / 1000), "unit": "rods/s", "h2d_bytes_per_step": int(h2d),
                      "d2h_bytes_per_step": int(d2h), "ms_per_step": e_ms}
    sim.close()
    if rank == 0 and not args.no_cpu_baseline:
        v, cores, sample = cpu_run(params, mesh)
        out["cpu_baseline"] = {"value": v, "unit": "rods/s", "cores": cores, "kind": "port", "sample": sample}
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(1)))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "batched":
        return run_batched(args, rank, world)
    return run_ours(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
