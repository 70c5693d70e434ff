"""Benchmark: IDG grid + degrid (w-stacked) on the 3072^2 workload.

One step = IDG.GridW (gridder, subgrid IFFT, w-stack adder) + IDG.DeGridW (splitter,
subgrid FFT, degridder) over the whole synthetic observation: 2016 baselines x 2000
times x 16 channels (64.5M visibilities, 42M of them gridded after the partitioner's
channel-span drop), N = 3072, S = 32, 8 w layers.  The metric counts visibilities
processed by the gridder plus the degridder per second.

  value : device-resident buffers (C ABI device entry points), CUDA events on the plan's stream
  e2e   : the reference-facing host API (IDG.GridW / IDG.DeGridW with Complex[...] host
          arrays in pinned memory), host<->device copies inside the timed region
  --impl reference : the CPU restatement of the reference gridder (oracle/) on all host cores
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

import __graft_entry__ as entry  # noqa: E402

WORKLOAD = "meerkat_3072"
METRIC = "Mvis/s grid+degrid at 3072², TC split-precision vs FP32, rel-L2 err vs FP64"
MODES = {"fp32": 0, "tc_bf16x3": 1, "tc_fp16x3": 2}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class NvmlClockSampler:
    """SM clock and clock-event (throttle) reasons read through NVML every ~2 ms in a thread during
    the timed region (read-only queries).  None when NVML cannot be loaded."""
    NAMES = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self, gpu_index):
        import ctypes
        self.ct = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        bus = _pci_bus_id(gpu_index)  # the CUDA device's own GPU, whatever CUDA_VISIBLE_DEVICES says
        if bus is None or self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h)) != 0:
            if self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(gpu_index), ctypes.byref(self.h)) != 0:
                raise OSError("no NVML handle")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(self.lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        self.rows = []
        self.stop_flag = threading.Event()

    def _sample(self):
        ct = self.ct
        mhz, mx, rs = ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, ct.c_int(1), ct.byref(mx))  # NVML_CLOCK_SM
        while not self.stop_flag.is_set():
            if self.lib.nvmlDeviceGetClockInfo(self.h, ct.c_int(1), ct.byref(mhz)) == 0 and \
                    self.reasons_fn(self.h, ct.byref(rs)) == 0:
                self.rows.append((mhz.value, mx.value, rs.value))
            time.sleep(0.002)

    def start(self):
        self.t = threading.Thread(target=self._sample, daemon=True)
        self.t.start()

    def stop(self):
        self.stop_flag.set()
        self.t.join(timeout=5)
        self.lib.nvmlShutdown()
        sm = [r[0] for r in self.rows]
        reasons = sorted({n for r in self.rows for bit, n in self.NAMES.items() if r[2] & bit})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(r[1] for r in self.rows) if self.rows else None,
                "reasons": reasons, "samples": len(self.rows), "source": "nvml"}


def _pci_bus_id(cuda_index):
    """NVML's "domain:bus:device.0" id of a CUDA device, or None."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(cuda_index)
        return f"{pr.pci_domain_id:08X}:{pr.pci_bus_id:02X}:{pr.pci_device_id:02X}.0"
    except (ImportError, AttributeError, RuntimeError):
        return None


def clock_sampler(gpu_index):
    """NVML sampler where the library loads, else nvidia-smi."""
    try:
        return NvmlClockSampler(gpu_index)
    except (OSError, AttributeError):
        return ClockSampler(gpu_index)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def gpu_local_cpus(gpu_index):
    """Host CPUs on the GPU's own NUMA node (sysfs local_cpulist of its PCI function), or None."""
    try:
        bus = subprocess.run(["nvidia-smi", "--query-gpu=pci.bus_id", "--format=csv,noheader", "-i", str(gpu_index)],
                             capture_output=True, text=True, timeout=20).stdout.strip()
        dom, rest = bus.split(":", 1)
        path = f"/sys/bus/pci/devices/{int(dom, 16):04x}:{rest.lower()}/local_cpulist"
        cpus = set()
        with open(path) as f:
            for part in f.read().strip().split(","):
                a, _, b = part.partition("-")
                cpus.update(range(int(a), int(b or a) + 1))
        cpus &= os.sched_getaffinity(0)
        return cpus or None
    except (OSError, ValueError, subprocess.SubprocessError):
        return None


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def traffic_per_launch(kernel):
    """Per-launch DRAM bytes from the committed ncu summary (profiles/traffic_per_launch.txt)."""
    p = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3 and not line.startswith("#") and parts[0] == kernel and parts[1] == WORKLOAD:
                return float(parts[2])
    return None


def pick_sample(subs, nch, target_vis, seed=0):
    rng = np.random.default_rng(seed)
    take, tot = [], 0
    for i in rng.permutation(len(subs)):
        take.append(i)
        tot += int(subs[i]["time_sample_count"]) * nch
        if tot >= target_vis:
            break
    return subs[np.sort(np.array(take, dtype=np.int64))], tot


def cpu_reference_step(oracle, cd, sample, obs, model_grid):
    """One sample of the reference gridder restated on the CPU: GridW + DeGridW of the sample."""
    layers = oracle.idg_grid_w(cd, sample, obs.vis, obs.uvw, obs.frequencies)
    vis, _ = oracle.idg_degrid(cd, sample, model_grid, obs.uvw, obs.frequencies, wstack=True)
    return layers, vis


def calibrate_cpu_sample(oracle, cd, subs, obs, model_grid, budget_s):
    """A seeded subgrid sample whose CPU grid+degrid takes about budget_s (from a short pilot)."""
    nch = obs.vis.shape[2]
    # two pilots: the fixed cost (w-layer allocation and shifts) and the per-visibility cost
    t0 = time.perf_counter()
    cpu_reference_step(oracle, cd, subs[:0], obs, model_grid)
    fixed = time.perf_counter() - t0
    sample, n1 = pick_sample(subs, nch, 250000, seed=1)
    t0 = time.perf_counter()
    cpu_reference_step(oracle, cd, sample, obs, model_grid)
    t1 = time.perf_counter() - t0
    per_vis = max((t1 - fixed) / max(n1, 1), 1e-9)
    target = int(max(budget_s - fixed, 0.5 * budget_s) / per_vis)
    sample, nv = pick_sample(subs, nch, target)
    return sample, nv, fixed


def load_oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # noqa: E402  (CPU baseline leg only)
    oracle.lib()
    return oracle


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))
    oracle = load_oracle()
    obs, cd = synth.build(WORKLOAD)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    model_grid = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    cores = oracle.num_threads()
    budget = max(3.0, min(20.0, 120.0 / max(1, args.steps + args.warmup)))
    sample, nv, _ = calibrate_cpu_sample(oracle, cd, subs, obs, model_grid, budget)
    for _ in range(args.warmup):
        cpu_reference_step(oracle, cd, sample, obs, model_grid)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu_reference_step(oracle, cd, sample, obs, model_grid)
        times.append(time.perf_counter() - t0)
    t = sum(times)
    value = 2 * nv * args.steps / t / 1e6
    gridded = int(subs["time_sample_count"].sum()) * obs.vis.shape[2]
    desc = (f"{len(sample)} of {len(subs)} subgrids ({nv} of {gridded} gridded visibilities), seeded; "
            f"GridW + DeGridW of the sample, FP64, {cores} OpenMP threads")
    out = {"metric": METRIC, "value": value, "unit": "Mvis/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, 3072^2 workload)",
           "impl": "reference",
           "config": {"workload": "3072^2 IDG grid+degrid: 2016 bl x 2000 t x 16 ch, S=32, W=8",
                      "sample": desc},
           "cpu_baseline": {"value": value, "unit": "Mvis/s", "cores": cores, "kind": "port", "sample": desc},
           "e2e": {"value": value, "unit": "Mvis/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


def link_rates(nbytes=256 << 20, reps=3):
    """This machine's host-link rates (GB/s): copies of nbytes between device memory and page-locked
    host memory, best of reps after one warm-up.  The e2e figure moves its bytes over this link, so
    the rates say whether a low e2e comes from the box."""
    import torch

    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    s = torch.cuda.current_stream()
    out = {}
    for name, copy in (("h2d", lambda: d.copy_(h, non_blocking=True)),
                       ("d2h", lambda: h.copy_(d, non_blocking=True))):
        best = 0.0
        for i in range(reps + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            copy()
            e1.record(s)
            e1.synchronize()
            if i:
                best = max(best, nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9)
        out[name] = round(best, 1)
    out["bytes"] = nbytes
    return out


def run_cd(args):
    """FastSerialCD alone at the 3072^2 workload's sizes: a 3072^2 image and a 384^2 PSF (cut 8,
    so a 768^2 PSF^2 window); a seeded synthetic PSF (Gaussian main lobe + noise sidelobes) and
    gradient map.  The CPU oracle (float, as the C#) runs the first iterations beside it."""
    pkg = entry.load_package()
    n, p = 3072, 384
    rng = np.random.default_rng(0)
    yy, xx = np.mgrid[:p, :p] - p // 2
    psf = (np.exp(-(yy ** 2 + xx ** 2) / 50.0) + 0.01 * rng.standard_normal((p, p))).astype(np.float32)
    g0 = (rng.standard_normal((n, n)) * 10).astype(np.float32)
    x0 = np.zeros((n, n), np.float32)
    cd = pkg.FastSerialCD(pkg.Rectangle(0, 0, n, n), psf)
    lam, alpha, eps = 0.5, 0.2, 1e-9
    cd.Deconvolve(x0.copy(), g0.copy(), lam, alpha, 300, eps)  # warm-up: graph capture
    clocks = clock_sampler(0)
    clocks.start()
    x, g = x0.copy(), g0.copy()
    r = cd.Deconvolve(x, g, lam, alpha, args.cd, eps)
    clk = clocks.stop()
    per_iter = r.ElapsedMs * 1e-3 / max(1, r.IterationCount)
    cpu = None
    if not args.no_cpu_baseline:
        oracle = load_oracle()
        psf2, amap = cd.maps()
        k = 60
        xs, gs = x0.copy(), g0.copy()
        cd.Deconvolve(xs, gs, lam, alpha, k, eps)
        t0 = time.perf_counter()
        ox, og, _, oit = oracle.deconvolve(x0, g0, amap, psf2, lam, alpha, k, eps)
        cpu_s = time.perf_counter() - t0
        cpu = {"value": oit / cpu_s, "unit": "iterations/s", "cores": oracle.num_threads(), "kind": "port",
               "sample": f"the first {k} iterations from the same start, FastSerialCD restated in C (float)",
               "bit_identical_to_gpu": bool(xs.tobytes() == ox.tobytes() and gs.tobytes() == og.tobytes())}
    out = {"metric": "FastSerialCD iterations/s at 3072^2 (384^2 PSF, 768^2 update window)",
           "value": 1.0 / per_iter, "unit": "iterations/s", "n_gpus": 1, "steps": 1, "warmup": 1,
           "ms_per_step": r.ElapsedMs, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded PSF and gradient map)",
           "config": {"workload": f"{n}^2 image, {p}^2 PSF, lambda {lam}, alpha {alpha}",
                      "iterations": r.IterationCount, "us_per_iteration": per_iter * 1e6},
           "cpu_baseline": cpu, "clocks": clk}
    print(json.dumps(out), flush=True)
    return 0


def run_major_cycle(args):
    """The full imaging loop on the 3072^2 workload: serial-CD major cycles (MajorCycle.cs:33-134,
    lambda 1.0, alpha 0.01, PSF cut 8) with the BF16x3 gridder, beside the same loop with the
    FP32 gridder; the FP64 CPU oracle runs the same loop on a small sample observation."""
    import torch

    pkg = entry.load_package()
    synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))
    kw = dict(psfCutFactor=8, maxMajorCycle=args.mc_cycles, lambda_=1.0, alpha=0.01,
              deconvIterations=args.mc_iterations, deconvEpsilon=1e-5)

    def gpu_loop(obs, cd, mode_name, kwargs):
        c = pkg.GriddingConstants.from_dict(cd)
        N = cd["grid_size"]
        part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
        part.plan.set_mode(MODES[mode_name])
        d_vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
        d_flags = torch.from_numpy(obs.flags.astype(np.uint8)).cuda()
        img = [torch.empty((N, N), dtype=torch.float32, device="cuda") for _ in range(3)]
        ptrs = (part.plan, d_vis.data_ptr(), d_flags.data_ptr(), img[0].data_ptr(), img[1].data_ptr(),
                img[2].data_ptr())
        warm = dict(kwargs, maxMajorCycle=1, deconvIterations=min(10, kwargs["deconvIterations"]))
        pkg.MajorCycle.reconstruct_serial_cd_device(*ptrs, **warm)  # module load, FFT plans
        torch.cuda.synchronize()
        clocks = clock_sampler(0)
        clocks.start()
        t0 = time.perf_counter()
        cycles = pkg.MajorCycle.reconstruct_serial_cd_device(*ptrs, **kwargs)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clk = clocks.stop()
        return dict(wall_s=wall, cycles=cycles, model=img[0].cpu().numpy(), residual=img[1].cpu().numpy(),
                    psf=img[2].cpu().numpy(), clocks=clk)

    obs, cd = synth.build(WORKLOAD)
    runs = {m: gpu_loop(obs, cd, m, kw) for m in ("tc_bf16x3", "fp32")}
    tc, fp = runs["tc_bf16x3"], runs["fp32"]
    iters = sum(int(c["iterations"]) for c in tc["cycles"])
    deconv_s = sum(c["deconv_ms"] for c in tc["cycles"]) / 1e3

    def rel(a, b):
        return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))

    cpu = None
    if not args.no_cpu_baseline:
        oracle = load_oracle()
        sobs, scd = synth.build(synth.scaled_workload("small_256", n_ant=16, nt=480, nch=8, seed=7))
        subs = oracle.partition(scd, sobs.uvw, sobs.frequencies)
        skw = dict(kw, maxMajorCycle=args.mc_cycles)
        t0 = time.perf_counter()
        ref = oracle.major_cycle(scd, subs, sobs.uvw, sobs.frequencies, sobs.vis, sobs.flags.astype(np.uint8),
                                 skw["psfCutFactor"], skw["maxMajorCycle"], skw["lambda_"], skw["alpha"],
                                 skw["deconvIterations"], skw["deconvEpsilon"])
        cpu_s = time.perf_counter() - t0
        g = gpu_loop(sobs, scd, "fp32", skw)
        gt = gpu_loop(sobs, scd, "tc_bf16x3", skw)
        nvis = int(np.prod(sobs.vis.shape))
        cpu = {"value": cpu_s, "unit": "s per reconstruction", "cores": oracle.num_threads(), "kind": "port",
               "sample": (f"the same loop on a 256^2 observation (16 antennas, 480 times, 8 channels: {nvis} "
                          f"visibilities, {len(ref['cycles'])} cycles, "
                          f"{int(ref['cycles']['iterations'].sum())} CD iterations), FP64 gridder"),
               "gpu_fp32_same_sample_s": g["wall_s"], "gpu_tc_same_sample_s": gt["wall_s"],
               "model_rel_l2_gpu_fp32_vs_cpu": rel(g["model"], ref["model"]),
               "residual_rel_l2_gpu_fp32_vs_cpu": rel(g["residual"], ref["residual"]),
               "model_rel_l2_gpu_tc_vs_cpu": rel(gt["model"], ref["model"]),
               "residual_rel_l2_gpu_tc_vs_cpu": rel(gt["residual"], ref["residual"])}
        cpu["objective_per_cycle_cpu_gpu_fp32_gpu_tc"] = [
            (float(r), float(x["objective"]), float(y["objective"]))
            for r, x, y in zip(ref["cycles"]["objective"], g["cycles"], gt["cycles"])]
    first = None
    if args.mc_cpu_full and not args.no_cpu_baseline:
        # the FP64 oracle on the full 3072^2 observation: PSF, first dirty image, gradients and the
        # first CD decisions of the first major cycle, against the GPU loop run to the same point
        oracle = load_oracle()
        n_it = 200
        subs = oracle.partition(cd, obs.uvw, obs.frequencies)
        t0 = time.perf_counter()
        ref = oracle.major_cycle(cd, subs, obs.uvw, obs.frequencies, obs.vis, obs.flags.astype(np.uint8),
                                 kw["psfCutFactor"], 1, kw["lambda_"], kw["alpha"], n_it, kw["deconvEpsilon"])
        cpu_full_s = time.perf_counter() - t0
        part_kw = dict(kw, maxMajorCycle=1, deconvIterations=n_it)
        first = {"cpu_s": cpu_full_s, "cd_iterations": n_it, "cores": oracle.num_threads()}
        for m in ("fp32", "tc_bf16x3"):
            gg = gpu_loop(obs, cd, m, part_kw)
            same_px = np.array_equal(np.flatnonzero(gg["model"]), np.flatnonzero(ref["model"]))
            first[m] = {"psf_rel_l2": rel(gg["psf"], ref["psf"]),
                        "first_dirty_image_rel_l2": rel(gg["residual"], ref["residual"]),
                        "max_b_gpu_cpu": (float(gg["cycles"][0]["max_b"]), float(ref["cycles"]["max_b"][0])),
                        "objective_gpu_cpu": (float(gg["cycles"][0]["objective"]),
                                              float(ref["cycles"]["objective"][0])),
                        "model_rel_l2": rel(gg["model"], ref["model"]),
                        "same_selected_pixels": bool(same_px),
                        "nonzero_pixels_gpu_cpu": (int(np.count_nonzero(gg["model"])),
                                                   int(np.count_nonzero(ref["model"])))}
    slim = [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in c.items()} for c in tc["cycles"]]
    out = {"metric": f"s per {args.mc_cycles}-cycle serial-CD reconstruction at 3072^2 (BF16x3 gridder)",
           "value": tc["wall_s"], "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 1,
           "ms_per_step": 1e3 * tc["wall_s"], "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "tc_bf16x3 gridder, f32 images / coordinate descent, f64 correlation",
           "data": "synthetic (seeded 3072^2 observation and sky)",
           "config": {"workload": "3072^2: 2016 bl x 2000 t x 16 ch, S=32, W=8; PSF cut 8; "
                                  f"lambda 1.0, alpha 0.01, <= {args.mc_iterations} CD iterations per cycle, eps 1e-5",
                      "cycles_run": len(tc["cycles"])},
           "cycles": slim,
           "cd_iterations": iters, "cd_iterations_per_s": iters / deconv_s if deconv_s > 0 else None,
           "fp32_gridder_s": fp["wall_s"],
           "model_rel_l2_tc_vs_fp32": rel(tc["model"], fp["model"]),
           "residual_rel_l2_tc_vs_fp32": rel(tc["residual"], fp["residual"]),
           "psf_rel_l2_tc_vs_fp32": rel(tc["psf"], fp["psf"]),
           "objective_per_cycle_tc_fp32": [(float(x["objective"]), float(y["objective"]))
                                           for x, y in zip(tc["cycles"], fp["cycles"])],
           "first_cycle_vs_cpu_full_size": first,
           "cpu_baseline": cpu, "clocks": tc["clocks"]}
    print(json.dumps(out), flush=True)
    return 0


def run_batched(args):
    """N independent problems (512^2..2048^2, 200-2000 times, 4-32 channels, 16-64 antennas):
    autotuned on the largest, gridded + degridded as one batch replayed from a CUDA graph."""
    import torch

    pkg = entry.load_package()
    synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))
    mode_name = "tc_bf16x3" if args.mode == "auto" else args.mode
    t0 = time.perf_counter()
    geos = [synth.build_geometry(w) for w in synth.batched_workloads(args.batched, seed=4, mix=args.mix)]
    big = max(range(len(geos)), key=lambda i: geos[i][0].shape[0] * geos[i][0].shape[1] * len(geos[i][1]))
    uvw_b, f_b, cd_b = geos[big]
    tune = pkg.autotune(pkg.GriddingConstants.from_dict(cd_b), uvw_b, f_b, MODES[mode_name],
                        [32] if mode_name != "fp32" else [24, 32, 48])
    S = tune["subgrid_size"]
    plans, bufs, info = [], [], []
    gen = torch.Generator(device="cuda").manual_seed(11)
    for uvw, freq, cd in geos:
        d = dict(cd)
        d["subgrid_size"] = S
        c = pkg.GriddingConstants.from_dict(d)
        part = pkg.Partitioner.CreatePartition(c, uvw, freq)
        part.plan.set_mode(MODES[mode_name])
        pkg.set_chunking(part.plan, tune["gridder_max_vis"], tune["degridder_max_vis"])
        N, W = d["grid_size"], d["wlayer_count"]
        shape = (uvw.shape[0], uvw.shape[1], len(freq))
        bufs.append(dict(vis=torch.randn(shape, dtype=torch.complex64, device="cuda", generator=gen),
                         layers=torch.empty((W, N, N), dtype=torch.complex64, device="cuda"),
                         grid=torch.randn((N, N), dtype=torch.complex64, device="cuda", generator=gen),
                         out=torch.empty(shape, dtype=torch.complex64, device="cuda")))
        plans.append(part.plan)
        info.append(part.plan.info())
    setup_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    batch = pkg.Batch(plans, [b["vis"].data_ptr() for b in bufs], [b["layers"].data_ptr() for b in bufs],
                      [b["grid"].data_ptr() for b in bufs], [b["out"].data_ptr() for b in bufs])
    batch.capture_graph()
    stream = torch.cuda.ExternalStream(batch.stream())
    for _ in range(max(3, args.warmup)):
        batch.run()
    batch.synchronize()
    clocks = clock_sampler(0)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        batch.run()
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    batch.synchronize()
    ms = e0.elapsed_time(e1)
    lat = batch.latencies_ms()
    gridded = sum(i["gridded_visibilities"] for i in info)
    value = 2 * gridded * args.steps / (ms * 1e-3) / 1e6
    # the same batch with the problems run smallest first (per-problem latency over throughput)
    batch.set_schedule(pkg.Batch.SMALL_FIRST)
    batch.capture_graph()
    for _ in range(2):
        batch.run()
    batch.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        batch.run()
    f1.record(stream)
    f1.synchronize()
    batch.synchronize()
    ms_small = f0.elapsed_time(f1)
    lat_small = batch.latencies_ms()
    # the same problems one after the other through the single-plan device entry points
    seq_stream = torch.cuda.Stream()
    for p in plans:
        p.set_stream(seq_stream.cuda_stream)
    def seq_step():
        for p, b in zip(plans, bufs):
            p.grid_w_device(b["vis"].data_ptr(), b["layers"].data_ptr())
            p.degrid_w_device(b["grid"].data_ptr(), b["out"].data_ptr())
    seq_step()
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(seq_stream)
    for _ in range(args.steps):
        seq_step()
    s1.record(seq_stream)
    s1.synchronize()
    seq_ms = s0.elapsed_time(s1)
    sizes = [(g[2]["grid_size"], g[0].shape[0], g[0].shape[1], len(g[1])) for g in geos]
    out = {"metric": f"Mvis/s grid+degrid, {len(geos)} independent problems in one graph-replayed batch",
           "value": value, "unit": "Mvis/s", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup),
           "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": mode_name, "data": "synthetic geometry (seeded); random complex64 visibilities and model grids",
           "config": {"workload": (f"{len(geos)} problems: N 512-2048, 200-2000 times, 4-32 channels, 16-64 antennas"
                                   if args.mix == "config" else
                                   f"{len(geos)} small problems: N 512-1024, 200-500 times, 4-16 channels, "
                                   f"16-32 antennas"),
                      "mode": mode_name, "tuning": tune, "gridded_visibilities": int(gridded),
                      "input_visibilities": int(sum(i["input_visibilities"] for i in info)),
                      "subgrids": int(sum(i["num_subgrids"] for i in info)), "setup_s": round(setup_s, 2),
                      "problems": sizes},
           "per_problem_latency_ms": {"min": float(lat.min()), "median": float(np.median(lat)),
                                      "max": float(lat.max()),
                                      "note": "degrid phase: from its start to each problem's last visibility"},
           "small_first_schedule": {"value": 2 * gridded * args.steps / (ms_small * 1e-3) / 1e6,
                                    "ms_per_step": ms_small / args.steps,
                                    "per_problem_latency_ms": {"min": float(lat_small.min()),
                                                               "median": float(np.median(lat_small)),
                                                               "max": float(lat_small.max())}},
           "sequential_per_plan_ms_per_step": seq_ms / args.steps,
           "batch_speedup_over_sequential": seq_ms / ms,
           "clocks": clk}
    print(json.dumps(out), flush=True)
    batch.destroy()
    return 0


def time_mode(plan, pkg, mode, step, stream, steps, warmup, ws, clock_gpu=None):
    """Warm-up, then K timed steps between CUDA events on the plan's stream (max over ranks)."""
    import torch

    plan.set_mode(MODES[mode])
    for _ in range(max(3, warmup)):
        step()
    plan.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = clock_sampler(clock_gpu) if clock_gpu is not None else None
    if clocks:
        clocks.start()
    plan.reset_timing()
    plan.enable_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    e1.synchronize()
    plan.synchronize()
    clk = clocks.stop() if clocks else None
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    stages = plan.stage_times()
    plan.enable_timing(False)
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, stages, clk


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="auto", choices=["auto"] + list(MODES),
                    help="headline kernels; auto = tensor-core BF16x3, with the FP32 kernels timed beside it")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--antennas", type=int, default=None,
                    help="smaller array (fewer baselines) of the same workload, for profiling captures")
    ap.add_argument("--batched", type=int, default=0,
                    help="instead: N independent problems of mixed sizes in one batch (graph-replayed)")
    ap.add_argument("--mix", default="config", choices=["config", "small"],
                    help="--batched problem mix: the configured sizes, or problems too small to fill the GPU")
    ap.add_argument("--major-cycle", action="store_true",
                    help="instead: the serial-CD major-cycle loop on the same workload")
    ap.add_argument("--mc-cycles", type=int, default=6)
    ap.add_argument("--mc-iterations", type=int, default=30000)
    ap.add_argument("--mc-cpu-full", action="store_true",
                    help="--major-cycle: also run the FP64 oracle's first cycle (PSF, dirty image, 200 CD "
                         "iterations) on the full 3072^2 observation (about a minute of host cores)")
    ap.add_argument("--cd", type=int, default=0,
                    help="instead: this many FastSerialCD iterations at 3072^2 (iterations/s)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.batched:
        return run_batched(args)
    if args.major_cycle:
        return run_major_cycle(args)
    if args.cd:
        return run_cd(args)

    import torch

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkg = entry.load_package()
    synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))

    # one observation for the whole job (strong scaling): with N ranks it is split by baseline into
    # contiguous blocks balanced by gridded visibilities, as the reference's MPI driver splits it
    # (DistributedData.cs:94-96); each rank partitions and grids its block, the w layers are summed
    # and one N x N grid is all-reduced (MPIMajorCycle.cs:173), the model grid is broadcast before
    # DeGridW (MPIMajorCycle.cs:106), all inside the timed step
    wl = synth.scaled_workload(WORKLOAD, n_ant=args.antennas)
    obs, cd = synth.build(wl)
    c = pkg.GriddingConstants.from_dict(cd)
    t_plan = time.perf_counter()
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)  # the partitioner, on the host
    plan_ms = 1e3 * (time.perf_counter() - t_plan)
    total_gridded = part.plan.info()["gridded_visibilities"]
    reducer = None
    block = (0, obs.uvw.shape[0])
    if ws > 1:
        dmod = entry._load_module(entry.PKG_NAME + ".distributed", os.path.join(entry.PKG_DIR, "distributed.py"))
        weights = dmod.gridded_per_baseline(part.plan.subgrids(), obs.uvw.shape[0], len(obs.frequencies))
        block = dmod.balanced_baseline_blocks(weights, ws)[rank]
        part.plan.destroy()
        b0, b1 = block
        obs.uvw = np.ascontiguousarray(obs.uvw[b0:b1])
        obs.vis = np.ascontiguousarray(obs.vis[b0:b1])
        obs.flags = np.ascontiguousarray(obs.flags[b0:b1])
        part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
        reducer = dmod.GridReducer()
    plan = part.plan
    info = plan.info()
    headline = "tc_bf16x3" if args.mode == "auto" else args.mode
    # config 3 times both split-precision forms beside the FP32 kernels
    compare = ["fp32", "tc_fp16x3"] if args.mode == "auto" else []

    stream = torch.cuda.Stream()
    plan.set_stream(stream.cuda_stream)
    N, W, S = cd["grid_size"], cd["wlayer_count"], cd["subgrid_size"]
    model_img = obs.model_image.astype(np.float32)
    model_grid = pkg.FFT.Forward(np.fft.ifftshift(model_img) if N % 2 == 0 else model_img)
    with torch.cuda.stream(stream):
        d_vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
        d_layers = torch.empty((W, N, N), dtype=torch.complex64, device="cuda")
        d_grid = torch.from_numpy(model_grid.astype(np.complex64)).cuda()
        d_out = torch.empty_like(d_vis)
        d_img = torch.empty((N, N), dtype=torch.float32, device="cuda")
    stream.synchronize()

    def step():
        plan.grid_w_device(d_vis.data_ptr(), d_layers.data_ptr())
        if reducer is not None:
            with torch.cuda.stream(stream):  # collectives ordered on the plan's stream
                reducer.sum_layers_device_(d_layers)  # layer sum + all-reduce of one N x N grid
                reducer.broadcast_device_(d_grid, root=0)
        plan.degrid_w_device(d_grid.data_ptr(), d_out.data_ptr())

    gridded = info["gridded_visibilities"]  # this rank's block
    if ws > 1:
        tg = torch.tensor([gridded], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(tg, op=torch.distributed.ReduceOp.SUM)
        assert int(tg.item()) == total_gridded, "the blocks' partitions must add up to the global one" 
    results = {}
    for mode in compare + [headline]:  # headline last: its clocks are sampled
        ms, stages, clk = time_mode(plan, pkg, mode, step, stream, args.steps, args.warmup, ws,
                                    clock_gpu=local if mode == headline else None)
        results[mode] = dict(ms=ms, stages=stages, clk=clk,
                             value=2 * total_gridded * args.steps / (ms * 1e-3) / 1e6)
    head = results[headline]
    stages = head["stages"]
    # one launch per timed stage, plus the two zero-fills each step runs beside the gridder (w layers)
    # and the degridder (uncovered visibilities), outside the stages
    launches = sum(n for (_, n) in stages.values()) - stages["h2d"][1] - stages["d2h"][1] + 2 * args.steps

    # tensor-core vs FP32 kernels on the whole workload: w layers, degridded visibilities, dirty image
    tc_vs_fp32 = None
    if compare:
        outs = {}
        for mode in ("fp32", headline):
            plan.set_mode(MODES[mode])
            step()
            plan.wstack_image_device(d_layers.data_ptr(), d_img.data_ptr(), True)
            plan.synchronize()
            outs[mode] = (d_layers.clone(), d_out.clone(), d_img.clone())

        def rel_dev(a, b):
            return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))

        a, b = outs[headline], outs["fp32"]
        tc_vs_fp32 = {"grid_w": rel_dev(a[0], b[0]), "degrid_w": rel_dev(a[1], b[1]),
                      "dirty_image": rel_dev(a[2], b[2]), "visibilities": int(gridded)}
        del outs, a, b
        plan.set_mode(MODES[headline])

    # the full-grid w-layer FFT (FFT.WStackIFFTFloat + FFT.Shift), timed separately
    plan.reset_timing()
    plan.enable_timing(True)
    for _ in range(3):
        plan.wstack_image_device(d_layers.data_ptr(), d_img.data_ptr(), True)
    layer_fft = plan.stage_times()["layer_fft"]
    plan.enable_timing(False)
    layer_fft_ms = layer_fft[0] / max(1, layer_fft[1])

    # roofline of the dominant kernel of the headline path
    peaks, peak_src = measured_peaks()
    kern = max(("gridder", "degridder"), key=lambda k: stages[k][0])
    kt_ms = stages[kern][0] / max(1, stages[kern][1])
    if headline == "fp32":
        sincos_peak, _ = pkg.measure_sincos_peak()
        achieved = gridded * S * S / (kt_ms * 1e-3) / 1e9
        roofline = {"bound": "sfu", "achieved": achieved, "peak": sincos_peak / 1e9, "unit": "Gsincos/s",
                    "frac": achieved / (sincos_peak / 1e9), "traffic": traffic_per_launch(kern + "_fp32"),
                    "kernel": kern + "_fp32", "peak_source": "measured on this GPU (hardware sincos probe loop)",
                    "work_per_launch": f"{gridded} visibilities x {S * S} pixels, one sincos + 10 flop each"}
    else:
        achieved = gridded * 10 * S * S / (kt_ms * 1e-3) / 1e12
        # tcgen05 work actually issued per visibility: gridder one M128 N192 K16 MMA per 16 visibilities;
        # degridder 3 MMAs (N128 + N64 + N64, K16) per 128 visibilities x 4 K chunks / 128
        phys = (2 * 128 * 192 * 16 / 16) if kern == "gridder" else (2 * 128 * 256 * 64 / 128)
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                    "frac": achieved / peaks["bf16_tflops"], "traffic": traffic_per_launch(kern + "_" + headline),
                    "kernel": kern + "_" + headline,
                    "peak_source": f"{peak_src} dense bf16 (MEASURED_PEAKS.json bf16_tflops)",
                    "work_per_launch": f"{gridded} visibilities x {S * S} pixels x 10 algorithmic flop",
                    "physical_mma_tflops": gridded * phys / (kt_ms * 1e-3) / 1e12,
                    "physical_mma_frac": gridded * phys / (kt_ms * 1e-3) / 1e12 / peaks["bf16_tflops"],
                    "note": "algorithmic flop counts one complex MAC + phase per pixel and visibility (the FP32 "
                            "kernel's work); the tensor-core kernels issue the physical MMA flop instead"}

    # e2e through the reference-facing host API (IDG.GridW + IDG.DeGridW) with pinned host buffers
    e2e = None
    if not args.no_e2e:
        # the host arrays live on the GPU's NUMA node, as a deployment would place them: allocated
        # and first touched by this thread while it runs on that node's CPUs
        all_cpus = os.sched_getaffinity(0)
        local_cpus = gpu_local_cpus(local)
        if local_cpus:
            os.sched_setaffinity(0, local_cpus)
        link = link_rates()
        pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
        h_vis = pin(obs.vis.shape, torch.complex128)
        h_vis[...] = obs.vis
        h_uvw = pin(obs.uvw.shape, torch.float64)
        h_uvw[...] = obs.uvw
        h_grid = pin((N, N), torch.complex128)
        h_grid[...] = model_grid
        h_layers = pin((W, N, N), torch.complex128)
        h_layers[...] = 0
        h_vout = pin(obs.vis.shape, torch.complex128)
        h_vout[...] = 0
        plan.set_mode(MODES[headline])
        plan.set_stream(0)
        pkg.IDG.GridW(c, part, h_vis, h_uvw, obs.frequencies, out=h_layers)  # warm-up of the host path
        pkg.IDG.DeGridW(c, part, h_grid, h_uvw, obs.frequencies, out=h_vout)
        # ten steps: a transient stall of the host's page-locked copies (seen on this pool for tens of
        # milliseconds at a time) weighs half what it would over five; the per-step spread is reported
        steps_e2e = max(1, min(args.steps, 10))
        t_grid = t_degrid = 0.0
        step_ms = []
        plan.reset_timing()
        plan.enable_timing(True)  # CUDA events on the plan's stream between stages (boundary copies)
        t0 = time.perf_counter()
        for _ in range(steps_e2e):
            ta = time.perf_counter()
            pkg.IDG.GridW(c, part, h_vis, h_uvw, obs.frequencies, out=h_layers)
            tb = time.perf_counter()
            pkg.IDG.DeGridW(c, part, h_grid, h_uvw, obs.frequencies, out=h_vout)
            tc = time.perf_counter()
            t_grid += tb - ta
            t_degrid += tc - tb
            step_ms.append(1e3 * (tc - ta))
        t_e2e = time.perf_counter() - t0
        if ws > 1:  # the job's time is the slowest rank's (no host-side grid reduce in this form)
            tt = torch.tensor([t_e2e], dtype=torch.float64, device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t_e2e = float(tt.item())
        e2e_stages = plan.stage_times()
        plan.enable_timing(False)
        # the same calls with uvw=None (NULL in the C ABI): the plan keeps the uvw the partition was
        # made from on the device, so no call uploads or compares it (the first call puts it back
        # after the calls above passed the host copy: untimed)
        pkg.IDG.GridW(c, part, h_vis, None, obs.frequencies, out=h_layers)
        pkg.IDG.DeGridW(c, part, h_grid, None, obs.frequencies, out=h_vout)
        t0 = time.perf_counter()
        for _ in range(steps_e2e):
            pkg.IDG.GridW(c, part, h_vis, None, obs.frequencies, out=h_layers)
            pkg.IDG.DeGridW(c, part, h_grid, None, obs.frequencies, out=h_vout)
        t_res = time.perf_counter() - t0
        if ws > 1:
            tt = torch.tensor([t_res], dtype=torch.float64, device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t_res = float(tt.item())
        os.sched_setaffinity(0, all_cpus)
        nvis = obs.vis.size
        h2d = nvis * 16 + 2 * obs.uvw.nbytes + N * N * 16
        d2h = W * N * N * 16 + N * N * 16 + nvis * 16
        in_place = plan.host_access()
        e2e = {"value": 2 * total_gridded * steps_e2e / t_e2e / 1e6, "unit": "Mvis/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "host_arrays_in_place": in_place,
               "grid_w_ms": 1e3 * t_grid / steps_e2e, "degrid_w_ms": 1e3 * t_degrid / steps_e2e,
               "step_ms": {"min": min(step_ms), "median": float(np.median(step_ms)), "max": max(step_ms),
                           "steps": steps_e2e},
               "stage_ms_per_step": {k: round(v[0] / steps_e2e, 4) for k, v in e2e_stages.items() if v[1]},
               "uvw_kept_on_device": {"value": 2 * total_gridded * steps_e2e / t_res / 1e6, "unit": "Mvis/s",
                                      "ms_per_step": 1e3 * t_res / steps_e2e,
                                      "h2d_bytes_per_step": int(h2d - 2 * obs.uvw.nbytes),
                                      "note": "the same GridW + DeGridW with uvw=None: the partition's uvw stays "
                                              "on the device (the reference's callers pass the same uvw every "
                                              "cycle)"},
               "host_numa_local_cpus": len(local_cpus) if local_cpus else None,
               "link_gbs": link,
               "note": "IDG.GridW + IDG.DeGridW host API, Complex(double) arrays in pinned host memory, "
                       "wall clock incl. every host<->device transfer and complex128<->complex64 conversion"
                       + ("; the kernels read the visibilities and the model grid and write the degridded "
                          "visibilities and the w layers in host memory over NVLink-C2C" if in_place else "")}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        oracle = load_oracle()
        subs = plan.subgrids()
        sample, nv, _ = calibrate_cpu_sample(oracle, cd, subs, obs, model_grid, 12.0)
        t0 = time.perf_counter()
        layers_ref, vis_ref = cpu_reference_step(oracle, cd, sample, obs, model_grid)
        t_cpu = time.perf_counter() - t0
        # accuracy of each GPU mode on the same sample (plan restricted to the sampled subgrids)
        rl = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
        acc = {}
        # every precision mode (config 3: the BF16 and FP16 hi + lo forms beside FP32)
        for mode in [headline] + [m for m in MODES if m != headline]:
            sp = pkg.plan_from_subgrids(c, sample, obs.uvw, obs.frequencies)
            sp.set_mode(MODES[mode])
            spart = pkg.Partition([[]], sp)
            lay_gpu = pkg.IDG.GridW(c, spart, obs.vis, obs.uvw, obs.frequencies)
            vis_gpu = pkg.IDG.DeGridW(c, spart, model_grid.copy(), obs.uvw, obs.frequencies)
            acc[mode] = {"grid_w": rl(lay_gpu, layers_ref), "degrid_w": rl(vis_gpu, vis_ref)}
            sp.destroy()
        cpu = {"value": 2 * nv / t_cpu / 1e6, "unit": "Mvis/s", "cores": oracle.num_threads(), "kind": "port",
               "sample": f"{len(sample)} of {len(subs)} subgrids ({nv} of {gridded} gridded visibilities), "
                         f"GridW + DeGridW of the sample in FP64",
               "rel_l2_vs_fp64": dict(acc, visibilities=nv)}

    if rank == 0:
        modes = {m: {"value": r["value"], "ms_per_step": r["ms"] / args.steps,
                     "per_stage_ms": {k: round(v[0] / max(1, v[1]), 4) for k, v in r["stages"].items() if v[1]}}
                 for m, r in results.items()}
        if "fp32" in results and headline != "fp32":
            # the FP32 kernels against their own ceiling: one hardware sincos per pixel and visibility,
            # divided by the measured sincos rate of the same intrinsic on this GPU (an ncu capture shows
            # the probe and the FP32 gridder at the same XU-pipe limit, ~49 % of the XU instruction peak)
            sincos_peak, _ = pkg.measure_sincos_peak()
            st32 = results["fp32"]["stages"]
            k32 = max(("gridder", "degridder"), key=lambda k: st32[k][0])
            per_kernel = {}
            for k in ("gridder", "degridder"):
                ms_k = st32[k][0] / max(1, st32[k][1])
                per_kernel[k] = gridded * S * S / (ms_k * 1e-3) / 1e9
            modes["fp32"]["roofline"] = {
                "bound": "sfu", "achieved": per_kernel[k32], "peak": sincos_peak / 1e9, "unit": "Gsincos/s",
                "frac": per_kernel[k32] / (sincos_peak / 1e9), "kernel": k32 + "_fp32",
                "frac_per_kernel": {k: v / (sincos_peak / 1e9) for k, v in per_kernel.items()},
                "traffic": traffic_per_launch(k32 + "_fp32"),
                "peak_source": "measured on this GPU: p9idg_measure_sincos_peak (independent chains of __sincosf)",
                "work_per_launch": f"{gridded} visibilities x {S * S} pixels, one sincos each"}
        out = {"metric": METRIC, "value": head["value"], "unit": "Mvis/s", "n_gpus": ws, "steps": args.steps,
               "warmup": max(3, args.warmup), "ms_per_step": head["ms"] / args.steps, "higher_is_better": True,
               "scaling": "strong", "vs_baseline": None, "dtype": "f32" if headline == "fp32" else headline,
               "data": "synthetic (seeded; stands in for the reference's MeerKAT FITS data, absent)",
               "config": {"workload": "3072^2 IDG grid+degrid: 2016 bl x 2000 t x 16 ch (64.5M vis), S=32, W=8",
                          "mode": headline, "input_visibilities": info["input_visibilities"],
                          "gridded_visibilities": gridded, "subgrids": info["num_subgrids"],
                          "parallelism": (f"baseline blocks balanced by gridded visibilities over {ws} ranks "
                                          f"(rank 0: baselines {block[0]}-{block[1]}); per step: layer sum + "
                                          f"all-reduce of one {N}x{N} complex64 grid and a broadcast of the "
                                          f"model grid (NCCL)") if ws > 1 else "one GPU",
                          "job_gridded_visibilities": total_gridded,
                          "l2_flush": "inputs larger than L2 (vis 516 MB, layers 604 MB complex64)",
                          "value_counts": "gridded visibilities x 2 (gridder + degridder) per step",
                          "layer_fft_ms": round(layer_fft_ms, 4),
                          "plan_ms": round(plan_ms, 1)},
               "modes": modes,
               "tc_over_fp32": (head["value"] / results["fp32"]["value"]) if "fp32" in results and
               headline != "fp32" else None,
               "rel_l2_tc_vs_fp32_full_workload": tc_vs_fp32,
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
               "clocks": head["clk"]}
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
