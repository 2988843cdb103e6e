#!/usr/bin/env python3
"""Benchmark of the batched non-oriented scattering path on GB300.

One step = one pass of the hot path over one batch: for every neutron its
total cross-section and one sampled isotropic scatter (E', mu).

Default workload ("pe"): Polyethylene_CH2.ncmat;temp=293K (ElInc + two
S(alpha,beta) kernels), 2^24 neutrons with energies log-uniform in [1e-4, 1] eV
(seeded), FP64 I/O, the mixed-precision mode (FP64 for the Bragg sums, the
beta-CDF inversion and the kinematics; FP32 elsewhere), and the learned beta
proposal: its networks are trained on the GPU before timing (untimed; the
training's size and time are reported), and the plain sampler is timed on the
same handle and inputs beside it ("plain_sampler", "learned_vs_plain").
Other workloads: al2o3_large (Al2O3, dcutoff 0.2, 2,886 merged Bragg
d-spacings, 2^24 neutrons log-uniform in [1e-4, 1] eV, FP32 I/O), al_small
(Al, 2^20 neutrons, wavelengths uniform in [0.5, 5] Aa), crystal_batch (64
(material, T) instances of 16 crystals at 77/150/293/400 K, ragged counts
log-uniform in [1e3, 1e6]) and mixed_batch (32 instances: water, polyethylene
at 280/293/320 K with the learned proposal, 28 crystal instances; ragged counts
log-uniform in [1e4, 2e6], energies log-uniform in [1e-5, 2] eV); batches are
one launch pair replayed as a CUDA graph.  --mode exact computes in FP64
throughout (the reference's results to rounding).

  value  -- device-resident batch (two kernels: k_pick, k_sab), inputs
            already in HBM
  e2e    -- the same through the C ABI with host (pinned) arrays, copies
            inside the timed region

minimc: the reference's MiniMC run on the device (1e7 histories per step,
polyethylene sphere, pencil beam), metric histories/s, CPU baseline the
oracle's MiniMC engine.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
       [--workload pe|al2o3_large|al_small|crystal_batch|mixed_batch|minimc]
       [--mode mixed|exact] [--sampler auto|plain|learned]
Under torchrun (N>1) each rank runs an independent replica on its own GPU
(the path has no cross-neutron exchange: replicas only) and rank 0 prints the
JSON line with the whole-job throughput.
"""
import argparse
import gc
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

METRIC = "neutron scatters/s on 1 GB300, learned-proposal vs plain GPU sampler (KS p>0.01)"
UNIT = "scatters/s"
L2_BYTES = 129 * 1024 * 1024


def workload(name, rank):
    """-> dict(cfgs, counts, energies (list per material), io)."""
    import ncrystal_gb300.workloads as W
    if name == "al2o3_large":
        n = 1 << 24
        return dict(cfgs=[W.AL2O3], counts=[n], io="f32",
                    energies=[W.loguniform_energies(n, 1e-4, 1.0, 0x5EED0002 + rank)])
    if name == "al_small":
        n = 1 << 20
        return dict(cfgs=[W.AL], counts=[n], io="f64",
                    energies=[W.al_wavelength_energies(n, 0x5EED0001 + rank)])
    if name == "pe":
        n = 1 << 24
        return dict(cfgs=[W.PE293], counts=[n], io="f64",
                    energies=[W.loguniform_energies(n, 1e-4, 1.0, 0x5EED0004 + rank)])
    if name == "crystal_batch":
        cfg = W.config("crystal_batch")
        counts = [int(c) for c in cfg["counts"]]
        return dict(cfgs=cfg["cfgs"], counts=counts, io="f64",
                    energies=[W.loguniform_energies(c, 1e-4, 1.0, 0x5EED0003 + 1000 * rank + k)
                              for k, c in enumerate(counts)])
    if name == "mixed_batch":
        cfg = W.config("mixed_batch")
        counts = [int(c) for c in cfg["counts"]]
        return dict(cfgs=cfg["cfgs"], counts=counts, io="f64",
                    energies=[W.loguniform_energies(c, 1e-5, 2.0, 0x5EED0005 + 1000 * rank + k)
                              for k, c in enumerate(counts)])
    raise KeyError(name)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="pe",
                    choices=["pe", "al2o3_large", "al_small", "crystal_batch", "mixed_batch", "minimc"])
    ap.add_argument("--sampler", default="auto", choices=["auto", "plain", "learned"],
                    help="S(alpha,beta) beta sampling: plain percentile inversion, or the learned proposal "
                         "(trained on the GPU before timing; the plain sampler is timed beside it). "
                         "auto: learned for the workloads with polyethylene, plain otherwise")
    ap.add_argument("--train-samples", type=int, default=1 << 26)
    ap.add_argument("--train-steps", type=int, default=6000)
    ap.add_argument("--mode", default="mixed", choices=["exact", "mixed"],
                    help="arithmetic mode of the GPU path (mixed: FP32 incoherent-elastic exponentials "
                         "and alpha inversion, FP64 elsewhere)")
    ap.add_argument("--cpu-seconds", type=float, default=8.0,
                    help="wall-clock budget of the CPU baseline sample")
    ap.add_argument("--phase-profile", action="store_true",
                    help="instead of the benchmark line, print the S(alpha,beta) pass's phase shares "
                         "(SM-clock cycles per phase, ncgb_sab_phase_profile) for the plain sampler and, "
                         "where trained, the learned one (single-material workloads)")
    return ap.parse_args()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel, workload_name, key="dram_bytes_per_launch"):
    """DRAM bytes from the committed ncu summary, if any
    (profiles/<kernel>_<workload>.md, line '<key>: X'): per launch, or per
    unit of work with another key."""
    p = os.path.join(ROOT, "profiles", "%s_%s.md" % (kernel, workload_name))
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class NvmlClocks:
    """Read-only NVML queries through ctypes (no Python NVML package needed):
    the SM clock, its maximum and the clocks-event reasons of one GPU."""

    SM = 1  # NVML_CLOCK_SM
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index):
        import ctypes
        self.C = ctypes
        lib = None
        for name in ("libnvidia-ml.so.1", "libnvidia-ml.so"):
            try:
                lib = ctypes.CDLL(name)
                break
            except OSError:
                pass
        if lib is None or lib.nvmlInit_v2() != 0:
            raise OSError("NVML unavailable")
        self.lib = lib
        self.dev = ctypes.c_void_p()
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        nvml_index = int(vis) if vis.strip().isdigit() else index
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(nvml_index), ctypes.byref(self.dev)) != 0:
            raise OSError("NVML device %d unavailable" % nvml_index)
        self.max_mhz = self._clock(lib.nvmlDeviceGetMaxClockInfo)

    def _clock(self, fn):
        v = self.C.c_uint(0)
        return float(v.value) if fn(self.dev, self.SM, self.C.byref(v)) == 0 else None

    def sample(self):
        r = self.C.c_ulonglong(0)
        ok = self.lib.nvmlDeviceGetCurrentClocksEventReasons(self.dev, self.C.byref(r)) == 0
        names = [nm for bit, nm in self.REASONS.items() if ok and r.value & bit]
        return self._clock(self.lib.nvmlDeviceGetClockInfo), names


class ClockSampler:
    """Clock samples during the timed region: NVML every 2 ms where the
    driver's NVML library loads, else nvidia-smi every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        self.nvml, self.samples, self.stop = None, [], threading.Event()
        try:
            self.nvml = NvmlClocks(self.index)
            self.samples.append(self.nvml.sample())
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        except (OSError, AttributeError, ValueError):
            self.nvml = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
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

    def _poll(self):
        while not self.stop.wait(0.002):
            self.samples.append(self.nvml.sample())

    def __exit__(self, *a):
        if self.nvml is not None:
            self.stop.set()
            self.t.join(timeout=5)
            self.samples.append(self.nvml.sample())
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            sm = [c for c, _ in self.samples if c is not None]
            reasons = sorted({nm for _, names in self.samples for nm in names})
            if sm:
                return {"sm_mhz": statistics.median(sm), "sm_max_mhz": self.nvml.max_mhz, "reasons": reasons,
                        "samples": len(sm), "source": "nvml, 2 ms"}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi, 200 ms"}


def cpu_baseline(wl, seconds, threads=None):
    """The CPU oracle (a plain-C restatement of NCrystal's per-neutron
    evaluation, pinned to the reference neutron by neutron) timed on this
    host's cores on a bounded sample of the same workload: cross-section and
    one scatter per neutron.  For a multi-material workload the sample takes
    the same fraction of every material's neutrons."""
    from concurrent.futures import ThreadPoolExecutor

    import ncrystal_gb300._build as B
    from oracle.pyoracle import HostMaterial
    threads = threads or os.cpu_count() or 1
    mats = [HostMaterial(os.path.join(B.BUNDLES, B.bundle_file_name(c))) for c in wl["cfgs"]]
    total = sum(wl["counts"])

    def work(item):
        m, chunk, off = item
        m.xs(chunk)
        m.scatter(chunk, 12345, index_offset=off)

    def items(frac, parts):
        out = []
        for m, e in zip(mats, wl["energies"]):
            e = np.ascontiguousarray(e[:max(1, int(len(e) * frac))], dtype=np.float64)
            for ch in np.array_split(e, max(1, min(parts, len(e)))):
                if len(ch):
                    out.append((m, ch, 0))
        return out

    # calibrate on a small sample, then size the sample to the time budget
    t0 = time.perf_counter()
    cal = items(min(1.0, 20000.0 / total), 1)
    for it in cal:
        work(it)
    ncal = sum(len(it[1]) for it in cal)
    rate1 = ncal / max(time.perf_counter() - t0, 1e-6)
    frac = min(1.0, rate1 * threads * seconds / total)
    sample = items(frac, threads)
    nsample = sum(len(it[1]) for it in sample)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(work, sample))
    dt = time.perf_counter() - t0
    return {"value": nsample / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d neutrons (%.3g of each material's, xs + one scatter each), %d threads, %.1f s"
                      % (nsample, frac, threads, dt)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, dist, dev):
    """The largest value of x over all ranks (x itself without a process
    group): timings of replicas are combined by their slowest rank."""
    if not dist:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def config_of(args, wl, world):
    cfgs = wl["cfgs"]
    return {"workload": args.workload, "cfg": cfgs[0] if len(cfgs) == 1 else "%d instances" % len(cfgs),
            "neutrons_per_gpu": int(sum(wl["counts"])), "io": wl["io"],
            "sampler": "plain (Alg.1 tables)" if getattr(args, "sampler", "plain") != "learned"
            else "learned beta proposal (exact rejection), plain Alg.1 elsewhere",
            "mode": getattr(args, "mode", "exact"), "parallelism": "replicas%d" % world}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__
    __graft_entry__.build()
    wl = workload(args.workload, 0)
    if wl["io"] == "f32":
        wl["energies"] = [e.astype(np.float32).astype(np.float64) for e in wl["energies"]]
    vals = []
    base = None
    per_step = max(1.0, 60.0 / max(1, args.steps + args.warmup))
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(wl, min(per_step, args.cpu_seconds))
        if i >= args.warmup:
            vals.append(b["value"])
            base = b
    v = statistics.median(vals)
    base["value"] = v
    cfgd = config_of(args, wl, 1)
    # the CPU arm runs the reference's algorithm: FP64 throughout, plain sampler
    cfgd["mode"] = "exact"
    cfgd["sampler"] = "plain (Alg.1 tables)"
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfgd,
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


class SingleRunner:
    """One material, device arrays (ncgb_scatter_device) and host arrays
    (ncgb_xs_scatter_many[_f32])."""

    def __init__(self, NC, torch, wl, dev, seed, mode):
        self.torch = torch
        self.f32 = wl["io"] == "f32"
        self.dt = torch.float32 if self.f32 else torch.float64
        e = wl["energies"][0].astype(np.float32 if self.f32 else np.float64)
        self.n = len(e)
        self.sc = NC.createScatter(wl["cfgs"][0], seed=seed).set_mode(mode)
        self.d_e = torch.from_numpy(e).to(dev)
        self.d_xs, self.d_ef, self.d_mu = (torch.empty_like(self.d_e) for _ in range(3))
        self.h_e = torch.from_numpy(e).pin_memory()
        self.h_xs, self.h_ef, self.h_mu = (torch.empty(self.n, dtype=self.dt).pin_memory() for _ in range(3))

    def gate(self, stream):
        st = self.torch.zeros(self.n, dtype=self.torch.int32, device=self.d_e.device)
        self.sc.scatter_device(self.d_e, self.d_xs, self.d_ef, self.d_mu, st, stream=stream)
        self.torch.cuda.synchronize()
        return int((st != 0).sum().item())

    def step(self, stream):
        self.sc.scatter_device(self.d_e, self.d_xs, self.d_ef, self.d_mu, None, stream=stream)

    timed_step = step

    def set_sampler(self, sampler):
        self.sc.set_sampler(sampler)

    def e2e_step(self):
        self.sc.xs_scatter_host_ptr(self.h_e.data_ptr(), self.n, self.h_xs.data_ptr(), self.h_ef.data_ptr(),
                                    self.h_mu.data_ptr(), self.f32)

    def e2e_info(self):
        esz = 4 if self.f32 else 8
        zcv = os.environ.get("NCGB_ZERO_COPY", "")
        zc = (zcv != "0") if zcv else self.f32
        chunk = 1 << 22
        return {"h2d_bytes_per_step": self.n * esz, "d2h_bytes_per_step": 3 * self.n * esz,
                "gpu_launches_per_step": 2 if zc else 2 * ((self.n + chunk - 1) // chunk),
                "api": "ncgb_xs_scatter_many%s (C ABI, pinned host arrays; %s)"
                       % ("_f32" if self.f32 else "",
                          "the kernels read the energies from and write the results to host memory over "
                          "NVLink-C2C" if zc else "chunked copies: copy-in, kernel and copy-out streams")}

    def launches_per_step(self):
        return 2


class BatchRunner:
    """Ragged multi-material batch: autotuned shape, CUDA-graph replay on
    device arrays; host arrays through ncgb_batch_xs_scatter_many."""

    def __init__(self, NC, torch, wl, dev, seed, mode, prepare=None):
        self.torch = torch
        self.f32 = False
        e = np.concatenate(wl["energies"]).astype(np.float64)
        self.n = len(e)
        offs = np.concatenate([[0], np.cumsum(wl["counts"])]).astype(np.int64)
        scatters = [NC.createScatter(c, seed=seed + k) for k, c in enumerate(wl["cfgs"])]
        self.prepared = prepare(scatters) if prepare else None   # e.g. proposals, before the batch copies views
        self.batch = NC.Batch(scatters)
        self.batch.set_mode(mode)
        self.d_e = torch.from_numpy(e).to(dev)
        self.d_off = torch.from_numpy(offs).to(dev)
        self.d_xs, self.d_ef, self.d_mu = (torch.empty_like(self.d_e) for _ in range(3))
        self.h_e = torch.from_numpy(e).pin_memory()
        self.h_off = torch.from_numpy(offs).pin_memory()
        self.h_xs, self.h_ef, self.h_mu = (torch.empty(self.n, dtype=torch.float64).pin_memory() for _ in range(3))
        self.shape = None

    def gate(self, stream):
        self.shape = self.batch.autotune(self.d_e, self.d_off, self.d_xs, self.d_ef, self.d_mu, stream=stream)
        st = self.torch.zeros(self.n, dtype=self.torch.int32, device=self.d_e.device)
        self.batch.scatter_device(self.d_e, self.d_off, self.d_xs, self.d_ef, self.d_mu, st, stream=stream)
        self.torch.cuda.synchronize()
        return int((st != 0).sum().item())

    def step(self, stream):
        # plain launch (used for the per-kernel timing pass)
        self.batch.scatter_device(self.d_e, self.d_off, self.d_xs, self.d_ef, self.d_mu, None, stream=stream)

    def timed_step(self, stream):
        self.batch.graph_launch(self.d_e, self.d_off, self.d_xs, self.d_ef, self.d_mu, None, stream=stream)

    def set_sampler(self, sampler):
        self.batch.set_sampler(sampler)

    def e2e_step(self):
        self.batch.xs_scatter_host_ptr(self.h_e.data_ptr(), self.h_off.data_ptr(), self.n, self.h_xs.data_ptr(),
                                       self.h_ef.data_ptr(), self.h_mu.data_ptr())

    def e2e_info(self):
        zc = os.environ.get("NCGB_ZERO_COPY", "") == "1"
        return {"h2d_bytes_per_step": self.n * 8 + self.h_off.numel() * 8, "d2h_bytes_per_step": 3 * self.n * 8,
                "gpu_launches_per_step": 2,
                "api": "ncgb_batch_xs_scatter_many (C ABI, pinned host arrays; %s)"
                       % ("kernels read and write host memory over NVLink-C2C" if zc
                          else "chunked copies: copy-in, kernel and copy-out streams"),
                "autotuned_shape": {"pick_block": self.shape[0], "sab_blocks_per_sm": self.shape[1],
                                    "split_lists": self.batch.split_lists()}}

    def launches_per_step(self):
        return 2


def run_gb300(args):
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__
    if rank == 0 or world == 1:
        __graft_entry__.build()
    if dist:
        dist.barrier()
        __graft_entry__.build()  # no-op when up to date; loads the package
    import ncrystal_gb300 as NC

    wl = workload(args.workload, rank)
    is_pe = [c.startswith("Polyethylene_CH2.ncmat") for c in wl["cfgs"]]
    if args.sampler == "auto":
        args.sampler = "learned" if any(is_pe) else "plain"
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    learned = None
    attach = None
    if args.sampler == "learned":
        # Train the proposal networks on the GPU (untimed); attach them to the
        # polyethylene instances (the plain sampler serves the others).
        import ncrystal_gb300.learn as LR
        if not any(is_pe):
            raise SystemExit("bench: the learned proposal is trained for polyethylene workloads")
        t0 = time.perf_counter()
        nets, infos = LR.train_proposals(n_total=args.train_samples, steps=args.train_steps, seed=3 + rank)
        torch.cuda.synchronize()
        learned = {"train_wall_s": time.perf_counter() - t0,
                   "components": {str(c): {k: v for k, v in i.items() if k != "loss_trace"}
                                  for c, i in infos.items()},
                   "final_loss": {str(c): i["loss_trace"][-1] if i["loss_trace"] else None
                                  for c, i in infos.items()},
                   "network": "4x128 hidden, BF16 tcgen05 tensor-core GEMMs + FP32 accumulation in TMEM, trained by the library's kernels"}

        def attach(scatters):
            return [LR.attach(sc, nets) for sc, p in zip(scatters, is_pe) if p]
    if len(wl["cfgs"]) > 1:
        R = BatchRunner(NC, torch, wl, dev, 0xB0057 + 977 * rank, args.mode, prepare=attach)
        acc = R.prepared
    else:
        R = SingleRunner(NC, torch, wl, dev, 0xB0057 + 977 * rank, args.mode)
        acc = attach([R.sc]) if attach else None
    n = R.n
    if learned is not None:
        learned["mean_envelope_acceptance"] = acc
        R.set_sampler("learned")
    esz = 4 if R.f32 else 8
    io_bytes = 4 * esz * n  # energies in, xs / E' / mu out

    nbad = R.gate(stream)   # correctness gate before timing: no neutron may fail
    if nbad:
        raise SystemExit("bench: %d neutrons failed to sample" % nbad)
    if args.phase_profile:
        return phase_profile(args, R, learned is not None, torch)

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    # Between timed steps the L2 must not hold the previous step's arrays:
    # workloads whose I/O is smaller than twice the L2 flush it with a write
    # of a 2xL2 buffer, outside the timed events.
    flush = None
    if io_bytes < 2 * L2_BYTES:
        flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    for _ in range(args.warmup):
        R.timed_step(stream)
    barrier()

    # per-kernel durations (CUDA events on the launching stream, recorded by the library)
    NC.phase_times()
    NC.phase_timing(True)
    for _ in range(max(2, args.steps // 4)):
        if flush is not None:
            flush.fill_(1.0)
        R.step(stream)
    NC.phase_timing(False)
    ms_pick, ms_sab, nbatches, n_sab = NC.phase_times()
    barrier()

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for a, b in evs:
            if flush is not None:
                flush.fill_(1.0)
            a.record(stream)
            R.timed_step(stream)
            b.record(stream)
        barrier()
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs), dist, dev)
    ms_per_step = ms / args.steps
    value = world * n * args.steps / (ms / 1e3)

    plain = None
    if learned is not None:
        # the plain sampler on the same handle, same inputs, same timing rules
        R.set_sampler("plain")
        for _ in range(args.warmup):
            R.timed_step(stream)
        barrier()
        pev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for a, b in pev:
            if flush is not None:
                flush.fill_(1.0)
            a.record(stream)
            R.timed_step(stream)
            b.record(stream)
        barrier()
        pms = max_over_ranks(sum(a.elapsed_time(b) for a, b in pev), dist, dev)
        plain = {"value": world * n * args.steps / (pms / 1e3), "ms_per_step": pms / args.steps}
        R.set_sampler("learned")
    peak, peak_kind = measured_peaks()
    # Algorithmic bytes per launch (inputs read + results written, nothing
    # else): k_pick reads every energy, writes every xs and the (E', mu) of the
    # neutrons it finishes; k_sab writes (E', mu) of the n_sab queued ones.
    bytes_pick = n * (esz + esz) + (n - n_sab) * 2 * esz
    bytes_sab = n_sab * 2 * esz
    t_pick = ms_pick / max(1, nbatches) / 1e3
    t_sab = ms_sab / max(1, nbatches) / 1e3
    kernels = {
        "k_pick": {"ms_per_launch": t_pick * 1e3, "bytes_per_launch": bytes_pick,
                   "achieved_gbs": bytes_pick / t_pick / 1e9 if t_pick else None,
                   "share": t_pick / (t_pick + t_sab) if t_pick + t_sab else None},
        "k_sab": {"ms_per_launch": t_sab * 1e3, "bytes_per_launch": bytes_sab, "n_sab": n_sab,
                  "achieved_gbs": bytes_sab / t_sab / 1e9 if t_sab else None,
                  "share": t_sab / (t_pick + t_sab) if t_pick + t_sab else None},
    }
    dom = "k_sab" if t_sab >= t_pick else "k_pick"
    achieved = kernels[dom]["achieved_gbs"]

    # ---- e2e: host (pinned) arrays through the C ABI, copies timed ----------
    # (as many steps as the device-timed region: a short window is at the
    # mercy of one host-side stall)
    for _ in range(max(2, args.warmup)):
        R.e2e_step()
    barrier()
    e2e_steps = max(60, args.steps)
    step_s = []
    gc.disable()   # no interpreter collection pauses inside the timed host loop
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        R.e2e_step()   # synchronous: copies in, kernels, copies out
        step_s.append(time.perf_counter() - t1)
    barrier()
    gc.enable()
    print("e2e call times (ms): " + " ".join("%.2f" % (1e3 * t) for t in step_s), file=sys.stderr)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e = {"value": world * n * e2e_steps / e2e_s, "unit": UNIT, "steps": e2e_steps,
           "step_ms": {"min": 1e3 * min(step_s), "median": 1e3 * statistics.median(step_s),
                       "max": 1e3 * max(step_s)}}
    e2e.update(R.e2e_info())

    if not float(R.d_mu.abs().max().item()) <= 1.0:
        raise SystemExit("bench: mu outside [-1,1]")

    if rank == 0:
        base = cpu_baseline(wl, args.cpu_seconds)
        cfgd = config_of(args, wl, world)
        cfgd["l2"] = ("flushed between timed steps (2xL2 write)" if flush is not None
                      else "per-step I/O %d MB > 2xL2; material tables stay L2-resident" % (io_bytes >> 20))
        cfgd["inputs"] = "device-resident, not re-read from host"
        if len(wl["cfgs"]) > 1:
            cfgd["timed_launch"] = "CUDA graph replay of the autotuned batch launch"
        if learned is not None:
            cfgd["learned"] = learned
            cfgd["plain_sampler"] = plain
            cfgd["learned_vs_plain"] = value / plain["value"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.mode == "exact" else "f64+f32",
            "data": "synthetic", "config": cfgd,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None, "peak_kind": peak_kind,
                         "traffic": profiled_traffic(dom, args.workload), "kernel": dom, "kernels": kernels,
                         "step_bytes_per_neutron": 4 * esz,
                         "note": "latency-bound (table gathers and spill reloads, FP64 pipe about half busy), "
                                 "not HBM-bound: see profiles/%s_%s.md" % (dom, args.workload)},
            "cpu_baseline": base,
            "e2e": e2e,
            "clocks": clk.summary(),
            "gpu_launches": args.steps * R.launches_per_step(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def phase_profile(args, R, learned, torch):
    """Phase shares of the S(alpha,beta) pass (cycles summed over lanes) for
    the plain sampler and the learned one, on the workload's device arrays;
    the profiled pass's own duration (CUDA events) beside the plain pass's."""
    if not isinstance(R, SingleRunner) or R.f32:
        raise SystemExit("bench: --phase-profile needs a single-material FP64 workload")
    out = {"metric": "S(alpha,beta) pass phase shares (lane cycles)", "workload": args.workload,
           "mode": args.mode, "neutrons": R.n, "samplers": {}}
    for sampler in (["plain", "learned"] if learned else ["plain"]):
        R.set_sampler(sampler)
        for _ in range(2):
            R.sc.sab_phase_profile(R.d_e, R.d_xs, R.d_ef, R.d_mu)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        cyc, attempts = R.sc.sab_phase_profile(R.d_e, R.d_xs, R.d_ef, R.d_mu)
        b.record()
        torch.cuda.synchronize()
        tot = sum(cyc.values())
        out["samplers"][sampler] = {"shares": {k: v / tot for k, v in cyc.items()}, "lane_cycles": tot,
                                    "alg1_attempts": attempts, "profiled_batch_ms": a.elapsed_time(b)}
    print(json.dumps(out), flush=True)
    return 0


# ---- MiniMC workload -------------------------------------------------------------------
# The reference's MiniMC on a polyethylene sphere (r = 1 cm) under a pencil
# beam of 0.0253 eV neutrons, 1e7 histories per step, tallies theta, mu, e,
# nscat, w with breakdowns (the query of tests/golden/mmc_pe_sphere.npz).
MMC_METRIC = "MiniMC neutron histories/s on 1 GB300 (polyethylene sphere r=1cm, pencil beam 0.0253 eV)"
MMC_UNIT = "histories/s"
MMC_GEOM = "sphere;r=0.01"
MMC_ENGINE = "seed=11;tally=theta,mu,e,nscat,w"
MMC_N = 10000000
MMC_ENERGY = 0.0253
# algorithmic bytes: a transported neutron reads its state (position,
# direction, pending scatter result, energy, weight, cached xs, counters,
# stream key, initial energy and direction: 128 B) and, when it goes on to a
# collision, writes it to the next population (116 B); a collision reads
# energy, direction and stream key (36 B) and writes E', direction, status (36 B)
MMC_BYTES_READ, MMC_BYTES_WRITE, MMC_BYTES_SCATTER = 128, 116, 72


def mmc_src(n):
    return "constant;ekin=%g;z=-0.01;n=%d" % (MMC_ENERGY, n)


def mmc_cpu_baseline(seconds, threads=None):
    """The oracle's CPU MiniMC engine (oracle/ncgb_oracle_mmc.c, pinned to the
    reference's MiniMC by tests/test_oracle_mmc.py) on this host's cores, on
    a bounded number of histories of the same query."""
    import ncrystal_gb300._build as B
    import ncrystal_gb300.minimc as M
    import ncrystal_gb300.workloads as W
    from ncrystal_gb300.bundle.reader import read_bundle
    from oracle import pyoracle as P
    threads = threads or os.cpu_count() or 1
    path = os.path.join(B.BUNDLES, B.bundle_file_name(W.PE293))
    geom = M.decode_cfgstr(MMC_GEOM, "geom")["decoded"]
    src = M.decode_cfgstr(mmc_src(1000), "src")["decoded"]
    src["energy_ev"] = MMC_ENERGY
    eng = M.decode_cfgstr(MMC_ENGINE, "engine")["decoded"]
    bins = {"theta": (180, 0.0, 180.0), "mu": (200, -1.0, 1.0), "e": (200, 0.0, 0.5), "nscat": (22, -1.5, 20.5),
            "w": (200, 0.0, 1.0)}
    m = P.HostMaterial(path)
    c, nstat, nbuf = P.mmc_config(m, read_bundle(path), geom, src, eng, bins, seed=11)
    t0 = time.perf_counter()
    P.mmc_run(m, c, nbuf, 0, 2000, threads=1)
    rate1 = 2000 / max(time.perf_counter() - t0, 1e-6)
    n = int(min(MMC_N, max(threads * 1000, rate1 * threads * seconds)))
    t0 = time.perf_counter()
    _, cnt = P.mmc_run(m, c, nbuf, 0, n, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": MMC_UNIT, "cores": threads, "kind": "port",
            "sample": "%d histories of the same query (%.3g neutron-steps), %d threads, %.1f s"
                      % (n, cnt[5], threads, dt)}


def run_minimc_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__
    __graft_entry__.build()
    vals, base = [], None
    per_step = max(1.0, 60.0 / max(1, args.steps + args.warmup))
    for i in range(args.warmup + args.steps):
        b = mmc_cpu_baseline(min(per_step, args.cpu_seconds))
        if i >= args.warmup:
            vals.append(b["value"])
            base = b
    v = statistics.median(vals)
    base["value"] = v
    line = {"metric": MMC_METRIC, "value": v, "unit": MMC_UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "minimc", "cfg": "Polyethylene_CH2.ncmat;temp=293K", "geomcfg": MMC_GEOM,
                       "srccfg": mmc_src(MMC_N), "enginecfg": MMC_ENGINE, "parallelism": "replicas1"},
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": v, "unit": MMC_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_minimc(args):
    """value: histories per second of device time (CUDA events around the
    engine's step loop on its stream); e2e: the same runs through the C ABI
    call (ncgb_mmc_run: cfg strings in, the results document out), wall
    clock.  Each step is one complete MiniMC run of 1e7 histories; the tally
    histograms stay in shared memory / L2, the population (2 x 8.4M neutrons,
    ~2.8 GB) is far larger than L2."""
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__
    if rank == 0 or world == 1:
        __graft_entry__.build()
    if dist:
        dist.barrier()
        __graft_entry__.build()
    import ncrystal_gb300 as NC
    import ncrystal_gb300.workloads as W
    dev = torch.device("cuda", local)
    sc = NC.createScatter(W.PE293, seed=11 + rank)
    sc.set_mode(args.mode)
    src = mmc_src(MMC_N)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        sc.minimc_run(MMC_GEOM, src, MMC_ENGINE)
    # kernel shares (phase timing on; one untimed run)
    NC.phase_times()
    NC.phase_timing(True)
    res = sc.minimc_run(MMC_GEOM, src, MMC_ENGINE)
    NC.phase_timing(False)
    ms_pick, ms_sab, nbatches, _ = NC.phase_times()
    devmd = res["output"]["metadata"]["device"]
    barrier()
    secs = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            r = sc.minimc_run(MMC_GEOM, src, MMC_ENGINE)
            secs.append(r["output"]["metadata"]["device"]["seconds"])
        barrier()
    dev_s = max_over_ranks(sum(secs), dist, dev)
    value = world * MMC_N * args.steps / dev_s
    # e2e: the C ABI call, wall clock (cfg strings in, JSON document out)
    barrier()
    t0 = time.perf_counter()
    e2e_steps = max(3, args.steps // 2)
    for _ in range(e2e_steps):
        r = sc.minimc_run(MMC_GEOM, src, MMC_ENGINE)
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
    nbuf = sum(6 * (t["total"]["bindata"]["nbins"] + 2) * 2 + 30 for t in r["output"]["tally"].values())
    e2e = {"value": world * MMC_N * e2e_steps / e2e_s, "unit": MMC_UNIT, "steps": e2e_steps,
           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": nbuf * 8 + 64,
           "api": "ncgb_mmc_run (C ABI; cfg strings in, results JSON out)"}
    # roofline of the dominant kernel (algorithmic bytes per launch over the
    # launch's CUDA-event time)
    peak, peak_kind = measured_peaks()
    nst = devmd["neutron_steps"]
    launches = max(1, devmd["transport_launches"])
    t_tr = devmd["transport_ms"] / launches / 1e3
    nscat = nst - MMC_N
    bytes_tr = (MMC_BYTES_READ * nst + MMC_BYTES_WRITE * nscat) / launches
    nb = max(1, nbatches)
    t_pick, t_sab = ms_pick / nb / 1e3, ms_sab / nb / 1e3
    bytes_sc = MMC_BYTES_SCATTER * nscat / nb
    tot = t_tr + t_pick + t_sab
    kernels = {
        "k_mmc_transport": {"ms_per_launch": t_tr * 1e3, "launches": launches, "bytes_per_launch": bytes_tr,
                            "achieved_gbs": bytes_tr / t_tr / 1e9 if t_tr else None,
                            "share": t_tr / tot if tot else None},
        "k_pick": {"ms_per_launch": t_pick * 1e3, "launches": nb, "bytes_per_launch": bytes_sc,
                   "share": t_pick / tot if tot else None},
        "k_sab": {"ms_per_launch": t_sab * 1e3, "launches": nb, "share": t_sab / tot if tot else None},
    }
    achieved = kernels["k_mmc_transport"]["achieved_gbs"]
    # DRAM traffic per launch: the ncu capture's bytes per transported
    # neutron (profiles/k_mmc_transport_minimc.md) times this run's average
    per_neutron = profiled_traffic("k_mmc_transport", "minimc", "dram_bytes_per_neutron_step")
    traffic = per_neutron * nst / launches if per_neutron else None
    if rank == 0:
        base = mmc_cpu_baseline(args.cpu_seconds)
        line = {
            "metric": MMC_METRIC, "value": value, "unit": MMC_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.mode == "exact" else "f64+f32",
            "data": "synthetic",
            "config": {"workload": "minimc", "cfg": W.PE293, "geomcfg": MMC_GEOM, "srccfg": src,
                       "enginecfg": MMC_ENGINE, "mode": args.mode, "parallelism": "replicas%d" % world,
                       "neutron_steps_per_run": nst, "engine_steps_per_run": devmd["steps"],
                       "l2": "population 2 x 2^23 neutrons (~2.8 GB) > L2; tallies block-local in shared memory"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None, "peak_kind": peak_kind,
                         "traffic": traffic, "kernel": "k_mmc_transport",
                         "kernels": kernels,
                         "note": "latency / FP64 bound (warp reductions of the tally statistics), not HBM bound"},
            "cpu_baseline": base,
            "e2e": e2e,
            "clocks": clk.summary(),
            "gpu_launches": args.steps * (launches + 2 * nb + 1),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.workload == "minimc":
        return run_minimc_reference(args) if args.impl == "reference" else run_minimc(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
