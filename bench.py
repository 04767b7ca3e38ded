"""Benchmark: MPIDForce energy+force evaluations per second on one GB300.

Workload water24k (the default; one step = one full evaluation: sort/tiles, permanent
field, mutual induced dipoles to 1e-7 D, energy/forces/torques, torque mapping): 8,000
rigid waters (24,000 atoms) in a 62.14 A cubic box, PME cutoff 0.9 nm, alpha 3.4 /nm,
72^3 grid, B-spline order 5, mutual polarisation, seeded synthetic multipoles.
Workload water288k: 96,000 waters (288,000 atoms), 142.0 A, 144^3 grid, mutual
polarisation to 1e-6 D, and the same box with OPT3 extrapolation.

Arms
* default: the mixed-precision path (FP32 pair/PME/solver kernels, 64-bit fixed-point
  forces, FP64 energies and residual refinement).  `value` is evaluations/s with inputs
  resident in HBM (device-pointer API, CUDA events on the launching stream, L2 flushed
  between steps); `e2e` runs the host-buffer C-ABI call (positions and forces copied
  in, forces and energy copied out each step).  The FP64 path is timed the same way on
  the same box (device pointers, events, flush, the same steps) for the mixed-vs-FP64
  speed-up; both are compared with the oracle port's FP64 evaluation of the box.  A
  few further evaluations with serial stages (every stream folded onto one) give the
  additive per-stage device times, cuFFT among them.
* --impl reference: the reference's CPU algorithm on the host cores.  The reference's
  own build needs its source tree, absent where the benchmark runs, so the oracle port
  (oracle/mpid_port.cpp, pinned to the reference in tests) is timed with all host
  threads, one full evaluation per step.

With torchrun (N > 1) every rank evaluates its own replica (replicas only; no data is
exchanged) and `value` is the sum over ranks.
"""
import argparse
import ctypes
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

METRIC = "force+energy evals/s, 24k-atom water PME mutual pol: mixed vs FP64 at 5e-6"
WORKLOADS = {
    "water24k": ("water24k: 8000 waters (24,000 atoms), 62.14 A box, cutoff 0.9 nm, alpha 3.4/nm, 72^3 grid, "
                 "B-spline order 5, mutual polarisation to 1e-7 D, seeded synthetic multipoles"),
    "water288k": ("water288k: 96,000 waters (288,000 atoms), 142.0 A box, cutoff 0.9 nm, alpha 3.4/nm, 144^3 grid, "
                  "B-spline order 5, mutual polarisation to 1e-6 D (and OPT3 extrapolation), seeded synthetic "
                  "multipoles"),
}
WORKLOADS.update({
    "water648": ("water648: 216 waters (648 atoms), 18.64 A box, cutoff 0.8 nm, alpha 3.5/nm, 24^3 grid, B-spline "
                 "order 5, mutual polarisation to 1e-7 D, seeded synthetic multipoles"),
    "solution61k": ("solution61k: 20,000 waters + 200 ethane-like solutes (61,600 atoms; solutes with anisotropic "
                    "polarisabilities), 85.3 A box, cutoff 0.9 nm, alpha 3.4/nm, 96^3 grid, B-spline order 5, "
                    "mutual polarisation to 1e-7 D (and Direct, OPT3), seeded synthetic multipoles"),
})
WORKLOAD = WORKLOADS["water24k"]
METRIC_288K = "force+energy evals/s, 288k-atom water PME: mixed mutual (1e-6 D) vs OPT3 vs FP64"
METRICS = {
    "water24k": METRIC,
    "water288k": METRIC_288K,
    "water648": "force+energy evals/s, 648-atom water PME mutual pol: mixed vs FP64",
    "solution61k": "force+energy evals/s, 61.6k-atom solution PME: mixed mutual vs Direct vs OPT3 vs FP64",
}
L2_FLUSH_BYTES = 512 << 20


def dist_setup(ngpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# NVML clock-event reason bits (nvml.h, nvmlClocksEventReason*)
_NVML_REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
                 0x80: "hw_power_brake_slowdown"}


class ClockSampler:
    """SM clock and clock-event reasons of this process's GPU, sampled every `period`
    seconds during the timed region by a host thread through read-only NVML queries
    (libnvidia-ml); nothing is set.  The GPU is found by its PCI bus id."""

    def __init__(self, device_index, period=0.005):
        self.period = period
        self.samples = []
        self.nvml = None
        self.error = None
        self._stop = threading.Event()
        self._thread = None
        self._active = False
        try:
            import torch
            props = torch.cuda.get_device_properties(device_index)
            nvml = ctypes.CDLL("libnvidia-ml.so.1")
            if nvml.nvmlInit_v2() != 0:
                raise RuntimeError("nvmlInit failed")
            self.handle = ctypes.c_void_p()
            rc = -1
            if hasattr(props, "pci_bus_id"):
                bus = ("%08X:%02X:%02X.0" % (getattr(props, "pci_domain_id", 0), props.pci_bus_id,
                                             props.pci_device_id)).encode()
                rc = nvml.nvmlDeviceGetHandleByPciBusId_v2(ctypes.c_char_p(bus), ctypes.byref(self.handle))
            if rc != 0:
                rc = nvml.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(device_index), ctypes.byref(self.handle))
            if rc != 0:
                raise RuntimeError("no NVML handle for the device")
            self.reasons_fn = getattr(nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nvml.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = ctypes.c_uint(0)
            nvml.nvmlDeviceGetMaxClockInfo(self.handle, 1, ctypes.byref(mx))  # NVML_CLOCK_SM
            self.sm_max = mx.value or None
            self.nvml = nvml
        except Exception as exc:  # no NVML: the line says so
            self.error = "NVML unavailable: %s" % exc

    def _run(self):
        clk = ctypes.c_uint(0)
        rs = ctypes.c_ulonglong(0)
        pw = ctypes.c_uint(0)
        while not self._stop.is_set():
            if self._active:
                self.nvml.nvmlDeviceGetClockInfo(self.handle, 1, ctypes.byref(clk))
                self.reasons_fn(self.handle, ctypes.byref(rs))
                self.nvml.nvmlDeviceGetPowerUsage(self.handle, ctypes.byref(pw))
                self.samples.append((clk.value, rs.value, pw.value / 1000.0))
            time.sleep(self.period)

    def __enter__(self):
        if self.nvml is not None:
            self._thread = threading.Thread(target=self._run, daemon=True)
            self._thread.start()
        return self

    def __exit__(self, *a):
        if self._thread is not None:
            self._stop.set()
            self._thread.join()

    def mark(self, which):
        self._active = which == "start"

    def summary(self):
        if self.nvml is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [self.error], "samples": 0}
        sm = [s[0] for s in self.samples]
        reasons = set()
        for _, r, _ in self.samples:
            for bit, name in _NVML_REASONS.items():
                if r & bit:
                    reasons.add(name)
        return {"sm_mhz": float(statistics.median(sm)) if sm else None, "sm_max_mhz": self.sm_max,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max((s[2] for s in self.samples), default=None),
                "source": "NVML every %.0f ms during the timed steps" % (1e3 * self.period)}


def count_pairs_within(pos, box, cutoff):
    from scipy.spatial import cKDTree
    L = np.diag(box)
    wrapped = pos - L * np.floor(pos / L)
    tree = cKDTree(wrapped, boxsize=L)
    return int(tree.count_neighbors(tree, cutoff) - len(pos)) // 2


# FP32 operations per interacting pair (add/mul = 1, FMA = 2, div/sqrt/exp/erfc = 1),
# counted from the kernels' own source by tests/native/flop_count.cpp and averaged over the
# pair-distance distribution of a 0.9 nm cutoff with alpha = 3.4/nm.
FLOP_PER_PAIR = {"pair_kernel": 2728,          # k_electrostatics<float, MUTUAL>
                 "dipole_field_pairs": 154,    # k_dipole_field_cg (CG matrix-vector product)
                 "fixed_field_pairs": 472}     # k_fixed_field<float>
# DRAM bytes per launch (read + write) from one ncu capture of each kernel on the
# 24,000-atom box with the caches as the evaluation leaves them (--cache-control none),
# summarised under profiles/; ncu is not run by this script.
DRAM_BYTES_PER_LAUNCH = {"pair_kernel": 59.1e3 + 88.6e3, "dipole_field_pairs": 59.4e3 + 139.3e3}
DRAM_BYTES_SOURCE = ("ncu capture with warm caches (profiles/k_dipole_field_cg_water24k_mutual.md, "
                     "profiles/k_electrostatics_water24k_mutual.md)")
KERNEL_NAMES = {"pair_kernel": "k_electrostatics<float, mutual> (energy/force/torque pair kernel)",
                "dipole_field_pairs": "k_dipole_field_cg (FP32 T.mu pair kernel of the CG solver)",
                "fixed_field_pairs": "k_fixed_field<float> (permanent-field pair kernel)"}


REFERENCE_SECONDS = 150  # time bound of the reference arm's timed evaluations


def oracle_result(f, pos, box):
    """The oracle port's FP64 evaluation of the box on the host cores (time, result)."""
    from oracle import oracle as O
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import helpers
    O.build("port")
    s = helpers.oracle_system(f, pos, box)
    t0 = time.perf_counter()
    r = O.evaluate(s, "port")
    return time.perf_counter() - t0, r


def run_reference(args, world, rank):
    """CPU arm: the oracle port, all host threads, one full evaluation per step."""
    if rank != 0:
        return
    from oracle import oracle as O
    from mpidopenmmplugin_gb300 import MPIDForce, synthetic
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import helpers
    O.build("port")
    f, pos, box = synthetic.workload("water24k", polarization=MPIDForce.Mutual)
    s = helpers.oracle_system(f, pos, box)
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    # The port keeps no state between calls; warm-up evaluations are run as asked (at
    # most 10), then evaluations until the requested steps are done or REFERENCE_SECONDS
    # have passed.
    warm = min(args.warmup, 10)
    for _ in range(warm):
        O.evaluate(s, "port")
    done = 0
    t0 = time.perf_counter()
    while done < args.steps:
        O.evaluate(s, "port")
        done += 1
        if time.perf_counter() - t0 > REFERENCE_SECONDS:
            break
    dt = time.perf_counter() - t0
    val = done / dt
    sample = ("%d full evaluation(s) of the 24,000-atom box, one per step (at most %d s of the %d steps requested; "
              "oracle/mpid_port.cpp, FP64, OpenMP; the reference's own build needs its source tree, absent here)"
              % (done, REFERENCE_SECONDS, args.steps))
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "evals/s", "n_gpus": args.gpus,
            "steps": done, "warmup": warm, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": 1e3 * dt / done, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp64", "data": "synthetic", "config": {"workload": WORKLOAD, "precision": "fp64 CPU"},
            "cpu_baseline": {"value": val, "unit": "evals/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


FITTING_METRIC = "batched fitting steps/s: 64 water boxes, energy+forces+per-type gradients"
FITTING_WORKLOAD = ("fitting64: 64 independent water boxes of 128-512 waters (uniform, seeded; 59,370 atoms in "
                    "all), 1.0 g/cm^3, cutoff 0.7 nm, alpha 4.0/nm, grid >= 1 point/A (FFT-friendly), order 5, "
                    "mutual polarisation to 1e-7 D, 2 types x 24 parameters")


def run_fitting(args, world, rank, local):
    """The batched-fitting workload: one step evaluates every box (energy, forces, the
    20 multipole and 4 polarisation gradients per atom, summed per type) through the
    host-buffer C ABI, boxes driven concurrently from host threads.  Timed by the wall
    clock with a device synchronisation on both sides (the boxes run on many streams)."""
    import torch
    from mpidopenmmplugin_gb300 import fitting
    torch.cuda.set_device(local)
    all_systems, params = fitting.water_batch()
    all_systems = all_systems[:args.boxes]  # a prefix of the 64 boxes for profiling runs
    natoms = sum(len(sy[1]) for sy in all_systems)
    # N > 1: each rank takes a share of the boxes (balanced by atoms); the energies and
    # the per-type gradient are all-reduced once per step
    mine = fitting.shard_indices([len(sy[1]) for sy in all_systems], rank, world)
    systems = [all_systems[k] for k in mine]
    out = {}
    grads = {}
    # arms: (precision, host threads; 0 = one batched launch of all boxes' graphs)
    main = ("mixed", 0)
    arms = [main]
    if world == 1 and not args.main_only:
        arms = arms + [("mixed", args.threads)] + ([] if args.no_fp64 else [("double", 0)])
    for precision, threads in arms:
        with fitting.BoxBatch(systems, 2, precision=precision, threads=max(threads, 1), device=local,
                              batched=threads == 0) as b:

            if args.launch_config:
                m, q = (int(v) for v in args.launch_config.split(","))
                b.configure({"max_split": m, "launch": q})
                tuned = ({"max_split": m, "launch": q}, {})
            else:
                tuned = b.autotune()  # recorded per GPU; a later run reuses the choice

            def step():
                e, _, g = b.evaluate()
                if world > 1:
                    e, g = fitting.allreduce_results(e, mine, len(all_systems), g)
                return g

            for _ in range(args.warmup):
                step()
            torch.cuda.synchronize()
            steps = args.steps if (precision, threads) == main else max(3, args.steps // 4)
            with ClockSampler(local) as clocks:
                barrier(world)
                torch.cuda.synchronize()
                clocks.mark("start")
                t0 = time.perf_counter()
                for _ in range(steps):
                    g = step()
                torch.cuda.synchronize()
                dt = (time.perf_counter() - t0) / steps
                clocks.mark("stop")
            # kernel launches of one step: each box's last evaluation and gradient passes
            per_step = b.launches()
            label = "%s_%s" % (precision, "batched" if threads == 0 else "t%d" % threads)
            out[label] = {"ms_per_step": dt * 1e3, "steps": steps, "launches_per_step": per_step,
                          "launch_config": tuned[0], "autotune_ms": tuned[1]}
            if b.batched and b.batch_launch == 0:
                # device time of the last step's fused graph (CUDA events around its launch)
                out[label]["device_ms_per_step"] = b.contexts[0].stats()["ms_total"]
            if threads == 0:
                grads[precision] = g
                if precision == "mixed":
                    clock_summary = clocks.summary()
    main_label = "mixed_batched"
    ms = max_over_ranks(out[main_label]["ms_per_step"], world)
    if rank != 0:
        return
    gm = grads["mixed"]
    gd = grads.get("double")
    main_arm = out[main_label]
    line = {"metric": FITTING_METRIC, "value": 1000.0 / ms, "unit": "steps/s", "n_gpus": world,
            "steps": main_arm["steps"], "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded water boxes)",
            "config": {"workload": FITTING_WORKLOAD if args.boxes >= 64 else
                       "first %d boxes of %s" % (len(all_systems), FITTING_WORKLOAD),
                       "atoms": natoms, "launch": "all boxes in one mpid_evaluate_batch call with no per-box host "
                                                   "synchronisation: fused (one launch per operation over every box, "
                                                   "batched cuFFT per grid size, one CUDA graph) or per-box graphs "
                                                   "over a stream pool, as the autotuner chose",
                       "comparison_host_threads": args.threads,
                       "device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                       "l2": "inputs copied from host each step"},
            "gpu_launches": main_arm["launches_per_step"] * main_arm["steps"],
            "arms": out,
            "mixed_vs_fp64_gradient_rel": None if gd is None else float(np.linalg.norm(gm - gd) / np.linalg.norm(gd)),
            "clocks": clock_summary}
    print(json.dumps(line))


class DeviceArm:
    """One context evaluated through the device-pointer API on a created stream."""

    def __init__(self, torch, f, pos, n, local, precision, **kw):
        from mpidopenmmplugin_gb300 import MPIDContext
        self.torch = torch
        self.ctx = MPIDContext(f, precision=precision, device=local, **kw)
        self.stream = torch.cuda.Stream(device=local)
        self.d_pos = torch.tensor(pos, dtype=torch.float64, device="cuda").contiguous()
        self.d_force = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
        self.d_energy = torch.zeros(1, dtype=torch.float64, device="cuda")

    def step(self, box):
        self.ctx.evaluate_device(self.d_pos.data_ptr(), box, self.d_force.data_ptr(), self.d_energy.data_ptr(),
                                 self.stream.cuda_stream)

    def timed(self, box, steps, warmup, flush, clocks=None, on_step=None):
        """Mean device ms per evaluation: events on the launching stream around each step,
        L2 flushed before each step."""
        torch = self.torch
        with torch.cuda.stream(self.stream):
            for _ in range(warmup):
                self.d_force.zero_()
                self.step(box)
            torch.cuda.synchronize()
            starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
            ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
            if clocks:
                clocks.mark("start")
            for k in range(steps):
                flush.zero_()
                starts[k].record(self.stream)
                self.step(box)
                ends[k].record(self.stream)
                if on_step:
                    on_step(self.ctx.stats())
            torch.cuda.synchronize()
            if clocks:
                clocks.mark("stop")
        return sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / steps

    def results(self, box):
        """Energy, forces and induced dipoles of one more evaluation into zeroed forces (the
        timed steps add their forces into the same buffer)."""
        torch = self.torch
        with torch.cuda.stream(self.stream):
            self.d_force.zero_()
            self.step(box)
        torch.cuda.synchronize()
        return float(self.d_energy.item()), self.d_force.cpu().numpy(), self.ctx.getInducedDipoles()


def serial_breakdown(torch, f, pos, n, local, box, flush, steps):
    """Additive device-time breakdown: a context whose side streams fold onto the caller's
    stream (MPID_FLAG_SERIAL_STAGES), cuFFT as its own stage; per-evaluation means."""
    arm = DeviceArm(torch, f, pos, n, local, "mixed", serial_stages=True)
    acc = {}
    tot = []

    def on_step(st):
        tot.append(st["ms_total"])
        for k, v in st["ms_stage"].items():
            acc[k] = acc.get(k, 0.0) + v

    ms = arm.timed(box, steps, 2, flush, on_step=on_step)
    stages = {k: v / steps for k, v in acc.items()}
    total = sum(tot) / steps
    stages["untimed"] = total - sum(stages.values())  # solver vectors, field totals, host waits
    return {"ms_per_step": ms, "ms_total": total, "stages": stages,
            "note": "serial stages (every stream folded onto one, graphs replayed); stages + untimed = ms_total; "
                    "untimed = the solver's vector kernels, field-total kernels, memsets and host waits"}


def errors_against(e, forces, mu, ref_e, ref_f, ref_mu, rel_rms):
    return {"energy_rel_err": abs(e - ref_e) / abs(ref_e), "force_rel_rms_err": rel_rms(forces, ref_f),
            "dipole_rel_rms_err": rel_rms(mu, ref_mu)}


def run_evaluations(args, world, rank, local):
    import torch
    from mpidopenmmplugin_gb300 import MPIDForce, synthetic
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import helpers

    torch.cuda.set_device(local)
    name = args.workload
    pols = [("mutual", MPIDForce.Mutual)]
    if name == "water288k":
        pols.append(("opt3", MPIDForce.Extrapolated))
    if name == "solution61k":
        pols += [("direct", MPIDForce.Direct), ("opt3", MPIDForce.Extrapolated)]
    f, pos, box = synthetic.workload(name, polarization=MPIDForce.Mutual)
    n = f.getNumMultipoles()
    props = torch.cuda.get_device_properties(local)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    mixed = DeviceArm(torch, f, pos, n, local, "mixed")
    stage_ms, stage_n = {}, {}
    counts = {"launches": 0, "cg": 0}

    def on_step(st):
        counts["launches"] += st["kernel_launches"]
        counts["cg"] += st["solver_iterations"]
        for k, v in st["ms_stage"].items():
            stage_ms[k] = stage_ms.get(k, 0.0) + v
            stage_n[k] = stage_n.get(k, 0) + st["stage_launches"][k]

    with ClockSampler(local) as clocks:
        barrier(world)
        ms = mixed.timed(box, args.steps, args.warmup, flush, clocks=clocks, on_step=on_step)
        barrier(world)
    ms = max_over_ranks(ms, world)
    value = world * 1000.0 / ms
    stats = mixed.ctx.stats()
    e_mix, f_mix, mu_mix = mixed.results(box)

    # end to end through the host-buffer API: positions + forces in, forces + energy out,
    # pinned host buffers (the caller's positions and force array)
    hpos = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    hpos[:] = pos
    hforce = torch.zeros((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(args.warmup):
        mixed.ctx.evaluate(hpos, box, forces=hforce)
    torch.cuda.synchronize()
    e2e_calls = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        hforce[:] = 0.0
        t1 = time.perf_counter()
        mixed.ctx.evaluate(hpos, box, forces=hforce)
        e2e_calls.append(1e3 * (time.perf_counter() - t1))
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    e2e_ms = max_over_ranks(e2e_ms, world)
    if rank != 0:
        barrier(world)
        return

    extra = {}
    # FP64 path on the same box, timed exactly like the mixed path
    fp64 = None
    if not args.no_fp64:
        dbl = DeviceArm(torch, f, pos, n, local, "double")
        fp64_ms = dbl.timed(box, args.steps, args.warmup, flush)
        e_d, f_d, mu_d = dbl.results(box)
        fp64 = (e_d, f_d, mu_d)
        extra.update({"fp64_evals_per_s": 1000.0 / fp64_ms, "fp64_ms_per_step": fp64_ms,
                      "speedup_vs_fp64": fp64_ms / ms,
                      "fp64_timing": "device pointers, CUDA events on the launching stream, L2 flushed, %d steps after "
                                     "%d warm-up steps (as the mixed path)" % (args.steps, args.warmup)})
        extra.update({"vs_fp64": errors_against(e_mix, f_mix, mu_mix, e_d, f_d, mu_d, helpers.rel_rms)})
        del dbl
    # the oracle port on the host cores: the CPU baseline and the reference result
    cpu = None
    if not args.no_cpu_baseline:
        try:
            t_cpu, ref = oracle_result(f, pos, box)
            cpu = {"value": 1.0 / t_cpu, "unit": "evals/s",
                   "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)), "kind": "port",
                   "sample": "one full evaluation of the %d-atom box (oracle/mpid_port.cpp, FP64, OpenMP)" % n}
            extra["vs_oracle"] = errors_against(e_mix, f_mix, mu_mix, ref.energy, ref.forces, ref.induced,
                                                helpers.rel_rms)
            if fp64 is not None:
                extra["fp64_vs_oracle"] = errors_against(*fp64, ref.energy, ref.forces, ref.induced, helpers.rel_rms)
        except Exception as exc:
            cpu = {"value": None, "unit": "evals/s", "cores": 0, "kind": "port", "sample": "failed: %s" % exc}
    # further polarisation types of the workload (water288k: OPT3; solution61k: Direct, OPT3)
    for label, pol in pols[1:]:
        f2 = synthetic.workload(name, polarization=pol)[0]
        arm = DeviceArm(torch, f2, pos, n, local, "mixed")
        t_mix = arm.timed(box, args.steps, args.warmup, flush)
        res = arm.results(box)
        entry = {"evals_per_s": 1000.0 / t_mix, "ms_per_step": t_mix}
        del arm
        if not args.no_fp64:
            d2 = DeviceArm(torch, f2, pos, n, local, "double")
            t_d = d2.timed(box, max(3, args.steps // 4), args.warmup, flush)
            entry.update({"fp64_evals_per_s": 1000.0 / t_d, "speedup_vs_fp64": t_d / t_mix,
                          "vs_fp64": errors_against(*res, *d2.results(box), helpers.rel_rms)})
            del d2
        if fp64 is not None:
            # the extrapolated dipoles against the converged mutual ones (FP64)
            entry["vs_fp64_mutual"] = errors_against(*res, *fp64, helpers.rel_rms)
        extra[label] = entry
    serial = serial_breakdown(torch, f, pos, n, local, box, flush, max(3, min(args.steps, 10)))
    extra["stage_ms_per_step"] = serial["stages"]
    extra["serial_stages"] = {k: v for k, v in serial.items() if k != "stages"}
    extra["cufft_ms_per_step"] = serial["stages"].get("cufft")

    # roofline of the dominant kernel: the pair kernel with the largest share of the
    # serial (additive) stage times -- in the replayed graphs a stage's time also counts the
    # SMs it shares with the side streams; per launch = FLOP/pair x pairs within the cutoff
    npairs = count_pairs_within(pos, box, f.getCutoffDistance())
    dom = max(FLOP_PER_PAIR, key=lambda k: serial["stages"].get(k, 0.0))
    nl = max(1, stage_n.get(dom, 0))
    if dom == "dipole_field_pairs" and counts["cg"]:
        # the CG launches pairs once per iteration; the one launched while the host reads
        # the last iteration's convergence flag returns at once and does no pair work
        nl = min(nl, counts["cg"])
    pair_ms = stage_ms.get(dom, 0.0) / nl
    ncg = max(1, min(stage_n.get("dipole_field_pairs", 0), counts["cg"]))
    pair_ms_cg = stage_ms.get("dipole_field_pairs", 0.0) / ncg
    achieved = FLOP_PER_PAIR[dom] * npairs / (pair_ms * 1e-3) / 1e12 if pair_ms > 0 else None
    sn = serial["stages"]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    clk = clocks.summary()
    sms = props.multi_processor_count
    sm_mhz = clk.get("sm_max_mhz") or peaks.get("sm_max_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * sm_mhz * 1e6 / 1e12
    serial_launches = {"dipole_field_pairs": counts["cg"] / args.steps, "pair_kernel": 1.0, "fixed_field_pairs": 1.0}
    roofline = {"bound": "fp32", "kernel": KERNEL_NAMES[dom], "achieved": achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": (achieved / fp32_peak) if achieved else None,
                "traffic": DRAM_BYTES_PER_LAUNCH.get(dom) if name == "water24k" else None,
                "traffic_unit": "bytes per launch",
                "traffic_source": DRAM_BYTES_SOURCE,
                "peak_source": "%d SMs (queried) x 128 FP32 lanes x 2 x max SM clock %.0f MHz (no measured FP32 peak "
                               "in MEASURED_PEAKS.json)" % (sms, sm_mhz),
                "pairs_within_cutoff": npairs, "flop_per_pair": FLOP_PER_PAIR[dom],
                "ms_per_launch": pair_ms, "launches_per_step": nl / args.steps,
                "share_of_step": stage_ms.get(dom, 0.0) / args.steps / ms,
                "timing": "CUDA events around each launch inside the replayed graphs of the timed steps (shares the "
                          "SMs with the PME chain on its stream)"}
    if dom in sn and serial_launches.get(dom):
        alone = sn[dom] / serial_launches[dom]
        roofline["ms_per_launch_serial"] = alone
        roofline["achieved_serial"] = FLOP_PER_PAIR[dom] * npairs / (alone * 1e-3) / 1e12
    # every pair kernel: per launch in the serial schedule (alone on the GPU) and in the
    # timed steps, with its algorithmic FLOP rate against the computed FP32 peak
    pair_kernels = {}
    for k in FLOP_PER_PAIR:
        per = serial_launches.get(k)
        if not per or k not in sn:
            continue
        alone = sn[k] / per
        instep = stage_ms.get(k, 0.0) / max(1, stage_n.get(k, 0)) if k != "dipole_field_pairs" else pair_ms_cg
        rate = FLOP_PER_PAIR[k] * npairs / (alone * 1e-3) / 1e12 if alone > 0 else None
        pair_kernels[KERNEL_NAMES[k]] = {"ms_per_launch_serial": alone, "ms_per_launch_in_step": instep,
                                         "tflops_serial": rate, "frac_serial": rate / fp32_peak if rate else None}
    roofline["pair_kernels"] = pair_kernels
    nbytes = 3 * n * 8
    line = {
        "metric": METRICS[name], "value": value, "unit": "evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": WORKLOADS[name], "precision": "mixed (FP32 kernels, FP64 energies and refinement)",
                   "l2": "flushed between timed steps (512 MB write)", "replicas": world,
                   "parallelism": "replicas only", "sms": sms,
                   "launch": "evaluation segments and CG iterations replayed from CUDA graphs on a created stream"},
        "e2e": {"value": world * 1000.0 / e2e_ms, "unit": "evals/s", "h2d_bytes_per_step": 2 * nbytes,
                "d2h_bytes_per_step": nbytes + 8, "warmup": args.warmup,
                "ms_per_call": {"median": float(np.median(e2e_calls)), "max": float(np.max(e2e_calls)),
                                "first": float(e2e_calls[0])}},
        "gpu_launches": counts["launches"],
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk,
        "solver": {"iterations": stats["solver_iterations"], "refinement_steps": stats["refinement_steps"],
                   "residual_debye": stats["solver_residual"], "max_neighbours": stats["max_neighbours"]},
    }
    line.update(extra)
    print(json.dumps(line))
    barrier(world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--workload", default="water24k",
                    choices=["water24k", "water288k", "water648", "solution61k", "fitting64"],
                    help="water24k: the headline evaluation; water288k: the 288,000-atom box (mutual and OPT3); "
                         "water648: the 648-atom box; solution61k: the 61,600-atom solution (mutual, Direct, OPT3); "
                         "fitting64: the batched per-type gradient workload")
    ap.add_argument("--threads", type=int, default=16, help="host threads driving the boxes of fitting64 (comparison arm)")
    ap.add_argument("--boxes", type=int, default=64, help="fitting64: evaluate only the first N boxes (profiling)")
    ap.add_argument("--launch-config", default=None, metavar="SPLIT,LAUNCH",
                    help="fitting64: skip the autotuner; work-split bound and batched launch mode (0 fused, -1 one "
                         "parent graph, k > 0 per-box graphs on k streams), e.g. 8,0 (profiling)")
    ap.add_argument("--main-only", action="store_true", help="fitting64: time the batched mixed arm only (profiling)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.workload == "fitting64":
        # 64 contexts on 4 streams each: more hardware work queues than the default 8, so
        # that independent boxes do not queue behind one another (read at CUDA start-up)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "fitting64":
        run_fitting(args, world, rank, local)
        return
    run_evaluations(args, world, rank, local)


if __name__ == "__main__":
    main()
