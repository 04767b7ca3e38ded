"""Benchmark: MPIDForce energy+force evaluations per second on one GB300.

Workload (one step = one full evaluation: sort/tiles, permanent field, mutual induced
dipoles to 1e-7 D, energy/forces/torques, torque mapping): 8,000 rigid waters
(24,000 atoms) in a 62.14 A cubic box, PME cutoff 0.9 nm, alpha 3.4 /nm, 72^3 grid,
B-spline order 5, mutual polarisation, seeded synthetic multipoles.

Arms
* default: the mixed-precision path (FP32 pair/PME/solver kernels, 64-bit fixed-point
  forces, FP64 energies and residual refinement).  `value` is evaluations/s with inputs
  resident in HBM (device-pointer API); `e2e` runs the host-buffer C-ABI call
  (positions and forces copied in, forces and energy copied out each step).  The FP64
  path is timed on the same box for the mixed-vs-FP64 speed-up and accuracy.
* --impl reference: the reference's CPU algorithm on the host cores.  The reference's
  own build needs its source tree, absent where the benchmark runs, so the oracle port
  (oracle/mpid_port.cpp, pinned to the reference in tests) is timed with all host
  threads, one full evaluation per step.

With torchrun (N > 1) every rank evaluates its own replica (replicas only; no data is
exchanged) and `value` is the sum over ranks.
"""
import argparse
import datetime
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "force+energy evals/s, 24k-atom water PME mutual pol: mixed vs FP64 at 5e-6"
WORKLOAD = ("water24k: 8000 waters (24,000 atoms), 62.14 A box, cutoff 0.9 nm, alpha 3.4/nm, 72^3 grid, "
            "B-spline order 5, mutual polarisation to 1e-7 D, seeded synthetic multipoles")
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


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        # the raw samples (the summary goes into the JSON line)
        self.path = os.environ.get("MPID_BENCH_CLOCKS_CSV",
                                   os.path.join(tempfile.gettempdir(), "mpid_bench_clocks_%d.csv" % os.getpid()))

    def __enter__(self):
        q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def mark(self, which):
        setattr(self, which, datetime.datetime.now())

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0, t1 = getattr(self, "start", None), getattr(self, "stop", None)
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(p[0], "%Y/%m/%d %H:%M:%S.%f")
                if t0 and t1 and not (t0 <= ts <= t1):
                    continue
                sm.append(float(p[2]))
                smax = float(p[3])
            except ValueError:
                continue
            for nm, v in zip(names, p[6:10]):
                if v.lower() == "active":
                    reasons.add(nm)
        out = {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
               "samples": len(sm)}
        if not sm:
            out["note"] = "timed region shorter than the 200 ms sampling interval: run more --steps"
        return out


def count_pairs_within(pos, box, cutoff):
    from scipy.spatial import cKDTree
    L = np.diag(box)
    wrapped = pos - L * np.floor(pos / L)
    tree = cKDTree(wrapped, boxsize=L)
    return int(len(tree.query_pairs(cutoff, output_type="ndarray")))


# FP32 operations per interacting pair (add/mul = 1, FMA = 2, div/sqrt/exp/erfc = 1),
# counted from the kernels' own source by mpidopenmmplugin_gb300/csrc/flop_count.cpp and
# averaged over the pair-distance distribution of a 0.9 nm cutoff with alpha = 3.4/nm.
FLOP_PER_PAIR = {"pair_kernel": 2728,          # k_electrostatics<float, MUTUAL>
                 "dipole_field_pairs": 154,    # k_dipole_field_packed (CG matrix-vector product)
                 "fixed_field_pairs": 472}     # k_fixed_field<float>
# DRAM bytes per launch (read + write) from one ncu capture of each kernel on this
# workload (the captures summarised under profiles/); ncu is not run by this script.
DRAM_BYTES_PER_LAUNCH = {"pair_kernel": 29.42e6 + 0.39e6, "dipole_field_pairs": 32.86e6}
KERNEL_NAMES = {"pair_kernel": "k_electrostatics<float, mutual> (energy/force/torque pair kernel)",
                "dipole_field_pairs": "k_dipole_field_packed (FP32 T.mu pair kernel of the CG solver)",
                "fixed_field_pairs": "k_fixed_field<float> (permanent-field pair kernel)"}


REFERENCE_SECONDS = 60  # time bound of the reference arm's timed evaluations


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
    # A full evaluation takes seconds on the host cores, so the run is bounded in time:
    # one warm-up evaluation (the port keeps no state between calls), then evaluations
    # until the requested steps are done or REFERENCE_SECONDS have passed.
    warm = min(args.warmup, 1)
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


def cpu_baseline_sample():
    """The oracle port on the host cores, one 24k-atom evaluation (about 5-15 s)."""
    from oracle import oracle as O
    from mpidopenmmplugin_gb300 import MPIDForce, synthetic
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import helpers
    O.build("port")
    f, pos, box = synthetic.workload("water24k", polarization=MPIDForce.Mutual)
    s = helpers.oracle_system(f, pos, box)
    t0 = time.perf_counter()
    O.evaluate(s, "port")
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "evals/s", "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
            "kind": "port",
            "sample": "one full evaluation of the 24,000-atom box (oracle/mpid_port.cpp, FP64, OpenMP)"}


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
    arms = [("mixed", args.threads)]
    if world == 1:
        arms = ([("mixed", 1)] if args.threads != 1 else []) + arms + ([] if args.no_fp64 else [("double", args.threads)])
    for precision, threads in arms:
        with fitting.BoxBatch(systems, 2, precision=precision, threads=threads, device=local) as b:

            def step():
                e, _, g = b.evaluate()
                if world > 1:
                    e, g = fitting.allreduce_results(e, mine, len(all_systems), g)
                return g

            for _ in range(args.warmup):
                step()
            torch.cuda.synchronize()
            steps = args.steps if (precision, threads) == ("mixed", args.threads) else max(3, args.steps // 4)
            with ClockSampler(local) as clocks:
                time.sleep(0.5)
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
            per_step = sum(c.stats()["kernel_launches"] for c in b.contexts)
            out["%s_t%d" % (precision, threads)] = {"ms_per_step": dt * 1e3, "steps": steps,
                                                    "launches_per_step": per_step}
            if threads == args.threads:
                grads[precision] = g
                if precision == "mixed":
                    clock_summary = clocks.summary()
    ms = max_over_ranks(out["mixed_t%d" % args.threads]["ms_per_step"], world)
    if rank != 0:
        return
    gm = grads["mixed"]
    gd = grads.get("double")
    main_arm = out["mixed_t%d" % args.threads]
    line = {"metric": FITTING_METRIC, "value": 1000.0 / ms, "unit": "steps/s", "n_gpus": world,
            "steps": out["mixed_t%d" % args.threads]["steps"], "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded water boxes)",
            "config": {"workload": FITTING_WORKLOAD if args.boxes >= 64 else
                       "first %d boxes of %s" % (len(all_systems), FITTING_WORKLOAD),
                       "atoms": natoms, "host_threads": args.threads,
                       "solver_graphs": True,
                       "device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                       "l2": "inputs copied from host each step"},
            "gpu_launches": main_arm["launches_per_step"] * main_arm["steps"],
            "arms": out,
            "mixed_vs_fp64_gradient_rel": None if gd is None else float(np.linalg.norm(gm - gd) / np.linalg.norm(gd)),
            "clocks": clock_summary}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--workload", default="water24k", choices=["water24k", "fitting64"],
                    help="water24k: the headline evaluation; fitting64: the batched per-type gradient workload")
    ap.add_argument("--threads", type=int, default=8, help="host threads driving the boxes of fitting64")
    ap.add_argument("--boxes", type=int, default=64, help="fitting64: evaluate only the first N boxes (profiling)")
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

    import torch
    from mpidopenmmplugin_gb300 import MPIDContext, MPIDForce, synthetic
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import helpers

    torch.cuda.set_device(local)
    f, pos, box = synthetic.workload("water24k", polarization=MPIDForce.Mutual)
    n = f.getNumMultipoles()
    ctx = MPIDContext(f, precision="mixed", device=local)
    # a created stream: the evaluation's segments are replayed from CUDA graphs there (the
    # legacy default stream cannot be captured)
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    d_pos = torch.tensor(pos, dtype=torch.float64, device="cuda").contiguous()
    d_force = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    d_energy = torch.zeros(1, dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def step():
        ctx.evaluate_device(d_pos.data_ptr(), box, d_force.data_ptr(), d_energy.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        d_force.zero_()
        step()
    torch.cuda.synchronize()
    # timed region: events around each step on the launching stream, L2 flushed between steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stage_ms, stage_n = {}, {}
    launches = 0
    cg_iters = 0
    with ClockSampler(local) as clocks:
        time.sleep(0.5)  # let the sampler start
        barrier(world)
        torch.cuda.synchronize()
        clocks.mark("start")
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            step()
            ends[k].record(stream)
            st = ctx.stats()
            launches += st["kernel_launches"]
            cg_iters += st["solver_iterations"]
            for name, v in st["ms_stage"].items():
                stage_ms[name] = stage_ms.get(name, 0.0) + v
                stage_n[name] = stage_n.get(name, 0) + st["stage_launches"][name]
        torch.cuda.synchronize()
        clocks.mark("stop")
        barrier(world)
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / args.steps
    ms = max_over_ranks(ms, world)
    value = world * 1000.0 / ms
    stats = ctx.stats()

    # end to end through the host-buffer API: positions + forces in, forces + energy out
    # pinned host buffers (the caller's positions and force array)
    hpos = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    hpos[:] = pos
    hforce = torch.zeros((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(2):
        ctx.evaluate(hpos, box, forces=hforce)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        hforce[:] = 0.0
        e_mixed, fm = ctx.evaluate(hpos, box, forces=hforce)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    e2e_ms = max_over_ranks(e2e_ms, world)

    line = None
    if rank == 0:
        # FP64 path on the same box: throughput and accuracy of the mixed path against it
        fp64 = {}
        if not args.no_fp64:
            cd = MPIDContext(f, precision="double", device=local)
            ed, fd = cd.evaluate(pos, box)
            t0 = time.perf_counter()
            reps = 3
            for _ in range(reps):
                ed, fd = cd.evaluate(pos, box)
            fp64_ms = (time.perf_counter() - t0) * 1000.0 / reps
            em, fmix = ctx.evaluate(pos, box)
            fp64 = {"fp64_evals_per_s": 1000.0 / fp64_ms, "speedup_vs_fp64": fp64_ms / ms,
                    "energy_rel_err": abs(em - ed) / abs(ed), "force_rel_rms_err": helpers.rel_rms(fmix, fd),
                    "dipole_rel_rms_err": helpers.rel_rms(ctx.getInducedDipoles(), cd.getInducedDipoles())}
        # roofline of the dominant kernel: the pair kernel with the largest device time in
        # the timed region; per launch = FLOP/pair x pairs within the cutoff
        npairs = count_pairs_within(pos, box, 0.9)
        dom = max(FLOP_PER_PAIR, key=lambda k: stage_ms.get(k, 0.0))
        nl = max(1, stage_n.get(dom, 0))
        if dom == "dipole_field_pairs" and cg_iters:
            # the CG launches pairs once per iteration; the one launched while the host reads
            # the last iteration's convergence flag returns at once and does no pair work
            nl = min(nl, cg_iters)
        pair_ms = stage_ms.get(dom, 0.0) / nl
        achieved = FLOP_PER_PAIR[dom] * npairs / (pair_ms * 1e-3) / 1e12 if pair_ms > 0 else None
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        clk = clocks.summary()
        # FP32 CUDA-core peak: 152 SMs x 128 FP32 lanes x 2 FLOP/FMA x SM clock
        sm_mhz = clk.get("sm_max_mhz") or peaks.get("sm_max_mhz") or 2070.0
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        roofline = {"bound": "fp32", "kernel": KERNEL_NAMES[dom],
                    "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                    "frac": (achieved / fp32_peak) if achieved else None,
                    "traffic": DRAM_BYTES_PER_LAUNCH.get(dom),
                    "traffic_unit": "bytes per launch (ncu capture, profiles/)",
                    "peak_source": "152 SMs x 128 FP32 lanes x 2 x max SM clock (no measured FP32 peak in "
                                   "MEASURED_PEAKS.json)",
                    "pairs_within_cutoff": npairs, "flop_per_pair": FLOP_PER_PAIR[dom],
                    "ms_per_launch": pair_ms, "launches_per_step": nl / args.steps,
                    "share_of_step": stage_ms.get(dom, 0.0) / args.steps / ms}
        cpu = None
        if not args.no_cpu_baseline:
            try:
                cpu = cpu_baseline_sample()
            except Exception as exc:
                cpu = {"value": None, "unit": "evals/s", "cores": 0, "kind": "port", "sample": "failed: %s" % exc}
        nbytes = 3 * n * 8
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "precision": "mixed (FP32 kernels, FP64 energies and refinement)",
                       "l2": "flushed between timed steps (512 MB write)", "replicas": world,
                       "parallelism": "replicas only",
                       "launch": "evaluation segments and CG iterations replayed from CUDA graphs on a created stream"},
            "e2e": {"value": world * 1000.0 / e2e_ms, "unit": "evals/s", "h2d_bytes_per_step": 2 * nbytes,
                    "d2h_bytes_per_step": nbytes + 8},
            "gpu_launches": launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk,
            "stage_ms_per_step": {k: v / args.steps for k, v in stage_ms.items()},
            "solver": {"iterations": stats["solver_iterations"], "refinement_steps": stats["refinement_steps"],
                       "residual_debye": stats["solver_residual"], "max_neighbours": stats["max_neighbours"]},
        }
        line.update(fp64)
        print(json.dumps(line))
    barrier(world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
