"""Energies, forces and per-type parameter gradients over many independent boxes.

Parameter fitting evaluates one force field on many small systems (snapshots of uneven
size) and needs dE/d(per-type parameters).  `BoxBatch` keeps one device context per
box.  The boxes are small next to the GPU (a few hundred to a few thousand atoms), so
the batch drives them concurrently: every context has its own CUDA streams, and a pool
of host threads issues the evaluations (the C ABI runs without the GIL), which overlaps
the boxes' kernels on the device.

Per-type parameters (24 per type) are the molecular-frame multipole components of
MPIDForce::addMultipole (charge, dipole X Y Z, quadrupole XX XY YY XZ YZ ZZ, octopole XXX
XXY XYY YYY XXZ XYZ YYZ XZZ YZZ ZZZ), the molecular-frame polarisabilities X Y Z and the
Thole width; every atom of a type takes them in its own local frame.  The gradients
come from mpid_evaluate_with_gradients, summed over the atoms of each type and over the
boxes.
Quadrupoles and octopoles must stay traceless: `project_traceless` removes the trace
directions from a gradient before a step.
"""
import concurrent.futures as _cf

import numpy as np

from .context import MPIDContext, MPIDError
from .force import MPIDForce

NPARAM = 24
COLUMNS = (["charge", "dipoleX", "dipoleY", "dipoleZ", "quadXX", "quadXY", "quadYY", "quadXZ", "quadYZ", "quadZZ"] +
           ["oct" + c for c in ("XXX", "XXY", "XYY", "YYY", "XXZ", "XYZ", "YYZ", "XZZ", "YZZ", "ZZZ")] +
           ["polarizabilityX", "polarizabilityY", "polarizabilityZ", "thole"])


def per_type(grad, types, ntypes):
    """(n, k) per-atom gradients -> (ntypes, k) sums over the atoms of each type (one
    matrix product with the atoms' one-hot type matrix)."""
    t = np.asarray(types, dtype=np.int64)
    onehot = np.zeros((ntypes, len(t)))
    onehot[t, np.arange(len(t))] = 1.0
    return onehot @ np.asarray(grad, dtype=np.float64)


def project_traceless(g):
    """Remove the trace directions from the quadrupole (XX, YY, ZZ) and octopole gradient
    components so that a step along the result keeps the moments traceless."""
    g = np.array(g, dtype=np.float64, copy=True)
    q = g[..., 4:10]  # XX XY YY XZ YZ ZZ
    tr = (q[..., 0] + q[..., 2] + q[..., 5]) / 3.0
    for c in (0, 2, 5):
        q[..., c] -= tr
    o = g[..., 10:20]  # XXX XXY XYY YYY XXZ XYZ YYZ XZZ YZZ ZZZ
    # the three traces of an octopole: (XXX, XYY, XZZ), (XXY, YYY, YZZ), (XXZ, YYZ, ZZZ)
    for a, b, c in ((0, 2, 7), (1, 3, 8), (4, 6, 9)):
        t = (o[..., a] + o[..., b] + o[..., c]) / 3.0
        o[..., a] -= t
        o[..., b] -= t
        o[..., c] -= t
    return g


def atom_parameters(force, i):
    """The 24 per-type parameters of atom i."""
    q, d, Q, O, _, _, _, _, thole, pol = force.getMultipoleParameters(i)
    return np.concatenate([[q], d, Q, O, pol, [thole]])


def type_parameters(force, types, ntypes):
    """(ntypes, 24) parameters read from the first atom of each type."""
    out = np.zeros((ntypes, NPARAM))
    seen = np.zeros(ntypes, dtype=bool)
    for i, t in enumerate(types):
        if not seen[t]:
            out[t] = atom_parameters(force, i)
            seen[t] = True
    return out


def apply_type_parameters(force, types, params):
    """Give every atom its type's row of params (frames and covalent maps unchanged)."""
    for i, t in enumerate(types):
        p = list(force.getMultipoleParameters(i))
        row = params[t]
        p[0], p[1], p[2], p[3] = float(row[0]), list(row[1:4]), list(row[4:10]), list(row[10:20])
        p[8], p[9] = float(row[23]), list(row[20:23])
        force.setMultipoleParameters(i, *p)


class BoxBatch:
    """Independent boxes sharing per-type parameters.

    systems: list of (force, positions (n, 3) nm, box (3, 3) nm, types (n,) ints).
    precision: "mixed" or "double", as MPIDContext.  batched: all boxes evaluate in one
    call of mpid_evaluate_batch (energy, forces, gradient passes) with no host
    synchronisation per box; by default every operation of the evaluation is one kernel
    launch for all boxes (launch mode 0, see evaluate_batch).  Otherwise host threads
    drive the contexts concurrently, each replaying its evaluation's segments from graphs
    (solver_graphs).
    """

    def __init__(self, systems, ntypes, precision="mixed", threads=8, device=0, solver_graphs=True, batched=True):
        self.ntypes = int(ntypes)
        self.systems = [(f, np.asarray(p, dtype=np.float64), np.asarray(b, dtype=np.float64), np.asarray(t))
                        for f, p, b, t in systems]
        self.contexts = [MPIDContext(f, precision=precision, device=device, box=b, solver_graphs=solver_graphs)
                         for f, p, b, t in self.systems]
        self.threads = max(1, int(threads))
        self.batched = bool(batched)
        self.batch_launch = 0  # batched launch mode: 0 fused, -1 one parent graph, k > 0 per-box graphs on k streams
        if self.batched:
            # per-type gradient sums on the device
            for (f, p, b, t), ctx in zip(self.systems, self.contexts):
                ctx.setAtomTypes(t, self.ntypes)
        self._pool = _cf.ThreadPoolExecutor(max_workers=self.threads)

    def set_parameters(self, params):
        """Apply (ntypes, 24) parameters to every box (host update + upload)."""
        params = np.asarray(params, dtype=np.float64).reshape(self.ntypes, NPARAM)
        for (f, p, b, t), ctx in zip(self.systems, self.contexts):
            apply_type_parameters(f, t, params)
            ctx.update_parameters(f)

    def _one(self, k, forces):
        f, p, b, t = self.systems[k]
        e, fo, gm, gp = self.contexts[k].evaluateWithGradients(p, b, forces=forces)
        g = np.zeros((self.ntypes, NPARAM))
        g[:, :20] = per_type(gm, t, self.ntypes)
        g[:, 20:] = per_type(gp, t, self.ntypes)
        return e, fo, g

    def evaluate(self, forces=True):
        """Energies (nbox,) kJ/mol, per-box forces (list of (n, 3) or None) and the gradient
        of the summed energy with respect to the per-type parameters (ntypes, 24)."""
        if self.batched:
            from .context import evaluate_batch
            energies, fo, _, _, grad = evaluate_batch(self.contexts, [s[1] for s in self.systems],
                                                      [s[2] for s in self.systems], forces=forces, multipole=False,
                                                      polarization=False, launch=self.batch_launch, flat=True,
                                                      type_grad=True)
            if forces:
                ends = np.cumsum([len(s[1]) for s in self.systems])
                fo = np.split(fo, ends[:-1])
            else:
                fo = [None] * len(self.systems)
            return energies, fo, grad
        results = list(self._pool.map(lambda k: self._one(k, forces), range(len(self.systems))))
        energies = np.array([r[0] for r in results])
        grad = np.zeros((self.ntypes, NPARAM))
        for r in results:
            grad += r[2]
        return energies, [r[1] for r in results], grad

    def launches(self):
        """Kernel launches of the last evaluate(): those of the fused launch (which every
        box shares) in launch mode 0, else the sum over the boxes' own evaluations."""
        if not self.contexts:
            return 0
        if self.batched and self.batch_launch == 0:
            return self.contexts[0].stats()["kernel_launches"]
        return sum(c.stats()["kernel_launches"] for c in self.contexts)

    def tuning_key(self):
        """The workload class a tuning result applies to: GPU (name, multiprocessors),
        launch mode, precision and batch shape (boxes, mean atoms per box to 100)."""
        import torch
        props = torch.cuda.get_device_properties(self.contexts[0].device if self.contexts else 0)
        sizes = [len(sy[1]) for sy in self.systems]
        return "%s|%d|%s|%s|%dx%d" % (props.name, props.multi_processor_count, "batched" if self.batched else "threads",
                                      self.contexts[0].precision, len(sizes), int(round(np.mean(sizes) / 100.0)) * 100)

    def set_work_split(self, max_split):
        for c in self.contexts:
            c.setWorkSplit(max_split)

    def configure(self, config):
        """Apply a launch configuration {"max_split": bound of the pair kernels' work split
        (MPIDContext.setWorkSplit), "launch": batched launch mode (0 fused, -1 one parent
        graph, k > 0 per-box graphs on k streams)}."""
        self.set_work_split(int(config.get("max_split", 0)))
        self.batch_launch = int(config.get("launch", 0))

    def autotune(self, splits=(0, 1, 2, 4, 8), launches=(0, 32), repeats=3, path=None, use_cache=True):
        """Launch-configuration autotuner: times evaluate() of this batch under each
        combination of the pair kernels' work-split bound and (batched mode) the launch
        mode, keeps the fastest, and records it per GPU and workload class (tuning_key) in a
        JSON file beside the built library, where later batches of the same class find it.
        A configuration the batch cannot run (the fused mode with a box above its size
        limit) is skipped.  Returns (chosen configuration, {configuration label: ms per
        evaluate})."""
        import json
        import os
        import time
        path = path or os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "tuning.json")
        key = self.tuning_key()
        table = {}
        if os.path.exists(path):
            try:
                table = json.load(open(path))
            except ValueError:
                table = {}
        if use_cache and key in table:
            best = table[key]["config"]
            self.configure(best)
            return best, table[key]["ms"]
        configs = [{"max_split": int(m), "launch": int(q)} for m in splits for q in (launches if self.batched else (0,))]
        times, ran = {}, []
        for cfg in configs:
            self.configure(cfg)
            try:
                self.evaluate()  # records / captures the graphs of this configuration
            except MPIDError:
                continue
            t0 = time.perf_counter()
            for _ in range(repeats):
                self.evaluate()
            times["split%d_launch%d" % (cfg["max_split"], cfg["launch"])] = 1e3 * (time.perf_counter() - t0) / repeats
            ran.append(cfg)
        if not ran:
            raise MPIDError("autotune: no configuration ran")
        best = ran[min(range(len(ran)), key=lambda i: list(times.values())[i])]
        self.configure(best)
        table[key] = {"config": best, "ms": times}
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as fh:
            json.dump(table, fh, indent=1, sort_keys=True)
        return best, times

    def close(self):
        self._pool.shutdown(wait=True)
        for c in self.contexts:
            c.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def shard_indices(sizes, rank, world):
    """Boxes of one rank when independent boxes are spread over `world` GPUs: greedy
    longest-processing-time assignment by atom count (largest box first, to the least
    loaded rank; ties to the lower rank), so every rank gets a near-equal share of
    atoms.  Deterministic, so every rank computes the same partition without talking."""
    order = sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k))
    load = [0] * world
    owner = [0] * len(sizes)
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += int(sizes[k])
    return [k for k in range(len(sizes)) if owner[k] == rank]


def allreduce_results(energies, indices, nboxes, grad, group=None):
    """Combine per-rank results of a sharded batch: each rank holds the energies of its
    boxes (`indices`) and its partial per-type gradient.  Returns (energies of all
    boxes, summed gradient), identical on every rank.  One all-reduce of
    nboxes + ntypes x 24 doubles (torch.distributed; on the GPU under NCCL)."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    g = np.asarray(grad, dtype=np.float64)
    buf = np.zeros(nboxes + g.size)
    buf[np.asarray(list(indices), dtype=np.int64)] = np.asarray(energies, dtype=np.float64)
    buf[nboxes:] = g.reshape(-1)
    t = torch.as_tensor(buf, device=dev)
    dist.all_reduce(t, group=group)
    out = t.cpu().numpy()
    return out[:nboxes], out[nboxes:].reshape(g.shape)


def torch_energy(batch: BoxBatch):
    """A torch.autograd.Function for the batch: params (ntypes, 24) -> summed energy of the
    boxes, whose backward is the per-type gradient of the same evaluation."""
    import torch

    class _BatchEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, params):
            batch.set_parameters(params.detach().cpu().double().numpy())
            energies, _, grad = batch.evaluate(forces=False)
            ctx.save_for_backward(torch.as_tensor(grad, dtype=params.dtype, device=params.device))
            return torch.as_tensor(energies.sum(), dtype=params.dtype, device=params.device)

        @staticmethod
        def backward(ctx, grad_out):
            (grad,) = ctx.saved_tensors
            return grad_out * grad

    return _BatchEnergy.apply


FFT_FRIENDLY = (16, 18, 20, 24, 25, 27, 30, 32, 36)


def water_batch(nboxes=64, seed=2024, min_waters=128, max_waters=512, cutoff=0.7, alpha=4.0, order=5,
                polarization=MPIDForce.Mutual, eps=1e-7):
    """Batched-fitting workload: nboxes water boxes with a uniformly random (seeded) number
    of waters in [min_waters, max_waters], edge (n x 29.915 A^3)^(1/3) (1.0 g/cm^3), PME
    grid of at least 1 point per A rounded up to an FFT-friendly size, cutoff 0.7 nm and
    Ewald alpha 4.0 /nm.  Two types (0 = O, 1 = H) whose parameters are those of the first
    O and H of the first box.  Returns (systems, type parameters (2, 24))."""
    from . import synthetic
    rng = np.random.default_rng(seed)
    sizes = rng.integers(min_waters, max_waters + 1, size=nboxes)
    systems = []
    params = None
    for k, nw in enumerate(sizes):
        edge = (int(nw) * 29.915) ** (1.0 / 3.0)
        f, pos, box = synthetic.water_box(int(nw), edge, seed=seed + 1 + k, placement="random")
        grid = next(g for g in FFT_FRIENDLY if g >= int(np.ceil(edge)))
        f.setNonbondedMethod(MPIDForce.PME)
        f.setCutoffDistance(cutoff)
        f.setPMEParameters(alpha, grid, grid, grid)
        f.setPmeBSplineOrder(order)
        f.setPolarizationType(polarization)
        f.setMutualInducedTargetEpsilon(eps)
        f.setMutualInducedMaxIterations(200)
        types = np.tile([0, 1, 1], int(nw))
        if params is None:
            params = type_parameters(f, types, 2)
        apply_type_parameters(f, types, params)
        systems.append((f, pos, box, types))
    return systems, params
