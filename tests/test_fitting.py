"""Polarisation-parameter gradients and the batched per-type fitting interface.

CPU tests cover the host logic of mpidopenmmplugin_gb300.fitting (per-type sums,
traceless projection, parameter round trips, the batched-boxes workload's geometry).
GPU tests check, through the C ABI:
* dE/d(polarisability X Y Z, Thole width) of the device against the oracle port (itself
  checked against central differences of its own energy): FP64 to 1e-8, mixed to 1e-5
  relative RMS (the gradient pass runs in FP64 on both paths; on the mixed path the
  induced dipoles of the mixed solve carry its ~1e-6 error);
* the batch's per-type gradient (24 parameters per type, summed over boxes) along
  admissible parameter directions against the oracle port's (FP64 to 1e-6, mixed to
  1e-5) and against differences of the device's FP64 energy; the port's own per-type
  gradient is checked on the CPU against central differences with h = 1e-4;
* that boxes evaluated concurrently on several host threads give bit-identical results
  to one-by-one evaluation, and the torch.autograd.Function's backward.
"""
import numpy as np
import pytest

from mpidopenmmplugin_gb300 import MPIDContext, MPIDForce, fitting, synthetic

import helpers


def small_batch(nboxes=4, polarization=MPIDForce.Mutual, seed=11):
    """A few boxes of 128-160 waters, the batched-fitting workload at a test size."""
    return fitting.water_batch(nboxes=nboxes, seed=seed, min_waters=128, max_waters=160, polarization=polarization,
                               eps=1e-9)


# --------------------------------------------------------------------------- CPU


def test_per_type_sums_and_traceless_projection():
    rng = np.random.default_rng(0)
    g = rng.normal(size=(9, 24))
    types = np.array([0, 1, 1, 0, 2, 2, 2, 1, 0])
    s = fitting.per_type(g, types, 3)
    for t in range(3):
        assert np.allclose(s[t], g[types == t].sum(axis=0))
    p = fitting.project_traceless(g)
    assert np.allclose(p[:, 4] + p[:, 6] + p[:, 9], 0.0)
    o = p[:, 10:20]
    for a, b, c in ((0, 2, 7), (1, 3, 8), (4, 6, 9)):
        assert np.allclose(o[:, a] + o[:, b] + o[:, c], 0.0)
    # components off the trace directions are untouched
    for c in (0, 1, 2, 3, 5, 7, 8, 20, 21, 22, 23):
        assert np.array_equal(p[:, c], g[:, c])


def test_type_parameters_round_trip():
    f, pos, box = synthetic.water_box(8, 6.2, seed=3)
    types = np.tile([0, 1, 1], 8)
    params = np.arange(48, dtype=np.float64).reshape(2, 24) * 0.01 + 0.1
    fitting.apply_type_parameters(f, types, params)
    for i, t in enumerate(types):
        assert np.allclose(fitting.atom_parameters(f, i), params[t])
        assert f.getMultipoleParameters(i)[4] == MPIDForce.ZThenX  # frames kept
    assert np.allclose(fitting.type_parameters(f, types, 2), params)


def test_batch_workload_geometry():
    systems, params = fitting.water_batch(nboxes=4, seed=5)
    assert params.shape == (2, 24)
    for f, pos, box, types in systems:
        nw = len(pos) // 3
        assert 128 <= nw <= 512
        edge = box[0, 0] * 10.0
        assert abs(edge - (nw * 29.915) ** (1.0 / 3.0)) < 1e-9
        alpha, nx, ny, nz = f.getPMEParameters()
        assert nx == ny == nz and nx in fitting.FFT_FRIENDLY and nx >= edge and alpha == 4.0
        assert f.getCutoffDistance() < box[0, 0] / 2
        # every atom of a type has the type's parameters
        for i in (0, 1, 2, len(pos) - 3, len(pos) - 1):
            assert np.allclose(fitting.atom_parameters(f, i), params[types[i]])
        # molecules do not overlap: intermolecular atom distances >= 1.6 A
        d = pos[None] - pos[:, None]
        d -= box[0, 0] * np.round(d / box[0, 0])
        r = np.sqrt((d ** 2).sum(-1))
        mol = np.arange(len(pos)) // 3
        r[mol[:, None] == mol[None]] = 1.0
        assert r.min() >= 0.16 - 1e-12


# --------------------------------------------------------------------------- GPU


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name", ["frames_mutual.npz", "frames_direct.npz", "frames_extrapolated.npz"])
def test_polarization_gradients_match_oracle(name, precision):
    from oracle import oracle as O
    if not O.available("port"):
        O.build("port")
    fx = helpers.load_npz_fixture(name)
    s = helpers.system_from_fixture(fx)
    s.mutual_eps, s.max_iter = 1e-10, 500
    f = helpers.force_from_oracle_system(s)
    ctx = MPIDContext(f, precision=precision)
    e, forces, gm, gp = ctx.evaluateWithGradients(s.pos, s.box)
    ref = O.evaluate(s, "port", want_grad=True)
    err_p = helpers.rel_rms(gp[:, :3], ref.polgrad[:, :3])
    err_t = helpers.rel_rms(gp[:, 3], ref.polgrad[:, 3]) if np.any(ref.polgrad[:, 3]) else 0.0
    err_m = helpers.rel_rms(gm, ref.grad)
    print("%s %s: polarisability %.3e thole %.3e multipole %.3e" % (name, precision, err_p, err_t, err_m))
    tol = 1e-8 if precision == "double" else 1e-5
    assert err_p < tol and err_t < tol and err_m < tol
    # the combined call agrees with the separate entry points: energies and forces bit for
    # bit on the mixed path (fixed-point accumulation); the FP64 passes (all gradients,
    # and the FP64 path's evaluation) spread their PME grids with floating-point atomics
    e2, f2 = ctx.evaluate(s.pos, s.box)
    gm2 = ctx.getParameterGradients(s.pos, s.box)
    if precision == "mixed":
        assert e2 == e and np.array_equal(f2, forces)
    else:
        assert abs(e2 - e) <= 1e-12 * abs(e) and helpers.rel_rms(f2, forces) < 1e-12
    assert helpers.rel_rms(gm2, gm) < 1e-12


def _directions(rng):
    """Admissible per-type directions: (ntypes, 24) with traceless quadrupole and
    octopole parts, scaled to each parameter's size."""
    v = np.zeros((2, 24))
    v[:, 0] = rng.normal(size=2) * 0.1
    v[:, 1:4] = rng.normal(size=(2, 3)) * 0.01
    v[:, 4:10] = synthetic.traceless_quadrupole(rng, 0.002, 2)
    v[:, 10:20] = synthetic.traceless_octopole(rng, 0.0005, 2)
    v[:, 20:23] = rng.normal(size=(2, 3)) * 1e-4
    v[:, 23] = rng.normal(size=2) * 0.1
    return v


def _block_directions(rng):
    """One direction per parameter block (charge, dipole, quadrupole, octopole,
    polarisability, Thole width), then one along all of them."""
    blocks = [slice(0, 1), slice(1, 4), slice(4, 10), slice(10, 20), slice(20, 23), slice(23, 24)]
    vs = []
    for b in blocks:
        v = np.zeros((2, 24))
        v[:, b] = _directions(rng)[:, b]
        vs.append(v)
    vs.append(_directions(rng))
    return vs


def _port_per_type(systems):
    """Per-type gradient of the summed energy from the oracle port (FP64)."""
    from oracle import oracle as O
    if not O.available("port"):
        O.build("port")
    g = np.zeros((2, 24))
    for f, pos, box, types in systems:
        r = O.evaluate(helpers.oracle_system(f, pos, box), "port", want_grad=True)
        g[:, :20] += fitting.per_type(r.grad, types, 2)
        g[:, 20:] += fitting.per_type(r.polgrad, types, 2)
    return g


def test_port_per_type_gradient_matches_finite_differences():
    """The oracle port's per-type gradient (24 parameters per type) on a 128-water box of
    the batched-fitting workload against central differences, h = 1e-4, of its own FP64
    energy: to 1e-5 relative along each parameter block."""
    systems, params = small_batch(nboxes=1, seed=11)
    f, pos, box, types = systems[0]
    f.setMutualInducedTargetEpsilon(1e-11)
    g = _port_per_type(systems)
    from oracle import oracle as O

    def energy(p):
        fitting.apply_type_parameters(f, types, p)
        return O.evaluate(helpers.oracle_system(f, pos, box), "port").energy

    h = 1e-4
    for v in _block_directions(np.random.default_rng(7))[:6]:
        fd = (energy(params + h * v) - energy(params - h * v)) / (2 * h)
        an = float((g * v).sum())
        assert abs(an - fd) <= 1e-5 * max(abs(fd), 1.0), (fd, an)


@pytest.mark.gpu
@pytest.mark.parametrize("polarization", [MPIDForce.Mutual, MPIDForce.Direct, MPIDForce.Extrapolated])
def test_batch_per_type_gradients(polarization):
    """Per-type gradients of 4 boxes (128-160 waters) evaluated concurrently, along each
    parameter block: FP64 within 1e-6 and mixed within 1e-5 of the oracle port's FP64
    gradient; FP64 within 1e-6 of five-point differences (h = 1e-2) of the device's FP64
    summed energy.  (Central differences with h = 1e-4 are run on the port's energy on
    the CPU: the device's FP64 energy carries ~1e-8 kJ/mol of rounding noise from the
    floating-point atomics of its PME spread, 5e-5 in an h = 1e-4 quotient.)"""
    systems, params = small_batch(polarization=polarization)
    rng = np.random.default_rng(7)
    for f, _, _, _ in systems:
        f.setMutualInducedTargetEpsilon(1e-11)
    ref = _port_per_type(systems)
    dbl = fitting.BoxBatch(systems, 2, precision="double", threads=4)
    for f, _, _, _ in systems:
        f.setMutualInducedTargetEpsilon(1e-9)
    with dbl, fitting.BoxBatch(systems, 2, precision="mixed", threads=4) as mix:
        # the second call of a batch runs its fused launches (the first sizes them)
        dbl.evaluate(forces=False)
        mix.evaluate(forces=False)
        _, _, gd = dbl.evaluate(forces=False)
        _, _, gmx = mix.evaluate(forces=False)
        h = 1e-2

        def energy(p):
            dbl.set_parameters(p)
            return dbl.evaluate(forces=False)[0].sum()

        for v in _block_directions(rng):
            r, an_d, an_m = float((ref * v).sum()), float((gd * v).sum()), float((gmx * v).sum())
            fd = (energy(params - 2 * h * v) - 8 * energy(params - h * v) + 8 * energy(params + h * v) -
                  energy(params + 2 * h * v)) / (12 * h)
            dbl.set_parameters(params)
            print("pol %d: port %.10e double %.10e mixed %.10e fd %.10e" % (polarization, r, an_d, an_m, fd))
            scale = max(abs(r), 1.0)
            assert abs(an_d - r) <= 1e-6 * scale
            assert abs(an_m - r) <= 1e-5 * scale
            assert abs(an_d - fd) <= 1e-6 * scale


@pytest.mark.gpu
def test_concurrent_boxes_match_one_by_one():
    systems, params = small_batch(nboxes=6, seed=13)
    with fitting.BoxBatch(systems, 2, precision="mixed", threads=6) as par:
        e_par, f_par, g_par = par.evaluate()
        e_par2, f_par2, g_par2 = par.evaluate()
    with fitting.BoxBatch(systems, 2, precision="mixed", threads=1) as seq:
        e_seq, f_seq, g_seq = seq.evaluate()
    assert np.array_equal(e_par, e_seq) and np.array_equal(e_par, e_par2)
    for a, b in zip(f_par, f_seq):
        assert np.array_equal(a, b)
    # the FP64 gradient pass spreads its PME grids with floating-point atomics: equal to
    # rounding
    assert np.abs(g_par - g_seq).max() <= 1e-11 * np.abs(g_seq).max()
    assert np.abs(g_par - g_par2).max() <= 1e-11 * np.abs(g_seq).max()
    # and each box against its own plain context
    for (f, pos, box, types), e in zip(systems, e_seq):
        ctx = MPIDContext(f, precision="mixed", box=box)
        assert ctx.evaluate(pos, box)[0] == e


@pytest.mark.gpu
@pytest.mark.parametrize("precision,polarization", [("mixed", MPIDForce.Mutual), ("double", MPIDForce.Mutual),
                                                    ("mixed", MPIDForce.Direct), ("mixed", MPIDForce.Extrapolated)])
def test_graph_solver_matches_direct_launches(precision, polarization):
    """Evaluation segments and solver iterations replayed from captured CUDA graphs give
    the results of launching them one by one: on repeated evaluations (graphs reused), and
    after the box and positions change (graphs captured again for the new shape).  Bit for
    bit on the mixed path; to rounding on the FP64 path, whose PME spread uses
    floating-point atomics."""
    (f, pos, box, types), = small_batch(nboxes=1, seed=21, polarization=polarization)[0]
    plain = MPIDContext(f, precision=precision, box=box, solver_graphs=False)
    graph = MPIDContext(f, precision=precision, box=box, solver_graphs=True)
    tol = 0.0 if precision == "mixed" else 1e-12

    def same(a, b):
        a, b = np.asarray(a), np.asarray(b)
        return np.abs(a - b).max() <= tol * np.abs(a).max()

    scaled = [(pos, box), (pos, box), (pos * 1.01, box * 1.01), (pos, box)]
    for p, b in scaled:
        e0, f0 = plain.evaluate(p, b)
        e1, f1 = graph.evaluate(p, b)
        assert same(e0, e1)
        assert same(f0, f1)
        assert same(plain.getInducedDipoles(), graph.getInducedDipoles())
        s0, s1 = plain.stats(), graph.stats()
        assert s0["solver_iterations"] == s1["solver_iterations"]
        assert s0["solver_iterations"] > 1 or polarization != MPIDForce.Mutual
    g0 = plain.evaluateWithGradients(pos, box)
    g1 = graph.evaluateWithGradients(pos, box)
    assert same(g0[0], g1[0])
    for a, b in zip(g0[2:], g1[2:]):
        assert np.abs(a - b).max() <= 1e-11 * np.abs(a).max()
    # device buffers on the legacy default stream (not capturable: launched directly) and
    # on a created stream (replayed)
    import torch
    e_ref, f_ref = plain.evaluate(pos, box)
    d_pos = torch.tensor(pos, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()
    for stream in (0, side.cuda_stream):
        d_f = torch.zeros((len(pos), 3), dtype=torch.float64, device="cuda")
        d_e = torch.zeros(1, dtype=torch.float64, device="cuda")
        graph.evaluate_device(d_pos.data_ptr(), box, d_f.data_ptr(), d_e.data_ptr(), stream)
        torch.cuda.synchronize()
        assert same(float(d_e.cpu()[0]), e_ref)
        assert same(d_f.cpu().numpy(), f_ref)


@pytest.mark.gpu
def test_graph_replay_reuse_and_recapture_guard():
    """Graphs are captured once and replayed afterwards; a box that changes at every
    evaluation captures new graphs each time until the context pauses replay (captures
    in 5 evaluations in a row), after which it launches directly, with the same results."""
    (f, pos, box, types), = small_batch(nboxes=1, seed=23)[0]
    plain = MPIDContext(f, box=box, solver_graphs=False)
    graph = MPIDContext(f, box=box)
    for _ in range(3):
        graph.evaluate(pos, box)
    s = graph.stats()
    assert s["graph_captures"] == 0 and s["graph_replays"] >= 4
    paused = None
    for k in range(1, 9):
        b, p = box * (1.0 + 0.002 * k), pos * (1.0 + 0.002 * k)
        e1, f1 = graph.evaluate(p, b)
        e0, f0 = plain.evaluate(p, b)
        assert e0 == e1 and np.array_equal(f0, f1)
        s = graph.stats()
        if s["graph_replays"] == 0 and paused is None:
            paused = k
        if paused is None:
            assert s["graph_captures"] > 0
        else:  # paused for the following evaluations too
            assert s["graph_replays"] == 0 and s["graph_captures"] == 0
    # five rescaled boxes in a row captured: the sixth launches directly
    assert paused == 6
    assert plain.stats()["graph_replays"] == 0


@pytest.mark.gpu
def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    systems, params = small_batch(nboxes=2, seed=17)
    with fitting.BoxBatch(systems, 2, precision="mixed", threads=2) as batch:
        energies, _, grad = batch.evaluate(forces=False)
        p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
        e = fitting.torch_energy(batch)(p)
        (3.0 * e).backward()
        assert float(e.detach()) == energies.sum()
        # a second evaluation: the FP64 gradient pass agrees to rounding
        assert np.abs(p.grad.numpy() - 3.0 * grad).max() <= 1e-11 * np.abs(3.0 * grad).max()


def test_shard_indices_partition_and_balance():
    rng = np.random.default_rng(1)
    sizes = rng.integers(384, 1537, size=64)
    for world in (1, 2, 3, 4, 8):
        parts = [fitting.shard_indices(sizes, r, world) for r in range(world)]
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(64))
        loads = [int(sizes[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= sizes.max()


def _sharded_worker(rank, world, port, out):
    import os
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = np.arange(10) * 7 + 3
        mine = fitting.shard_indices(sizes, rank, world)
        # stand-ins for each box's energy and per-type gradient
        energies = [float(sizes[k]) * 0.5 for k in mine]
        grad = sum((np.full((2, 24), float(k)) for k in mine), np.zeros((2, 24)))
        e, g = fitting.allreduce_results(energies, mine, len(sizes), grad)
        out.put((rank, e.tolist(), g.tolist()))
    finally:
        dist.destroy_process_group()


def test_sharded_batch_allreduce_gloo():
    """Two ranks (gloo, CPU) split 10 boxes and combine energies and gradients."""
    import multiprocessing as mp
    import socket
    ctx = mp.get_context("spawn")
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    q = ctx.Queue()
    procs = [ctx.Process(target=_sharded_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sizes = np.arange(10) * 7 + 3
    for rank, e, g in res:
        assert np.allclose(e, sizes * 0.5)
        assert np.allclose(g, np.full((2, 24), float(sum(range(10)))))


@pytest.mark.gpu
@pytest.mark.parametrize("pol", [MPIDForce.Mutual, MPIDForce.Extrapolated])
def test_gradients_without_cutoff_match_oracle(pol):
    """Multipole and polarisation gradients of the 160-atom frames system under NoCutoff
    (no reciprocal or self terms; every pair in the lists), FP64 and mixed, against the
    oracle port."""
    from oracle import oracle as O
    if not O.available("port"):
        O.build("port")
    fx = helpers.load_npz_fixture("properties_frames_nocutoff.npz")
    s = helpers.system_from_fixture(fx)
    s.polarization_type = pol
    s.mutual_eps, s.max_iter = 1e-10, 500
    f = helpers.force_from_oracle_system(s)
    ref = O.evaluate(s, "port", want_grad=True)
    box = np.eye(3) * 10.0
    for precision, tol in (("double", 1e-8), ("mixed", 1e-5)):
        ctx = MPIDContext(f, precision=precision)
        e, forces, gm, gp = ctx.evaluateWithGradients(s.pos, box)
        errs = (helpers.rel_rms(gm, ref.grad), helpers.rel_rms(gp[:, :3], ref.polgrad[:, :3]),
                helpers.rel_rms(gp[:, 3], ref.polgrad[:, 3]))
        print("nocutoff pol %d %s: multipole %.2e polarisability %.2e thole %.2e" % ((pol, precision) + errs))
        assert max(errs) < tol, (precision, errs)


def _sharded_gpu_worker(rank, world, port, nboxes, out):
    import os
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        systems, _ = fitting.water_batch(nboxes=nboxes, min_waters=128, max_waters=192)
        sizes = [len(s[1]) for s in systems]
        mine = fitting.shard_indices(sizes, rank, world)
        with fitting.BoxBatch([systems[k] for k in mine], 2, precision="double", threads=2) as b:
            e, _, g = b.evaluate(forces=False)
        E, G = fitting.allreduce_results(e, mine, nboxes, g)
        out.put((rank, mine, E.tolist(), G.tolist()))
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_sharded_batch_on_gpu_matches_single_process():
    """The sharded fitting step end to end: two ranks (gloo processes sharing the one GPU;
    no kernel waits on another rank) each evaluate their shard_indices share of a 6-box
    batch with a BoxBatch (FP64) and combine with allreduce_results; every rank then holds
    the energies of all boxes and the per-type gradient of a single-process BoxBatch over
    all boxes, to 1e-12."""
    import multiprocessing as mp
    import socket
    nboxes = 6
    ctx = mp.get_context("spawn")
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    q = ctx.Queue()
    procs = [ctx.Process(target=_sharded_gpu_worker, args=(r, 2, port, nboxes, q)) for r in range(2)]
    for p in procs:
        p.start()
    systems, _ = fitting.water_batch(nboxes=nboxes, min_waters=128, max_waters=192)
    with fitting.BoxBatch(systems, 2, precision="double", threads=2) as b:
        e_ref, _, g_ref = b.evaluate(forces=False)
    res = [q.get(timeout=600) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    shards = sorted(k for _, mine, _, _ in res for k in mine)
    assert shards == list(range(nboxes)) and all(len(mine) > 0 for _, mine, _, _ in res)
    for rank, mine, e, g in res:
        assert np.allclose(e, e_ref, rtol=1e-12, atol=0), rank
        assert np.abs(np.asarray(g) - g_ref).max() <= 1e-12 * np.abs(g_ref).max(), rank


@pytest.mark.gpu
@pytest.mark.parametrize("launch", [0, -1, 8])
@pytest.mark.parametrize("precision", ["mixed", "double"])
def test_batched_graph_matches_per_box_evaluations(precision, launch):
    """mpid_evaluate_batch against the same boxes evaluated one context at a time, for
    three calls in a row (the first takes the ordinary evaluation and sizes the graphs,
    the later ones run batched) and for a call after one box's atoms moved.  Per-box
    graphs (launch -1: one parent graph, 8: eight streams) run the per-box kernels as
    they are: energies, forces and per-type gradients to 1e-10 relative.  The fused
    launches (0) run the same kernel bodies with the same per-box parameters, but each
    grid size's FFTs as one batched cuFFT plan, whose FP32 rounding differs from the
    single-box plan's: FP64 to 1e-10, mixed to 1e-7 (energies), 1e-5 (forces) and 1e-6
    (per-type gradients), relative."""
    systems, _ = fitting.water_batch(nboxes=6, min_waters=128, max_waters=192)
    tol = (1e-10, 1e-10, 1e-10) if precision == "double" or launch != 0 else (1e-7, 1e-5, 1e-6)
    with fitting.BoxBatch(systems, 2, precision=precision, threads=1, batched=False) as ref, \
            fitting.BoxBatch(systems, 2, precision=precision, batched=True) as bb:
        bb.configure({"launch": launch})
        e0, f0, g0 = ref.evaluate()

        def check(e1, f1, g1, e0, f0, g0):
            assert np.allclose(e1, e0, rtol=tol[0], atol=0), np.abs(e1 / e0 - 1).max()
            for a, b in zip(f1, f0):
                assert np.abs(a - b).max() <= tol[1] * np.abs(b).max(), np.abs(a - b).max() / np.abs(b).max()
            assert np.abs(g1 - g0).max() <= tol[2] * np.abs(g0).max(), np.abs(g1 - g0).max() / np.abs(g0).max()

        for step in range(3):
            e1, f1, g1 = bb.evaluate()
            check(e1, f1, g1, e0, f0, g0)
            if step > 0:
                assert all(c.stats()["graph_replays"] == 1 for c in bb.contexts)
        # one box moves: its list and solver may change; results follow the new positions
        f, pos, box, types = systems[2]
        moved = pos + np.random.default_rng(4).normal(scale=0.003, size=pos.shape)
        for b in (ref, bb):
            b.systems[2] = (f, moved, box, types)
        e0, f0, g0 = ref.evaluate()
        e1, f1, g1 = bb.evaluate()
        check(e1, f1, g1, e0, f0, g0)


@pytest.mark.gpu
def test_autotuner_records_and_reuses_its_choice(tmp_path):
    """BoxBatch.autotune times the batch under each launch configuration (work-split bound
    of the pair kernels, batched launch mode), keeps the fastest, records it per GPU and
    workload class and reuses the record; the results under any configuration are those of
    the default one up to the rounding of the FP32 partial sums, which the split groups
    differently (energies 1e-7, per-type gradients 1e-6 relative: within the mixed path's
    own accuracy against FP64)."""
    import json
    systems, _ = fitting.water_batch(nboxes=4, min_waters=128, max_waters=160)
    path = str(tmp_path / "tuning.json")
    with fitting.BoxBatch(systems, 2, precision="mixed", batched=True) as b:
        e0, _, g0 = b.evaluate()
        best, times = b.autotune(splits=(0, 2), launches=(0, 4), repeats=1, path=path)
        assert best in [{"max_split": m, "launch": q} for m in (0, 2) for q in (0, 4)] and len(times) == 4
        rec = json.load(open(path))
        assert rec[b.tuning_key()]["config"] == best
        again, times2 = b.autotune(splits=(0, 2), launches=(0, 4), repeats=1, path=path)  # from the record
        assert again == best and times2 == times
        for cfg in ({"max_split": 2, "launch": 4}, {"max_split": 0, "launch": 0}):
            b.configure(cfg)
            e1, _, g1 = b.evaluate()
            print(cfg, np.abs(e1 / e0 - 1).max(), np.abs(g1 - g0).max() / np.abs(g0).max())
            assert np.allclose(e1, e0, rtol=1e-7, atol=0)
            assert np.abs(g1 - g0).max() <= 1e-6 * np.abs(g0).max()


@pytest.mark.gpu
@pytest.mark.parametrize("launch", [0, 8])
def test_batch_type_sums_match_per_atom_gradients(launch):
    """mpid_evaluate_batch's per-type gradient sums (type_grad, summed on the device per
    box in the fused launch, on the host otherwise) against the per-type sums of the same
    call's per-atom gradients, to 1e-12 relative; the first call (ordinary evaluations)
    and a batched one."""
    from mpidopenmmplugin_gb300.context import evaluate_batch
    systems, _ = fitting.water_batch(nboxes=5, min_waters=128, max_waters=192)
    ctxs = [MPIDContext(f, precision="mixed", box=b) for f, p, b, t in systems]
    for (f, p, b, t), c in zip(systems, ctxs):
        c.setAtomTypes(t, 2)
    types = np.concatenate([t for _, _, _, t in systems])
    for call in range(2):
        e, fo, gm, gp, tg = evaluate_batch(ctxs, [s[1] for s in systems], [s[2] for s in systems], launch=launch,
                                           flat=True, type_grad=True)
        ref = np.hstack([fitting.per_type(gm, types, 2), fitting.per_type(gp, types, 2)])
        assert tg.shape == (2, 24)
        assert np.abs(tg - ref).max() <= 1e-12 * np.abs(ref).max(), (call, np.abs(tg - ref).max())
    for c in ctxs:
        c.close()


@pytest.mark.gpu
def test_fused_batch_beyond_one_launch_of_boxes():
    """70 boxes: more than the 64 (or fewer, for large parameter sets) boxes whose
    parameters one fused launch carries, so every fused operation is split into several
    launches.  Energies, forces and per-type gradients against the per-box graphs (launch
    mode 8), within the tolerances of the fused mixed path."""
    systems, _ = fitting.water_batch(nboxes=70, min_waters=128, max_waters=136)
    with fitting.BoxBatch(systems, 2, precision="mixed", batched=True) as fused, \
            fitting.BoxBatch(systems, 2, precision="mixed", batched=True) as ref:
        ref.configure({"launch": 8})
        for _ in range(2):
            e0, f0, g0 = ref.evaluate()
            e1, f1, g1 = fused.evaluate()
        assert fused.launches() < 600  # against about 126 per box (8,820) unfused
        assert np.allclose(e1, e0, rtol=1e-7, atol=0), np.abs(e1 / e0 - 1).max()
        for a, b in zip(f1, f0):
            assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max()
        assert np.abs(g1 - g0).max() <= 1e-6 * np.abs(g0).max()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["solution", "triclinic"])
def test_fused_batch_on_solutes_and_triclinic_boxes(kind):
    """The fused launch mode on boxes unlike the water batch: small solutions (ethanes with
    anisotropic polarisabilities, 1-4 scaled pairs, so every box has covalently scaled
    pair energies) and a triclinic box (the reference's triclinic fixture, its atoms
    jittered per box).  Energies, forces and per-atom gradients against per-box graphs
    (launch mode 8), within the tolerances of the fused mixed path, three calls in a row."""
    from mpidopenmmplugin_gb300.context import evaluate_batch
    systems = []
    if kind == "solution":
        for k in range(3):
            f, pos, box = synthetic.solution_box(150 + 10 * k, 3, 17.5 + 0.4 * k, seed=31 + k)
            f.setNonbondedMethod(MPIDForce.PME)
            f.setCutoffDistance(0.7)
            f.setPMEParameters(4.0, 18, 18, 18)
            f.setPmeBSplineOrder(5)
            f.setMutualInducedTargetEpsilon(1e-7)
            systems.append((f, pos, box))
    else:
        fx = helpers.load_npz_fixture("triclinic_mutual.npz")
        s = helpers.system_from_fixture(fx)
        for k in range(3):
            f = helpers.force_from_oracle_system(s)
            pos = np.asarray(s.pos) + np.random.default_rng(40 + k).normal(scale=0.002, size=np.shape(s.pos))
            systems.append((f, pos, np.asarray(s.box)))
    ctxs = {launch: [MPIDContext(f, precision="mixed", box=b) for f, p, b in systems] for launch in (0, 8)}
    pos = [p for _, p, _ in systems]
    boxes = [b for _, _, b in systems]
    for call in range(3):
        e1, f1, m1, p1 = evaluate_batch(ctxs[0], pos, boxes, launch=0)
        e0, f0, m0, p0 = evaluate_batch(ctxs[8], pos, boxes, launch=8)
        assert np.allclose(e1, e0, rtol=1e-7, atol=0), (call, np.abs(e1 / e0 - 1).max())
        for a, b in zip(f1, f0):
            assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max(), call
        for a, b in list(zip(m1, m0)) + list(zip(p1, p0)):
            assert helpers.rel_rms(a, b) <= 1e-5, call
    for cs in ctxs.values():
        for c in cs:
            c.close()
