"""mpid_evaluate_device_noalloc against mpid_evaluate_device, through the C ABI.

The allocation-free call serves callers that must not allocate device memory while they
evaluate (an integrator that reserved a fixed device-memory budget, a host whose own
allocator owns the device).  It runs the same evaluation with its neighbour lists and
per-task energies in a static device array, so on the same context and inputs it must
give the existing entry point's energy, forces and dipoles (tolerance 1e-12 relative;
the kernels and their summation order are the same), and it must make no device
allocation: the library's own count of cudaMalloc calls (mpid_stats.device_allocations)
and the device's free memory stay unchanged across it.  This file is collected last so
that it also runs after every other GPU test in the same process.
"""
import numpy as np
import pytest

from mpidopenmmplugin_gb300 import MPIDContext, MPIDError, MPIDForce, synthetic

import helpers

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _device_buffers(torch, pos):
    d_pos = torch.tensor(np.asarray(pos), dtype=torch.float64, device="cuda").contiguous()
    d_force = torch.zeros((len(pos), 3), dtype=torch.float64, device="cuda")
    d_energy = torch.zeros(1, dtype=torch.float64, device="cuda")
    return d_pos, d_force, d_energy


def _run(torch, ctx, fn, pos, box, bufs=None):
    d_pos, d_force, d_energy = bufs if bufs is not None else _device_buffers(torch, pos)
    if bufs is not None:
        d_pos.copy_(torch.tensor(np.asarray(pos), dtype=torch.float64))
        d_force.zero_()
    stream = torch.cuda.current_stream()
    fn(d_pos.data_ptr(), box, d_force.data_ptr(), d_energy.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    return float(d_energy.item()), d_force.cpu().numpy(), ctx.getInducedDipoles()


@pytest.mark.parametrize("pol", [MPIDForce.Mutual, MPIDForce.Direct, MPIDForce.Extrapolated])
@pytest.mark.parametrize("precision", ["mixed", "double"])
def test_noalloc_matches_evaluate_device(pol, precision):
    torch = pytest.importorskip("torch")
    f, pos, box = synthetic.workload("water648", polarization=pol, order=5)
    ctx = MPIDContext(f, precision=precision)
    e0, f0, mu0 = _run(torch, ctx, ctx.evaluate_device, pos, box)
    for _ in range(2):  # two consecutive calls
        e1, f1, mu1 = _run(torch, ctx, ctx.evaluate_device_noalloc, pos, box)
        assert abs(e1 - e0) <= TOL * abs(e0)
        assert helpers.rel_rms(f1, f0) <= TOL
        assert helpers.rel_rms(mu1, mu0) <= TOL
    # the context's own buffers are back in use afterwards
    e2, f2, _ = _run(torch, ctx, ctx.evaluate_device, pos, box)
    assert abs(e2 - e0) <= TOL * abs(e0)
    assert helpers.rel_rms(f2, f0) <= TOL


@pytest.mark.parametrize("precision", ["mixed", "double"])
def test_noalloc_makes_no_device_allocation(precision):
    """No cudaMalloc by the library (its own counter) and no change of the device's free
    memory across allocation-free calls at the first positions, at moved positions and in
    a rescaled box; each result equals mpid_evaluate_device's on the same inputs."""
    torch = pytest.importorskip("torch")
    f, pos, box = synthetic.workload("water648", polarization=MPIDForce.Mutual, order=5)
    ctx = MPIDContext(f, precision=precision)
    rng = np.random.default_rng(11)
    moved = pos + rng.normal(scale=0.004, size=pos.shape)
    scaled_box = np.asarray(box) * 1.003
    cases = [(pos, box), (moved, box), (moved * 1.003, scaled_box)]
    bufs = _device_buffers(torch, pos)
    # the ordinary entry point sizes the context (and loads every kernel) first
    _run(torch, ctx, ctx.evaluate_device, pos, box, bufs)
    _run(torch, ctx, ctx.evaluate_device_noalloc, pos, box, bufs)
    allocs0 = ctx.stats()["device_allocations"]
    free0 = torch.cuda.mem_get_info()[0]
    results = []
    for p, b in cases + cases:  # every case twice in a row
        results.append(_run(torch, ctx, ctx.evaluate_device_noalloc, p, b, bufs))
        assert ctx.stats()["device_allocations"] == allocs0
    assert torch.cuda.mem_get_info()[0] == free0
    for k, (p, b) in enumerate(cases):
        e0, f0, mu0 = _run(torch, ctx, ctx.evaluate_device, p, b, bufs)
        for e1, f1, mu1 in (results[k], results[k + len(cases)]):
            assert abs(e1 - e0) <= TOL * abs(e0), k
            assert helpers.rel_rms(f1, f0) <= TOL, k
            assert helpers.rel_rms(mu1, mu0) <= TOL, k


def test_gradients_after_noalloc_match_ordinary_evaluation():
    """The gradient calls after an allocation-free evaluation rebuild the context's own
    neighbour lists (the allocation-free call's lists lived in its scratch): they return
    what they return after an ordinary evaluation."""
    torch = pytest.importorskip("torch")
    f, pos, box = synthetic.workload("water648", polarization=MPIDForce.Mutual, order=5)
    ctx = MPIDContext(f, precision="mixed")
    _run(torch, ctx, ctx.evaluate_device, pos, box)
    e_ref, f_ref, gm_ref, gp_ref = ctx.evaluateWithGradients(pos, box)
    g_ref = ctx.getParameterGradients(pos, box)
    _run(torch, ctx, ctx.evaluate_device_noalloc, pos, box)
    g = ctx.getParameterGradients(pos, box)
    assert helpers.rel_rms(g, g_ref) <= TOL
    _run(torch, ctx, ctx.evaluate_device_noalloc, pos, box)
    e, fo, gm, gp = ctx.evaluateWithGradients(pos, box)
    assert abs(e - e_ref) <= TOL * abs(e_ref)
    assert helpers.rel_rms(fo, f_ref) <= TOL
    assert helpers.rel_rms(gm, gm_ref) <= TOL and helpers.rel_rms(gp, gp_ref) <= TOL


def test_noalloc_rejects_systems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    f, pos, box = synthetic.workload("water24k", polarization=MPIDForce.Direct)
    ctx = MPIDContext(f, precision="mixed")
    # one ordinary call sizes the context's tile lists (a fresh context is rejected
    # earlier, because its tile lists would have to grow)
    e0, f0, _ = _run(torch, ctx, ctx.evaluate_device, pos, box)
    d_pos, d_force, d_energy = _device_buffers(torch, pos)
    with pytest.raises(MPIDError, match="static scratch"):
        ctx.evaluate_device_noalloc(d_pos.data_ptr(), box, d_force.data_ptr(), d_energy.data_ptr(), 0)
    torch.cuda.synchronize()
    assert not d_force.abs().sum().item()  # nothing written to the caller's forces
    # still usable through the ordinary entry point, which matches the host-buffer call
    e1, f1 = ctx.evaluate(pos, box)
    assert abs(e1 - e0) <= TOL * abs(e0)
    assert helpers.rel_rms(f1, f0) <= TOL


def test_noalloc_rejects_no_cutoff():
    torch = pytest.importorskip("torch")
    f, pos, box = synthetic.workload("water648", polarization=MPIDForce.Direct, order=5)
    f.setNonbondedMethod(MPIDForce.NoCutoff)
    ctx = MPIDContext(f, precision="mixed")
    d_pos, d_force, d_energy = _device_buffers(torch, pos)
    with pytest.raises(MPIDError, match="PME only"):
        ctx.evaluate_device_noalloc(d_pos.data_ptr(), box, d_force.data_ptr(), d_energy.data_ptr(), 0)
