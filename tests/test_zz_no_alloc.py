"""mpid_evaluate_device_noalloc against mpid_evaluate_device, through the C ABI.

The allocation-free call runs the same evaluation with its neighbour lists and per-task
energies in a static device array, so on the same context and inputs it must give the
existing entry point's energy, forces and dipoles (tolerance 1e-12 relative; the kernels
and their summation order are the same).  This file is collected last so that it also
runs after every other GPU test in the same process.
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


def _run(torch, ctx, fn, pos, box):
    d_pos, d_force, d_energy = _device_buffers(torch, pos)
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
