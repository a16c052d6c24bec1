"""Capture-safe assembly: gales_asm_enqueue recorded into a CUDA graph and replayed.

A graph of several Newton-iteration assemblies (the use of the hex workload) must
give the same CSR values and rhs as the synchronous call, replay after replay, with
the state changed in place between replays.
"""
import numpy as np
import pytest

import cases
from cases import gm, rel


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["mixed", "fp64"])
def test_enqueue_in_cuda_graph_matches_synchronous_assembly(form, cuda_lib):
    torch = pytest.importorskip("torch")
    f = gm.FORM_MIXED if form == "mixed" else gm.FORM_FP64
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    dev = torch.device("cuda:0")
    fa = gm.FluidAssembly(mesh, mat, setup)
    ref = fa.linear_system(device=dev)
    lp = fa.linear_system(device=dev)
    Id = torch.tensor(I, device=dev)
    Pd = torch.tensor(P, device=dev)
    s = torch.cuda.Stream(device=dev)
    # warm up outside the capture (as a caller does before recording)
    with torch.cuda.stream(s):
        fa.enqueue(Id, Pd, dt, lp, form=f, stream=s.cuda_stream)
    fa.sync(stream=s.cuda_stream)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
        for _ in range(3):
            fa.enqueue(Id, Pd, dt, lp, form=f, stream=s.cuda_stream)
    rng = np.random.default_rng(0)
    for rep in range(3):
        Inew = I * (1.0 + 1e-3 * rng.normal(size=I.shape))
        Id.copy_(torch.tensor(Inew, device=dev))
        g.replay()
        torch.cuda.synchronize()
        fa.sync(stream=s.cuda_stream)
        fa.execute(Id, Pd, dt, ref, form=f)
        torch.cuda.synchronize()
        assert rel(lp.vals.cpu().numpy(), ref.vals.cpu().numpy()) <= 1e-12
        assert rel(lp.rhs.cpu().numpy(), ref.rhs.cpu().numpy()) <= 1e-12


@pytest.mark.gpu
def test_enqueue_reports_errors_at_sync(cuda_lib):
    torch = pytest.importorskip("torch")
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    dev = torch.device("cuda:0")
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp = fa.linear_system(device=dev)
    Ib = I.copy()
    Ib[int(mesh.conn[5, 0]) * fa.nd] = np.nan
    fa.enqueue(torch.tensor(Ib, device=dev), torch.tensor(P, device=dev), dt, lp)
    with pytest.raises(gm.GalesError) as ei:
        fa.sync()
    assert ei.value.code & gm.abi.ERR_NONFINITE
    # cleared: the next enqueue of a finite state syncs clean
    fa.enqueue(torch.tensor(I, device=dev), torch.tensor(P, device=dev), dt, lp)
    fa.sync()
