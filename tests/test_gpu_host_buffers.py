"""Host-buffer assemblies (the reference's interface: A and b filled in host memory).
Into page-locked memory the CSR rows are copied while the interior pass runs, prefix by
prefix in node order; into pageable memory after it.  Both equal the device-buffer
assembly (summation order aside)."""
import numpy as np
import pytest

from cases import gm, rel, syn


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["mixed", "fp64"])
def test_host_buffers_match_device_buffers(form, cuda_lib):
    torch = pytest.importorskip("torch")
    f = gm.FORM_MIXED if form == "mixed" else gm.FORM_FP64
    mesh = syn.box_tet_delaunay(22, seed=3)          # ~60k tets; pinned buffers: 8 interior chunks
    mat, setup = syn.material_for(3, 0), syn.setup_for(3, 3)
    I, P = syn.state_for(mesh, 3, 0)
    dt = 1e-3
    fa = gm.FluidAssembly(mesh, mat, setup)
    dev = torch.device("cuda:0")
    ref = fa.linear_system(device=dev)
    fa.execute(torch.tensor(I, device=dev), torch.tensor(P, device=dev), dt, ref, form=f)
    rv, rb = ref.vals.cpu().numpy(), ref.rhs.cpu().numpy()
    pinned = gm.LinearSystem(ref.row_ptr, ref.col, torch.zeros(len(rv), dtype=torch.float64).pin_memory(),
                             torch.zeros(len(rb), dtype=torch.float64).pin_memory())
    pageable = fa.linear_system()
    for lp, Ih, Ph in ((pinned, torch.from_numpy(I).pin_memory(), torch.from_numpy(P).pin_memory()),
                       (pageable, I, P)):
        for _ in range(2):                              # reuse of the handle's copy events
            fa.execute(Ih, Ph, dt, lp, form=f)
            v = lp.vals.numpy() if hasattr(lp.vals, "numpy") else lp.vals
            b = lp.rhs.numpy() if hasattr(lp.rhs, "numpy") else lp.rhs
            assert rel(v, rv) <= 1e-12 and rel(b, rb) <= 1e-12
