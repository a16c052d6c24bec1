"""The allocation-free assembly entry point (gales_asm_assemble_noalloc).

It serves callers that must not allocate device memory while assembling (memory
owned by another allocator or a fixed quota, loops with a fixed footprint).  Its
output must equal the regular entry point's, call after call, although every call
reuses the same library-wide scratch array.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from cases import rel


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc,form", [("tet", 3, 0), ("tet", 3, 1), ("hex", 4, 0), ("tri", 2, 1)])
def test_noalloc_matches_assemble_twice(kind, nc, form, cuda_lib, gm):
    import torch
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    Id, Pd = torch.from_numpy(I).cuda(), torch.from_numpy(P).cuda()
    ref = fa.linear_system(device="cuda")
    fa.execute(Id, Pd, dt, ref, form=form)
    tol = 1e-12 if form == 0 else 1e-6
    for _ in range(2):                       # two calls in a row on the shared scratch
        lp = fa.linear_system(device="cuda")
        lp.vals.fill_(np.nan)
        lp.rhs.fill_(np.nan)
        fa.execute_noalloc(Id, Pd, dt, lp, form=form)
        torch.cuda.synchronize()
        assert rel(lp.vals.cpu().numpy(), ref.vals.cpu().numpy()) <= tol
        assert rel(lp.rhs.cpu().numpy(), ref.rhs.cpu().numpy()) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_noalloc_many_scratch_chunks(form, cuda_lib, gm):
    """A mesh far larger than one scratch chunk: the chunks (multiples of a matrix CTA's
    elements) keep every block of point records inside the scratch."""
    import torch
    syn = cases.syn
    mesh = syn.box_tet_delaunay(22, seed=3)
    mat, setup = syn.material_for(3, 0), syn.setup_for(3, 3)
    I, P = syn.state_for(mesh, 3, 0)
    fa = gm.FluidAssembly(mesh, mat, setup)
    Id, Pd = torch.from_numpy(I).cuda(), torch.from_numpy(P).cuda()
    ref = fa.linear_system(device="cuda")
    fa.execute(Id, Pd, 1e-3, ref, form=form)
    lp = fa.linear_system(device="cuda")
    n0 = fa.launch_count()
    fa.execute_noalloc(Id, Pd, 1e-3, lp, form=form)
    torch.cuda.synchronize()
    # one point and one matrix launch per scratch chunk (plus the boundary pass): more
    # than two interior launches means the records went through several chunks
    assert fa.launch_count() - n0 >= 6
    tol = 1e-12 if form == 0 else 1e-6
    assert rel(lp.vals.cpu().numpy(), ref.vals.cpu().numpy()) <= tol
    assert rel(lp.rhs.cpu().numpy(), ref.rhs.cpu().numpy()) <= tol


@pytest.mark.gpu
def test_noalloc_rejects_host_buffers(cuda_lib, gm):
    mesh, mat, setup, I, P, dt = cases.make("tri", 2)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp = fa.linear_system()
    L = gm.abi.lib()
    rc = L.gales_asm_assemble_noalloc(fa._h, I.ctypes.data, P.ctypes.data, dt, 0, lp.vals.ctypes.data,
                                      lp.rhs.ctypes.data, None)
    assert rc == gm.abi.ERR_BAD_INPUT
    assert b"device pointers" in L.gales_asm_last_error(fa._h)
