"""The allocation-free kinetic-energy reduction (mg_mvv_noalloc).

Callers that cannot allocate device memory (a host loop under CUDA-graph capture, a plugin inside a
process whose allocator owns the GPU, a real-time loop that must not block on the allocator) use
mg_mvv_noalloc instead of mg_thermo. This file checks, through the C ABI, that it gives mg_thermo's
sum m v^2 on two different states in a row (its scratch array keeps the previous call's values), and
that it rejects an atom count beyond its fixed scratch. It sorts last so that a failure here stops a
-x run only after every other test has run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A0 = 2.855
RCF = 5.6 / A0


def test_mvv_noalloc_matches_thermo_twice(pkg, wl, potentials, gpu_lib):
    import torch

    cells = (12, 10, 11)
    lib = pkg.load_library()
    ctx = pkg.Context(cells, A0, RCF)
    ctx.pot_init_setfl(potentials["fe"])
    loc = wl.local_slot_indices(cells, RCF)
    stream = torch.cuda.current_stream()
    for seed, temp in ((3, 600.0), (4, 250.0)):
        atoms = wl.build_state(cells, A0, RCF, temperature=temp, seed=seed)
        atoms["type"][loc[7::53]] = -1  # a few vacancies, skipped by both
        atoms["v"][loc[7::53]] = 0.0
        ctx.upload(atoms)
        want = ctx.thermo()["mvv"]
        a = atoms[loc]
        v = torch.tensor(np.ascontiguousarray(a["v"].T), dtype=torch.float64, device="cuda")
        ty = torch.tensor(a["type"].astype(np.int8), device="cuda")
        out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        st = lib.mg_mvv_noalloc(v[0].data_ptr(), v[1].data_ptr(), v[2].data_ptr(), ty.data_ptr(), a.size,
                                out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, lib.mg_last_error(None)
        torch.cuda.synchronize()
        assert out.item() == pytest.approx(want, rel=1e-12)
    ctx.close()


def test_mvv_noalloc_rejects_oversize(pkg, gpu_lib):
    import torch

    lib = pkg.load_library()
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    t = torch.zeros(4, dtype=torch.int8, device="cuda")
    st = lib.mg_mvv_noalloc(x.data_ptr(), x.data_ptr(), x.data_ptr(), t.data_ptr(), 33_554_433, x.data_ptr(), None)
    assert st == 1
    assert b"33,554,432" in lib.mg_last_error(None)
