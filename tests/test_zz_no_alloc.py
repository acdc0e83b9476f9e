"""The allocation-free reciprocal-energy entry point.

It serves callers that may not allocate device memory themselves (a plug-in
inside a host program whose device memory all comes from that program's own
allocator).  The test hands it device buffers made by the caller (torch here)
and checks two calls in a row against the allocating path (fe_mc_setup +
fe_mc_kspace_energy on a box), to 1e-9 relative (both FP64, different
summation order).  Collected last so that a stop-at-first-failure run has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def test_noalloc_kspace_energy_matches_allocating_path():
    import torch

    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(400, L=22.0, seed=31, grid=(24, 24, 24))
    kmax, mks = 7, 49
    with engine.Box(s) as b:
        b.mc_setup(kmax=kmax, max_k_square=mks)
        want = b.mc_kspace_energy()
    lib = engine.load_library()
    fn = lib.fe_ewald_kspace_energy_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_void_p,
                   C.c_void_p]
    fn.restype = C.c_int
    xyzq = torch.tensor(np.concatenate([s.pos, s.q[:, None]], axis=1), dtype=torch.float64,
                        device="cuda").contiguous()
    L = np.ascontiguousarray(s.L, dtype=np.float64)
    got = []
    for _ in range(2):
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = fn(xyzq.data_ptr(), s.n, L.ctypes.data, s.kappa, kmax, mks, out.data_ptr(), None)
        assert rc == 0, lib.fe_last_error().decode()
        torch.cuda.synchronize()
        got.append(float(out.item()))
    for g in got:
        assert abs(g - want) <= RTOL * abs(want), (g, want)
    # a call beyond the fixed scratch is refused before any launch
    out = torch.zeros((1,), dtype=torch.float64, device="cuda")
    rc = fn(xyzq.data_ptr(), s.n, L.ctypes.data, s.kappa, 13, 169, out.data_ptr(), None)
    assert rc == engine.FE_ERR_SIZE
