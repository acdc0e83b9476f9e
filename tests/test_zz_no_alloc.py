"""The allocation-free reciprocal-energy entry point.

It serves callers that may not allocate device memory themselves (a plug-in
inside a host program whose device memory all comes from that program's own
allocator).  The tests hand it device buffers made by the caller (torch here)
and check two calls in a row against the allocating path (fe_mc_setup +
fe_mc_kspace_energy on a box), to 1e-9 relative (both FP64, different
summation order): a cubic box at kmax 7 on the legacy default stream, a
non-cubic box at the size limit (kmax 12, 8,112 candidate k-vectors) on a side
stream, refusals of host pointers and of sizes beyond the limit (made on the
host, nothing launched), and a second call after the host program reset the
device.  Collected last so that a stop-at-first-failure run has already run
every other test.
"""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-9
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _fn():
    from thecodecombo_7_gb300 import engine
    lib = engine.load_library()
    fn = lib.fe_ewald_kspace_energy_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_void_p,
                   C.c_void_p]
    fn.restype = C.c_int
    return lib, fn


def _box(L):
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(400, L=22.0, seed=31, grid=(24, 24, 24))
    s.L = np.asarray(L, dtype=np.float64)  # sites stay inside [-11, 11): wrapped in every L
    return s


def _allocating(s, kmax, mks):
    from thecodecombo_7_gb300 import engine
    with engine.Box(s) as b:
        b.mc_setup(kmax=kmax, max_k_square=mks)
        return b.mc_kspace_energy()


def _noalloc_twice(s, kmax, mks, stream=None):
    import torch
    lib, fn = _fn()
    xyzq = torch.tensor(np.concatenate([s.pos, s.q[:, None]], axis=1), dtype=torch.float64,
                        device="cuda").contiguous()
    L = np.ascontiguousarray(s.L, dtype=np.float64)
    got = []
    for _ in range(2):
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        sp = stream.cuda_stream if stream is not None else None
        rc = fn(xyzq.data_ptr(), s.n, L.ctypes.data, s.kappa, kmax, mks, out.data_ptr(), sp)
        assert rc == 0, lib.fe_last_error().decode()
        torch.cuda.synchronize()
        got.append(float(out.item()))
    return got


def test_noalloc_kspace_energy_matches_allocating_path():
    s = _box([22.0, 22.0, 22.0])
    want = _allocating(s, 7, 49)
    for g in _noalloc_twice(s, 7, 49):
        assert abs(g - want) <= RTOL * abs(want), (g, want)


def test_noalloc_non_cubic_box_at_the_size_limit_on_a_side_stream():
    import torch
    s = _box([22.0, 25.0, 28.5])
    want = _allocating(s, 12, 144)
    stream = torch.cuda.Stream()
    for g in _noalloc_twice(s, 12, 144, stream=stream):
        assert abs(g - want) <= RTOL * abs(want), (g, want)


def test_noalloc_refusals_launch_nothing():
    import torch
    from thecodecombo_7_gb300 import engine
    lib, fn = _fn()
    s = _box([22.0, 22.0, 22.0])
    L = np.ascontiguousarray(s.L, dtype=np.float64)
    host = np.ascontiguousarray(np.concatenate([s.pos, s.q[:, None]], axis=1))
    dev = torch.tensor(host, device="cuda")
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    host_out = np.zeros(1)
    torch.cuda.synchronize()
    # host memory for the sites or the result: refused on the host
    assert fn(host.ctypes.data, s.n, L.ctypes.data, s.kappa, 7, 49, out.data_ptr(),
              None) == engine.FE_ERR_ARG
    assert fn(dev.data_ptr(), s.n, L.ctypes.data, s.kappa, 7, 49, host_out.ctypes.data,
              None) == engine.FE_ERR_ARG
    # beyond the fixed scratch (kmax 13), and a kmax whose candidate count
    # would overflow 32-bit arithmetic
    for kmax in (13, 2**30):
        assert fn(dev.data_ptr(), s.n, L.ctypes.data, s.kappa, kmax, 169, out.data_ptr(),
                  None) == engine.FE_ERR_SIZE
    torch.cuda.synchronize()
    assert float(out.item()) == 7.0 and host_out[0] == 0.0  # nothing was written


_RESET_CHILD = textwrap.dedent(r"""
    import ctypes as C, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    from thecodecombo_7_gb300 import engine, systems
    lib = engine.load_library()
    rt = C.CDLL("libcudart.so.13")
    fn = lib.fe_ewald_kspace_energy_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_void_p,
                   C.c_void_p]
    s = systems.water_box(400, L=22.0, seed=31, grid=(24, 24, 24))
    host = np.ascontiguousarray(np.concatenate([s.pos, s.q[:, None]], axis=1))
    L = np.ascontiguousarray(s.L)
    def call():
        d_x, d_e = C.c_void_p(), C.c_void_p()
        assert rt.cudaMalloc(C.byref(d_x), C.c_size_t(host.nbytes)) == 0
        assert rt.cudaMalloc(C.byref(d_e), C.c_size_t(8)) == 0
        assert rt.cudaMemcpy(d_x, host.ctypes.data, C.c_size_t(host.nbytes), 1) == 0
        rc = fn(d_x, s.n, L.ctypes.data, s.kappa, 7, 49, d_e, None)
        assert rc == 0, lib.fe_last_error().decode()
        e = np.zeros(1)
        assert rt.cudaMemcpy(e.ctypes.data, d_e, C.c_size_t(8), 2) == 0
        rt.cudaFree(d_x)
        rt.cudaFree(d_e)
        return float(e[0])
    e1 = call()
    assert rt.cudaDeviceReset() == 0  # the host program ends its context
    e2 = call()
    print(repr(e1), repr(e2))
""")


def test_noalloc_after_device_reset():
    """A host program that resets the device between two calls gets the
    same result from the second (the scratch address is looked up in the new
    context).  Run in a child process: the reset ends only that process's
    context."""
    s = _box([22.0, 22.0, 22.0])
    want = _allocating(s, 7, 49)
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, ROOT], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    e1, e2 = (float(x) for x in r.stdout.split()[-2:])
    for g in (e1, e2):
        assert abs(g - want) <= RTOL * abs(want), (e1, e2, want)
