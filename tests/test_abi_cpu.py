"""CPU-side checks of the C ABI and host logic (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from thecodecombo_7_gb300 import build, engine
    build.build()
    return engine.load_library()


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char \*)\s*\*?\s*(fe_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_declared_symbol(lib):
    from thecodecombo_7_gb300 import engine
    declared = _declared("fe.h")
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(engine.EXPORTS) == declared
    out = subprocess.run(["nm", "-D", "--defined-only", engine.LIB_PATH], capture_output=True,
                         text=True).stdout
    for name in declared:
        assert re.search(rf"\bT {name}\b", out), name


def _param_counts(header):
    """Number of parameters of every fe_* prototype in the header."""
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(fe_\w+)\s*\(([^;{]*?)\)\s*;", txt, re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_ctypes_signatures_match_header(lib):
    """Every argtypes list the host mirror sets has the header's arity."""
    counts = _param_counts("fe.h")
    checked = 0
    for name, n in counts.items():
        at = getattr(lib, name).argtypes
        if at is not None:
            assert len(at) == n, (name, len(at), n)
            checked += 1
    assert checked >= 10


def test_abi_version(lib):
    assert lib.fe_abi_version() == 2


def test_non_neutral_box_is_rejected_with_code_20(lib):
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(20, L=12.0, seed=1, grid=(8, 8, 8))
    s.q = s.q.copy()
    s.q[0] += 0.01
    with pytest.raises(engine.FeError) as ei:
        engine.Box(s)
    assert ei.value.code == engine.FE_ERR_CHARGE


def test_bad_arguments_are_rejected(lib):
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(20, L=12.0, seed=1, grid=(8, 8, 8))
    s.order = 2
    with pytest.raises(engine.FeError) as ei:
        engine.Box(s)
    assert ei.value.code == engine.FE_ERR_ARG


def test_no_cpu_fallback_without_device(lib):
    """With no usable GPU the engine fails loudly instead of computing on the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(20, L=12.0, seed=1, grid=(8, 8, 8))
    with pytest.raises(engine.FeError) as ei:
        engine.Box(s)
    assert ei.value.code == engine.FE_ERR_CUDA


def test_water_box_recipe():
    from thecodecombo_7_gb300 import systems
    s = systems.water_box(1365, density=0.1, seed=3)
    assert s.n == 4095
    assert abs(s.L[0] - 34.4683) < 1e-3 and s.grid == (32, 32, 32)
    assert abs(s.q.sum()) < 1e-12
    o = s.pos[0::3]
    d = o[:, None, :] - o[None, :, :]
    d -= s.L * np.rint(d / s.L)
    r = np.sqrt((d ** 2).sum(-1)) + np.eye(len(o)) * 100
    assert r.min() >= 2.6
    oh = s.pos[1::3] - s.pos[0::3]
    oh -= s.L * np.rint(oh / s.L)
    np.testing.assert_allclose(np.linalg.norm(oh, axis=1), 1.0, atol=1e-12)
    assert np.all(np.abs(s.pos) <= s.L / 2)
    p = (s.vel * s.mass[:, None]).sum(0)
    np.testing.assert_allclose(p, 0.0, atol=1e-9)
    assert systems.fft_friendly(97) == 100 and systems.fft_friendly(96) == 96
    assert systems.fft_friendly_below(99) == 96 and systems.fft_friendly_below(34) == 32


@pytest.mark.skipif(O.reference_dir() is None, reason="reference sources not present")
def test_reference_program_links_against_the_engine(lib):
    """The reference's own program, with the replaced routines taken out of
    its SRCS and the drop-in shim added, compiles and links against libfe.so
    in both forms (MD with SPME, Monte Carlo with classic Ewald); the
    replaced symbols resolve to the shim."""
    script = os.path.join(ROOT, "thecodecombo_7_gb300", "dropin", "build_reference_with_engine.sh")
    subprocess.check_call(["sh", script], stdout=subprocess.DEVNULL,
                          env=dict(os.environ, REF_DIR=O.reference_dir()))
    out = os.path.join(ROOT, "thecodecombo_7_gb300", "dropin", "_build")
    forms = {
        "md": ("nblist", "forces", "cnonbondnl", "pme_calc", "pme_force", "charge_grid", "pme_init",
               "pme_clean", "fillspline", "integrate_vverlet", "integrate_nhc", "pbc_all",
               "kinet", "drift", "isokin", "swap_box", "force_short", "force_long",
               "integrate_mts", "integrate_mts_nhc"),
        "mc": ("forces_mc", "enbnd_mc", "ewald_kspace_mc", "ewald_rspace_mc", "nblist_pivot",
               "drift"),
    }
    for form, names in forms.items():
        assert os.path.exists(os.path.join(out, form, "spidey_gpu")), form
        obj = os.path.join(out, form, "fe_dropin.o")
        syms = subprocess.run(["nm", "--defined-only", obj], capture_output=True, text=True).stdout
        for name in names:
            assert re.search(rf"\bT {name}\b", syms), (form, name)
        need = subprocess.run(["nm", "-u", obj], capture_output=True, text=True).stdout
        assert "fe_box_create" in need
    need_md = subprocess.run(["nm", "-u", os.path.join(out, "md", "fe_dropin.o")],
                             capture_output=True, text=True).stdout
    assert "fe_forces" in need_md and "fe_drift" in need_md and "fe_bspline" in need_md
    assert "fe_integrate_mts" in need_md and "fe_set_forces_mts" in need_md
    need_mc = subprocess.run(["nm", "-u", os.path.join(out, "mc", "fe_dropin.o")],
                             capture_output=True, text=True).stdout
    assert "fe_mc_delta_terms" in need_mc and "fe_mc_site_energy" in need_mc
