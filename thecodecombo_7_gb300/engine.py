"""Host-side mirror of the reference's hot-path interface over libfe.so.

``Box`` wraps one fe_box (the reference's ``ibox``) and exposes the
reference's routine names -- nblist, forces, cnonbondnl, charge_grid,
pme_calc, pbc_all, kinet, integrate_vverlet, integrate_nhc -- plus the
production step loop (run_md) and the classic-Ewald MC energy path.  Every
call goes through the C ABI of include/fe.h; there is no CPU fallback: without
the compiled library or a CUDA device the constructor raises.

Errors: the reference prints and exit()s (nblist.c:185-197 exit 5,
ewald.c:185-194 exit 20); here the same conditions raise ``FeError`` carrying
the same code.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfe.so")

FE_OK = 0
FE_ERR_CUDA = 1
FE_ERR_ARG = 2
FE_ERR_OVERFLOW = 5
FE_ERR_CHARGE = 20
FE_ERR_STATE = 30
FE_ERR_DEVICE = 31
FE_ERR_SIZE = 32
FE_PREC_FP64 = 0
FE_PREC_MIXED = 1
EN_KEYS = ["kinet", "bond", "bend", "nbond", "nbonds", "coulomb", "rewald", "rewalds",
           "kewald", "sewald", "iewald", "tewald", "urey", "tors", "impr"]
FE_EN_COUNT = len(EN_KEYS)

# symbols of include/fe.h (checked by the tests against the built library)
EXPORTS = [
    "fe_box_create", "fe_box_destroy", "fe_box_set_stream", "fe_last_error", "fe_abi_version",
    "fe_set_positions", "fe_get_positions", "fe_set_positions_nopbc", "fe_get_positions_nopbc",
    "fe_set_velocities", "fe_get_velocities", "fe_get_forces", "fe_set_forces", "fe_set_nhc_state",
    "fe_get_nhc_state", "fe_nblist", "fe_nblist_download", "fe_forces", "fe_cnonbondnl",
    "fe_pme_calc", "fe_charge_grid", "fe_get_charge_grid", "fe_bonded", "fe_zero_forces",
    "fe_pbc_all", "fe_kinet", "fe_integrate_vverlet", "fe_integrate_nhc", "fe_run_md",
    "fe_force_short", "fe_force_long", "fe_integrate_mts", "fe_get_forces_mts",
    "fe_set_forces_mts", "fe_integrate_mts_nhc", "fe_integrate_vverlet_host", "fe_pme_force",
    "fe_box_set_lj_form",
    "fe_mc_setup", "fe_mc_delta", "fe_mc_accept", "fe_mc_kspace_energy",
    "fe_time_kernel", "fe_step_launches", "fe_list_stats", "fe_inner_list_stats", "fe_nl_check",
    "fe_ewald_kspace_energy_noalloc",
    "fe_batch_create", "fe_batch_destroy", "fe_batch_run", "fe_batch_state",
    "fe_batch_step_launches", "fe_batch_get_stream",
    "fe_mc_chains_setup", "fe_mc_chains_run", "fe_mc_chains_state",
    "fe_mc_chains_kspace_energy", "fe_mc_chains_log",
    "fe_mlp_create", "fe_mlp_destroy", "fe_mlp_param_count", "fe_mlp_set_params",
    "fe_mlp_get_params", "fe_mlp_grad", "fe_mlp_train", "fe_tc_gemm_bf16",
    "fe_mc_chains_collect", "fe_mc_chains_samples", "fe_mc_chains_train_surrogate",
    "fe_mc_chains_set_surrogate", "fe_mc_chains_set_mode", "fe_mc_chains_stats",
    "fe_go_create", "fe_go_destroy", "fe_go_run", "fe_go_forces", "fe_go_state",
    "fe_go_get_stream", "fe_go_layout", "fe_go_set_reference_form", "fe_autotune", "fe_pipe_peak", "fe_pair_counts",
    "fe_mc_delta_terms", "fe_mc_site_energy", "fe_drift", "fe_box_set_temperature",
    "fe_bspline", "fe_batch_set_fused", "fe_set_ureys", "fe_set_torsions", "fe_set_impropers",
    "fe_get_torsion_angles", "fe_bonded_ext",
]
FE_KERNEL_PAIR = 0
FE_KERNEL_SPREAD = 1
FE_KERNEL_LIST = 2


class FeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[fe error {code}] {msg}")
        self.code = code


class FeMdIo(C.Structure):
    """fe_md_io: the host arrays of one fe_integrate_vverlet_host call."""
    _fields_ = [("atoms", C.c_void_p), ("atoms_stride", C.c_size_t), ("atoms_off", C.c_size_t),
                ("nopbc", C.c_void_p), ("nopbc_stride", C.c_size_t), ("nopbc_off", C.c_size_t),
                ("vv", C.c_void_p), ("uu", C.c_void_p), ("ff", C.c_void_p)]


class FeBoxParams(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("ntypes", C.c_int), ("L", C.c_double * 3), ("rc", C.c_double),
        ("rclist", C.c_double), ("rclist_ew", C.c_double), ("kappa", C.c_double),
        ("epsRF", C.c_double), ("dt", C.c_double), ("T", C.c_double), ("grid", C.c_int * 3),
        ("order", C.c_int), ("r_switch", C.c_double), ("precision", C.c_int),
        ("max_neighbors", C.c_int), ("device", C.c_int),
        ("q", C.c_void_p), ("mass", C.c_void_p), ("type", C.c_void_p),
        ("lj_eps", C.c_void_p), ("lj_sig", C.c_void_p),
        ("nbond", C.c_int), ("bond_ab", C.c_void_p), ("bond_req", C.c_void_p),
        ("bond_k", C.c_void_p),
        ("nbend", C.c_int), ("bend_abc", C.c_void_p), ("bend_theta0", C.c_void_p),
        ("bend_k", C.c_void_p),
        ("nexcl", C.c_int), ("excl_ab", C.c_void_p), ("excl_flag", C.c_void_p),
        ("nhc_M", C.c_int), ("nhc_Q", C.c_double), ("nfree", C.c_double),
    ]


class FeGoParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("sigma_rep", C.c_double), ("rc_rep", C.c_double),
                ("k_bond", C.c_double), ("r_bond", C.c_double), ("mass", C.c_double),
                ("gamma", C.c_double), ("dt", C.c_double), ("min_sep", C.c_int),
                ("device", C.c_int)]


_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load libfe.so; raises if it has not been built (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FeError(FE_ERR_CUDA, f"{path} not built: run __graft_entry__.build() "
                      "or python -m thecodecombo_7_gb300.build")
    lib = C.CDLL(path)
    lib.fe_last_error.restype = C.c_char_p
    lib.fe_box_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(FeBoxParams)]
    lib.fe_box_destroy.argtypes = [C.c_void_p]
    lib.fe_box_destroy.restype = None
    for name in EXPORTS:
        fn = getattr(lib, name)
        if name not in ("fe_last_error", "fe_box_destroy", "fe_box_create",
                        "fe_batch_destroy", "fe_mlp_destroy", "fe_go_destroy"):
            fn.restype = C.c_int
    lib.fe_go_destroy.argtypes = [C.c_void_p]
    lib.fe_go_destroy.restype = None
    lib.fe_go_create.argtypes = [C.POINTER(C.c_void_p), C.c_int] + [C.c_void_p] * 7 + [
        C.POINTER(FeGoParams), C.c_uint64]
    lib.fe_go_run.argtypes = [C.c_void_p, C.c_int64, C.c_int]
    lib.fe_mlp_destroy.argtypes = [C.c_void_p]
    lib.fe_mlp_destroy.restype = None
    lib.fe_mlp_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_uint64]
    lib.fe_mlp_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                C.c_void_p, C.c_void_p]
    lib.fe_mlp_train.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int,
                                 C.c_float, C.c_uint64, C.c_void_p]
    lib.fe_tc_gemm_bf16.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_int, C.c_int]
    lib.fe_batch_destroy.argtypes = [C.c_void_p]
    lib.fe_batch_destroy.restype = None
    lib.fe_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_int, C.c_uint64]
    lib.fe_batch_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_long, C.c_int]
    lib.fe_mc_chains_setup.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                       C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_uint64, C.c_int]
    lib.fe_mc_chains_run.argtypes = [C.c_void_p, C.c_int64]
    lib.fe_mc_chains_log.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    lib.fe_mc_chains_collect.argtypes = [C.c_void_p, C.c_int64]
    lib.fe_mc_chains_samples.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    lib.fe_mc_chains_train_surrogate.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                                 C.c_float, C.c_uint64, C.c_void_p]
    lib.fe_mc_chains_set_surrogate.argtypes = [C.c_void_p, C.c_void_p]
    lib.fe_mc_chains_set_mode.argtypes = [C.c_void_p, C.c_int]
    lib.fe_mc_chains_stats.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    _lib = lib
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Box:
    """One simulation box resident on the GPU (the reference's ``ibox``)."""

    def __init__(self, sysm, precision: int = FE_PREC_FP64, device: int = 0,
                 max_neighbors: int = 0):
        self.lib = load_library()
        self.sysm = sysm
        eps, sig = sysm.lj_tables()
        k = dict(q=_c(sysm.q, np.float64), mass=_c(sysm.mass, np.float64),
                 type=_c(sysm.type, np.int32), eps=_c(eps, np.float64), sig=_c(sig, np.float64),
                 bond_ab=_c(sysm.bonds, np.int32), bond_req=_c(sysm.bond_req, np.float64),
                 bond_k=_c(sysm.bond_k, np.float64), bend_abc=_c(sysm.bends, np.int32),
                 bend_t0=_c(sysm.bend_theta0, np.float64), bend_k=_c(sysm.bend_k, np.float64),
                 excl_ab=_c(sysm.excl, np.int32), excl_flag=_c(sysm.excl_flag, np.int32))
        self._keep = k
        p = FeBoxParams()
        p.n = sysm.n
        p.ntypes = sysm.ntypes
        p.L[:] = [float(x) for x in sysm.L]
        p.rc, p.rclist, p.rclist_ew = sysm.rc, sysm.rclist, sysm.rclist_ew
        p.kappa, p.epsRF, p.dt, p.T = sysm.kappa, sysm.epsRF, sysm.dt, sysm.T
        p.grid[:] = list(sysm.grid)
        p.order = sysm.order
        p.r_switch = sysm.r_switch
        p.precision = precision
        p.max_neighbors = max_neighbors
        p.device = device
        p.q, p.mass, p.type = _p(k["q"]), _p(k["mass"]), _p(k["type"])
        p.lj_eps, p.lj_sig = _p(k["eps"]), _p(k["sig"])
        p.nbond = k["bond_ab"].shape[0]
        p.bond_ab, p.bond_req, p.bond_k = _p(k["bond_ab"]), _p(k["bond_req"]), _p(k["bond_k"])
        p.nbend = k["bend_abc"].shape[0]
        p.bend_abc, p.bend_theta0, p.bend_k = _p(k["bend_abc"]), _p(k["bend_t0"]), _p(k["bend_k"])
        p.nexcl = k["excl_ab"].shape[0]
        p.excl_ab, p.excl_flag = _p(k["excl_ab"]), _p(k["excl_flag"])
        p.nhc_M = sysm.nhc_M
        p.nhc_Q = sysm.nhc_Q
        p.nfree = 0.0
        self.params = p
        h = C.c_void_p()
        self.lib.fe_box_set_temperature.argtypes = [C.c_void_p, C.c_double]
        self._check(self.lib.fe_box_create(C.byref(h), C.byref(p)))
        self.h = h
        self.n = sysm.n
        self.set_positions(sysm.pos, nopbc=True)
        self.set_velocities(sysm.vel)
        if getattr(sysm, "has_ext_bonded", False):
            self.set_ext_bonded(sysm)

    # ---- plumbing ----
    def _check(self, rc):
        if rc != FE_OK:
            raise FeError(rc, self.lib.fe_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fe_box_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr: int | None):
        self._check(self.lib.fe_box_set_stream(self.h, C.c_void_p(stream_ptr or 0)))

    # ---- state ----
    def set_positions(self, pos, nopbc=False):
        a = _c(pos, np.float64).reshape(-1, 3)
        self._check(self.lib.fe_set_positions(self.h, _p(a), C.c_size_t(24), C.c_size_t(0),
                                              int(nopbc)))

    def set_positions_records(self, records: np.ndarray, stride: int, off_x: int, nopbc=False):
        """Positions straight from reference-layout records (e.g. struct atoms)."""
        self._check(self.lib.fe_set_positions(self.h, _p(records), C.c_size_t(stride),
                                              C.c_size_t(off_x), int(nopbc)))

    def get_positions(self):
        out = np.empty((self.n, 3))
        self._check(self.lib.fe_get_positions(self.h, _p(out), C.c_size_t(24), C.c_size_t(0)))
        return out

    def get_positions_records(self, records: np.ndarray, stride: int, off_x: int):
        self._check(self.lib.fe_get_positions(self.h, _p(records), C.c_size_t(stride),
                                              C.c_size_t(off_x)))

    def set_positions_nopbc_array(self, pos):
        """Unwrapped positions (atnopbc) from an n x 3 array."""
        a = _c(pos, np.float64).reshape(-1, 3)
        self._check(self.lib.fe_set_positions_nopbc(self.h, _p(a), C.c_size_t(24),
                                                    C.c_size_t(0)))

    def get_positions_nopbc(self):
        out = np.empty((self.n, 3))
        self._check(self.lib.fe_get_positions_nopbc(self.h, _p(out), C.c_size_t(24),
                                                    C.c_size_t(0)))
        return out

    def set_velocities(self, vv, uu=None):
        v = _c(vv, np.float64).reshape(-1, 3)
        u = v if uu is None else _c(uu, np.float64).reshape(-1, 3)
        self._check(self.lib.fe_set_velocities(self.h, _p(v), _p(u)))

    def get_velocities(self):
        v = np.empty((self.n, 3))
        u = np.empty((self.n, 3))
        self._check(self.lib.fe_get_velocities(self.h, _p(v), _p(u)))
        return v, u

    def get_forces(self):
        f = np.empty((self.n, 3))
        self._check(self.lib.fe_get_forces(self.h, _p(f)))
        return f

    def set_forces(self, ff):
        f = _c(ff, np.float64).reshape(-1, 3)
        self._check(self.lib.fe_set_forces(self.h, _p(f)))

    def get_nhc_state(self):
        z = np.empty((max(self.sysm.nhc_M, 1), 3))
        self._check(self.lib.fe_get_nhc_state(self.h, _p(z)))
        return z

    def set_nhc_state(self, zeta):
        z = _c(zeta, np.float64)
        self._check(self.lib.fe_set_nhc_state(self.h, _p(z)))

    # ---- the reference's routines ----
    def nblist(self):
        self._check(self.lib.fe_nblist(self.h))

    def nblist_download(self):
        cnt = np.empty(self.n, np.int32)
        tot = C.c_int64()
        self._check(self.lib.fe_nblist_download(self.h, _p(cnt), None, None, C.c_int64(0),
                                                C.byref(tot)))
        idx = np.empty(max(tot.value, 1), np.int32)
        flg = np.empty(max(tot.value, 1), np.int32)
        self._check(self.lib.fe_nblist_download(self.h, _p(cnt), _p(idx), _p(flg),
                                                C.c_int64(idx.size), C.byref(tot)))
        return cnt, idx[:tot.value], flg[:tot.value]

    def forces(self):
        en = np.empty(FE_EN_COUNT)
        self._check(self.lib.fe_forces(self.h, _p(en)))
        return dict(zip(EN_KEYS, en.tolist()))

    def set_lj_form(self, form):
        """The pair loop's LJ form: 0 the reference's default, 2 its BGO
        build (eps [13 (R/r)^12 - 18 (R/r)^10 + 4 (R/r)^6])."""
        self._check(self.lib.fe_box_set_lj_form(self.h, int(form)))

    def pme_force(self):
        """pme_force (pme_calc.c:122): reciprocal forces from the grid of the
        last pme_calc, accumulated into ff."""
        self._check(self.lib.fe_pme_force(self.h))

    def cnonbondnl(self):
        e = np.empty(8)
        self._check(self.lib.fe_cnonbondnl(self.h, _p(e)))
        return e

    def pme_calc(self):
        e = np.empty(3)
        self._check(self.lib.fe_pme_calc(self.h, _p(e)))
        return e

    def charge_grid(self):
        self._check(self.lib.fe_charge_grid(self.h))
        g = np.empty(int(np.prod(self.sysm.grid)))
        self._check(self.lib.fe_get_charge_grid(self.h, _p(g)))
        return g.reshape(self.sysm.grid)

    def bonded(self):
        e = np.empty(2)
        self._check(self.lib.fe_bonded(self.h, _p(e)))
        return e

    def set_ext_bonded(self, sysm):
        """Urey-Bradley, proper and improper torsion terms of sysm."""
        ab = _c(sysm.ureys, np.int32)
        self._check(self.lib.fe_set_ureys(self.h, ab.shape[0], _p(ab),
                                          _p(_c(sysm.urey_seq, np.float64)),
                                          _p(_c(sysm.urey_k, np.float64))))
        t = _c(sysm.tors, np.int32)
        self._check(self.lib.fe_set_torsions(self.h, t.shape[0], _p(t),
                                             _p(_c(sysm.tors_kphi, np.float64)),
                                             _p(_c(sysm.tors_nphi, np.float64)),
                                             _p(_c(sysm.tors_delphi, np.float64))))
        m = _c(sysm.impr, np.int32)
        self._check(self.lib.fe_set_impropers(self.h, m.shape[0], _p(m),
                                              _p(_c(sysm.impr_k, np.float64)),
                                              _p(_c(sysm.impr_eq, np.float64))))
        self.ntors = t.shape[0]

    def bonded_ext(self):
        """curey, ctorsion, cimproper energies (forces added into ff)."""
        e = np.empty(3)
        self._check(self.lib.fe_bonded_ext(self.h, _p(e)))
        return e

    def torsion_angles(self):
        tau = np.empty(max(getattr(self, "ntors", 0), 1))
        self._check(self.lib.fe_get_torsion_angles(self.h, _p(tau)))
        return tau[:getattr(self, "ntors", 0)]

    def zero_forces(self):
        self._check(self.lib.fe_zero_forces(self.h))

    def pbc_all(self):
        self._check(self.lib.fe_pbc_all(self.h))

    def kinet(self):
        ken = np.empty(6)
        k = C.c_double()
        self._check(self.lib.fe_kinet(self.h, _p(ken), C.byref(k)))
        return k.value, ken

    def integrate_vverlet(self, vscal=1.0):
        en = np.empty(FE_EN_COUNT)
        self._check(self.lib.fe_integrate_vverlet(self.h, C.c_double(vscal), _p(en)))
        return dict(zip(EN_KEYS, en.tolist()))

    def force_short(self):
        """force_short.c: bonds, bends and Urey-Bradley terms into ff_short
        (and ff); returns the energies."""
        en = np.empty(FE_EN_COUNT)
        self._check(self.lib.fe_force_short(self.h, _p(en)))
        return dict(zip(EN_KEYS, en.tolist()))

    def force_long(self):
        """force_long.c: torsions, impropers and the non-bonded terms with
        SPME into ff_long (and ff); returns the energies."""
        en = np.empty(FE_EN_COUNT)
        self._check(self.lib.fe_force_long(self.h, _p(en)))
        return dict(zip(EN_KEYS, en.tolist()))

    def integrate_mts(self, nshort, vscal=1.0):
        """integrate_mts.c: one RESPA long step of `nshort` short steps."""
        en = np.empty(FE_EN_COUNT)
        self._check(self.lib.fe_integrate_mts(self.h, C.c_double(vscal), int(nshort), _p(en)))
        return dict(zip(EN_KEYS, en.tolist()))

    def integrate_mts_nhc(self, nshort, xrespa=0):
        """integrate_mts_nhc.c: one RESPA long step with the Nose-Hoover chain
        per long step (xrespa 0) or per short step (xrespa 1)."""
        en = np.empty(FE_EN_COUNT)
        self._check(self.lib.fe_integrate_mts_nhc(self.h, int(nshort), int(xrespa), _p(en)))
        return dict(zip(EN_KEYS, en.tolist()))

    def forces_mts(self):
        """(ff_short, ff_long) as two (n, 3) arrays."""
        fs, fl = np.empty((self.n, 3)), np.empty((self.n, 3))
        self._check(self.lib.fe_get_forces_mts(self.h, _p(fs), _p(fl)))
        return fs, fl

    def integrate_vverlet_host(self, pos, pos_nopbc, vv, uu, ff, vscal=1.0):
        """integrate_vverlet with its host state in one call: the five (n, 3)
        float64 arrays are read before the step and overwritten after it
        (one synchronisation when they are in pinned memory)."""
        arrs = (pos, pos_nopbc, vv, uu, ff)
        for a in arrs:
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != 3 * self.n:
                raise ValueError("integrate_vverlet_host needs contiguous float64 (n, 3) arrays")
        io = FeMdIo(pos.ctypes.data, 24, 0, pos_nopbc.ctypes.data, 24, 0, vv.ctypes.data,
                    uu.ctypes.data, ff.ctypes.data)
        en = np.empty(FE_EN_COUNT)
        self._check(self.lib.fe_integrate_vverlet_host(self.h, C.c_double(vscal), C.byref(io),
                                                       _p(en)))
        return dict(zip(EN_KEYS, en.tolist()))

    def integrate_nhc(self, time_step=None):
        ts = self.sysm.dt if time_step is None else time_step
        self._check(self.lib.fe_integrate_nhc(self.h, C.c_double(ts)))

    def run_md(self, nsteps, nlist_freq=None, use_nhc=False, first_step=1, record=True):
        nl = self.sysm.nlist_freq if nlist_freq is None else nlist_freq
        rec = np.empty((max(nsteps, 1), FE_EN_COUNT)) if record else None
        self._check(self.lib.fe_run_md(self.h, int(nsteps), int(nl), int(use_nhc),
                                       C.c_long(first_step), _p(rec) if record else None))
        return rec[:nsteps] if record else None

    def autotune(self):
        """Picks the pair kernel's launch shape for this box (mixed precision);
        returns (warps per block, registers per thread, blocks, us per launch)."""
        ch = np.zeros(3, np.int32)
        us = C.c_double()
        self._check(self.lib.fe_autotune(self.h, _p(ch), C.byref(us)))
        return int(ch[0]), int(ch[1]), int(ch[2]), us.value

    # ---- instrumentation ----
    def time_kernel(self, which=FE_KERNEL_PAIR, reps=20):
        us = C.c_double()
        self._check(self.lib.fe_time_kernel(self.h, int(which), int(reps), C.byref(us)))
        return us.value

    def list_stats(self):
        e, m = C.c_int64(), C.c_int()
        self._check(self.lib.fe_list_stats(self.h, C.byref(e), C.byref(m)))
        return e.value, m.value

    def nl_check(self, lb=0, ub=None):
        """nl_check (nblist.c:607-647): 1 if a site of [lb, ub) moved more than
        (rclist - rc)/4 since the last nblist, else 0."""
        f = C.c_int()
        ub = self.sysm.n if ub is None else ub
        self._check(self.lib.fe_nl_check(self.h, int(lb), int(ub), C.byref(f)))
        return f.value

    def pair_counts(self):
        """FP64 boxes: (half-list entries, evaluated pairs within rc, those
        with LJ, excluded pairs within rc)."""
        v = np.zeros(4, np.int64)
        self._check(self.lib.fe_pair_counts(self.h, _p(v)))
        return tuple(int(x) for x in v)

    def inner_list_stats(self):
        """Mixed mode: (entries, longest row, prunes so far) of the inner list."""
        e, m, p = C.c_int64(), C.c_int(), C.c_int64()
        self._check(self.lib.fe_inner_list_stats(self.h, C.byref(e), C.byref(m), C.byref(p)))
        return e.value, m.value, p.value

    def step_launches(self, use_nhc=False):
        a, b = C.c_int(), C.c_int()
        self._check(self.lib.fe_step_launches(self.h, int(use_nhc), C.byref(a), C.byref(b)))
        return a.value, b.value

    # ---- Monte Carlo energy path ----
    def mc_setup(self, kmax=7, max_k_square=None, rc_ew=None):
        mks = kmax * kmax if max_k_square is None else max_k_square
        rc = self.sysm.rc_ew if rc_ew is None else rc_ew
        self._check(self.lib.fe_mc_setup(self.h, int(kmax), int(mks), C.c_double(rc)))

    def mc_delta(self, lb, ub, new_pos):
        npos = _c(new_pos, np.float64).reshape(-1, 3)
        de = C.c_double()
        parts = np.empty(3)
        self._check(self.lib.fe_mc_delta(self.h, int(lb), int(ub), _p(npos), C.byref(de),
                                         _p(parts)))
        return de.value, parts

    def mc_delta_terms(self, lb, ub, new_pos):
        """Change of the six MC energy terms (reciprocal, LJ, LJ shift,
        real, real shift, intramolecular) for moving [lb, ub) to new_pos."""
        npos = _c(new_pos, np.float64).reshape(-1, 3)
        t = np.empty(6)
        self._check(self.lib.fe_mc_delta_terms(self.h, int(lb), int(ub), _p(npos), _p(t)))
        return t

    def mc_site_energy(self, lb, ub):
        """The six terms of the pairs touching [lb, ub) (whole reciprocal)."""
        t = np.empty(6)
        self._check(self.lib.fe_mc_site_energy(self.h, int(lb), int(ub), _p(t)))
        return t

    def drift(self):
        """drift.c:21: remove the net momentum from the velocities."""
        self._check(self.lib.fe_drift(self.h))

    def set_temperature(self, T):
        self._check(self.lib.fe_box_set_temperature(self.h, C.c_double(T)))

    def mc_accept(self):
        self._check(self.lib.fe_mc_accept(self.h))

    def mc_kspace_energy(self):
        e = C.c_double()
        self._check(self.lib.fe_mc_kspace_energy(self.h, C.byref(e)))
        return e.value

    # ---- Monte Carlo chains resident on the device ----
    def mc_chains_setup(self, nchains=1, mol_first=None, kmax=7, max_k_square=None, rc_ew=None,
                        T=None, delta=0.6, rot_max=0.2617993877991494, p_rot=0.5, seed=1,
                        log_cap=0):
        s = self.sysm
        if mol_first is None:  # 3-site molecules in order
            mol_first = np.arange(0, s.n + 1, 3, dtype=np.int32)
        mf = _c(mol_first, np.int32)
        mks = kmax * kmax if max_k_square is None else max_k_square
        self._mc_nmol = len(mf) - 1
        self._check(self.lib.fe_mc_chains_setup(
            self.h, int(nchains), _p(mf), self._mc_nmol, int(kmax), int(mks),
            float(s.rc_ew if rc_ew is None else rc_ew), float(s.T if T is None else T),
            float(delta), float(rot_max), float(p_rot), C.c_uint64(seed), int(log_cap)))

    def mc_chains_run(self, nmoves):
        self._check(self.lib.fe_mc_chains_run(self.h, int(nmoves)))

    def mc_chains_state(self, chain=0):
        xyz = np.empty((self.sysm.n, 3))
        mv, acc = C.c_int64(), C.c_int64()
        self._check(self.lib.fe_mc_chains_state(self.h, int(chain), _p(xyz), C.byref(mv),
                                                C.byref(acc)))
        return xyz, mv.value, acc.value

    def mc_chains_kspace_energy(self, chain=0):
        e = C.c_double()
        self._check(self.lib.fe_mc_chains_kspace_energy(self.h, int(chain), C.byref(e)))
        return e.value

    def mc_chains_collect(self, per_chain):
        self._check(self.lib.fe_mc_chains_collect(self.h, int(per_chain)))

    def mc_chains_samples(self):
        cnt = C.c_int64()
        self._check(self.lib.fe_mc_chains_samples(self.h, None, 0, C.byref(cnt)))
        out = np.zeros((cnt.value, 129), np.float32)
        self._check(self.lib.fe_mc_chains_samples(self.h, _p(out), cnt.value, C.byref(cnt)))
        return out[:cnt.value]

    def mc_chains_train_surrogate(self, mlp, epochs=20, batch=512, lr=1e-3, seed=1):
        hist = np.empty(epochs, np.float32)
        self._check(self.lib.fe_mc_chains_train_surrogate(self.h, mlp.h, int(epochs), int(batch),
                                                          C.c_float(lr), C.c_uint64(seed),
                                                          _p(hist)))
        return hist

    def mc_chains_set_surrogate(self, mlp):
        self._check(self.lib.fe_mc_chains_set_surrogate(self.h, mlp.h))

    def mc_chains_set_mode(self, mode):
        self._check(self.lib.fe_mc_chains_set_mode(self.h, int(mode)))

    def mc_chains_stats(self, chain=0):
        v = np.zeros(4, np.int64)
        self._check(self.lib.fe_mc_chains_stats(self.h, int(chain), _p(v)))
        return dict(moves=int(v[0]), accepted=int(v[1]), stage1=int(v[2]), kspace=int(v[3]))

    def mc_chains_log(self, cap):
        rec = np.zeros((cap, 12))
        fx = np.zeros((cap, 8, 3), np.uint32)
        cnt = C.c_int64()
        self._check(self.lib.fe_mc_chains_log(self.h, _p(rec), _p(fx), int(cap), C.byref(cnt)))
        return rec[:cnt.value], fx[:cnt.value]


class Batch:
    """Several boxes stepped together in one CUDA graph per step, with replica
    exchange on the device (repexch.c:139-305, swap_box.c:5-86).

    Slot s starts at box s and its temperature ``boxes[s].sysm.T``; an
    accepted exchange swaps the slots (temperature and Nose-Hoover chain
    state) of two boxes and rescales their velocities as swap_box does.
    """

    def __init__(self, boxes, seed: int = 1):
        self.lib = load_library()
        self.boxes = list(boxes)
        arr = (C.c_void_p * len(self.boxes))(*[b.h for b in self.boxes])
        h = C.c_void_p()
        rc = self.lib.fe_batch_create(C.byref(h), arr, len(self.boxes), C.c_uint64(seed))
        if rc != FE_OK:
            raise FeError(rc, self.lib.fe_last_error().decode())
        self.h = h

    def _check(self, rc):
        if rc != FE_OK:
            raise FeError(rc, self.lib.fe_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fe_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, nsteps, nlist_freq=10, swap_freq=0, first_step=1, use_nhc=True):
        self._check(self.lib.fe_batch_run(self.h, int(nsteps), int(nlist_freq), int(swap_freq),
                                          int(first_step), int(use_nhc)))

    def state(self):
        R = len(self.boxes)
        slot = np.empty(R, np.int32)
        T = np.empty(R)
        acc = np.empty(R, np.int64)
        att = np.empty(R, np.int64)
        n = C.c_uint64()
        self._check(self.lib.fe_batch_state(self.h, _p(slot), _p(T), _p(acc), _p(att),
                                            C.byref(n)))
        return dict(slot_box=slot, T_box=T, accepted=acc[:R - 1], attempted=att[:R - 1],
                    attempts=n.value)

    def step_launches(self):
        v = np.empty(4, np.int32)
        self._check(self.lib.fe_batch_step_launches(self.h, _p(v)))
        return v.tolist()

    def set_fused(self, on: bool):
        """All boxes per kernel launch (True, the default where allowed) or
        one graph branch per box (False)."""
        self._check(self.lib.fe_batch_set_fused(self.h, int(on)))

    def stream(self) -> int:
        """cudaStream_t (as an integer) the step graphs run on."""
        s = C.c_void_p()
        self._check(self.lib.fe_batch_get_stream(self.h, C.byref(s)))
        return s.value or 0


def pipe_peak(which: int, device: int = 0) -> float:
    """Measured FP32 FMA (which=0) or FP64 FMA (1) TFLOP/s, or ex2.approx
    Tera-ops/s (2), of the device."""
    lib = load_library()
    v = C.c_double()
    rc = lib.fe_pipe_peak(int(device), int(which), C.byref(v))
    if rc != FE_OK:
        raise FeError(rc, lib.fe_last_error().decode())
    return v.value


def tc_gemm_bf16(A_bits, B_bits, bias=None):
    """D = A B^T (+ bias) on the tensor cores; A (M x K), B (N x K) uint16 bf16 bits."""
    lib = load_library()
    A = _c(A_bits, np.uint16)
    B = _c(B_bits, np.uint16)
    M, K = A.shape
    N = B.shape[0]
    D = np.empty((M, N), np.float32)
    bb = _c(bias, np.float32) if bias is not None else None
    rc = lib.fe_tc_gemm_bf16(_p(A), _p(B), _p(bb) if bb is not None else None, _p(D), M, N, K)
    if rc != FE_OK:
        raise FeError(rc, lib.fe_last_error().decode())
    return D


class Mlp:
    """The Monte Carlo surrogate network (tensor-core training kernels)."""

    N_IN = 64

    def __init__(self, device: int = 0, seed: int = 1):
        self.lib = load_library()
        h = C.c_void_p()
        self._check(self.lib.fe_mlp_create(C.byref(h), int(device), C.c_uint64(seed)))
        self.h = h
        self.n_params = self.lib.fe_mlp_param_count()

    def _check(self, rc):
        if rc != FE_OK:
            raise FeError(rc, self.lib.fe_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fe_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        P = np.empty(self.n_params, np.float32)
        mean = np.empty(self.N_IN, np.float32)
        istd = np.empty(self.N_IN, np.float32)
        self._check(self.lib.fe_mlp_get_params(self.h, _p(P), _p(mean), _p(istd)))
        return P, mean, istd

    def set_params(self, P, mean=None, istd=None):
        P = _c(P, np.float32)
        m = _c(mean, np.float32) if mean is not None else None
        s = _c(istd, np.float32) if istd is not None else None
        self._check(self.lib.fe_mlp_set_params(self.h, _p(P), _p(m) if m is not None else None,
                                               _p(s) if s is not None else None))

    def grad(self, data, y):
        data = _c(data, np.float32)
        y = _c(y, np.float32)
        B = data.shape[0]
        G = np.empty(self.n_params, np.float32)
        out = np.empty(2 * B, np.float32)
        loss = C.c_float()
        self._check(self.lib.fe_mlp_grad(self.h, _p(data), _p(y), B, _p(G), C.byref(loss),
                                         _p(out)))
        return loss.value, G, out

    def train(self, data, y, epochs=10, batch=256, lr=1e-3, seed=1):
        data = _c(data, np.float32)
        y = _c(y, np.float32)
        hist = np.empty(epochs, np.float32)
        self._check(self.lib.fe_mlp_train(self.h, _p(data), _p(y), data.shape[0], int(epochs),
                                          int(batch), C.c_float(lr), C.c_uint64(seed),
                                          _p(hist)))
        return hist


class GoBatch:
    """Replicas of Go-model chains with Langevin dynamics and replica exchange
    on the device (one persistent launch per exchange segment)."""

    def __init__(self, g, device: int = 0, seed: int = 1):
        self.lib = load_library()
        self.g = g
        self._keep = dict(nb=_c(g.nbeads, np.int32), pos=_c(g.pos, np.float64),
                          vel=_c(g.vel, np.float64), ns=_c(g.nat_start, np.int32),
                          nj=_c(g.nat_j, np.int32), r0=_c(g.nat_r0, np.float64),
                          T=_c(g.T, np.float64))
        k = self._keep
        p = FeGoParams(g.eps, g.sigma_rep, g.rc_rep, g.k_bond, g.r_bond, g.mass, g.gamma, g.dt,
                       g.min_sep, device)
        h = C.c_void_p()
        rc = self.lib.fe_go_create(C.byref(h), len(g.nbeads), _p(k["nb"]), _p(k["pos"]),
                                   _p(k["vel"]), _p(k["ns"]), _p(k["nj"]), _p(k["r0"]),
                                   _p(k["T"]), C.byref(p), C.c_uint64(seed))
        if rc != FE_OK:
            raise FeError(rc, self.lib.fe_last_error().decode())
        self.h = h

    def _check(self, rc):
        if rc != FE_OK:
            raise FeError(rc, self.lib.fe_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fe_go_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, nsteps, swap_freq=0):
        self._check(self.lib.fe_go_run(self.h, int(nsteps), int(swap_freq)))

    def forces(self):
        n = int(self.g.nbeads.sum())
        f = np.empty((n, 3))
        e = np.empty(len(self.g.nbeads))
        self._check(self.lib.fe_go_forces(self.h, _p(f), _p(e)))
        return f, e

    def state(self):
        n, R = int(self.g.nbeads.sum()), len(self.g.nbeads)
        pos, vel = np.empty((n, 3)), np.empty((n, 3))
        T, e = np.empty(R), np.empty(R)
        slot = np.empty(R, np.int32)
        acc, att = np.empty(R, np.int64), np.empty(R, np.int64)
        steps = C.c_uint64()
        self._check(self.lib.fe_go_state(self.h, _p(pos), _p(vel), _p(T), _p(e), _p(slot),
                                         _p(acc), _p(att), C.byref(steps)))
        return dict(pos=pos, vel=vel, T=T, epot=e, slot_rep=slot, accepted=acc[:R - 1],
                    attempted=att[:R - 1], steps=steps.value)

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.fe_go_get_stream(self.h, C.byref(s)))
        return s.value or 0

    def set_reference_form(self, d_rep=4.0, rc=12.0, native=None):
        """Switches to the reference's own Go model (cgolik.c) with the bond
        lengths and bend angles of each chain's native structure (`native`,
        (total, 3); default the starting coordinates), non-native cut d_rep
        and native cutoff rc."""
        g = self.g
        st = g.start
        nat = g.pos if native is None else native
        br, bt = np.zeros(int(st[-1])), np.zeros(int(st[-1]))
        for r in range(len(g.nbeads)):
            a, b = int(st[r]), int(st[r + 1])
            x = np.asarray(nat[a:b], np.float64)
            d = x[1:] - x[:-1]
            br[a:b - 1] = np.sqrt((d * d).sum(axis=1))
            u, v = -d[:-1], d[1:]
            bt[a + 1:b - 1] = np.arccos((u * v).sum(axis=1) / np.sqrt(
                (u * u).sum(axis=1) * (v * v).sum(axis=1)))
        self._keep.update(br=br, bt=bt)
        self._check(self.lib.fe_go_set_reference_form(self.h, _p(br), _p(bt), C.c_double(d_rep),
                                                       C.c_double(rc)))

    def layout(self):
        """The launch's load-balance plan: CTAs launched, CTAs resident at
        once, and the CTAs that share each replica's chain."""
        ncta, slots = C.c_int(), C.c_int()
        parts = np.empty(len(self.g.nbeads), np.int32)
        self._check(self.lib.fe_go_layout(self.h, C.byref(ncta), C.byref(slots), _p(parts)))
        return dict(ncta=ncta.value, slots=slots.value, parts=parts)
