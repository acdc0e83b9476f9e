"""ctypes front end of the CPU oracle (fe_oracle.c) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
legs may import this module, and only as the checker or the timed CPU
baseline.  The product path (thecodecombo_7_gb300) never imports it.

Also writes the binary system file read by ref_harness.c (the driver of the
reference's own routines) and reads its tagged output.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
LIB_FAST = os.path.join(HERE, "liboracle_fast.so")
SRC = [os.path.join(HERE, "fe_oracle.c"), os.path.join(HERE, "fe_fft.c")]
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")
REF_BIN_FAST = os.path.join(HERE, "_ref", "ref_harness_fast")
REF_BIN_DLIST = os.path.join(HERE, "_ref", "ref_harness_dlist")
REF_BIN_MC = os.path.join(HERE, "_ref", "ref_harness_mc")
REF_BIN_GO = os.path.join(HERE, "_ref", "ref_harness_go")
REF_BIN_BGO = os.path.join(HERE, "_ref", "ref_harness_bgo")

# strict IEEE: no FMA contraction, no fast-math, so results are reproducible
# on x86-64 and aarch64 alike and match a strict build of the reference
CFLAGS = ["-O2", "-std=gnu99", "-fPIC", "-shared", "-ffp-contract=off",
          "-fno-fast-math"]


# the reference makefile's own optimisation flags (makefile:84-88), used only
# for timing the CPU baseline
CFLAGS_FAST = ["-O3", "-ffast-math", "-funroll-all-loops", "-std=gnu99", "-fPIC", "-shared"]


def build(force: bool = False, fast: bool = False) -> str:
    lib, flags = (LIB_FAST, CFLAGS_FAST) if fast else (LIB, CFLAGS)
    newest = max(os.path.getmtime(p) for p in SRC + [os.path.join(HERE, "fe_oracle.h")])
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        tmp = lib + ".tmp"
        subprocess.check_call(["gcc", *flags, "-o", tmp, *SRC, "-lm"])
        os.replace(tmp, lib)
    return lib


def reference_dir():
    """The reference's source tree: the directory named by the environment
    variable FE_REFERENCE_DIR, or else a checkout named ``reference`` next to
    this repository; None when neither holds its defines.h."""
    cands = [os.environ.get("FE_REFERENCE_DIR"),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.exists(os.path.join(c, "defines.h")):
            return c
    return None


def build_reference() -> bool:
    """Compile the reference's own routines into oracle/_ref (only where the
    reference sources exist).  Returns True when the binary is available."""
    script = os.path.join(HERE, "build_ref.sh")
    ref = reference_dir()
    if ref:
        subprocess.check_call(["sh", script], env=dict(os.environ, REF_DIR=ref))
    return os.path.exists(REF_BIN)


class OrSystem(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("ntypes", C.c_int), ("L", C.c_double * 3),
        ("rc", C.c_double), ("rclist", C.c_double), ("rclist_ew", C.c_double),
        ("kappa", C.c_double), ("epsRF", C.c_double), ("dt", C.c_double),
        ("T", C.c_double), ("grid", C.c_int * 3), ("order", C.c_int),
        ("r_switch", C.c_double),
        ("q", C.c_void_p), ("mass", C.c_void_p), ("type", C.c_void_p),
        ("lj_eps", C.c_void_p), ("lj_sig", C.c_void_p),
        ("nbond", C.c_int), ("bond_ab", C.c_void_p), ("bond_req", C.c_void_p),
        ("bond_k", C.c_void_p),
        ("nbend", C.c_int), ("bend_abc", C.c_void_p),
        ("bend_theta0", C.c_void_p), ("bend_k", C.c_void_p),
        ("nexcl", C.c_int), ("excl_ab", C.c_void_p), ("excl_flag", C.c_void_p),
        ("lj_form", C.c_int),
    ]


class OrEnergy(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "bond", "bend", "nbond", "nbonds", "coulomb", "rewald", "rewalds",
        "kewald", "sewald", "iewald", "tewald")]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


EN_KEYS = ["kinet", "bond", "bend", "nbond", "nbonds", "coulomb", "rewald",
           "rewalds", "kewald", "sewald", "iewald", "tewald"]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """Holds one system's arrays alive and exposes the restated routines."""

    def __init__(self, sysm, fast: bool = False):
        self.lib = C.CDLL(build(fast=fast))
        L = self.lib
        L.or_nblist.restype = C.c_int64
        L.or_ewald_self.restype = C.c_double
        L.or_kinet.restype = C.c_double
        L.or_cbond.restype = C.c_double
        L.or_cbend.restype = C.c_double
        L.or_run_md.restype = C.c_int
        L.or_ewald_kspace_energy.restype = C.c_double
        L.or_mc_delta_energy.restype = C.c_double
        L.or_ewald_nk.restype = C.c_int
        self.sysm = sysm
        eps, sig = sysm.lj_tables()
        self._keep = dict(
            q=np.ascontiguousarray(sysm.q, np.float64),
            mass=np.ascontiguousarray(sysm.mass, np.float64),
            type=np.ascontiguousarray(sysm.type, np.int32),
            eps=np.ascontiguousarray(eps), sig=np.ascontiguousarray(sig),
            bond_ab=np.ascontiguousarray(sysm.bonds, np.int32),
            bond_req=np.ascontiguousarray(sysm.bond_req, np.float64),
            bond_k=np.ascontiguousarray(sysm.bond_k, np.float64),
            bend_abc=np.ascontiguousarray(sysm.bends, np.int32),
            bend_t0=np.ascontiguousarray(sysm.bend_theta0, np.float64),
            bend_k=np.ascontiguousarray(sysm.bend_k, np.float64),
            excl_ab=np.ascontiguousarray(sysm.excl, np.int32),
            excl_flag=np.ascontiguousarray(sysm.excl_flag, np.int32),
        )
        k = self._keep
        s = OrSystem()
        s.n = sysm.n
        s.ntypes = sysm.ntypes
        s.L[:] = [float(x) for x in sysm.L]
        s.rc, s.rclist, s.rclist_ew = sysm.rc, sysm.rclist, sysm.rclist_ew
        s.kappa, s.epsRF, s.dt, s.T = sysm.kappa, sysm.epsRF, sysm.dt, sysm.T
        s.grid[:] = list(sysm.grid)
        s.order = sysm.order
        s.r_switch = sysm.r_switch
        s.q, s.mass, s.type = _p(k["q"]), _p(k["mass"]), _p(k["type"])
        s.lj_eps, s.lj_sig = _p(k["eps"]), _p(k["sig"])
        s.nbond = k["bond_ab"].shape[0]
        s.bond_ab, s.bond_req, s.bond_k = _p(k["bond_ab"]), _p(k["bond_req"]), _p(k["bond_k"])
        s.nbend = k["bend_abc"].shape[0]
        s.bend_abc, s.bend_theta0, s.bend_k = _p(k["bend_abc"]), _p(k["bend_t0"]), _p(k["bend_k"])
        s.nexcl = k["excl_ab"].shape[0]
        s.excl_ab, s.excl_flag = _p(k["excl_ab"]), _p(k["excl_flag"])
        s.lj_form = int(getattr(sysm, "lj_form", 0))
        self.s = s
        self.sp = C.byref(s)

    # ---- neighbour list ----
    def nblist(self, pos, with_ew=False):
        n = self.sysm.n
        pos = np.ascontiguousarray(pos, np.float64)
        cap = n * 800 + 64
        cnt = np.zeros(n, np.int32)
        idx = np.zeros(cap, np.int32)
        flg = np.zeros(cap, np.int32)
        if with_ew:
            cnt_e = np.zeros(n, np.int32)
            idx_e = np.zeros(cap, np.int32)
            flg_e = np.zeros(cap, np.int32)
            tot = self.lib.or_nblist(self.sp, _p(pos), _p(cnt), _p(idx), _p(flg), C.c_int64(cap),
                                     _p(cnt_e), _p(idx_e), _p(flg_e), C.c_int64(cap))
        else:
            tot = self.lib.or_nblist(self.sp, _p(pos), _p(cnt), _p(idx), _p(flg), C.c_int64(cap),
                                     None, None, None, C.c_int64(0))
        if tot < 0:
            raise RuntimeError("oracle neighbour list overflow")
        out = (cnt, idx[:tot].copy(), flg[:tot].copy())
        if with_ew:
            te = int(cnt_e.sum())
            out = out + (cnt_e, idx_e[:te].copy(), flg_e[:te].copy())
        return out

    # ---- forces ----
    def forces(self, pos, lst=None):
        pos = np.ascontiguousarray(pos, np.float64)
        if lst is None:
            lst = self.nblist(pos)
        cnt, idx, flg = lst
        ff = np.zeros((self.sysm.n, 3))
        en = OrEnergy()
        sew = self.lib.or_ewald_self(self.sp)
        self.lib.or_forces(self.sp, _p(pos), _p(cnt), _p(idx), _p(flg), C.c_double(sew),
                           _p(ff), C.byref(en))
        return ff, en.asdict()

    def pair_forces(self, pos, lst):
        pos = np.ascontiguousarray(pos, np.float64)
        cnt, idx, flg = lst
        ff = np.zeros((self.sysm.n, 3))
        e5 = np.zeros(5)
        self.lib.or_cnonbond_pairs(self.sp, _p(pos), _p(cnt), _p(idx), _p(flg), _p(ff), _p(e5))
        return ff, e5

    def pme(self, pos):
        pos = np.ascontiguousarray(pos, np.float64)
        ff = np.zeros((self.sysm.n, 3))
        e3 = np.zeros(3)
        sew = self.lib.or_ewald_self(self.sp)
        self.lib.or_pme_calc(self.sp, _p(pos), C.c_double(sew), _p(ff), _p(e3))
        return ff, e3

    def charge_grid(self, pos):
        pos = np.ascontiguousarray(pos, np.float64)
        g = np.zeros(int(np.prod(self.sysm.grid)))
        self.lib.or_charge_grid(self.sp, _p(pos), _p(g))
        return g.reshape(self.sysm.grid)

    def bspline_moduli(self):
        gx, gy, gz = self.sysm.grid
        bx, by, bz = np.zeros(gx + 2), np.zeros(gy + 2), np.zeros(gz + 2)
        self.lib.or_pme_bspline(self.sp, _p(bx), _p(by), _p(bz))
        return bx[1:gx + 1], by[1:gy + 1], bz[1:gz + 1]

    def bonded(self, pos):
        pos = np.ascontiguousarray(pos, np.float64)
        ff = np.zeros((self.sysm.n, 3))
        eb = self.lib.or_cbond(self.sp, _p(pos), _p(ff))
        ea = self.lib.or_cbend(self.sp, _p(pos), _p(ff))
        return ff, eb, ea

    def bonded_ext(self, pos):
        """Urey-Bradley, torsion and improper terms (curey.c, ctorsion.c,
        cimproper.c): a dict of forces (n, 3) and energies per term and the
        torsion angles."""
        sm = self.sysm
        pos = np.ascontiguousarray(pos, np.float64)
        L = self.lib
        for f in (L.or_curey, L.or_ctorsion, L.or_cimproper):
            f.restype = C.c_double
        k = dict(ab=np.ascontiguousarray(sm.ureys, np.int32),
                 seq=np.ascontiguousarray(sm.urey_seq, np.float64),
                 uk=np.ascontiguousarray(sm.urey_k, np.float64),
                 t=np.ascontiguousarray(sm.tors, np.int32),
                 kp=np.ascontiguousarray(sm.tors_kphi, np.float64),
                 np_=np.ascontiguousarray(sm.tors_nphi, np.float64),
                 dp=np.ascontiguousarray(sm.tors_delphi, np.float64),
                 m=np.ascontiguousarray(sm.impr, np.int32),
                 mk=np.ascontiguousarray(sm.impr_k, np.float64),
                 me=np.ascontiguousarray(sm.impr_eq, np.float64))
        out = {}
        f = np.zeros((sm.n, 3))
        out["e_urey"] = L.or_curey(self.sp, _p(pos), C.c_int(len(k["ab"])), _p(k["ab"]),
                                   _p(k["seq"]), _p(k["uk"]), _p(f))
        out["f_urey"] = f
        f = np.zeros((sm.n, 3))
        tau = np.zeros(max(len(k["t"]), 1))
        out["e_tors"] = L.or_ctorsion(self.sp, _p(pos), C.c_int(len(k["t"])), _p(k["t"]),
                                      _p(k["kp"]), _p(k["np_"]), _p(k["dp"]), _p(f), _p(tau))
        out["f_tors"] = f
        out["tau"] = tau[:len(k["t"])]
        f = np.zeros((sm.n, 3))
        out["e_impr"] = L.or_cimproper(self.sp, _p(pos), C.c_int(len(k["m"])), _p(k["m"]),
                                       _p(k["mk"]), _p(k["me"]), _p(f))
        out["f_impr"] = f
        return out

    def ewald_self(self):
        return self.lib.or_ewald_self(self.sp)

    def kinet(self, vv, uu=None):
        vv = np.ascontiguousarray(vv, np.float64)
        uu = vv if uu is None else np.ascontiguousarray(uu, np.float64)
        ken = np.zeros(6)
        k = self.lib.or_kinet(self.sp, _p(vv), _p(uu), _p(ken))
        return k, ken

    def integrate_nhc(self, vv, uu, zeta, M, Q, nfree=None):
        vv = np.ascontiguousarray(vv, np.float64)
        uu = np.ascontiguousarray(uu, np.float64)
        zeta = np.ascontiguousarray(zeta, np.float64)
        if nfree is None:
            nfree = 3.0 * self.sysm.n - 3.0
        self.lib.or_integrate_nhc(self.sp, C.c_double(self.sysm.dt), C.c_int(M),
                                  C.c_double(Q), C.c_double(nfree), _p(zeta), _p(vv), _p(uu))
        return vv, uu, zeta

    def run_md(self, nsteps, use_nhc=False, pos=None, vel=None, zeta=None, pos_nopbc=None,
               T=None, timed=False):
        """or_run_md from the given state; zeta / pos_nopbc / T (the
        thermostat temperature, sim.T[k]) default to a fresh start.  With
        timed=True the result also holds ``tstamp`` (monotonic seconds at the
        end of each step, index 0 after the initial list and forces)."""
        s = self.sysm
        pos = np.ascontiguousarray(s.pos if pos is None else pos, np.float64).copy()
        nop = pos.copy() if pos_nopbc is None else np.ascontiguousarray(pos_nopbc,
                                                                        np.float64).copy()
        vv = np.ascontiguousarray(s.vel if vel is None else vel, np.float64).copy()
        ff = np.zeros_like(pos)
        M = s.nhc_M
        self.s.T = s.T if T is None else float(T)
        if zeta is None:
            zeta = np.zeros(3 * max(M, 1))
            kT = 1.380662e-23 * s.T * 1e-4
            for i in range(M - 1):  # read_config.c:369-370
                zeta[3 * (i + 1) + 2] = (s.nhc_Q * zeta[3 * i + 1] ** 2 - kT) / s.nhc_Q
        else:
            zeta = np.ascontiguousarray(zeta, np.float64).reshape(-1).copy()
        rec = np.zeros((nsteps + 1, 12))
        ts = np.zeros(nsteps + 1)
        rc = self.lib.or_run_md_timed(self.sp, nsteps, s.nlist_freq, int(use_nhc), M,
                                      C.c_double(s.nhc_Q), _p(pos), _p(nop), _p(vv), _p(ff),
                                      _p(zeta), _p(rec), _p(ts) if timed else None)
        self.s.T = s.T
        if rc != 0:
            raise RuntimeError("oracle md failed (list overflow)")
        out = dict(en=rec, pos=pos, pos_nopbc=nop, vel=vv, force=ff, zeta=zeta.reshape(-1, 3))
        if timed:
            out["tstamp"] = ts
        return out

    def drift(self, vel):
        v = np.ascontiguousarray(vel, np.float64).copy()
        self.lib.or_drift(self.sp, _p(v))
        return v

    # ---- MC ----
    def ewald_kspace_energy(self, pos, kmax=7, max_k_square=49):
        pos = np.ascontiguousarray(pos, np.float64)
        return self.lib.or_ewald_kspace_energy(self.sp, _p(pos), kmax, max_k_square)

    def mc_delta_energy(self, pos, pos_new, lb, ub, kmax=7, max_k_square=49, rc_ew=None):
        pos = np.ascontiguousarray(pos, np.float64)
        pos_new = np.ascontiguousarray(pos_new, np.float64)
        parts = np.zeros(3)
        rc_ew = self.sysm.rc_ew if rc_ew is None else rc_ew
        de = self.lib.or_mc_delta_energy(self.sp, _p(pos), _p(pos_new), lb, ub, kmax,
                                         max_k_square, C.c_double(rc_ew), _p(parts))
        return de, parts


# ---------------------------------------------------------------------------
# binary system file for ref_harness.c, and its tagged output

def write_system_file(path, sysm):
    n = sysm.n
    hi = [n, sysm.ntypes, sysm.bonds.shape[0], sysm.bends.shape[0], sysm.excl.shape[0],
          *sysm.grid, sysm.order, sysm.nhc_M, sysm.nlist_freq, 0]
    hd = [*sysm.L, sysm.rc, sysm.rclist, sysm.rclist_ew, sysm.rc_ew, sysm.kappa,
          sysm.epsRF, sysm.dt, sysm.T, sysm.nhc_Q]
    with open(path, "wb") as f:
        f.write(b"FESYS01\0")
        f.write(struct.pack("<12i", *hi))
        f.write(struct.pack("<12d", *hd))
        for t in range(sysm.ntypes):
            f.write(struct.pack("<2d", sysm.type_eps_kcal[t], sysm.type_rmin_half[t]))
        rec = np.zeros(n, dtype=[("r", "<f8", 5), ("t", "<i4")])
        rec["r"][:, :3] = sysm.pos
        rec["r"][:, 3] = sysm.q
        rec["r"][:, 4] = sysm.mass
        rec["t"] = sysm.type
        f.write(rec.tobytes())
        f.write(np.ascontiguousarray(sysm.vel, "<f8").tobytes())
        b = np.zeros(sysm.bonds.shape[0], dtype=[("ab", "<i4", 2), ("p", "<f8", 2)])
        b["ab"] = sysm.bonds
        b["p"][:, 0] = sysm.bond_req
        b["p"][:, 1] = sysm.bond_k
        f.write(b.tobytes())
        a = np.zeros(sysm.bends.shape[0], dtype=[("abc", "<i4", 3), ("p", "<f8", 2)])
        a["abc"] = sysm.bends
        a["p"][:, 0] = sysm.bend_theta0
        a["p"][:, 1] = sysm.bend_k
        f.write(a.tobytes())
        x = np.zeros((sysm.excl.shape[0], 3), "<i4")
        x[:, :2] = sysm.excl
        x[:, 2] = sysm.excl_flag
        f.write(x.tobytes())
        if getattr(sysm, "has_ext_bonded", False):
            # trailer: Urey-Bradley, torsion and improper records
            f.write(b"FEXT")
            f.write(struct.pack("<3i", len(sysm.ureys), len(sysm.tors), len(sysm.impr)))
            u = np.zeros(len(sysm.ureys), dtype=[("ab", "<i4", 2), ("p", "<f8", 2)])
            u["ab"] = sysm.ureys
            u["p"][:, 0] = sysm.urey_seq
            u["p"][:, 1] = sysm.urey_k
            f.write(u.tobytes())
            t = np.zeros(len(sysm.tors), dtype=[("abcd", "<i4", 4), ("p", "<f8", 18)])
            t["abcd"] = sysm.tors
            t["p"][:, 0:6] = sysm.tors_kphi
            t["p"][:, 6:12] = sysm.tors_nphi
            t["p"][:, 12:18] = sysm.tors_delphi
            f.write(t.tobytes())
            m = np.zeros(len(sysm.impr), dtype=[("abcd", "<i4", 4), ("p", "<f8", 2)])
            m["abcd"] = sysm.impr
            m["p"][:, 0] = sysm.impr_k
            m["p"][:, 1] = sysm.impr_eq
            f.write(m.tobytes())


def read_tagged(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    p = 0
    while p < len(data):
        tag = data[p:p + 16].split(b"\0", 1)[0].decode()
        (nb,) = struct.unpack("<q", data[p + 16:p + 24])
        p += 24
        raw = data[p:p + nb]
        p += nb
        if tag.endswith(("_cnt", "_idx", "_flg")):
            out[tag] = np.frombuffer(raw, "<i4").copy()
        else:
            out[tag] = np.frombuffer(raw, "<f8").copy()
    return out


def run_reference(mode, sysm, workdir, nsteps=None, fast=False, extra=(), binary=None):
    """Run the reference's own routines (oracle/_ref) on sysm; `extra` are
    further integer arguments of the mode (mts: the short steps per long
    step); `binary` another build of the harness (REF_BIN_BGO)."""
    binp = binary or (REF_BIN_FAST if fast else REF_BIN)
    os.makedirs(workdir, exist_ok=True)
    sp = os.path.join(workdir, "system.bin")
    op = os.path.join(workdir, f"out_{mode}.bin")
    write_system_file(sp, sysm)
    cmd = [binp, mode, sp, op] + ([str(nsteps)] if nsteps is not None else [])
    cmd += [str(x) for x in extra]
    subprocess.check_call(cmd)
    return read_tagged(op)


def run_reference_nlcheck(sysm, cases, workdir):
    """The reference's own nl_check (-DDLIST build) on sysm: cases are
    (lb, ub, [(site, dx, dy, dz), ...]) applied to the list-time positions,
    wrapped by the reference's pbc_all, then checked."""
    os.makedirs(workdir, exist_ok=True)
    sp = os.path.join(workdir, "system.bin")
    cp = os.path.join(workdir, "cases.bin")
    op = os.path.join(workdir, "out_nlcheck.bin")
    write_system_file(sp, sysm)
    with open(cp, "wb") as f:
        f.write(struct.pack("<i", len(cases)))
        for lb, ub, moves in cases:
            f.write(struct.pack("<iii", lb, ub, len(moves)))
            for i, dx, dy, dz in moves:
                f.write(struct.pack("<iddd", i, dx, dy, dz))
    subprocess.check_call([REF_BIN_DLIST, "nlcheck", sp, op, cp])
    return read_tagged(op)


def fillspline(order, w):
    """or_fillspline: (array, darray) of order + 1 doubles each."""
    L = C.CDLL(build())
    a = np.zeros(order + 1)
    d = np.zeros(order + 1)
    L.or_fillspline(C.c_int(order), C.c_double(w), _p(a), _p(d))
    return a, d


def run_reference_mc(sysm, kmax, max_k_square, moves, workdir):
    """The reference's classic-Ewald MC energies (-DMC build): enbnd_mc
    (ewald_kspace_mc + ewald_rspace_mc + LJ) of the whole box, then before
    and after each move (lb, ub, new_positions[(ub - lb), 3]), each move undone
    after.  Returns energy[(nmoves + 1), 16] (whole box in [0, :8]; per move
    8 before, 8 after, enbnd_mc's energy[] order) and the move ranges."""
    os.makedirs(workdir, exist_ok=True)
    sp = os.path.join(workdir, "system.bin")
    mp = os.path.join(workdir, "moves.bin")
    op = os.path.join(workdir, "out_mc.bin")
    write_system_file(sp, sysm)
    with open(mp, "wb") as f:
        f.write(struct.pack("<3i", kmax, max_k_square, len(moves)))
        for lb, ub, new in moves:
            f.write(struct.pack("<2i", lb, ub))
            f.write(np.ascontiguousarray(new, "<f8").reshape(ub - lb, 3).tobytes())
    subprocess.check_call([REF_BIN_MC, "mc", sp, op, mp])
    r = read_tagged(op)
    return dict(energy=r["mc_energy"].reshape(len(moves) + 1, 16),
                ranges=r["mc_rng_idx"].reshape(len(moves) + 1, 2), nk=int(r["mc_nk"][0]))


# ---- counter-based random numbers and replica exchange (no system needed) ----

def _lib():
    L = C.CDLL(build())
    L.or_uniform.restype = C.c_double
    L.or_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32]
    L.or_rex_attempt.restype = C.c_int
    L.or_rex_attempt.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                 C.c_uint64, C.c_void_p, C.c_void_p]
    return L


TAG_EXCHANGE = 0x52455831


def philox4x32_10(ctr, key):
    L = _lib()
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    L.or_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def uniform(seed, tag, event, lane):
    return _lib().or_uniform(seed, tag, event, lane)


def rex_attempt(T_slot, potens_box, slot_box, attempt, seed):
    """One exchange attempt; returns (slot_box, vmode, vfac, n_accepted)."""
    L = _lib()
    T = np.ascontiguousarray(T_slot, np.float64)
    U = np.ascontiguousarray(potens_box, np.float64)
    slot = np.ascontiguousarray(slot_box, np.int32).copy()
    R = len(T)
    vmode = np.zeros(R, np.int32)
    vfac = np.zeros(R)
    n = L.or_rex_attempt(R, _p(T), _p(U), _p(slot), attempt, seed, _p(vmode), _p(vfac))
    return slot, vmode, vfac, n


# ---- Go-model chains ----

class OrGoParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("sigma_rep", C.c_double), ("rc_rep", C.c_double),
                ("k_bond", C.c_double), ("r_bond", C.c_double), ("mass", C.c_double),
                ("gamma", C.c_double), ("dt", C.c_double), ("min_sep", C.c_int)]


def _go_params(g):
    return OrGoParams(g.eps, g.sigma_rep, g.rc_rep, g.k_bond, g.r_bond, g.mass, g.gamma, g.dt,
                      g.min_sep)


def _go_lib():
    L = C.CDLL(build())
    L.or_go_forces.restype = C.c_double
    L.or_go_baoab.restype = C.c_double
    return L


def go_forces(g, r, pos=None):
    """(forces (N x 3), potential energy) of replica r of a GoChains."""
    L = _go_lib()
    st = g.start
    a, b = int(st[r]), int(st[r + 1])
    x = np.ascontiguousarray(g.pos[a:b] if pos is None else pos, np.float64)
    f = np.zeros_like(x)
    ns = np.ascontiguousarray(g.nat_start, np.int32)
    nj = np.ascontiguousarray(g.nat_j, np.int32)
    r0 = np.ascontiguousarray(g.nat_r0, np.float64)
    p = _go_params(g)
    e = L.or_go_forces(b - a, _p(x), a, _p(ns), _p(nj), _p(r0), C.byref(p), _p(f))
    return f, e


def go_baoab(g, r, nsteps, seed, step0=0, T=None, pos=None, vel=None):
    """nsteps Langevin steps of replica r; returns (pos, vel, final potential)."""
    L = _go_lib()
    st = g.start
    a, b = int(st[r]), int(st[r + 1])
    x = np.ascontiguousarray(g.pos[a:b] if pos is None else pos, np.float64).copy()
    v = np.ascontiguousarray(g.vel[a:b] if vel is None else vel, np.float64).copy()
    ns = np.ascontiguousarray(g.nat_start, np.int32)
    nj = np.ascontiguousarray(g.nat_j, np.int32)
    r0 = np.ascontiguousarray(g.nat_r0, np.float64)
    p = _go_params(g)
    e = L.or_go_baoab(b - a, _p(x), _p(v), a, _p(ns), _p(nj), _p(r0), C.byref(p),
                      C.c_double(g.T[r] if T is None else T), C.c_uint64(seed),
                      C.c_uint64(step0), int(nsteps))
    return x, v, e


def nl_check(pos, pos0, L, rclist, rc, lb=0, ub=None):
    """nl_check (nblist.c:607-647, DLIST), restated: 1 if any site of
    [lb, ub) has moved more than (rclist - rc)/4 from pos0 along one axis or
    in distance; per axis |d| > L/2 subtracts L, as the reference does."""
    ub = len(pos) if ub is None else ub
    L = np.asarray(L, float)
    h = L / 2.0
    rcut = (rclist - rc) / 4.0
    for i in range(lb, ub):
        d = np.abs(np.asarray(pos[i], float) - np.asarray(pos0[i], float))
        d = np.where(d > h, d - L, d)
        if (d > rcut).any():
            return 1
        if d[0] * d[0] + d[1] * d[1] + d[2] * d[2] > rcut * rcut:
            return 1
    return 0


# ---- the reference's own Go model (cgolik.c) ----

class OrGoHcParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("d_rep", C.c_double), ("rc", C.c_double)]


def go_native_geometry(g, r):
    """Bond lengths (N-1) and bend angles (N-2) of replica r's native
    structure (its starting coordinates), as set_go_params takes them
    (read_golik.c:300-355 with GOBT)."""
    a, b = int(g.start[r]), int(g.start[r + 1])
    x = np.asarray(g.pos[a:b], np.float64)
    d = x[1:] - x[:-1]
    r0 = np.sqrt((d * d).sum(axis=1))
    u, v = -d[:-1], d[1:]
    cos = (u * v).sum(axis=1) / np.sqrt((u * u).sum(axis=1) * (v * v).sum(axis=1))
    return r0, np.arccos(cos)


def go_hc_terms(g, r, hc, pos=None):
    """The four terms of the reference's Go model (or_go_hc_term) of replica
    r: dict of forces (N, 3) and energies per term (pairs: shifted, and
    e_nb2 = (unshifted, shifted))."""
    L = _go_lib()
    L.or_go_hc_term.restype = C.c_double
    a, b = int(g.start[r]), int(g.start[r + 1])
    x = np.ascontiguousarray(g.pos[a:b] if pos is None else pos, np.float64)
    ns = np.ascontiguousarray(g.nat_start, np.int32)
    nj = np.ascontiguousarray(g.nat_j, np.int32)
    r0 = np.ascontiguousarray(g.nat_r0, np.float64)
    br0, bt0 = (np.ascontiguousarray(v) for v in go_native_geometry(g, r))
    p = OrGoHcParams(*hc)
    out = {}
    for t, name in enumerate(("bond", "bend", "tors", "nb")):
        f = np.zeros((b - a, 3))
        e2 = np.zeros(2)
        out["e_" + name] = L.or_go_hc_term(b - a, _p(x), a, _p(ns), _p(nj), _p(r0), C.byref(p),
                                           _p(br0), _p(bt0), t, _p(f), _p(e2))
        out["f_" + name] = f
        if name == "nb":
            out["e_nb2"] = e2
    return out


def run_reference_go(g, r, hc, workdir, pos=None, L_box=1.0e4):
    """The reference's own cbb_golik / cba_golik / cda_golik / cnbnd_golik
    (oracle/_ref/ref_harness_go) on replica r with parameters hc = (eps,
    d_rep, rc), at pos (default: the native structure, whose geometry sets
    the bond lengths and bend angles either way)."""
    os.makedirs(workdir, exist_ok=True)
    a, b = int(g.start[r]), int(g.start[r + 1])
    N = b - a
    br0, bt0 = go_native_geometry(g, r)
    pairs = []
    for i in range(N):
        for q in range(int(g.nat_start[a + i]), int(g.nat_start[a + i + 1])):
            j = int(g.nat_j[q]) - a
            if j > i:
                pairs.append((i, j, float(g.nat_r0[q])))
    sp = os.path.join(workdir, "go.bin")
    op = os.path.join(workdir, "out_go.bin")
    with open(sp, "wb") as f:
        f.write(struct.pack("<i", N))
        f.write(struct.pack("<4d", L_box, hc[0], hc[1], hc[2]))
        f.write(np.ascontiguousarray(g.pos[a:b] if pos is None else pos, "<f8").tobytes())
        f.write(np.ascontiguousarray(br0, "<f8").tobytes())
        f.write(np.ascontiguousarray(bt0, "<f8").tobytes())
        f.write(struct.pack("<i", len(pairs)))
        for i, j, r0 in pairs:
            f.write(struct.pack("<iid", i, j, r0))
    subprocess.check_call([REF_BIN_GO, sp, op])
    return read_tagged(op)


def go_hc_forces(g, r, hc, pos=None):
    """(forces (N, 3), potential energy) of replica r under the reference's
    Go model: the sum of the four terms."""
    t = go_hc_terms(g, r, hc, pos)
    f = t["f_bond"] + t["f_bend"] + t["f_tors"] + t["f_nb"]
    return f, t["e_bond"] + t["e_bend"] + t["e_tors"] + t["e_nb"]


def go_hc_baoab(g, r, hc, nsteps, seed, step0=0):
    """nsteps Langevin steps of replica r under the reference's Go model;
    returns (pos, vel, final potential)."""
    L = _go_lib()
    L.or_go_baoab_hc.restype = C.c_double
    a, b = int(g.start[r]), int(g.start[r + 1])
    x = np.ascontiguousarray(g.pos[a:b], np.float64).copy()
    v = np.ascontiguousarray(g.vel[a:b], np.float64).copy()
    ns = np.ascontiguousarray(g.nat_start, np.int32)
    nj = np.ascontiguousarray(g.nat_j, np.int32)
    r0 = np.ascontiguousarray(g.nat_r0, np.float64)
    br0, bt0 = (np.ascontiguousarray(w) for w in go_native_geometry(g, r))
    e = L.or_go_baoab_hc(b - a, _p(x), _p(v), a, _p(ns), _p(nj), _p(r0), C.byref(_go_params(g)),
                         C.byref(OrGoHcParams(*hc)), _p(br0), _p(bt0), C.c_double(g.T[r]),
                         C.c_uint64(seed), C.c_uint64(step0), int(nsteps))
    return x, v, e
