"""Generates the golden fixtures in this folder from the REFERENCE itself.

The reference's own hot-path routines are compiled from its unmodified C
sources (oracle/build_ref.sh -> oracle/_ref/ref_harness, strict IEEE build)
and driven by oracle/ref_harness.c on seeded synthetic water boxes; their
outputs are stored as compressed .npz files.  Needs the reference sources, so
it runs on the development machine only:

    python tests/golden/make_golden.py

Fixtures:
  water600.npz   600 sites, L = 25 A, SPME grid 24x25x27 (odd, non-cubic):
                 full pair lists (nlist + nlist_ew with xflags), spread grid,
                 force breakdown, energies, 12-step NVE and NHC trajectories
                 (list rebuilt every 5 steps)
  water4095.npz  the 4,095-site box at 0.1 sites/A^3 (L = 34.47 A, grid 32^3):
                 per-atom list counts, a SHA-256 of the sorted pair list,
                 forces and energies
  nlcheck600.npz the DLIST rebuild trigger (nl_check, -DDLIST build) on the
                 600-site box: list-time positions, the positions of 10
                 displacement cases after the reference's pbc_all, the site
                 ranges and the reference's nl_flag for each
  drift600.npz   drift() (drift.c:21) on velocities of the 600-site box given
                 a net momentum: velocities before and after
  chain900.npz   150 flexible 6-site chains (L = 31.07 A, grid 30^3): every
                 bonded term of forces() -- bonds, bends, Urey-Bradley,
                 proper torsions (cosine series, one stopping early) and
                 impropers -- with 1-4 pairs (xflag 4); the topology, the
                 forces of curey / ctorsion / cimproper alone, their energies
                 and torsion angles, the full forces() and en[k], and a
                 12-step NVE trajectory
  mc.npz         the classic-Ewald Monte Carlo energies (-DMC build): the
                 reference's enbnd_mc (ewald_kspace_mc + ewald_rspace_mc + LJ)
                 before and after fixed trial molecule moves, on a periodic
                 600-site box (k-space 297 vectors; its real space carries
                 the reference's minimum-image slip, ewald_mc.c:432-437, so
                 only the k-space and LJ parts are compared there) and on a
                 330-site cluster inside a larger box (no pair needs an
                 image: every part is compared)
"""
import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from thecodecombo_7_gb300 import systems  # noqa: E402


def sys_arrays(s):
    return dict(L=s.L, pos=s.pos, vel=s.vel, q=s.q, mass=s.mass, type=s.type,
                grid=np.array(s.grid), nlist_freq=np.array(s.nlist_freq))


def pair_hash(cnt, idx):
    rows = np.repeat(np.arange(cnt.shape[0], dtype=np.int64), cnt)
    key = rows * (1 << 32) + idx.astype(np.int64)
    return hashlib.sha256(np.sort(key).tobytes()).hexdigest()


def main():
    if not O.build_reference():
        raise SystemExit("reference sources not available")
    tmp = tempfile.mkdtemp(prefix="fe_golden_")
    # ---- small system, full detail ----
    s = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27))
    s.nlist_freq = 5
    nb = O.run_reference("nblist", s, tmp)
    fo = O.run_reference("forces", s, tmp)
    nve = O.run_reference("nve", s, tmp, nsteps=12)
    nhc = O.run_reference("nhc", s, tmp, nsteps=12)
    out = sys_arrays(s)
    for k, v in nb.items():
        out["nblist_" + k] = v
    for k, v in fo.items():
        out["forces_" + k] = v
    for k, v in nve.items():
        out["nve_" + k] = v
    for k, v in nhc.items():
        out["nhc_" + k] = v
    np.savez_compressed(os.path.join(HERE, "water600.npz"), **out)
    # ---- the 4,095-site box ----
    s = systems.water_box(1365, density=0.1, seed=2024)
    nb = O.run_reference("nblist", s, tmp)
    fo = O.run_reference("forces", s, tmp)
    out = sys_arrays(s)
    out["nl_cnt"] = nb["nl_cnt"]
    out["nl_hash"] = np.array(pair_hash(nb["nl_cnt"], nb["nl_idx"]))
    out["nl_nflag"] = np.array([(nb["nl_flg"] == f).sum() for f in range(5)])
    for k in ("f_total", "f_pme", "f_nonbond", "f_bonded", "e_pme", "e_nonbond",
              "e_bonded", "en"):
        out["forces_" + k] = fo[k]
    np.savez_compressed(os.path.join(HERE, "water4095.npz"), **out)
    make_nlcheck(tmp)
    make_mc(tmp)
    make_drift(tmp)
    make_chain(tmp)
    make_mts_water(tmp)
    make_go_hc(tmp)
    make_bgo(tmp)
    print("golden fixtures written to", HERE)


def nlcheck_cases(s):
    """Displacement cases around the DLIST threshold (rclist - rc)/4."""
    rcut = (s.rclist - s.rc) / 4.0
    n = s.n
    rng = np.random.default_rng(11)
    edge = int(np.argmax(s.pos[:, 0]))  # the site nearest +L/2 along x
    to_edge = s.L[0] / 2 - s.pos[edge, 0]
    small = [(int(i), *(rng.uniform(-0.35, 0.35, 3) * rcut)) for i in rng.choice(n, 40, False)]
    return [
        (0, n, []),
        (0, n, [(17, 0.98 * rcut, 0.0, 0.0)]),
        (0, n, [(17, 1.02 * rcut, 0.0, 0.0)]),
        (0, n, [(33, 0.6 * rcut, 0.6 * rcut, 0.6 * rcut)]),  # each axis below, distance above
        (0, n, [(edge, to_edge + 0.4 * rcut, 0.0, 0.0)]),      # wraps, moved 0.4 rcut
        (0, n, [(edge, to_edge + 1.2 * rcut, 0.0, 0.0)]),      # wraps, moved 1.2 rcut
        (0, n // 2, [(n - 3, 0.0, 2.0 * rcut, 0.0)]),          # outside the range
        (n // 2, n, [(n - 3, 0.0, 2.0 * rcut, 0.0)]),          # inside the range
        (0, n, small),
        (0, n, small + [(5, 0.0, 0.0, -1.1 * rcut)]),
    ]


def mc_moves(s, nmol, seed, count=8, delta=0.6):
    """Rigid translations of random molecules, (u - 0.5) delta per axis
    (mcmove_displ.c:92-94)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m = int(rng.integers(0, nmol))
        new = s.pos[3 * m:3 * m + 3] + (rng.uniform(size=3) - 0.5) * delta
        out.append((3 * m, 3 * m + 3, new))
    return out


def make_mc(tmp):
    out = {}
    # periodic box
    s = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27), helper=False)
    mv = mc_moves(s, 200, 5)
    r = O.run_reference_mc(s, 5, 25, mv, tmp)
    out.update(per_pos=s.pos, per_L=s.L, per_q=s.q, per_kmax=5, per_mks=25,
               per_energy=r["energy"], per_ranges=r["ranges"], per_nk=r["nk"],
               per_new=np.stack([m[2] for m in mv]))
    # cluster: molecules inside a 15 A cube, box 36 x 38 x 40 A
    s = systems.water_box(110, L=15.0, seed=8, grid=(24, 24, 24), helper=False)
    s.pos -= 15.0 * np.floor(s.pos / 15.0 + 0.5)
    s.L = np.array([36.0, 38.0, 40.0])
    mv = mc_moves(s, 110, 6)
    r = O.run_reference_mc(s, 7, 49, mv, tmp)
    out.update(clu_pos=s.pos, clu_L=s.L, clu_q=s.q, clu_kmax=7, clu_mks=49,
               clu_energy=r["energy"], clu_ranges=r["ranges"], clu_nk=r["nk"],
               clu_new=np.stack([m[2] for m in mv]))
    np.savez_compressed(os.path.join(HERE, "mc.npz"), **out)


CHAIN_KEYS = ("bonds", "bond_req", "bond_k", "bends", "bend_theta0", "bend_k", "excl",
              "excl_flag", "type_eps_kcal", "type_rmin_half", "ureys", "urey_seq", "urey_k",
              "tors", "tors_kphi", "tors_nphi", "tors_delphi", "impr", "impr_k", "impr_eq")


def make_chain(tmp):
    s = systems.chain_box(150, 6, seed=3)
    s.nlist_freq = 5
    fo = O.run_reference("forces", s, tmp)
    nve = O.run_reference("nve", s, tmp, nsteps=12)
    # RESPA (integrate_mts.c): 6 long steps of 4 short steps
    mts = O.run_reference("mts", s, tmp, nsteps=6, extra=(4,))
    out = sys_arrays(s)
    for k, v in mts.items():
        out["mts_" + k] = v
    for k in CHAIN_KEYS:
        out["top_" + k] = getattr(s, k)
    for k, v in fo.items():
        out["forces_" + k] = v
    for k, v in nve.items():
        out["nve_" + k] = v
    np.savez_compressed(os.path.join(HERE, "chain900.npz"), **out)


def make_mts_water(tmp):
    """RESPA on the 600-site water box: 8 long steps of 4 short steps."""
    s = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27))
    s.nlist_freq = 5
    r = O.run_reference("mts", s, tmp, nsteps=8, extra=(4,))
    out = sys_arrays(s)
    for k, v in r.items():
        out["mts_" + k] = v
    # integrate_mts_nhc.c with the thermostat per long step (xRESPA 0) and
    # per short step (xRESPA 1)
    for x in (0, 1):
        r = O.run_reference("mtsnhc", s, tmp, nsteps=8, extra=(4, x))
        for k, v in r.items():
            out[f"mtsnhc{x}_" + k] = v
    np.savez_compressed(os.path.join(HERE, "mts_water600.npz"), **out)


def make_go_hc(tmp):
    """The reference's own Go model (cgolik.c) on three chains of 60-150
    beads at perturbed coordinates: forces and energies per term."""
    g = systems.go_chains(3, nmin=60, nmax=150, seed=31)
    rng = np.random.default_rng(8)
    hc = (g.eps, 4.0, 12.0)  # eps, d_repulsive, rc
    out = dict(nbeads=g.nbeads, pos0=g.pos, nat_start=g.nat_start, nat_j=g.nat_j,
               nat_r0=g.nat_r0, hc=np.array(hc))
    pos = g.pos + rng.normal(0.0, 0.15, g.pos.shape)
    out["pos"] = pos
    for r in range(len(g.nbeads)):
        a, b = int(g.start[r]), int(g.start[r + 1])
        ref = O.run_reference_go(g, r, hc, tmp, pos=pos[a:b])
        for k, v in ref.items():
            out[f"r{r}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "go_hc.npz"), **out)


def make_bgo(tmp):
    """The BGO build's pair form (cnonbond_nblist.c:294-307) on the 600-site
    water box: forces() and its breakdown from the reference's -DBGO build."""
    s = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27))
    fo = O.run_reference("forces", s, tmp, binary=O.REF_BIN_BGO)
    out = sys_arrays(s)
    for k, v in fo.items():
        out["forces_" + k] = v
    np.savez_compressed(os.path.join(HERE, "bgo600.npz"), **out)


def make_drift(tmp):
    s = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27), helper=False)
    s.vel = s.vel + np.array([0.7, -0.4, 0.25])
    r = O.run_reference("drift", s, tmp)
    np.savez_compressed(os.path.join(HERE, "drift600.npz"), vel0=s.vel, mass=s.mass,
                        vel=r["vel"].reshape(-1, 3), uu=r["vel_uu"].reshape(-1, 3))


def make_nlcheck(tmp):
    s = systems.water_box(200, L=25.0, seed=7, grid=(24, 25, 27))
    cases = nlcheck_cases(s)
    r = O.run_reference_nlcheck(s, cases, tmp)
    np.savez_compressed(os.path.join(HERE, "nlcheck600.npz"), L=s.L, rclist=s.rclist, rc=s.rc,
                        pos0=r["pos0"].reshape(-1, 3),
                        pos_cases=r["pos_cases"].reshape(len(cases), -1, 3),
                        lb=np.array([c[0] for c in cases]), ub=np.array([c[1] for c in cases]),
                        flags=r["nl_flg"])


if __name__ == "__main__":
    if sys.argv[1:] in (["nlcheck"], ["mc"], ["drift"], ["chain"], ["mts"], ["go"], ["bgo"]):
        if not O.build_reference():
            raise SystemExit("reference sources not available")
        {"nlcheck": make_nlcheck, "mc": make_mc, "drift": make_drift,
         "chain": make_chain, "mts": make_mts_water, "go": make_go_hc,
         "bgo": make_bgo}[sys.argv[1]](
            tempfile.mkdtemp(prefix="fe_golden_"))
    else:
        main()
