"""Shared helpers for the tests: rebuild a System from a golden fixture."""
import numpy as np

from thecodecombo_7_gb300 import systems


def system_from_golden(g, n_mol):
    L = float(g["L"][0])
    s = systems.water_box(n_mol, L=L, seed=0, grid=tuple(int(x) for x in g["grid"]))
    s.pos = np.ascontiguousarray(g["pos"])
    s.vel = np.ascontiguousarray(g["vel"])
    s.nlist_freq = int(g["nlist_freq"])
    return s


def mc_case(g, which):
    """(System, kmax, max_k_square, moves, reference energies) of one box of
    the Monte Carlo fixture: which = "per" (periodic 600-site box) or "clu"
    (cluster inside a larger box).  moves are (lb, ub, new positions)."""
    pos = np.ascontiguousarray(g[which + "_pos"])
    n_mol = pos.shape[0] // 3
    s = systems.water_box(n_mol, L=25.0, seed=0, grid=(24, 24, 24), helper=False)
    s.pos = pos
    s.L = np.ascontiguousarray(g[which + "_L"], dtype=np.float64)
    rng = g[which + "_ranges"][1:]
    new = g[which + "_new"]
    moves = [(int(a), int(b), new[i]) for i, (a, b) in enumerate(rng)]
    return s, int(g[which + "_kmax"]), int(g[which + "_mks"]), moves, g[which + "_energy"]


def mc_reference_parts(e):
    """(dE_kspace, dE_real, dE_lj) of each move from the reference's
    enbnd_mc energy[] before (e[:8]) and after (e[8:]): k-space energy[4];
    real space energy[7] - energy[6] (unshifted real minus intramolecular);
    shifted LJ energy[1] - energy[7] + energy[6] - energy[4] + energy[5]."""
    def parts(x):
        return np.array([x[4], x[7] - x[6], x[1] - x[7] + x[6] - x[4] + x[5]])
    return np.array([parts(r[8:]) - parts(r[:8]) for r in e[1:]])


CHAIN_KEYS = ("bonds", "bond_req", "bond_k", "bends", "bend_theta0", "bend_k", "excl",
              "excl_flag", "type_eps_kcal", "type_rmin_half", "ureys", "urey_seq", "urey_k",
              "tors", "tors_kphi", "tors_nphi", "tors_delphi", "impr", "impr_k", "impr_eq")


def chain_from_golden(g):
    """The chain box of chain900.npz, topology and state from the fixture."""
    L = np.ascontiguousarray(g["L"], dtype=np.float64)
    kw = {k: np.ascontiguousarray(g["top_" + k]) for k in CHAIN_KEYS}
    s = systems.System(L=L, pos=np.ascontiguousarray(g["pos"]), q=np.ascontiguousarray(g["q"]),
                       mass=np.ascontiguousarray(g["mass"]),
                       type=np.ascontiguousarray(g["type"], dtype=np.int32),
                       vel=np.ascontiguousarray(g["vel"]),
                       grid=tuple(int(x) for x in g["grid"]), **kw)
    s.nlist_freq = int(g["nlist_freq"])
    return s


def go_from_golden(g):
    """The chains of go_hc.npz (native structure as the starting coordinates,
    velocities zero, temperatures 300 K) and the perturbed coordinates the
    reference's terms were evaluated at."""
    nb = np.asarray(g["nbeads"], np.int32)
    n = int(nb.sum())
    chains = systems.GoChains(nbeads=nb, pos=np.ascontiguousarray(g["pos0"]),
                              vel=np.zeros((n, 3)), nat_start=np.asarray(g["nat_start"], np.int32),
                              nat_j=np.asarray(g["nat_j"], np.int32),
                              nat_r0=np.asarray(g["nat_r0"], np.float64),
                              T=np.full(len(nb), 300.0))
    return chains, np.ascontiguousarray(g["pos"]), tuple(float(x) for x in g["hc"])
