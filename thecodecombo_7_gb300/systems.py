"""Synthetic systems in the reference's vocabulary (boxes of sites).

The reference reads its systems from INPUT/ files (read_config.c,
read_topology.c); the workloads here are generated instead, seeded, with the
shapes the engine is measured on:

* ``water_box`` -- rigid-geometry 3-site bent molecules (O, H, H) with charges
  -0.8/+0.4/+0.4 e, O-H 1.0 A (k = 450 kcal/mol/A^2), H-O-H 104.5 deg
  (k = 55 kcal/mol/rad^2), LJ on O only (eps = 0.15 kcal/mol, sigma = 3.15 A,
  stored the reference's way as CHARMM eps < 0 and R_min/2), masses 16/1/1
  amu; 1-2 pairs (xflag 1) and the 1-3 pair (xflag 2) excluded.  Molecule
  centres are placed uniformly at random in a periodic cube at the requested
  site density, rejecting any O-O distance below 2.6 A, with uniformly random
  orientations, and Maxwell-Boltzmann velocities (net momentum removed).

* ``go_chains`` -- replicas of C-alpha Go-model chains for batched replica
  exchange: compact self-avoiding-walk native structures, native contacts,
  geometric temperatures.

Units are the reference's internal ones (A, ps, amu, e, kJ/mol;
defines.h:62-75, integrate_vverlet.c:56).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np
from scipy.spatial import cKDTree

KB = 1.380662e-23  # defines.h:63
AU = 1.6605655e-27  # defines.h:66
KCAL = 4.184  # read_topology.c:212 (kcal -> kJ)


@dataclasses.dataclass
class System:
    """One box: sites, topology and the run parameters of the hot path."""

    L: np.ndarray  # (3,) box lengths
    pos: np.ndarray  # (n, 3) float64, wrapped into [-L/2, L/2]
    q: np.ndarray  # (n,)
    mass: np.ndarray  # (n,)
    type: np.ndarray  # (n,) int32 site type (atom[k][i].atomid)
    vel: np.ndarray  # (n, 3) A/ps
    type_eps_kcal: np.ndarray  # (ntypes,) CHARMM eps (<= 0)
    type_rmin_half: np.ndarray  # (ntypes,) R_min/2
    bonds: np.ndarray  # (nb, 2) int32
    bond_req: np.ndarray
    bond_k: np.ndarray  # kJ/mol/A^2, E = k (r - r0)^2
    bends: np.ndarray  # (na, 3) int32 (a, b=apex, c)
    bend_theta0: np.ndarray  # rad
    bend_k: np.ndarray  # kJ/mol/rad^2, E = k (theta - theta0)^2
    excl: np.ndarray  # (nx, 2) int32
    excl_flag: np.ndarray  # (nx,) int32, 1 bond / 2 bend / 3 exNB / 4 1-4
    rc: float = 10.0
    rclist: float = 12.0
    rclist_ew: float = 12.0
    rc_ew: float = 10.0
    kappa: float = 0.32
    epsRF: float = 1.0
    dt: float = 0.0005  # ps
    T: float = 300.0
    grid: tuple = (32, 32, 32)
    order: int = 4
    nlist_freq: int = 10
    r_switch: float = 0.0  # 0 = no switch (the reference); 8.0 = CHARMM switch 8->rc
    nhc_M: int = 3
    nhc_Q: float = 1.0e-18
    seed: int = 0
    # Urey-Bradley 1-3 terms (curey.c), E = k (r - Seq)^2
    ureys: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 2), np.int32))
    urey_seq: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    urey_k: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    # proper torsions (ctorsion.c): E = sum_t kphi (1 + cos(nphi tau - delphi)),
    # six terms per torsion, the series ending at the first kphi == 0
    tors: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 4), np.int32))
    tors_kphi: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 6)))
    tors_nphi: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 6)))
    tors_delphi: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 6)))
    # improper torsions (cimproper.c): E = kimpr (tau - angeq)^2
    impr: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 4), np.int32))
    impr_k: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    impr_eq: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    @property
    def ntypes(self) -> int:
        return int(self.type_eps_kcal.shape[0])

    @property
    def has_ext_bonded(self) -> bool:
        """Urey-Bradley, torsion or improper terms present."""
        return bool(len(self.ureys) or len(self.tors) or len(self.impr))

    def lj_tables(self):
        """Mixed (eps [kJ/mol], R_min [A]) per type pair, setlj.c:181-191."""
        e = self.type_eps_kcal
        s = self.type_rmin_half
        eps = KCAL * np.sqrt(np.outer(e, e))
        sig = 0.5 * (2.0 * s[:, None] + 2.0 * s[None, :])
        return np.ascontiguousarray(eps), np.ascontiguousarray(sig)

    def copy(self) -> "System":
        return dataclasses.replace(
            self, pos=self.pos.copy(), vel=self.vel.copy(), L=self.L.copy())


def fft_friendly(n: int) -> int:
    """Smallest m >= n whose prime factors are 2, 3 and 5."""
    m = max(int(n), 1)
    while True:
        k = m
        for p in (2, 3, 5):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


def fft_friendly_below(n: int) -> int:
    """Largest m <= n whose prime factors are 2, 3 and 5."""
    m = max(int(n), 1)
    while m > 1:
        k = m
        for p in (2, 3, 5):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m -= 1
    return 1


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices from unit quaternions."""
    qv = rng.normal(size=(n, 4))
    qv /= np.linalg.norm(qv, axis=1, keepdims=True)
    w, x, y, z = qv.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def _place_centres(rng: np.random.Generator, n_mol: int, L: float,
                   dmin: float, max_tries: int = 400) -> np.ndarray:
    """Random sequential placement in a periodic cube with an O-O minimum.

    Candidates are drawn in batches of 4096; each batch is first screened in
    one vectorised pass against the molecules accepted before it (a dense
    cell grid, cell >= dmin, 8 slots per cell), then the survivors are taken
    in order against the grid as it fills -- the same outcome as testing
    every candidate sequentially against all earlier acceptances.
    """
    m = max(1, int(L // dmin))
    cell = L / m
    slots = 8
    occ = np.full((m, m, m, slots, 3), np.nan)
    nocc = np.zeros((m, m, m), dtype=np.int64)
    out = np.empty((n_mol, 3))
    d2 = dmin * dmin
    offs = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    count = 0
    tries = 0

    def conflicts(cs, ci):
        nb = (ci[:, None, :] + offs[None, :, :]) % m
        pts = occ[nb[..., 0], nb[..., 1], nb[..., 2]]  # (B, 27, slots, 3)
        d = pts - cs[:, None, None, :]
        d -= L * np.rint(d / L)
        r2 = np.einsum("bkst,bkst->bks", d, d)
        return np.any(r2 < d2, axis=(1, 2))  # NaN slots compare False

    while count < n_mol:
        cand = rng.uniform(-L / 2, L / 2, size=(4096, 3))
        ci = ((cand + L / 2) / cell).astype(np.int64) % m
        bad = conflicts(cand, ci)
        surv = np.nonzero(~bad)[0]
        keep = np.ones(surv.size, dtype=bool)
        if surv.size > 1:
            # conflicts among this batch's survivors: an earlier accepted one wins
            tree = cKDTree(np.mod(cand[surv] + L / 2, L), boxsize=L)
            pairs = tree.query_pairs(dmin, output_type="ndarray")
            if len(pairs):
                pairs = pairs[np.lexsort((pairs[:, 0], pairs[:, 1]))]
                for i, j in pairs:
                    if keep[i]:
                        keep[j] = False
        for k in surv[keep][: n_mol - count]:
            cc = ci[k]
            slot = nocc[cc[0], cc[1], cc[2]]
            if slot >= slots:
                raise RuntimeError("cell over capacity in the placement grid")
            occ[cc[0], cc[1], cc[2], slot] = cand[k]
            nocc[cc[0], cc[1], cc[2]] += 1
            out[count] = cand[k]
            count += 1
        tries += 4096
        if tries > max_tries * n_mol:
            raise RuntimeError(
                f"could not place {n_mol} molecules at L={L:.3f} with O-O >= {dmin}")
    return out


def _place_centres_fast(rng: np.random.Generator, n_mol: int, L: float, dmin: float,
                        max_tries: int = 400):
    """Same placement as _place_centres (same candidate stream, same result)
    through the C helper libfe_sysgen.so; None if the helper is not built."""
    import ctypes as C
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libfe_sysgen.so")
    if not os.path.exists(path):
        return None
    lib = C.CDLL(path)
    lib.fe_sysgen_place.restype = C.c_long
    lib.fe_sysgen_place.argtypes = [C.c_void_p, C.c_long, C.c_double, C.c_double, C.c_long,
                                    C.c_void_p, C.POINTER(C.c_long)]
    out = np.zeros((n_mol, 3))
    done = C.c_long(0)
    drawn = 0
    chunk = 4096 * 64
    while True:
        state = rng.bit_generator.state
        cand = np.ascontiguousarray(rng.uniform(-L / 2, L / 2, size=(chunk, 3)))
        used = lib.fe_sysgen_place(cand.ctypes.data, chunk, L, dmin, n_mol, out.ctypes.data,
                                   C.byref(done))
        if used == -2:
            raise RuntimeError("cell over capacity in the placement grid")
        if used > 0:
            # advance the stream exactly as the batch-of-4096 version would
            rng.bit_generator.state = state
            rng.uniform(-L / 2, L / 2, size=(-(-used // 4096) * 4096, 3))
            return out
        drawn += chunk
        if drawn > max_tries * n_mol:
            raise RuntimeError(
                f"could not place {n_mol} molecules at L={L:.3f} with O-O >= {dmin}")


def water_box(n_mol: int, density: float = 0.1, seed: int = 1234,
              grid=None, T: float = 300.0, L: float | None = None,
              dmin: float = 2.6, helper: bool = True, **params) -> System:
    """The 3-site bent-molecule box of the configured workloads.

    ``density`` is sites per A^3 (0.1 gives L = 34.47 A at 1,365 molecules and
    L = 98.65 A at 32,000).  ``grid`` defaults to about 1 point/A: round(L)
    lowered to the nearest FFT-friendly size (32^3 and 96^3 for the two sizes
    above).  ``helper=False`` places the molecules with numpy only (same
    result, no compiled helper loaded).
    """
    rng = np.random.default_rng(seed)
    n = 3 * n_mol
    if L is None:
        L = (n / density) ** (1.0 / 3.0)
    if grid is None:
        g = fft_friendly_below(int(round(L)))
        grid = (g, g, g)
    centres = _place_centres_fast(rng, n_mol, L, dmin) if helper else None
    if centres is None:
        centres = _place_centres(rng, n_mol, L, dmin)
    R = _random_rotations(rng, n_mol)
    half = math.radians(104.5) / 2.0
    body = np.array([[0.0, 0.0, 0.0],
                     [math.sin(half), math.cos(half), 0.0],
                     [-math.sin(half), math.cos(half), 0.0]])  # O-H = 1.0 A
    pos = centres[:, None, :] + np.einsum("mij,kj->mki", R, body)
    pos = pos.reshape(n, 3)
    pos -= L * np.floor(pos / L + 0.5)  # wrap into [-L/2, L/2)
    q = np.tile([-0.8, 0.4, 0.4], n_mol)
    mass = np.tile([16.0, 1.0, 1.0], n_mol)
    typ = np.tile(np.array([0, 1, 1], dtype=np.int32), n_mol)
    # Maxwell-Boltzmann at T: sigma = sqrt(kT/m) m/s = 0.01 * that A/ps
    sd = np.sqrt(KB * T / (mass * AU)) * 1.0e-2
    vel = rng.normal(size=(n, 3)) * sd[:, None]
    p = (vel * mass[:, None]).sum(0) / mass.sum()
    vel -= p
    base = 3 * np.arange(n_mol, dtype=np.int32)
    bonds = np.stack([np.stack([base, base + 1], 1),
                      np.stack([base, base + 2], 1)], 1).reshape(-1, 2)
    bends = np.stack([base + 1, base, base + 2], 1)
    excl = np.concatenate([np.stack([base, base + 1], 1),
                           np.stack([base, base + 2], 1),
                           np.stack([base + 1, base + 2], 1)], 0)
    excl_flag = np.concatenate([np.ones(n_mol, np.int32), np.ones(n_mol, np.int32),
                                2 * np.ones(n_mol, np.int32)])
    rmin_half = 2.0 ** (1.0 / 6.0) * 3.15 / 2.0
    sysm = System(
        L=np.array([L, L, L], dtype=np.float64),
        pos=np.ascontiguousarray(pos, dtype=np.float64),
        q=q.astype(np.float64), mass=mass, type=typ,
        vel=np.ascontiguousarray(vel),
        type_eps_kcal=np.array([-0.15, 0.0]),
        type_rmin_half=np.array([rmin_half, 0.0]),
        bonds=bonds.astype(np.int32),
        bond_req=np.full(bonds.shape[0], 1.0),
        bond_k=np.full(bonds.shape[0], 450.0 * KCAL),
        bends=bends.astype(np.int32),
        bend_theta0=np.full(n_mol, math.radians(104.5)),
        bend_k=np.full(n_mol, 55.0 * KCAL),
        excl=excl.astype(np.int32), excl_flag=excl_flag,
        T=T, grid=tuple(int(x) for x in grid), seed=seed)
    for k, v in params.items():
        setattr(sysm, k, v)
    return sysm


def _grow_chain(rng, n_site, bond, theta, L):
    """One chain grown site by site: bond lengths and bend angles around
    (bond, theta) with a small spread, dihedrals uniform in (-pi, pi]."""
    x = np.zeros((n_site, 3))
    x[1] = [bond, 0.0, 0.0]
    if n_site > 2:
        th = theta + rng.normal(0.0, 0.05)
        x[2] = x[1] + bond * np.array([-math.cos(th), math.sin(th), 0.0])
    for k in range(3, n_site):
        b = bond * (1.0 + rng.normal(0.0, 0.02))
        th = theta + rng.normal(0.0, 0.05)
        phi = rng.uniform(-math.pi, math.pi)
        a, bb, c = x[k - 3], x[k - 2], x[k - 1]
        bc = c - bb
        bc /= np.linalg.norm(bc)
        nrm = np.cross(bb - a, bc)
        nrm /= np.linalg.norm(nrm)
        m = np.stack([bc, np.cross(nrm, bc), nrm], 1)
        d = np.array([-b * math.cos(th), b * math.sin(th) * math.cos(phi),
                      b * math.sin(th) * math.sin(phi)])
        x[k] = c + m @ d
    return x - x.mean(0)


def chain_box(n_mol: int = 150, n_site: int = 6, density: float = 0.03, seed: int = 0,
              T: float = 300.0, L: float | None = None, dmin: float = 2.5, grid=None,
              **params) -> System:
    """Flexible united-atom chains with every bonded term of forces():
    bonds, bends, Urey-Bradley 1-3 terms, proper torsions (three-term cosine
    series; the first torsion of each chain has a zero second term, so its
    series stops after one term) and one improper per chain; charges
    +-0.25 / +-0.1 e (neutral chains), 1-2 / 1-3 pairs excluded (xflag 1 / 2)
    and 1-4 pairs modified (xflag 4).  Chains are grown with random
    dihedrals, rotated at random and placed one by one, rejecting any site
    closer than ``dmin`` to a site of another chain."""
    rng = np.random.default_rng(seed)
    n = n_mol * n_site
    if L is None:
        L = (n / density) ** (1.0 / 3.0)
    if grid is None:
        g = fft_friendly_below(int(round(L)))
        grid = (g, g, g)
    bond, theta = 1.53, math.radians(111.0)
    placed = np.zeros((0, 3))
    chains = []
    tries = 0
    while len(chains) < n_mol:
        tries += 1
        if tries > 200 * n_mol:
            raise RuntimeError(f"could not place {n_mol} chains at L={L:.2f}")
        x = _grow_chain(rng, n_site, bond, theta, L)
        dd = np.linalg.norm(x[:, None] - x[None], axis=-1)
        if n_site > 4 and np.triu(dd < dmin, 4).any():  # the chain folds onto itself
            continue
        x = x @ _random_rotations(rng, 1)[0].T + rng.uniform(-L / 2, L / 2, 3)
        x -= L * np.floor(x / L + 0.5)
        if len(placed):
            tree = cKDTree(np.mod(placed + L / 2, L), boxsize=L)
            if np.isfinite(tree.query(np.mod(x + L / 2, L), distance_upper_bound=dmin)[0]).any():
                continue
        chains.append(x)
        placed = np.concatenate([placed, x])
    pos = np.concatenate(chains)
    pattern_q = np.array([0.25, -0.25, 0.1, -0.1, 0.25, -0.25])
    q = np.tile(np.resize(pattern_q, n_site), n_mol)
    q -= np.repeat(q.reshape(n_mol, n_site).mean(1), n_site)  # neutral chains
    typ1 = np.ones(n_site, np.int32)
    typ1[0] = typ1[-1] = 0
    typ = np.tile(typ1, n_mol)
    mass = np.where(typ == 0, 15.0, 14.0)
    sd = np.sqrt(KB * T / (mass * AU)) * 1.0e-2
    vel = rng.normal(size=(n, 3)) * sd[:, None]
    vel -= (vel * mass[:, None]).sum(0) / mass.sum()
    base = n_site * np.arange(n_mol, dtype=np.int32)[:, None]
    def idx(*offs):
        ks = np.arange(n_site - max(offs), dtype=np.int32)
        return np.stack([(base + ks[None, :] + o) for o in offs], -1).reshape(-1, len(offs))
    bonds, bends, ureys, tors = idx(0, 1), idx(0, 1, 2), idx(0, 2), idx(0, 1, 2, 3)
    nt = len(tors)
    kphi = np.zeros((nt, 6))
    nphi = np.zeros((nt, 6))
    delphi = np.zeros((nt, 6))
    kphi[:, :3] = np.array([0.20, 0.25, 0.40]) * KCAL
    nphi[:, :3] = [1.0, 2.0, 3.0]
    delphi[:, :3] = [0.0, math.pi, 0.0]
    first = (np.arange(nt) % (n_site - 3)) == 0
    kphi[first, 1] = 0.0  # the series stops here (ctorsion.c:178-186)
    impr = (base[:, 0:1] + np.array([[1, 0, 2, 3]], np.int32)).astype(np.int32)
    excl = np.concatenate([bonds, ureys, idx(0, 3)])
    excl_flag = np.concatenate([np.ones(len(bonds), np.int32), 2 * np.ones(len(ureys), np.int32),
                                4 * np.ones(len(tors), np.int32)])
    sysm = System(
        L=np.array([L, L, L], dtype=np.float64),
        pos=np.ascontiguousarray(pos), q=q.astype(np.float64), mass=mass.astype(np.float64),
        type=typ, vel=np.ascontiguousarray(vel),
        type_eps_kcal=np.array([-0.175, -0.118]),
        type_rmin_half=np.array([2.06, 2.20]),
        bonds=bonds, bond_req=np.full(len(bonds), bond), bond_k=np.full(len(bonds), 222.5 * KCAL),
        bends=bends, bend_theta0=np.full(len(bends), theta),
        bend_k=np.full(len(bends), 58.35 * KCAL),
        excl=excl.astype(np.int32), excl_flag=excl_flag,
        T=T, grid=tuple(int(x) for x in grid), seed=seed,
        ureys=ureys, urey_seq=np.full(len(ureys), 2.53), urey_k=np.full(len(ureys), 11.16 * KCAL),
        tors=tors.astype(np.int32), tors_kphi=kphi, tors_nphi=nphi, tors_delphi=delphi,
        impr=impr, impr_k=np.full(n_mol, 20.0 * KCAL), impr_eq=np.full(n_mol, math.radians(35.0)))
    for k, v in params.items():
        setattr(sysm, k, v)
    return sysm


# ---------------------------------------------------------------------------
# Go-model chains (the batched replica-exchange workload)

@dataclasses.dataclass
class GoChains:
    """Replicas of C-alpha chains: concatenated beads, natives as CSR over
    the global bead index (both directions), per-replica temperatures."""

    nbeads: np.ndarray      # (R,)
    pos: np.ndarray         # (total, 3) native (starting) coordinates [A]
    vel: np.ndarray         # (total, 3) [A/ps]
    nat_start: np.ndarray   # (total + 1,)
    nat_j: np.ndarray       # global partner index
    nat_r0: np.ndarray      # native distance [A]
    T: np.ndarray           # (R,) [K]
    eps: float = 1.0 * KCAL        # 1 kcal/mol
    sigma_rep: float = 4.0
    rc_rep: float = 10.0
    k_bond: float = 100.0 * KCAL   # E = k (r - r0)^2
    r_bond: float = 3.8
    mass: float = 110.0
    gamma: float = 1.0
    dt: float = 0.01
    min_sep: int = 3
    seed: int = 0

    @property
    def start(self):
        return np.concatenate([[0], np.cumsum(self.nbeads)]).astype(np.int64)


def _compact_saw(rng: np.random.Generator, n: int, bias: float = 1.5) -> np.ndarray:
    """A compact self-avoiding walk of n sites on the unit cubic lattice:
    grown site by site, each step choosing among the free neighbours with
    weight exp(bias x occupied neighbours of the candidate); restarts on a
    dead end."""
    steps = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]])
    while True:
        path = [(0, 0, 0)]
        occ = {(0, 0, 0)}
        ok = True
        for _ in range(n - 1):
            x = np.array(path[-1])
            cands, w = [], []
            for s in steps:
                c = tuple(x + s)
                if c in occ:
                    continue
                k = sum(tuple(np.array(c) + t) in occ for t in steps)
                cands.append(c)
                w.append(math.exp(bias * k))
            if not cands:
                ok = False
                break
            w = np.array(w) / sum(w)
            c = cands[rng.choice(len(cands), p=w)]
            path.append(c)
            occ.add(c)
        if ok:
            return np.array(path, dtype=np.float64)


def go_chains(n_rep: int = 64, nmin: int = 60, nmax: int = 400, seed: int = 2025,
              T_min: float = 280.0, T_max: float = 450.0, lattice: float = 3.8,
              jitter: float = 0.25, native_cut: float = 6.5, native_min_sep: int = 4,
              **params) -> GoChains:
    """Chain lengths uniform in [nmin, nmax]; native structures are compact
    self-avoiding walks on a cubic lattice of spacing `lattice` with each bead
    jittered uniformly by +-`jitter` per axis; natives are pairs closer than
    `native_cut` with |i - j| >= native_min_sep; temperatures geometric from
    T_min to T_max; Maxwell-Boltzmann velocities at each replica's T."""
    rng = np.random.default_rng(seed)
    nb = rng.integers(nmin, nmax + 1, n_rep)
    T = np.geomspace(T_min, T_max, n_rep) if n_rep > 1 else np.array([T_min])
    mass = params.get("mass", 110.0)
    pos, vel, starts, js, r0s = [], [], [0], [], []
    base = 0
    for r in range(n_rep):
        n = int(nb[r])
        x = _compact_saw(rng, n) * lattice
        x += rng.uniform(-jitter, jitter, x.shape)
        x -= x.mean(axis=0)
        d = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
        for i in range(n):
            nat = [j for j in range(n) if abs(i - j) >= native_min_sep and d[i, j] < native_cut]
            js.extend(base + j for j in nat)
            r0s.extend(d[i, j] for j in nat)
            starts.append(starts[-1] + len(nat))
        sv = math.sqrt(KB * T[r] / (mass * AU)) * 0.01
        v = rng.normal(0.0, sv, (n, 3))
        v -= v.mean(axis=0)
        pos.append(x)
        vel.append(v)
        base += n
    return GoChains(nbeads=nb.astype(np.int32), pos=np.concatenate(pos), vel=np.concatenate(vel),
                    nat_start=np.array(starts, dtype=np.int32),
                    nat_j=np.array(js, dtype=np.int32), nat_r0=np.array(r0s, dtype=np.float64),
                    T=T.astype(np.float64), seed=seed, **params)
