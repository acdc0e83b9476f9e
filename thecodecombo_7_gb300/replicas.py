"""Replica exchange decisions on the host, for boxes spread over several
processes (one process per GPU).

On one GPU the exchange runs on the device (``engine.Batch``).  With boxes
on several GPUs, every rank steps its own boxes and, at an exchange step,
the ranks all-gather one potential energy per box (8 bytes each), then each
rank takes the same decision: the draws are Philox4x32-10 keyed by the seed
and the attempt number, so no further message is needed.  Swaps exchange
temperature slots, not coordinates; a rank only rescales the velocities of
its own boxes (``vmode``/``vfac``) and moves their chain states.

The arithmetic is the device kernel's: swap_box.c:5-86 on slots, pairs
alternating as repexch.c:273-301, kT as read_sim.c:351.
"""
from __future__ import annotations

import numpy as np

KB = 1.380662e-23
NA = 6.022045e23
TAG_EXCHANGE = 0x52455831

_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = 0x9E3779B9, 0xBB67AE85
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) of one counter."""
    c = [np.uint64(int(x) & 0xFFFFFFFF) for x in ctr]
    k0, k1 = int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF
    for r in range(10):
        if r:
            k0 = (k0 + _W0) & 0xFFFFFFFF
            k1 = (k1 + _W1) & 0xFFFFFFFF
        p0 = _M0 * c[0]
        p1 = _M1 * c[2]
        c = [(p1 >> np.uint64(32)) ^ c[1] ^ np.uint64(k0), p1 & _MASK,
             (p0 >> np.uint64(32)) ^ c[3] ^ np.uint64(k1), p0 & _MASK]
    return np.array([int(x) for x in c], dtype=np.uint32)


def uniform(seed: int, tag: int, event: int, lane: int) -> float:
    o = philox4x32_10([lane, event & 0xFFFFFFFF, (event >> 32) & 0xFFFFFFFF, tag],
                      [seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF])
    w = (int(o[0]) << 32) | int(o[1])
    return float(w >> 11) * (1.0 / 9007199254740992.0)


def exchange_decision(T_slot, potens_box, slot_box, attempt: int, seed: int):
    """One attempt over all slots.  Returns (slot_box, vmode, vfac) where
    vmode[b] is 1 (vv *= vfac[b]), 2 (vv /= vfac[b]) or 0 for box b."""
    T = np.asarray(T_slot, np.float64)
    U = np.asarray(potens_box, np.float64)
    slot = np.array(slot_box, dtype=np.int32, copy=True)
    R = len(T)
    vmode = np.zeros(R, np.int32)
    vfac = np.zeros(R)
    s = attempt & 1
    while s + 1 < R:
        r1, r2 = int(slot[s]), int(slot[s + 1])
        kT1 = ((KB * NA) * T[s]) * .001
        kT2 = ((KB * NA) * T[s + 1]) * .001
        with np.errstate(over="ignore"):  # exp overflow is +inf, as in C: accepted
            crit = np.exp((1.0 / kT1 - 1.0 / kT2) * (U[r1] - U[r2]))
        if crit > uniform(seed, TAG_EXCHANGE, attempt, s):
            slot[s], slot[s + 1] = r2, r1
            f = np.sqrt(T[s] / T[s + 1])
            vmode[r2], vfac[r2] = 1, f
            vmode[r1], vfac[r1] = 2, f
        s += 2
    return slot, vmode, vfac


def partition_boxes(n_atoms, world: int):
    """Whole boxes per rank, balanced by atom count (largest first onto the
    least-loaded rank).  Returns the owning rank of every box."""
    order = np.argsort(-np.asarray(n_atoms), kind="stable")
    load = np.zeros(world)
    owner = np.zeros(len(n_atoms), np.int32)
    for b in order:
        r = int(np.argmin(load))
        owner[b] = r
        load[r] += n_atoms[b]
    return owner


class RankExchange:
    """Exchange state shared by all ranks: slots, temperatures, attempt
    counter.  ``attempt(local_potens)`` all-gathers the potentials of the
    boxes each rank owns and applies one decision everywhere."""

    def __init__(self, T_slot, owner, rank: int, seed: int, group=None):
        self.T_slot = np.asarray(T_slot, np.float64)
        self.owner = np.asarray(owner, np.int32)
        self.rank = rank
        self.seed = seed
        self.group = group
        self.slot_box = np.arange(len(self.T_slot), dtype=np.int32)
        self.attempts = 0
        self.local = np.nonzero(self.owner == rank)[0]

    def temperature_of(self, box: int) -> float:
        return float(self.T_slot[int(np.nonzero(self.slot_box == box)[0][0])])

    def attempt(self, local_potens):
        import torch
        import torch.distributed as dist
        R = len(self.T_slot)
        mine = torch.zeros(R, dtype=torch.float64)
        mine[torch.as_tensor(self.local, dtype=torch.long)] = torch.as_tensor(
            np.asarray(local_potens, np.float64))
        if dist.is_available() and dist.is_initialized():
            dist.all_reduce(mine, group=self.group)  # each box has one owner
        U = mine.numpy()
        self.slot_box, vmode, vfac = exchange_decision(self.T_slot, U, self.slot_box,
                                                       self.attempts, self.seed)
        self.attempts += 1
        return {int(b): (int(vmode[b]), float(vfac[b])) for b in self.local}
