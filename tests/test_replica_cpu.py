"""Replica-exchange decisions without a GPU: the Philox draws against the
published known-answer vectors, the host decision against the oracle's
swap_box restatement, and the multi-process exchange (gloo, 2 ranks)
against a single-process run."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from thecodecombo_7_gb300 import replicas

# Philox4x32-10 known-answer vectors published with the algorithm
# (counter, key) -> output
KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(ctr, key, want):
    assert list(O.philox4x32_10(ctr, key)) == want
    assert list(replicas.philox4x32_10(ctr, key)) == want


def test_uniform_host_equals_oracle():
    rng = np.random.default_rng(5)
    for _ in range(200):
        seed = int(rng.integers(0, 2**63))
        ev = int(rng.integers(0, 2**40))
        lane = int(rng.integers(0, 4096))
        a = replicas.uniform(seed, replicas.TAG_EXCHANGE, ev, lane)
        b = O.uniform(seed, O.TAG_EXCHANGE, ev, lane)
        assert a == b and 0.0 <= a < 1.0


def test_exchange_decision_equals_oracle():
    rng = np.random.default_rng(9)
    for trial in range(50):
        R = int(rng.integers(2, 12))
        T = np.sort(rng.uniform(280, 450, R))
        U = rng.normal(-5000, 40, R)
        slot = rng.permutation(R).astype(np.int32)
        a = int(rng.integers(0, 1000))
        s1, m1, f1 = replicas.exchange_decision(T, U, slot, a, 77)
        s2, m2, f2, n = O.rex_attempt(T, U, slot, a, 77)
        assert np.array_equal(s1, s2) and np.array_equal(m1, m2)
        assert np.array_equal(f1[m1 > 0], f2[m2 > 0])
        assert n == int((m1 > 0).sum()) // 2


def test_exchange_schedule_alternates():
    T = np.array([300.0, 310.0, 320.0, 330.0, 340.0])
    U = np.array([0.0, -1e6, 0.0, -1e6, 0.0])  # every pair with the low box below accepts
    s, m, _ = replicas.exchange_decision(T, U, np.arange(5), 0, 1)
    # attempt 0 pairs (0,1) and (2,3): box 0 (U=0) at the colder slot swaps up
    assert list(s) == [1, 0, 3, 2, 4]
    s, m, _ = replicas.exchange_decision(T, U, np.arange(5), 1, 1)
    # attempt 1 pairs (1,2) and (3,4): U1 < U2 at the colder slot: never accepted
    assert list(s) == [0, 1, 2, 3, 4] and not m.any()


def test_partition_balanced():
    sizes = np.array([6000, 36000, 12000, 30000, 9000, 21000, 18000, 24000])
    owner = replicas.partition_boxes(sizes, 2)
    loads = [sizes[owner == r].sum() for r in range(2)]
    assert abs(loads[0] - loads[1]) <= sizes.max()
    assert set(owner.tolist()) == {0, 1}


def _potens(box, attempt):
    return -5000.0 + 7.0 * np.sin(1.3 * box + 0.7 * attempt) - 3.0 * box


def _rank_main(rank, world, port, T, owner, n_att, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ex = replicas.RankExchange(T, owner, rank, seed=99)
        scales = []
        for a in range(n_att):
            local = [_potens(int(b), a) for b in ex.local]
            scales.append(ex.attempt(local))
        np.save(f"{out}_{rank}.npy", ex.slot_box)
        np.save(f"{out}_{rank}_scales.npy", np.array(
            [(a, b, m, f) for a, sc in enumerate(scales) for b, (m, f) in sc.items()]))
    finally:
        dist.destroy_process_group()


def test_rank_exchange_gloo_two_ranks(tmp_path):
    import socket

    import torch.multiprocessing as mp
    R, n_att = 8, 9
    T = np.geomspace(280.0, 450.0, R)
    owner = replicas.partition_boxes(np.arange(R) * 100 + 600, 2)
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    out = str(tmp_path / "slots")
    mp.start_processes(_rank_main, args=(2, port, T, owner, n_att, out), nprocs=2,
                       join=True, start_method="spawn")
    # single process reference
    slot = np.arange(R, dtype=np.int32)
    want_scales = {}
    for a in range(n_att):
        U = np.array([_potens(b, a) for b in range(R)])
        slot, vm, vf = replicas.exchange_decision(T, U, slot, a, 99)
        for b in range(R):
            want_scales[(a, b)] = (vm[b], vf[b])
    for rank in range(2):
        assert np.array_equal(np.load(f"{out}_{rank}.npy"), slot)
        for a, b, m, f in np.load(f"{out}_{rank}_scales.npy"):
            assert owner[int(b)] == rank
            wm, wf = want_scales[(int(a), int(b))]
            assert int(m) == wm and (wm == 0 or f == wf)
