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
