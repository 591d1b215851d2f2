"""Shared test helpers: build oracle tensors from fixtures and compare layouts."""
import numpy as np

from oracle.blocksparse import BSTensor, QN
from oracle import models


def T(j):
    return BSTensor.from_json(j)


def layout_and_maxerr(X, refj):
    """(same block list & offsets, max abs difference) of X against a fixture tensor."""
    R = T(refj)
    X = X.permuted_to(R.inds)
    cs, offs, tot = X.layout()
    rcs, roffs, rtot = R.layout()
    if cs != rcs or offs != roffs:
        return False, np.inf
    return True, (float(np.max(np.abs(X.flat() - R.flat()))) if tot else 0.0)


def link_sectors(I):
    return [(q.key(), d) for q, d in I.sectors]


def json_sectors(j):
    return [(QN.from_json(q).key(), d) for q, d in j["sectors"]]


def model_from_json(m, N):
    """(Hamiltonian, initial product-state labels) for a fixture model entry."""
    t = m["type"]
    neel = ["Up" if i % 2 == 0 else "Dn" for i in range(N)]
    if t in ("heisenberg", "xxz"):
        return models.heisenberg(N, J=m["J"], Jz=m["Jz"]), neel
    if t == "j1j2":
        return models.heisenberg(N, J2=m["J2"]), neel
    if t == "tfi":
        return models.tfi(N, m["h"]), ["Up"] * N
    if t == "hubbard":
        return models.hubbard(m["Lx"], m["Ly"], m["t"], m["U"], m.get("yperiodic", False)), neel
    raise ValueError(t)
