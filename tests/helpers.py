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


# ---------------------------------------------------------------- fixtures -> device tensors
def qn_names(obj, acc=None):
    """All QN names appearing in a fixture (sorted), used as the slot order."""
    if acc is None:
        acc = set()
    if isinstance(obj, dict):
        if "sectors" in obj and "id" in obj:
            for q, _ in obj["sectors"]:
                for name, _, _ in q:
                    acc.add(name)
        for v in obj.values():
            qn_names(v, acc)
    elif isinstance(obj, list):
        for v in obj:
            qn_names(v, acc)
    return sorted(acc)


def gpu_index(j, names):
    import itensor_gb300 as itg
    qns, mods = [], [0, 0, 0, 0]
    for q, d in j["sectors"]:
        row = [0, 0, 0, 0]
        for name, v, m in q:
            k = names.index(name)
            row[k] = v
            mods[k] = m
        qns.append(row)
    for k in range(len(names)):
        if mods[k] == 0:
            mods[k] = 1
    return itg.Index(int(j["id"]), j["plev"], j["dir"], qns, [d for _, d in j["sectors"]], mods)


def gpu_tensor(ctx, j, names):
    inds = [gpu_index(x, names) for x in j["inds"]]
    if not inds:
        data = j.get("data") or [j.get("scalar", 0.0)]
        return ctx.tensor([], [], np.asarray(data, np.float64))
    return ctx.tensor(inds, np.asarray(j["blocks"], np.int32).reshape(-1), np.asarray(j["data"], np.float64))


def gpu_layout_matches(t, refj):
    """(same index order/ids, same blocks+offsets) of a device tensor against a fixture tensor."""
    inds = t.inds
    same_inds = [(I.id, I.plev, I.dir) for I in inds] == [(int(x["id"]), x["plev"], x["dir"]) for x in refj["inds"]]
    coords, offs = t.blocks()
    rb = np.asarray(refj["blocks"], np.int64).reshape(len(refj["blocks"]), -1) if refj["blocks"] else np.zeros((0, len(inds)))
    same_blocks = coords.shape[0] == rb.shape[0] and np.array_equal(coords.reshape(rb.shape), rb) and \
        list(offs) == list(refj["offsets"])
    return same_inds, same_blocks


def bst_json(X):
    """An oracle tensor in the fixture format (for uploading through gpu_tensor)."""
    inds = [dict(id=I.id, plev=I.plev, dir=I.dir, sectors=[[q.to_json(), d] for q, d in I.sectors])
            for I in X.inds]
    if not X.inds:
        return dict(inds=[], data=[float(X.scalar or 0.0)])
    blocks, offsets, data, off = [], [], [], 0
    for c in X.sorted_coords():
        b = X.blocks[c]
        blocks.append(list(c))
        offsets.append(off)
        data.extend(np.asarray(b).reshape(-1, order="F").tolist())
        off += b.size
    return dict(inds=inds, blocks=blocks, offsets=offsets, data=data)


def to_gpu(ctx, X, names):
    return gpu_tensor(ctx, bst_json(X), names)
