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


def device_to_oracle(t, names):
    """A device tensor (itensor_gb300.Tensor) as an oracle BSTensor; QN slot k is `names[k]`."""
    from oracle.blocksparse import BSTensor, Index as OIndex
    inds = []
    for I in t.inds:
        secs = []
        for q, d in zip(I.qns, I.dims):
            items = [(names[k], int(q[k]), int(I.mods[k])) for k in range(len(names)) if I.mods[k] != 0]
            secs.append((QN(*items), int(d)))
        inds.append(OIndex(secs, dir=I.dir, id=str(I.id), plev=I.plev))  # fixture ids are strings
    X = BSTensor(inds)
    coords, offs = t.blocks()
    data = t.numpy()
    for c, o in zip(coords.reshape(len(offs), -1) if len(offs) else [], offs):
        c = tuple(int(x) for x in c)
        shp = X.block_shape(c)
        n = int(np.prod(shp))
        X.blocks[c] = np.reshape(data[o:o + n], shp, order="F").copy(order="F")
    return X


def workload_to_oracle(t):
    """A synthetic workload tensor (itensor_gb300.workloads form: Sz in QN slot 0)
    as an oracle BSTensor holding the same bytes."""
    from oracle.blocksparse import BSTensor, Index as OIndex
    inds = [OIndex([(QN(("Sz", q, 1)), d) for q, d in zip(I["qn"], I["dims"])], dir=I["dir"], id=str(I["id"]),
                   plev=I["plev"]) for I in t["inds"]]
    X = BSTensor(inds)
    off = 0
    for c in t["coords"]:
        c = tuple(int(x) for x in c)
        shp = X.block_shape(c)
        n = int(np.prod(shp))
        X.blocks[c] = np.reshape(t["data"][off:off + n], shp, order="F").copy(order="F")
        off += n
    return X


def check_dmrg_record(res, ref, names, energy_tol=1e-10, trunc_tol=1e-12):
    """A device DMRG result against a recorded reference run: final energy and
    every bond step's energy within energy_tol, truncation errors within
    trunc_tol, kept dimensions exact; final link layouts (arrow, QN sectors and
    sizes) exact. QN slot k of the device indices is `names[k]`."""
    assert abs(res.energy - ref["energy"]) < energy_tol, (res.energy, ref["energy"])
    assert len(res.bonds) == len(ref["bonds"])
    for a, b in zip(res.bonds, ref["bonds"]):
        assert tuple(a[:3]) == tuple(b[:3])
        assert abs(a[3] - b[3]) < energy_tol, (a, b)
        assert abs(a[4] - b[4]) < trunc_tol, (a, b)
        assert a[5] == b[5], (a, b)
    assert len(res.links) == len(ref["links"])
    for (dr, qn, dims), r in zip(res.links, ref["links"]):
        assert dr == r["dir"]
        got = [(tuple(sorted((names[k], int(q[k])) for k in range(len(names)) if q[k] != 0)), int(d))
               for q, d in zip(qn, dims)]
        assert got == json_sectors(r)


def mps_energy(psi, W):
    """<psi|H|psi> / <psi|psi> of an MPS (oracle BSTensors) under an MPO (oracle
    BSTensors): the site of tensor j is the index it shares with W[j]."""
    from oracle.blocksparse import contract
    E = nrm = None
    for A, Wj in zip(psi, W):
        site_ids = {I.id for I in Wj.inds}
        links = {I.id for I in A.inds if I.id not in site_ids}
        Ad_all = A.dag().prime()
        Ad_links = A.dag().prime(which=links)
        E = contract(contract(contract(E, A) if E is not None else A, Wj), Ad_all)
        nrm = contract(contract(nrm, A) if nrm is not None else A, Ad_links)
    return float(E.scalar) / float(nrm.scalar)
