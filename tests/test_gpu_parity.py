"""Parity of the sm_103a path (called through the C-ABI) with the reference's
golden fixtures and with the CPU oracle. GPU only.

Tolerances: contractions 1e-12 relative to the largest output entry; DMRG
energies 1e-10; truncation errors 1e-12; kept dimensions and QN layouts exact.
"""
import numpy as np
import pytest

from helpers import (T, gpu_tensor, gpu_layout_matches, qn_names, json_sectors, model_from_json)

pytestmark = pytest.mark.gpu

CONTRACT_RTOL = 1e-12
ENERGY_TOL = 1e-10


@pytest.fixture(scope="module")
def ctx():
    import itensor_gb300 as itg
    import itensor_gb300.build as b
    b.build()
    c = itg.Context(0)
    yield c
    c.close()


def _relerr(x, ref):
    ref = np.asarray(ref, np.float64)
    if ref.size == 0:
        return 0.0
    return float(np.max(np.abs(np.asarray(x) - ref)) / max(1.0, np.max(np.abs(ref))))


@pytest.mark.parametrize("prec", [0, 1])
def test_contract_golden(ctx, golden, prec):
    d = golden("contract")
    names = qn_names(d)
    for c in d["cases"]:
        A, B = gpu_tensor(ctx, c["A"], names), gpu_tensor(ctx, c["B"], names)
        Cg = ctx.contract(A, B, precision=prec)
        ref = c["C"]
        # split form: ~2^-42 of row/column maxima per product (6 BF16 slices)
        tol = CONTRACT_RTOL if prec == 0 else 1e-11
        if not ref["inds"]:
            val = ref["data"][0] if ref.get("data") else ref.get("scalar", 0.0)
            assert abs(Cg.scalar() - val) <= tol * max(1, abs(val)), c["name"]
            continue
        same_inds, same_blocks = gpu_layout_matches(Cg, ref)
        assert same_inds and same_blocks, c["name"]
        assert _relerr(Cg.numpy(), ref["data"]) <= tol, c["name"]


def test_plan_exec_raw_boundary(ctx, golden):
    """itg_contract_plan/itg_contract_exec: layouts + Lind/Rind labels + device pointers."""
    d = golden("contract")
    names = qn_names(d)
    c = [x for x in d["cases"] if x["name"] == "perm2"][0]
    A, B = gpu_tensor(ctx, c["A"], names), gpu_tensor(ctx, c["B"], names)
    ia = [(int(x["id"]), x["plev"]) for x in c["A"]["inds"]]
    ib = [(int(x["id"]), x["plev"]) for x in c["B"]["inds"]]
    la, lb = [], []
    nxt = 1
    for k in ia:
        if k in ib:
            la.append(-(ib.index(k) + 1))
        else:
            la.append(nxt); nxt += 1
    for k in ib:
        lb.append(-(ib.index(k) + 1) if k in ia else 100 + len(lb))
    dimsA = [[s[1] for s in x["sectors"]] for x in c["A"]["inds"]]
    dimsB = [[s[1] for s in x["sectors"]] for x in c["B"]["inds"]]
    plan = ctx.plan((dimsA, c["A"]["blocks"]), la, (dimsB, c["B"]["blocks"]), lb)
    coords, offs, size = plan.output()
    assert coords.tolist() == c["C"]["blocks"]
    assert offs.tolist() == c["C"]["offsets"]
    import itensor_gb300 as itg
    out = ctx.tensor(gpu_tensor(ctx, c["C"], names).inds, np.asarray(c["C"]["blocks"], np.int32).reshape(-1))
    ctx.contract_exec(plan, A.device_ptr(), B.device_ptr(), out.device_ptr(), precision=itg.PREC_F64)
    assert _relerr(out.numpy(), c["C"]["data"]) <= CONTRACT_RTOL


def _op(ctx, c, names):
    L = gpu_tensor(ctx, c["L"], names) if c["L"]["inds"] else None
    R = gpu_tensor(ctx, c["R"], names) if c["R"]["inds"] else None
    return L, gpu_tensor(ctx, c["W1"], names), gpu_tensor(ctx, c["W2"], names), R


@pytest.mark.parametrize("prec", [0, 1])
def test_heff_golden(ctx, golden, prec):
    d = golden("heff")
    names = qn_names(d)
    for c in d["cases"]:
        if "Hphi" not in c:
            continue
        L, W1, W2, R = _op(ctx, c, names)
        phi = gpu_tensor(ctx, c["phi"], names)
        out = ctx.heff_apply(L, W1, W2, R, phi, precision=prec)
        same_inds, same_blocks = gpu_layout_matches(out, c["Hphi"])
        assert same_inds and same_blocks, c["name"]
        assert _relerr(out.numpy(), c["Hphi"]["data"]) <= (CONTRACT_RTOL if prec == 0 else 1e-11), c["name"]


def test_davidson_golden(ctx, golden):
    d = golden("heff")
    names = qn_names(d)
    for c in d["cases"]:
        for key, mi in (("davidson_niter2", 2), ("davidson_niter9", 9)):
            if key not in c:
                continue
            L, W1, W2, R = _op(ctx, c, names)
            phi = gpu_tensor(ctx, c["phi"], names)
            e, v = ctx.davidson(L, W1, W2, R, phi, maxiter=mi)
            assert abs(e - c[key]["energy"]) < 1e-12, (c["name"], key, e)
            # compare the Ritz vector on the reference's blocks (others are zero)
            ref = T(c[key]["phi"])
            coords, offs = v.blocks()
            data = v.numpy()
            got = {tuple(cc): data[o:o + int(np.prod(ref.block_shape(tuple(cc))))] for cc, o in zip(coords.tolist(), offs)}
            for cc, blk in ref.blocks.items():
                assert np.max(np.abs(got[cc] - blk.reshape(-1, order="F"))) < 1e-10
    # reference unit value: 4-site Heisenberg, E = -0.95710678118
    c = [x for x in d["cases"] if x["name"] == "heis4_b2"][0]
    L, W1, W2, R = _op(ctx, c, names)
    e, _ = ctx.davidson(L, W1, W2, R, gpu_tensor(ctx, c["phi"], names), maxiter=9)
    assert abs(e + 0.95710678118) < 1e-10


def test_denmat_golden(ctx, golden):
    from oracle.blocksparse import contract as ocontract
    d = golden("bondsplit")
    names = qn_names(d)
    for c in d["cases"]:
        if c["usesvd"]:
            continue
        AA, A, B = (gpu_tensor(ctx, c[k], names) for k in ("AA", "A", "B"))
        Ao, Bo, eigs, te = ctx.denmat_decomp(AA, A, B, c["fromleft"], c["cutoff"], c["maxdim"], c["mindim"],
                                             normalize=False)
        e = np.asarray(c["spec"]["eigs"])
        assert len(eigs) == len(e), c["name"]
        assert np.max(np.abs(eigs - e)) < 1e-12 * max(1.0, e[0]), c["name"]
        assert abs(te - c["spec"]["truncerr"]) < 1e-12 * max(1.0, e[0])
        link = [I for I in Ao.inds if any(I.same(J) for J in Bo.inds)][0]
        ref_secs = json_sectors(c["link"])
        assert [int(x) for x in link.dims] == [dd for _, dd in ref_secs], c["name"]
        assert link.dir == c["link"]["dir"]
        # A*B reconstructs the reference's (gauge-free) product
        AB = ctx.contract(Ao, Bo)
        from helpers import layout_and_maxerr
        from oracle.blocksparse import BSTensor
        ref = T(c["AB"])
        coords, offs = AB.blocks()
        inds_map = [[(int(x["id"]), x["plev"]) for x in c["AB"]["inds"]].index((I.id, I.plev)) for I in AB.inds]
        data = AB.numpy()
        for cc, o in zip(coords.tolist(), offs):
            rc = [0] * len(cc)
            for k, p in enumerate(inds_map):
                rc[p] = cc[k]
            blk_ref = ref.blocks.get(tuple(rc))
            shp = tuple(int(AB.inds[k].dims[cc[k]]) for k in range(len(cc)))
            blk = data[o:o + int(np.prod(shp))].reshape(shp, order="F")
            if blk_ref is None:
                assert np.max(np.abs(blk)) < 1e-12
            else:
                assert np.max(np.abs(np.transpose(blk_ref, inds_map) - blk)) < 1e-11 * max(1, np.abs(ref.flat()).max())


@pytest.mark.parametrize("name", ["heis20", "heis20_noise", "xxz16", "j1j2_16", "tfi16", "hubbard8", "hubbard4x2"])
def test_dmrg_golden(ctx, golden, name):
    c = [x for x in golden("dmrg")["cases"] if x["name"] == name][0]
    m = c["model"]
    if m["type"] in ("heisenberg", "xxz"):
        model = dict(type=0, N=c["N"], J=m["J"], Jz=m["Jz"])
    elif m["type"] == "j1j2":
        model = dict(type=0, N=c["N"], J=1.0, Jz=1.0, J2=m["J2"])
    elif m["type"] == "tfi":
        model = dict(type=1, N=c["N"], h=m["h"])
    else:
        model = dict(type=2, Lx=m["Lx"], Ly=m["Ly"], t=m["t"], U=m["U"], yperiodic=int(m.get("yperiodic", False)))
    res = ctx.dmrg(model, c["sweeps"], precision=0)
    assert abs(res.energy - c["energy"]) < ENERGY_TOL
    assert len(res.bonds) == len(c["bonds"])
    # noise splits rho's SU(2) multiplets only by noise*drho, so rounding-level
    # changes move the kept vectors inside a multiplet: in the first, noisiest
    # sweep a bond's (2-iteration) Davidson energy moves by up to ~3e-8 between
    # summation orders (the oracle moves 3e-9 when rho changes by 1e-14), and a
    # truncation error by ~2e-12; the final energy and kept dims stay tight.
    noisy = any(s.get("noise", 0.0) > 0 for s in c["sweeps"])
    bond_tol, trunc_tol = (1e-7, 1e-11) if noisy else (ENERGY_TOL, 1e-12)
    for a, b in zip(res.bonds, c["bonds"]):
        assert tuple(a[:3]) == tuple(b[:3])
        assert abs(a[3] - b[3]) < bond_tol, (a, b)
        assert abs(a[4] - b[4]) < trunc_tol
        assert a[5] == b[5]
    for (dr, qn, dims), ref in zip(res.links, c["links"]):
        assert [int(x) for x in dims] == [d for _, d in ref["sectors"]]
        assert dr == ref["dir"]


def test_dmrg_ozaki_energy_within_1e9(ctx, golden):
    """Split-precision block GEMMs (6 BF16 slices) keep |dE| <= 1e-9 on the N=20 chain."""
    c = [x for x in golden("dmrg")["cases"] if x["name"] == "heis20"][0]
    res = ctx.dmrg(dict(type=0, N=20, J=1.0, Jz=1.0), c["sweeps"], precision=1)
    assert abs(res.energy - c["energy"]) <= 1e-9


def test_svd_split_golden(ctx, golden):
    """SVD route of the bond split against the reference's svd cases."""
    d = golden("bondsplit")
    names = qn_names(d)
    n = 0
    for c in d["cases"]:
        if not c["usesvd"]:
            continue
        n += 1
        AA, A, B = (gpu_tensor(ctx, c[k], names) for k in ("AA", "A", "B"))
        Ao, Bo, eigs, te = ctx.svd_split(AA, A, B, c["fromleft"], c["cutoff"], c["maxdim"], c["mindim"],
                                         normalize=False)
        e = np.asarray(c["spec"]["eigs"])
        assert len(eigs) == len(e), c["name"]
        assert np.max(np.abs(eigs - e)) < 1e-12 * max(1.0, e[0]), c["name"]
        assert abs(te - c["spec"]["truncerr"]) < 1e-12 * max(1.0, e[0])
        link = [I for I in Ao.inds if any(I.same(J) for J in Bo.inds)][0]
        assert [int(x) for x in link.dims] == [dd for _, dd in json_sectors(c["link"])], c["name"]
        # A*B reproduces the reference's truncated product
        AB = ctx.contract(Ao, Bo)
        ref = T(c["AB"])
        coords, offs = AB.blocks()
        pos = [[(int(x["id"]), x["plev"]) for x in c["AB"]["inds"]].index((I.id, I.plev)) for I in AB.inds]
        data = AB.numpy()
        scale = max(1.0, np.abs(ref.flat()).max())
        for cc, o in zip(coords.tolist(), offs):
            rc = [0] * len(cc)
            for k, p in enumerate(pos):
                rc[p] = cc[k]
            shp = tuple(int(AB.inds[k].dims[cc[k]]) for k in range(len(cc)))
            blk = data[o:o + int(np.prod(shp))].reshape(shp, order="F")
            ref_blk = ref.blocks.get(tuple(rc))
            err = np.max(np.abs(blk)) if ref_blk is None else np.max(np.abs(np.transpose(ref_blk, pos) - blk))
            assert err < 1e-11 * scale, (c["name"], err)
    assert n >= 2


def test_dmrg_svd_route_matches_oracle(ctx):
    """DMRG with the SVD bond split (UseSVD) against the CPU oracle's SVD route."""
    from oracle import models
    from oracle.dmrg import dmrg as odmrg
    sweeps = [dict(maxdim=m, mindim=1, cutoff=1e-13, niter=2, use_svd=1) for m in (8, 16, 24)]
    res = ctx.dmrg(dict(type=0, N=10, J=1.0, Jz=1.0), sweeps, precision=0)
    H = models.heisenberg(10)
    sites, W, _ = models.build_mpo(H)
    psi = models.product_mps(sites, H.st, ["Up" if i % 2 == 0 else "Dn" for i in range(10)])
    E, _, recs = odmrg(W, psi, sweeps, usesvd=True)
    assert abs(res.energy - E) < 1e-10
    for a, b in zip(res.bonds, recs):
        assert abs(a[3] - b[3]) < 1e-10
        assert a[5] == b[5]


def test_dmrg_noise_matches_oracle(ctx):
    """Noise term on a fermionic MPO (Hubbard 4x2, Jordan-Wigner strings in the
    channels) against the CPU oracle's deltaRho."""
    from oracle import models
    from oracle.dmrg import dmrg as odmrg
    sweeps = [dict(maxdim=m, mindim=1, cutoff=1e-9, niter=2, noise=nz)
              for m, nz in ((8, 1e-5), (16, 1e-6), (24, 1e-7), (32, 0.0))]
    res = ctx.dmrg(dict(type=2, Lx=4, Ly=2, t=1.0, U=4.0, yperiodic=0), sweeps, precision=0)
    H = models.hubbard(4, 2, 1.0, 4.0)
    sites, W, _ = models.build_mpo(H)
    labels = ["Up" if i % 2 == 0 else "Dn" for i in range(8)]
    psi = models.product_mps(sites, H.st, labels)
    E, _, recs = odmrg(W, psi, sweeps)
    assert abs(res.energy - E) < 1e-10
    assert len(res.bonds) == len(recs)
    for a, b in zip(res.bonds, recs):
        assert tuple(a[:3]) == tuple(b[:3])
        assert abs(a[3] - b[3]) < 1e-8, (a, b)
        assert abs(a[4] - b[4]) < 1e-11
        assert a[5] == b[5]


def test_denmat_noise_single_bond(ctx):
    """One noisy density-matrix split, from the left and from the right, against
    the oracle: trace-normalised eigenvalues and truncation error."""
    from oracle import models
    from oracle.blocksparse import contract as ocontract
    from oracle.dmrg import LocalMPO, dmrg as odmrg
    from oracle.decomp import denmat_decomp as odenmat
    from helpers import to_gpu
    N = 6
    H = models.heisenberg(N)
    sites, W, _ = models.build_mpo(H)
    psi = models.product_mps(sites, H.st, ["Up" if i % 2 == 0 else "Dn" for i in range(N)])
    _, psi, _ = odmrg(W, psi, [dict(maxdim=4, mindim=1, cutoff=1e-12, niter=2)])
    for b in (1, 3, 5):  # chain end (no L), middle, other end (no R)
        op = LocalMPO(W).position(b, psi)
        A, B = psi[b - 1], psi[b]
        AA = ocontract(A, B)
        names = ["Sz"]
        g = lambda X: to_gpu(ctx, X, names) if X is not None else None
        for fromleft in (True, False):
            _, _, probs, te = odenmat(AA, A, B, fromleft, 3, 1, 1e-12, normalize=False, noise=1e-3, op=op)
            _, _, eigs, gte = ctx.denmat_decomp(g(AA), g(A), g(B), fromleft, 1e-12, 3, 1, normalize=False,
                                                noise=1e-3, op=(g(op.L), g(op.W1), g(op.W2), g(op.R)))
            assert len(eigs) == len(probs), (b, fromleft)
            assert np.max(np.abs(eigs - probs)) < 1e-13, (b, fromleft)
            assert abs(gte - te) < 1e-13, (b, fromleft)


def _big_split_problem(seed=3):
    """A two-site tensor whose density-matrix blocks are several hundred wide."""
    from oracle.blocksparse import BSTensor, Index, QN, OUT, IN
    rng = np.random.default_rng(seed)
    q = lambda v: QN(("Sz", v, 1))
    l = Index([(q(-4), 90), (q(-2), 200), (q(0), 260), (q(2), 200), (q(4), 90)], dir=IN, tags="l")
    s1 = Index([(q(1), 1), (q(-1), 1)], dir=OUT, tags="s1")
    s2 = Index([(q(1), 1), (q(-1), 1)], dir=OUT, tags="s2")
    r = Index([(q(-2), 30), (q(0), 60), (q(2), 30)], dir=OUT, tags="r")
    a = Index([(q(0), 4), (q(2), 4), (q(-2), 4)], dir=OUT, tags="a")
    AA = BSTensor.random([l, s1, s2, r], QN(("Sz", 0, 1)), rng)
    # a decaying spectrum, as in a density matrix: scale the right index's columns
    for c, b in AA.blocks.items():
        b *= np.exp(-np.arange(b.shape[3]) / 6.0)[None, None, None, :]
    A = BSTensor.random([l, s1, a], QN(("Sz", 0, 1)), rng)
    B = BSTensor.random([a.dag(), s2, r], QN(("Sz", 0, 1)), rng)
    return AA, A, B


def _small_split_problem(seed=5):
    """A two-site tensor whose density-matrix blocks have 1, 2, 3, 15, 16 and 3
    rows from the left (combined l, s1 sectors) and several sizes from the right."""
    from oracle.blocksparse import BSTensor, Index, QN, OUT, IN
    rng = np.random.default_rng(seed)
    q = lambda v: QN(("Sz", v, 1))
    l = Index([(q(-4), 1), (q(-2), 1), (q(0), 2), (q(2), 13), (q(4), 3)], dir=IN, tags="l")
    s1 = Index([(q(1), 1), (q(-1), 1)], dir=OUT, tags="s1")
    s2 = Index([(q(1), 1), (q(-1), 1)], dir=OUT, tags="s2")
    r = Index([(q(-2), 5), (q(0), 9), (q(2), 7)], dir=OUT, tags="r")
    a = Index([(q(0), 2), (q(2), 2), (q(-2), 2)], dir=OUT, tags="a")
    AA = BSTensor.random([l, s1, s2, r], QN(("Sz", 0, 1)), rng)
    A = BSTensor.random([l, s1, a], QN(("Sz", 0, 1)), rng)
    B = BSTensor.random([a.dag(), s2, r], QN(("Sz", 0, 1)), rng)
    return AA, A, B


def test_denmat_small_blocks(ctx, monkeypatch):
    """Density-matrix blocks of 1 to 16 rows through the small-block Jacobi
    (the tridiagonal threshold raised past 16, so a 16-row block takes it too)
    against the oracle's eigh: every eigenvalue, the truncation error, and the
    kept weight of A' B'."""
    from oracle.decomp import denmat_decomp as odenmat
    from helpers import to_gpu
    monkeypatch.setenv("ITG_EIG_TRI_MIN", "17")
    AA, A, B = _small_split_problem()
    names = ["Sz"]
    for fromleft in (True, False):
        _, _, probs, te = odenmat(AA, A, B, fromleft, 100, 1, 1e-14, normalize=False)
        gA, gB, eigs, gte = ctx.denmat_decomp(to_gpu(ctx, AA, names), to_gpu(ctx, A, names), to_gpu(ctx, B, names),
                                              fromleft, 1e-14, 100, 1, normalize=False)
        assert len(eigs) == len(probs), fromleft
        assert np.max(np.abs(eigs - probs)) < 1e-13 * probs[0], fromleft
        assert abs(gte - te) < 1e-13, fromleft
        AB = ctx.contract(gA, gB)
        nrm2 = float(np.sum(AB.numpy() ** 2))
        assert abs(nrm2 - np.sum(probs)) < 1e-12 * np.sum(probs)


@pytest.mark.parametrize("tri_min", ["64", "300", "100000"])
def test_denmat_large_blocks(ctx, tri_min, monkeypatch):
    """Density-matrix blocks of 90..460 rows through the tridiagonal eigensolver
    (and, for comparison, the Jacobi one) against the oracle's eigh."""
    from oracle.decomp import denmat_decomp as odenmat
    from helpers import to_gpu
    monkeypatch.setenv("ITG_EIG_TRI_MIN", tri_min)
    AA, A, B = _big_split_problem()
    names = ["Sz"]
    for fromleft in (True, False):
        _, _, probs, te = odenmat(AA, A, B, fromleft, 400, 1, 1e-10, normalize=False)
        gA, gB, eigs, gte = ctx.denmat_decomp(to_gpu(ctx, AA, names), to_gpu(ctx, A, names), to_gpu(ctx, B, names),
                                              fromleft, 1e-10, 400, 1, normalize=False)
        assert len(eigs) == len(probs), fromleft
        assert np.max(np.abs(eigs - probs)) < 1e-12 * probs[0], fromleft
        assert abs(gte - te) < 1e-12, fromleft
        # A' B' reproduces the truncated product: compare norms of the kept weight
        AB = ctx.contract(gA, gB)
        nrm2 = float(np.sum(AB.numpy() ** 2))
        assert abs(nrm2 - np.sum(probs)) < 1e-10 * np.sum(probs)


@pytest.mark.parametrize("pairs", ["0", "1000000"])
def test_planners_agree(golden, pairs, monkeypatch):
    """Every plan by the device planner (threshold 0), then every plan by the
    host one: the contraction fixtures and a DMRG run match the reference
    either way (block lists, offsets and index order exact)."""
    import itensor_gb300 as itg
    monkeypatch.setenv("ITG_HOST_PLAN_PAIRS", pairs)
    c = itg.Context(0)  # a fresh plan cache
    try:
        test_contract_golden(c, golden, 0)
        test_dmrg_golden(c, golden, "hubbard4x2")
    finally:
        c.close()


@pytest.mark.parametrize("name", ["heis20", "hubbard4x2", "heis20_noise"])
def test_dmrg_golden_tridiagonal_eigh(ctx, golden, name, monkeypatch):
    """Every density-matrix block through the tridiagonal path (down to 1x1)."""
    monkeypatch.setenv("ITG_EIG_TRI_MIN", "1")
    test_dmrg_golden(ctx, golden, name)


@pytest.mark.parametrize("prec", [0, 1])
def test_dmrg_excited_golden(ctx, golden, prec):
    """Excited-state DMRG through the C-ABI (ground state, then H + 20 |psi0><psi0|)
    against the reference's N=12 Heisenberg fixture; FP64 to 1e-10 per bond, the
    split form to 1e-9 on the energies."""
    c = [x for x in golden("dmrg")["cases"] if x["name"] == "heis12_excited"][0]
    res = ctx.dmrg_states(dict(type=0, N=c["N"], J=1.0, Jz=1.0), [c["ground_sweeps"], c["sweeps"]], c["weight"],
                          precision=prec)
    tol = ENERGY_TOL if prec == 0 else 1e-9
    assert abs(res[0].energy - c["ground_energy"]) < tol
    assert abs(res[1].energy - c["energy"]) < tol
    if prec == 0:
        assert len(res[1].bonds) == len(c["bonds"])
        for a, b in zip(res[1].bonds, c["bonds"]):
            assert tuple(a[:3]) == tuple(b[:3])
            assert abs(a[3] - b[3]) < ENERGY_TOL, (a, b)
            assert abs(a[4] - b[4]) < 1e-12
            assert a[5] == b[5]
        for (dr, qn, dims), ref in zip(res[1].links, c["links"]):
            assert [int(x) for x in dims] == [d for _, d in ref["sectors"]]


def test_dmrg_mpo_sum_golden(ctx, golden):
    """DMRG of a sum of two MPOs (the J1-J2 chain as nearest- plus next-nearest-
    neighbour MPOs) through the C-ABI against the reference's LocalMPOSet run."""
    c = [x for x in golden("dmrg")["cases"] if x["name"] == "j1j2_16_set"][0]
    N, J2 = c["N"], c["model"]["J2"]
    res = ctx.dmrg_sum([dict(type=0, N=N, J=1.0, Jz=1.0), dict(type=0, N=N, J=0.0, Jz=0.0, J2=J2)], c["sweeps"],
                       precision=0)
    assert abs(res.energy - c["energy"]) < ENERGY_TOL
    assert len(res.bonds) == len(c["bonds"])
    for a, b in zip(res.bonds, c["bonds"]):
        assert tuple(a[:3]) == tuple(b[:3])
        assert abs(a[3] - b[3]) < ENERGY_TOL, (a, b)
        assert abs(a[4] - b[4]) < 1e-12
        assert a[5] == b[5]


def test_dmrg_mpo_sum_noise_matches_oracle(ctx):
    """The noise term of a sum of MPOs (every MPO's deltaRho added, LocalMPOSet)
    against the oracle on the same MPOs: the J1-J2 chain N=10 as two MPOs."""
    from oracle import models
    from oracle.dmrg import dmrg as odmrg
    N, J2 = 10, 0.3
    sweeps = [dict(maxdim=m, mindim=1, cutoff=1e-10, niter=2, noise=nz)
              for m, nz in ((8, 1e-5), (16, 1e-6), (24, 0.0))]
    res = ctx.dmrg_sum([dict(type=0, N=N, J=1.0, Jz=1.0), dict(type=0, N=N, J=0.0, Jz=0.0, J2=J2)], sweeps,
                       precision=0)
    H1 = models.heisenberg(N)
    H2 = models.heisenberg(N, J=0.0, J2=J2)
    H2.two = [t for t in H2.two if t[0] != 0.0]
    sites, W1, _ = models.build_mpo(H1)
    _, W2, _ = models.build_mpo(H2, sites=sites)
    psi = models.product_mps(sites, H1.st, ["Up" if i % 2 == 0 else "Dn" for i in range(N)])
    E, _, recs = odmrg([W1, W2], psi, sweeps)
    assert abs(res.energy - E) < 1e-10
    assert len(res.bonds) == len(recs)
    for a, b in zip(res.bonds, recs):
        assert tuple(a[:3]) == tuple(b[:3])
        assert abs(a[3] - b[3]) < 1e-7, (a, b)
        assert abs(a[4] - b[4]) < 1e-11
        assert a[5] == b[5]
