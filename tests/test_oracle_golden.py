"""Pins the CPU oracle against golden fixtures produced by the ITensor C++
reference (tests/golden/make_golden.py). CPU only."""
import numpy as np
import pytest

from oracle.blocksparse import contract, dot
from oracle.decomp import truncate, denmat_decomp, svd_split
from oracle.dmrg import LocalOp, davidson, dmrg
from oracle import models
from helpers import T, layout_and_maxerr, link_sectors, json_sectors, model_from_json

CONTRACT_RTOL = 1e-12   # contractions agree to 1e-12 relative
ENERGY_TOL = 1e-10      # DMRG energies agree to 1e-10


def test_contract_cases(golden):
    d = golden("contract")
    assert len(d["cases"]) >= 10
    for c in d["cases"]:
        A, B = T(c["A"]), T(c["B"])
        C = contract(A, B)
        R = T(c["C"])
        assert [(I.id, I.plev, I.dir) for I in C.inds] == [(I.id, I.plev, I.dir) for I in R.inds], c["name"]
        if R.scalar is not None:
            assert C.scalar == pytest.approx(R.scalar, rel=CONTRACT_RTOL)
            continue
        same, err = layout_and_maxerr(C, c["C"])
        assert same, c["name"]
        scale = max(1.0, float(np.max(np.abs(R.flat())))) if R.blocks else 1.0
        assert err <= CONTRACT_RTOL * scale, (c["name"], err)


def test_heff_and_davidson(golden):
    d = golden("heff")
    for c in d["cases"]:
        L = T(c["L"]) if c["L"]["inds"] else None
        R = T(c["R"]) if c["R"]["inds"] else None
        op = LocalOp(T(c["W1"]), T(c["W2"]), L, R)
        phi = T(c["phi"])
        if "Hphi" in c:
            same, err = layout_and_maxerr(op.product(phi), c["Hphi"])
            assert same and err < 1e-12 * max(1, np.abs(T(c["Hphi"]).flat()).max()), (c["name"], err)
        for key, mi in (("davidson_niter2", 2), ("davidson_niter9", 9)):
            if key in c:
                e, p = davidson(op, phi, maxiter=mi)
                assert abs(e - c[key]["energy"]) < 1e-12, (c["name"], key)
                same, err = layout_and_maxerr(p, c[key]["phi"])
                assert same and err < 1e-10, (c["name"], key, err)


def test_davidson_unit_value(golden):
    # reference unit test: 4-site Heisenberg, E = -0.95710678118
    c = [x for x in golden("heff")["cases"] if x["name"] == "heis4_b2"][0]
    op = LocalOp(T(c["W1"]), T(c["W2"]), T(c["L"]) if c["L"]["inds"] else None, T(c["R"]) if c["R"]["inds"] else None)
    e, _ = davidson(op, T(c["phi"]), maxiter=9)
    assert abs(e - (-0.95710678118)) < 1e-10


def test_truncate_bit_exact(golden):
    d = golden("truncate")
    for c in d["cases"]:
        P, te, lo, up, nd = truncate(c["P"], c["maxdim"], c["mindim"], c["cutoff"], c["absoluteCutoff"],
                                     c["doRelCutoff"], c["respectDegenerate"])
        assert list(P) == c["Pout"]
        assert (te, lo, up, nd) == (c["truncerr"], c["docut_lower"], c["docut_upper"], c["ndegen"])


def test_bond_split(golden):
    d = golden("bondsplit")
    for c in d["cases"]:
        AA, A, B = T(c["AA"]), T(c["A"]), T(c["B"])
        if c["usesvd"]:
            Uinds = [I for I in A.inds if B.find(I) < 0]
            Ao, Bo, probs, te = svd_split(AA, Uinds, c["maxdim"], c["mindim"], c["cutoff"],
                                          fromleft=c["fromleft"], normalize=False)
        else:
            Ao, Bo, probs, te = denmat_decomp(AA, A, B, c["fromleft"], c["maxdim"], c["mindim"], c["cutoff"],
                                              normalize=False)
        link = [I for I in Ao.inds if Bo.find(I) >= 0][0]
        assert link_sectors(link) == json_sectors(c["link"]), c["name"]
        assert link.dir == c["link"]["dir"]
        e = np.asarray(c["spec"]["eigs"])
        assert len(probs) == len(e)
        assert np.max(np.abs(probs - e)) < 1e-12 * max(1.0, e[0])
        assert abs(te - c["spec"]["truncerr"]) < 1e-12 * max(1.0, e[0])
        same, err = layout_and_maxerr(contract(Ao, Bo), c["AB"])
        assert same and err < 1e-12 * max(1.0, np.abs(T(c["AA"]).flat()).max()), (c["name"], err)


@pytest.mark.parametrize("name", ["heis20", "heis20_noise", "xxz16", "j1j2_16", "tfi16", "hubbard8", "hubbard4x2"])
def test_dmrg_energies_and_structure(golden, name):
    c = [x for x in golden("dmrg")["cases"] if x["name"] == name][0]
    N = c["N"]
    H, labels = model_from_json(c["model"], N)
    sites, W, _ = models.build_mpo(H)
    psi = models.product_mps(sites, H.st, labels)
    E, psi2, recs = dmrg(W, psi, c["sweeps"])
    assert abs(E - c["energy"]) < ENERGY_TOL
    ref = c["bonds"]
    assert len(recs) == len(ref)
    # With noise on, rho's SU(2) multiplets are split only by noise*drho, so a
    # rounding-level change of rho (1e-16) rotates the kept vectors inside a
    # multiplet and moves the next bond's (2-iteration) Davidson energy by
    # ~1e-9 and a truncation error by ~1e-12 (measured by rescaling the noise
    # by 1+1e-9); the final energy and the kept dims stay tight.
    noisy = any(s.get("noise", 0.0) > 0 for s in c["sweeps"])
    bond_tol, trunc_tol = (1e-8, 1e-11) if noisy else (ENERGY_TOL, 1e-12)
    for a, b in zip(recs, ref):
        assert tuple(a[:3]) == tuple(b[:3])
        assert abs(a[3] - b[3]) < bond_tol
        assert abs(a[4] - b[4]) < trunc_tol
        assert a[5] == b[5]          # kept states: exact
    for b in range(N - 1):
        link = [I for I in psi2[b].inds if psi2[b + 1].find(I) >= 0][0]
        assert link_sectors(link) == json_sectors(c["links"][b])
        assert link.dir == c["links"][b]["dir"]


def test_dmrg_excited_state(golden):
    """Excited-state DMRG (H + weight |psi0><psi0|, itensor/mps/dmrg.h:245-266):
    the ground state, then the first excited state against the reference."""
    c = [x for x in golden("dmrg")["cases"] if x["name"] == "heis12_excited"][0]
    N = c["N"]
    H, labels = model_from_json(c["model"], N)
    sites, W, _ = models.build_mpo(H)
    psi = models.product_mps(sites, H.st, labels)
    E0, psi0, _ = dmrg(W, psi, c["ground_sweeps"])
    assert abs(E0 - c["ground_energy"]) < ENERGY_TOL
    E1, psi1, recs = dmrg(W, psi, c["sweeps"], psis=[psi0], weight=c["weight"], site_ids=[I.id for I in sites])
    assert abs(E1 - c["energy"]) < ENERGY_TOL
    assert len(recs) == len(c["bonds"])
    for a, b in zip(recs, c["bonds"]):
        assert tuple(a[:3]) == tuple(b[:3])
        assert abs(a[3] - b[3]) < ENERGY_TOL
        assert abs(a[4] - b[4]) < 1e-12
        assert a[5] == b[5]


def test_dmrg_mpo_sum(golden):
    """dmrg with a sum of MPOs (LocalMPOSet, itensor/mps/localmposet.h): the J1-J2
    chain as nearest- plus next-nearest-neighbour MPOs, against the reference."""
    c = [x for x in golden("dmrg")["cases"] if x["name"] == "j1j2_16_set"][0]
    N = c["N"]
    H1 = models.heisenberg(N)
    H2 = models.heisenberg(N, J=0.0, J2=c["model"]["J2"])
    H2.two = [t for t in H2.two if t[0] != 0.0]
    sites, W1, _ = models.build_mpo(H1)
    _, W2, _ = models.build_mpo(H2, sites=sites)
    psi = models.product_mps(sites, H1.st, ["Up" if i % 2 == 0 else "Dn" for i in range(N)])
    E, psi2, recs = dmrg([W1, W2], psi, c["sweeps"])
    assert abs(E - c["energy"]) < ENERGY_TOL
    assert len(recs) == len(c["bonds"])
    for a, b in zip(recs, c["bonds"]):
        assert tuple(a[:3]) == tuple(b[:3])
        assert abs(a[3] - b[3]) < ENERGY_TOL
        assert abs(a[4] - b[4]) < 1e-12
        assert a[5] == b[5]
