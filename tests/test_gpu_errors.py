"""Malformed block metadata through the C-ABI is refused with ITG_ERR_ARG, as
the reference raises ITError for it (itensor/util/error.h:26-37): block
coordinates out of range, a block listed twice or out of storage order,
blocks of different flux in one tensor, a contracted index whose sector sizes
differ between the operands, and a caller MPO that does not act on the MPS's
sites. The context stays usable after each refusal."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_ARG = 1


@pytest.fixture(scope="module")
def ctx():
    import itensor_gb300 as itg
    import itensor_gb300.build as b
    b.build()
    c = itg.Context(0)
    yield c
    c.close()


def _sz(id_, qns, dims, dir_=1, plev=0):
    import itensor_gb300 as itg
    return itg.Index(id_, plev, dir_, [[q, 0, 0, 0] for q in qns], dims, [1, 0, 0, 0])


def _refused(fn):
    import itensor_gb300 as itg
    with pytest.raises(itg.ITGError) as e:
        fn()
    assert e.value.code == ERR_ARG, str(e.value)
    return str(e.value)


def test_tensor_metadata_errors(ctx):
    i = _sz(101, [-1, 1], [2, 3])
    j = _sz(102, [-1, 1], [2, 2], dir_=-1)
    # a valid matrix: blocks (0,0) and (1,1), divergence 0
    good = ctx.tensor([i, j], np.array([0, 0, 1, 1], np.int32), np.arange(10.0))
    assert good.numpy().shape == (10,)
    _refused(lambda: ctx.tensor([i, j], np.array([0, 0, 2, 1], np.int32), np.zeros(10)))        # out of range
    _refused(lambda: ctx.tensor([i, j], np.array([0, 0, 0, 0], np.int32), np.zeros(8)))         # listed twice
    _refused(lambda: ctx.tensor([i, j], np.array([1, 1, 0, 0], np.int32), np.zeros(10)))        # out of order
    msg = _refused(lambda: ctx.tensor([i, j], np.array([0, 0, 1, 0], np.int32), np.zeros(10)))  # two fluxes
    assert "flux" in msg
    # still usable
    assert np.array_equal(good.numpy(), np.arange(10.0))


def test_contraction_metadata_errors(ctx):
    # raw plan: the contracted label -1 has sector sizes (2, 3) on A and (2, 2) on B
    A = ([[2, 3], [4]], [[0, 0], [1, 0]])
    B = ([[2, 2], [5]], [[0, 0], [1, 0]])
    msg = _refused(lambda: ctx.plan(A, [-1, 1], B, [-1, 2]))
    assert "sector sizes" in msg
    ok = ctx.plan(A, [-1, 1], ([[2, 3], [5]], [[0, 0], [1, 0]]), [-1, 2])
    assert ok.output()[2] == 4 * 5


def test_dmrg_mpo_errors(ctx, golden):
    from helpers import gpu_tensor, qn_names
    d = golden("mpo_io")
    names = qn_names(d)
    c = [x for x in d["cases"] if x["run"]["name"] == "heis20"][0]
    W = [gpu_tensor(ctx, j, names) for j in c["W"]]
    psi0 = [gpu_tensor(ctx, j, names) for j in c["psi0"]]
    sw = [dict(maxdim=10, cutoff=1e-10, niter=2)]
    # MPO tensors shifted by one site: they act on the neighbours' site indices
    msg = _refused(lambda: ctx.dmrg_mpo(W[1:] + W[:1], psi0, sw))
    assert "site" in msg
    _refused(lambda: ctx.dmrg_mpo(W, psi0[:-1] + [psi0[0]], sw))   # the last MPS tensor on the wrong site
    res = ctx.dmrg_mpo(W, psi0, sw)  # the context still works
    assert res.energy < 0
