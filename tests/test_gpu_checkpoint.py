"""Checkpoints of device tensors and CTM environments (the fields of the reference's
StorageType_contiguous::serialize and CTM::serialize): byte round trips and a resumed
CTM run that continues exactly like the uninterrupted one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tensor(sym, pairs_a, pairs_b, seed):
    from xped_gb300 import Basis, Tensor
    rng = np.random.default_rng(seed)
    A, B = Basis.from_pairs(sym, pairs_a), Basis.from_pairs(sym, pairs_b)
    t = Tensor.zeros([A, B], [A.conj(), B])
    t.set_data(rng.standard_normal(t.size))
    return t


@pytest.mark.parametrize("sym,pa,pb", [
    ("U1", [(-1, 2), (0, 3), (1, 2)], [(-2, 1), (1, 2)]),
    ("fZ2", [(0, 2), (1, 3)], [(1, 2), (0, 1)]),
    ("SU2", [(1, 2), (2, 1), (3, 1)], [(1, 1), (2, 2)]),
])
def test_tensor_round_trip(sym, pa, pb):
    from xped_gb300 import ensure_device
    from xped_gb300.tensor import Tensor
    ensure_device(0)
    t = _tensor(sym, pa, pb, 3)
    u = Tensor.from_bytes(t.to_bytes())
    assert u.sectors() == t.sectors()
    assert u.rank == t.rank
    assert np.array_equal(u.data(), t.data())
    # push_back-ordered outputs (tSVD) keep their storage order
    U, S, V, *_ = t.tSVD(5, 1e-10)
    for x in (U, S, V):
        y = Tensor.from_bytes(x.to_bytes())
        assert y.sectors() == x.sectors() and np.array_equal(y.data(), x.data())


def test_corrupt_checkpoint_is_rejected():
    from xped_gb300 import XgbError, ensure_device
    from xped_gb300.tensor import Tensor
    ensure_device(0)
    b = bytearray(_tensor("U1", [(-1, 2), (0, 3)], [(0, 2)], 1).to_bytes())
    with pytest.raises(XgbError):
        Tensor.from_bytes(bytes(b[:-8]))   # truncated
    b[0:4] = b"XXXX"
    with pytest.raises(XgbError):
        Tensor.from_bytes(bytes(b))        # wrong record


def test_resumed_ctm_continues_identically():
    from xped_gb300 import CTM, Basis, Tensor, ensure_device
    ensure_device(0)
    aux = Basis.from_pairs("U1", [(-1, 1), (0, 2), (1, 1)])
    phys = Basis.from_pairs("U1", [(-1, 1), (1, 1)])
    A = Tensor.zeros([aux, aux], [aux, aux, phys])
    A.set_data(np.random.default_rng(7).standard_normal(A.size))
    run = CTM(A, 12).init()
    run.grow_all()
    blob = run.to_bytes()
    resumed = CTM.from_bytes(A, blob)
    run.grow_all()
    resumed.grow_all()
    for name in ("C1", "C2", "C3", "C4", "T1", "T2", "T3", "T4"):
        a, b = run.get(name), resumed.get(name)
        assert a.sectors() == b.sectors()
        assert np.array_equal(a.data(), b.data())
