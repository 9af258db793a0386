"""The tensor-core Gram product of the mixed SOMMG reduction (tcgen05,
gram.cuh) through the C ABI against FP64 products on the same data.

Bound: |G - G_fp64| <= 1e-6 * (|Q| |W|') entrywise.  The operands enter as
exact TF32 pieces (Q) and pieces good to about 2^-35 (W), and every piece
product is exact; what remains is the FP32 summation inside tensor memory
over one 32-value chunk (four MMAs) between readouts: random-signed sums
were measured at 1.6e-8 of sum |q w|, same-signed sums (the diagonal of an
orthonormal basis) lose about 6e-8 per accumulated MMA.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _gram(Q, W, n, kb):
    from topopt_in_petsc_transient_gb300 import _lib
    L = _lib.load()
    out = np.zeros((kb, kb))
    _lib.check(L.topo_sommg_gram_dev(Q.data_ptr(), Q.shape[1], W.data_ptr(), W.shape[1], n, kb, out.ctypes.data),
               "gram")
    return out


@pytest.mark.parametrize("kb,n,ldpad", [(32, 1000, 0), (5, 100003, 7), (32, 2_000_003, 0), (1, 33, 3), (17, 4096, 0)])
def test_tensor_core_gram_matches_fp64(gpu, kb, n, ldpad):
    g = torch.Generator(device="cuda").manual_seed(kb * 7919 + n)
    Q = torch.randn(kb, n + ldpad, dtype=torch.float32, device="cuda", generator=g)
    W = torch.randn(kb, n + ldpad, dtype=torch.float64, device="cuda", generator=g) * 1e3
    got = _gram(Q, W, n, kb)
    Qd = Q[:, :n].double()
    ref = (Qd @ W[:, :n].T).cpu().numpy()
    bound = (Qd.abs() @ W[:, :n].abs().T).cpu().numpy()
    err = np.abs(got - ref) / bound
    assert err.max() < 1e-6, err.max()


def test_tensor_core_gram_of_an_orthonormal_basis(gpu):
    # Q Q' of orthonormal rows: the diagonal sums are same-signed (the worst
    # case of the TMEM summation); the bound is 1e-6 of sum |q_a| |q_b| <= 1
    n, kb = 300_000, 32
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(n, kb, dtype=torch.float64, device="cuda", generator=g)
    Qd, _ = torch.linalg.qr(A)
    Q = Qd.T.contiguous().float()
    W = Q.double()
    got = _gram(Q, W, n, kb)
    ref = (W @ W.T).cpu().numpy()
    assert np.abs(got - ref).max() < 1e-6
    assert np.abs(got - np.eye(kb)).max() < 1e-6  # FP32 rounding of the rows


def test_gram_rejects_bad_sizes(gpu):
    from topopt_in_petsc_transient_gb300 import TopoError
    Q = torch.zeros(33, 64, dtype=torch.float32, device="cuda")
    W = torch.zeros(33, 64, dtype=torch.float64, device="cuda")
    with pytest.raises(TopoError):
        _gram(Q, W, 64, 33)
