"""Allocation-free volume constraint (topo_volume_constraint_noalloc_dev).

Collected last on purpose: it must give the same answers whether it runs alone
or after every other test has used the device.  It is compared with the
object-based entry point topo_le_volume_constraint_dev (LinearElasticity.cc:
1283-1296) on two calls in a row: gx to 1e-14 relative (the two sums use
different CTA partitions), dgdx bit-exact.
"""
import ctypes as C

import numpy as np
import pytest

from topopt_in_petsc_transient_gb300 import LinearElasticity, _lib

MAX_NEL = 8192 * 256 * 8


def _call(L, n, dg, x, volfrac):
    gx = C.c_double()
    rc = L.topo_volume_constraint_noalloc_dev(n, C.byref(gx), C.c_void_p(dg.data_ptr()), C.c_void_p(x.data_ptr()),
                                              volfrac)
    return rc, gx.value


@pytest.mark.gpu
@pytest.mark.parametrize("nel", [(24, 12, 12), (96, 48, 48)])
def test_noalloc_volume_constraint_matches_object_entry_point(gpu, nel):
    import torch
    L = _lib.load()
    n = int(np.prod(nel))
    rng = np.random.default_rng(11)
    x = torch.tensor(rng.uniform(0.0, 1.0, n), dtype=torch.float64, device=gpu)
    le = LinearElasticity(*nel, nlvls=2, ncp=1, tsc=2, t1=0.02)
    dg_ref = torch.zeros_like(x)
    gx_ref = le.VolumeConstraint(dg_ref, x, 0.12)
    assert abs(gx_ref - (x.mean().item() - 0.12)) < 1e-13
    for _ in range(2):
        dg = torch.full_like(x, -1.0)
        torch.cuda.synchronize()
        rc, gx = _call(L, n, dg, x, 0.12)
        assert rc == 0, L.topo_last_error()
        assert abs(gx - gx_ref) <= 1e-14 * max(1.0, abs(gx_ref))
        assert torch.equal(dg, dg_ref)


@pytest.mark.gpu
def test_noalloc_volume_constraint_rejects_sizes_beyond_its_scratch(gpu):
    import torch
    L = _lib.load()
    x = torch.zeros(16, dtype=torch.float64, device=gpu)
    dg = torch.zeros_like(x)
    for n in (0, MAX_NEL + 1):
        rc, _ = _call(L, n, dg, x, 0.5)
        assert rc == 1  # TOPO_ERR_ARG, before any launch
        assert b"outside 1..16777216" in L.topo_last_error()
    rc, gx = _call(L, 16, dg, x, 0.5)
    assert rc == 0 and gx == -0.5 and torch.all(dg == 1.0 / 16)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [MAX_NEL, MAX_NEL - 1, 16_777_216 - 8 * 256 * 8 + 1])
def test_noalloc_volume_constraint_at_the_scratch_limit(gpu, n):
    # the last partial slot in use (a full last CTA, and a last CTA with one
    # element or one thread's share missing), two calls in a row: gx against
    # torch's FP64 mean, dgdx exactly 1/n
    import torch
    L = _lib.load()
    g = torch.Generator(device=gpu).manual_seed(n)
    x = torch.rand(n, dtype=torch.float64, device=gpu, generator=g)
    ref = x.mean().item() - 0.12
    for _ in range(2):
        dg = torch.full_like(x, -1.0)
        torch.cuda.synchronize()
        rc, gx = _call(L, n, dg, x, 0.12)
        assert rc == 0, L.topo_last_error()
        assert abs(gx - ref) <= 1e-14 * max(1.0, abs(ref))
        assert bool(torch.all(dg == 1.0 / n))
