"""GPU parity of the alternative kernel forms: the z-marching slab form of the
FP32 and double-float operator kernels (tile_form = 1) and the register
line-segment form of the Kronecker passes (kron_form = 1) against the brick
and staged-line forms, on the 192x96x96 cantilever where the slab grid fills
the resident CTA slots (smaller grids keep bricks), and on a small mesh
against the oracle.

Both forms reorder no arithmetic inside an element product or a Kronecker
tap row; the FCG dot products of the slab form sum in a different order, so
end-to-end results agree to the solve tolerance: objective 1e-10 relative,
sensitivities 1e-9 of max|dfdx| at rtol 1e-12.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

M6 = (1e-9, 1.0, 1e-3, 1.0, 3.0, 1.0)


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def _run(n, x, tile_form, kron_form, **kw):
    from topopt_in_petsc_transient_gb300 import LinearElasticity
    le = LinearElasticity(*n, tile_form=tile_form, kron_form=kron_form, **kw)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    df = torch.zeros_like(xd)
    le.CompleteInitialState(xd, *M6)
    le.GenerateCheckPoints()
    fx = le.ComputeObjectiveSensitivities(df)
    out = (fx, df.cpu().numpy(), le.state(0, kw["tsc"] - 1))
    del le
    return out


@pytest.mark.parametrize("forms", [(1, 0), (0, 1), (1, 1)])
def test_kernel_forms_agree_on_the_192x96x96_cantilever(gpu, forms):
    n = (192, 96, 96)
    rng = np.random.default_rng(0x7A11)
    x = 0.12 + rng.uniform(-0.02, 0.02, int(np.prod(n)))
    kw = dict(nlvls=6, ncp=2, tsc=3, t1=0.015, objective=3, loadsignal=1, dalpha=0.0, dbeta=1e-3, mixed=True,
              rtol=1e-12, sens_fp32=False)
    f0, d0, u0 = _run(n, x, 0, 0, **kw)
    f1, d1, u1 = _run(n, x, *forms, **kw)
    assert abs(f1 - f0) <= 1e-10 * abs(f0), (f0, f1)
    assert _rel(d1, d0) < 1e-9
    assert _rel(u1, u0) < 1e-9


@pytest.mark.parametrize("forms", [(1, 1)])
def test_kernel_forms_match_oracle(gpu, forms):
    n = (16, 8, 8)
    kw = dict(ncp=2, tsc=4, t1=0.08, objective=5, loadsignal=1, dalpha=1e-3, dbeta=1e-3)
    rng = np.random.default_rng(44)
    x = 0.1 + 0.5 * rng.random(int(np.prod(n)))
    fx, df, _ = _run(n, x, *forms, nlvls=2, mixed=True, rtol=1e-12, sens_fp32=False, **kw)
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert rc == 0
    assert abs(fx - fx_r) <= 1e-10 * abs(fx_r)
    assert _rel(df, df_r) < 1e-9
