"""The allocation-free volume entry point against simp_evaluate.

simp_filter_volume_noalloc serves callers that cannot allocate device memory
where they evaluate a design's volume (an optimiser trying many designs per
iteration without device synchronisation, an application whose device memory
belongs to its own pool).  It must give the physical density and volume that
simp_evaluate reports for the same design: the density bit for bit (same
filter and projection arithmetic) and the volume within 1e-13 relative (the
partial sums are grouped differently).

The grids hold several 4096-element chunks with a ragged last chunk, and the
calls alternate between a larger and a smaller problem, so a call reads fewer
partials than the one before it wrote: the shared scratch array must leave
nothing behind between calls.  One problem has the Heaviside projection on,
where the physical density is the projected filtered field.  This file is
named to be collected last."""
import numpy as np
import pytest

from sparlab_gb300 import problems as P
from sparlab_gb300.topopt import GpuSimpProblem

pytestmark = pytest.mark.gpu


def _check(prob, x):
    import torch
    dev = torch.device("cuda", 0)
    prob.set_design(x)
    ev = prob.evaluate()
    xd = torch.from_numpy(x).to(dev)
    rho = torch.full((prob.ne,), -1.0, dtype=torch.float64, device=dev)
    vol = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    prob.filter_volume_noalloc(xd.data_ptr(), rho.data_ptr(), vol.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(rho.cpu().numpy(), ev.physical_density)
    v = float(vol.item())
    assert abs(v - ev.volume) <= 1e-13 * abs(ev.volume)
    return v


def test_noalloc_volume_matches_evaluate_across_sizes():
    # 48 x 24 x 23 = 26,496 elements: 7 chunks, the last one ragged;
    # 20 x 12 x 11 = 2,640 elements: a single partial chunk
    big = GpuSimpProblem(P.hex8_cantilever(48, 24, 23, 0.3, "noalloc_big"))
    small = GpuSimpProblem(P.hex8_cantilever(20, 12, 11, 0.3, "noalloc_small"))
    vols = []
    for seed in (3, 4):
        for prob in (big, small):
            x = P.SplitMix64(seed).uniform_array(prob.ne, 0.05, 1.0)
            vols.append(_check(prob, x))
    assert len(set(vols)) == 4


def test_noalloc_volume_matches_evaluate_with_projection():
    spec = P.hex8_cantilever(40, 20, 13, 0.3, "noalloc_projected")
    spec.projection, spec.beta_start, spec.beta_max = True, 4.0, 8.0
    prob = GpuSimpProblem(spec)
    for seed in (5, 6):
        x = P.SplitMix64(seed).uniform_array(prob.ne, 0.05, 1.0)
        _check(prob, x)


def test_noalloc_rejects_null_pointers():
    from sparlab_gb300._lib import SolverError
    spec = P.hex8_cantilever(8, 4, 4, 0.3, "noalloc_null")
    prob = GpuSimpProblem(spec)
    with pytest.raises(SolverError):
        prob.filter_volume_noalloc(0, 0, 0)
