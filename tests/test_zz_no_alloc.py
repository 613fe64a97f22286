"""The allocation-free volume entry point against simp_evaluate.

simp_filter_volume_noalloc serves callers that cannot allocate device memory
where they evaluate a design's volume (an optimiser trying many designs per
iteration without device synchronisation, an application whose device memory
belongs to its own pool).  It must give the physical density and volume that
simp_evaluate reports for the same design: the density bit for bit (same
filter arithmetic) and the volume within 1e-13 relative (the partial sums
are grouped differently).  Two calls in a row check that the shared scratch
array leaves nothing behind between calls.  This file is named to be
collected last."""
import ctypes as C

import numpy as np
import pytest

from sparlab_gb300 import problems as P
from sparlab_gb300.topopt import GpuSimpProblem

pytestmark = pytest.mark.gpu


def test_noalloc_volume_matches_evaluate_twice():
    import torch
    spec = P.hex8_cantilever(24, 12, 12, 0.3, "noalloc")
    spec.rtol = 1e-8
    prob = GpuSimpProblem(spec)
    dev = torch.device("cuda", 0)
    for seed in (3, 4):
        x = P.SplitMix64(seed).uniform_array(prob.ne, 0.05, 1.0)
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


def test_noalloc_rejects_null_pointers():
    from sparlab_gb300._lib import SolverError
    spec = P.hex8_cantilever(8, 4, 4, 0.3, "noalloc_null")
    prob = GpuSimpProblem(spec)
    with pytest.raises(SolverError):
        prob.filter_volume_noalloc(0, 0, 0)
