"""The tensor-core matrix-free level-0 operator (csrc/mfree_tc.cuh).

Each cell layer's element products K_e^0 x_e run as TF32 tensor-core GEMMs
with hi + lo operand splits (3 x TF32, FP32 accumulation in tensor memory).
Checked here:

- the product y = K_ff x (V-cycle level 0, mixed precision) against the FP64
  CG operator of an FP64 problem with the same design (its assembled K_ff is
  bit-exact against the oracle elsewhere): FP32-level error, within a small
  multiple of the FMA kernel's own error, on grids whose node counts are not
  multiples of the kernel's 31 x 7 node columns, with a clamped face and a
  seeded density, in every z-chunking of the march, which all give the same
  bits;
- solves: the compliance of the oracle's FP64 solve and the FMA kernel's CG
  iteration counts (within one with the V-cycle's level 0 on the tensor
  cores, within two with the CG operator itself on them, matrix_free = 2).

Reference for the operator: the uniform-element assembly it replaces
(src/fem/Assembler.cpp:44-58) and the level-0 products of the reference's
V-cycle (src/fem/Multigrid.cpp:783-885)."""
import ctypes as C

import numpy as np
import pytest

from sparlab_gb300 import _lib
from sparlab_gb300 import problems as P
from sparlab_gb300.topopt import GpuSimpProblem

pytestmark = pytest.mark.gpu


def _vector(n, seed):
    return P.SplitMix64(seed).uniform_array(n, -1.0, 1.0)


def _products(spec, design, v, **opts):
    """(FP64 CG-operator product, level-0 product with the given options)."""
    import torch
    dev = torch.device("cuda", 0)
    out = []
    for prec, kw in (("fp64", {}), ("mixed", opts)):
        prob = GpuSimpProblem(spec, precision=prec, **kw)
        prob.set_design(design)
        prob.evaluate()
        x = torch.from_numpy(v).to(dev)
        y = torch.full_like(x, np.nan)
        if prec == "fp64":
            prob.apply_operator(x.data_ptr(), y.data_ptr())
        else:
            prob.apply_level0(x.data_ptr(), y.data_ptr())
        torch.cuda.synchronize()
        out.append(y.cpu().numpy())
        prob.close()
    return out


def _rel(y, ref):
    return float(np.linalg.norm(y - ref) / np.linalg.norm(ref))


@pytest.mark.parametrize("grid", [(37, 21, 19), (30, 6, 7), (62, 13, 3)])
def test_tensor_core_product_against_fp64(grid):
    nx, ny, nz = grid
    spec = P.hex8_cantilever(nx, ny, nz, 0.3, "mf_tc_%dx%dx%d" % grid)
    design = P.seeded_density(spec, seed=11)
    v = _vector(GpuSimpProblem(spec, precision="fp64").nfree, 5)
    ref, y_tc = _products(spec, design, v, tensor_cores=1)
    _, y_fma = _products(spec, design, v, tensor_cores=0)
    assert np.all(np.isfinite(y_tc))
    e_tc, e_fma = _rel(y_tc, ref), _rel(y_fma, ref)
    # FP32 products of an FP32-rounded input: ~1e-7 relative
    assert e_tc < 2e-6 and e_tc <= 4.0 * e_fma + 1e-7, (e_tc, e_fma)
    assert np.abs(y_tc - ref).max() <= 1e-5 * np.abs(ref).max()


def test_every_chunking_gives_the_same_bits():
    # 94 x 43 x 41 nodes: 4 x 7 node columns, so the four chunkings of the
    # z march (about 2, 4, 1 and 8 CTAs per SM) give different layer counts
    spec = P.hex8_cantilever(93, 42, 40, 0.3, "mf_tc_chunks")
    design = P.seeded_density(spec, seed=12)
    lib = _lib.load()
    v = None
    ys = []
    for variant in range(4):
        lib.simp_autotune_set(b"mf3tc:94x43x41", C.c_int32(variant))
        if v is None:
            v = _vector(GpuSimpProblem(spec, precision="fp64").nfree, 6)
        ref, y = _products(spec, design, v, tensor_cores=1)
        ys.append(y)
        assert _rel(y, ref) < 2e-6
    for y in ys[1:]:
        np.testing.assert_array_equal(y, ys[0])


@pytest.mark.parametrize("matrix_free", [1, 2])
def test_solves_keep_iterations_and_match_the_oracle(matrix_free):
    import oracle
    spec = P.hex8_cantilever(48, 24, 24, 0.3, "mf_tc_solve")
    spec.rtol = 1e-10
    design = P.seeded_density(spec, seed=3)
    ref = oracle.Problem(spec).evaluate(design)
    runs = {}
    for tc in (0, 1):
        prob = GpuSimpProblem(spec, precision="mixed", matrix_free=matrix_free, tensor_cores=tc)
        prob.set_design(design)
        ev = prob.evaluate()
        runs[tc] = (ev.compliance, ev.linear_iterations)
        prob.close()
    (c0, it0), (c1, it1) = runs[0], runs[1]
    assert abs(c1 / ref["compliance"] - 1) < 1e-8, (c1, ref["compliance"])
    assert abs(c1 / c0 - 1) < 1e-9
    # the V-cycle's level 0 keeps the count; with the CG operator itself an
    # FP32 product (matrix_free = 2) the two kernels' roundings can move the
    # refinement rounds' counts by a little more
    assert abs(it1 - it0) <= (1 if matrix_free == 1 else 2), (it1, it0)

