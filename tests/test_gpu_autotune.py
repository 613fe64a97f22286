"""The launch-shape tuner changes speed, never results: every tile shape of
the matrix-free operator (both halo layouts), every Galerkin launch
variant and both unrolls of the double-float CG operator give the same
iteration history bit for bit, and the tuner records its choices."""
import ctypes as C

import pytest

from sparlab_gb300 import _lib
from sparlab_gb300 import problems as P
from sparlab_gb300.topopt import GpuSimpProblem

pytestmark = pytest.mark.gpu


def history(iterations=3):
    spec = P.hex8_cantilever(28, 14, 13, 0.25, "tune")
    spec.rtol = 1e-9
    prob = GpuSimpProblem(spec, precision="mixed", tensor_cores=0)   # the FMA kernel's tile shapes
    recs = [prob.iterate() for _ in range(iterations)]
    prob.close()
    return [(r.compliance, r.linear_iterations, r.lam) for r in recs]


def test_every_launch_shape_gives_the_same_iterations():
    lib = _lib.load()
    base = history()                       # tuned shapes
    report = _lib.autotune_report()
    mf_keys = [k for k in report if k.startswith("mf3:29x15x14")]
    row_keys = [k for k in report if "_rows" in k]
    df_keys = [k for k in report if k.startswith("df0:")]
    assert mf_keys and row_keys and df_keys
    assert len(mf_keys) >= 7                          # one key per mode of the operator
    assert len(report[mf_keys[0]][1]) == 10           # five tile shapes x two halo layouts timed
    assert len(report[df_keys[0]][1]) == 2            # the CG operator's two unrolls timed
    for v in range(10):
        for k in mf_keys:
            lib.simp_autotune_set(k.encode(), C.c_int32(v))
        for k in row_keys:
            lib.simp_autotune_set(k.encode(), C.c_int32(v % 4))
        for k in df_keys:
            lib.simp_autotune_set(k.encode(), C.c_int32(v % 2))
        assert history() == base, v
    lib.simp_autotune_enable(0)
    try:
        assert history() == base
    finally:
        lib.simp_autotune_enable(1)
