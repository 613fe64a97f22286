"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports
every entry point include/simp_gpu.h declares, and its host-only helpers
agree with the oracle.  No kernel runs here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle
from sparlab_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "simp_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(simp_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_for_sm103a():
    path = build.build()
    assert os.path.exists(path)
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)


def test_every_declared_symbol_is_exported():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_lib.EXPORTS)


def test_default_options_match_reference_defaults():
    o = _lib.default_options()
    assert o.strength_threshold == 0.02 and o.max_levels == 12 and o.coarse_size == 1500
    assert o.smoother_degree == 3 and o.chebyshev_ratio == 30.0
    assert o.prolongator_damping == pytest.approx(4.0 / 3.0) and o.lanczos_steps == 12
    assert o.coarse_pivot_tolerance == 1e-13 and o.reuse_aggregates == 1
    assert o.iterative_tolerance == 1e-12


@pytest.mark.parametrize("dim,h", [(2, (1.0, 1.0, 0.0)), (2, (0.25, 0.1, 0.0)),
                                   (3, (1.0, 1.0, 1.0)), (3, (0.25, 0.25, 0.25)),
                                   (3, (0.5, 0.2, 0.125))])
def test_element_stiffness_matches_oracle(dim, h):
    from sparlab_gb300.topopt import element_stiffness
    ke = element_stiffness(dim, *h, 70e9, 0.3, 0.01 if dim == 2 else 1.0)
    ko = oracle.element_stiffness(dim, *h, 70e9, 0.3, 0.01 if dim == 2 else 1.0)
    assert np.abs(ke - ko).max() <= 1e-14 * np.abs(ko).max()
    assert np.array_equal(ke, ke.T)
    # rigid translations are in the null space
    n = ke.shape[0]
    for k in range(dim):
        t = np.zeros(n)
        t[k::dim] = 1.0
        assert np.abs(ke @ t).max() <= 1e-12 * np.abs(ke).max()


@pytest.mark.parametrize("field,value,words", [
    ("strength_threshold", 1.5, "strength_threshold"),
    ("strength_threshold", -0.1, "strength_threshold"),
    ("max_levels", 0, "max_levels"),
    ("coarse_size", 0, "coarse_size"),
    ("smoother_degree", 0, "smoother_degree"),
    ("chebyshev_ratio", 1.0, "chebyshev_ratio"),
    ("prolongator_damping", 2.0, "prolongator_damping"),
    ("lanczos_steps", 1, "lanczos_steps"),
    ("iterative_tolerance", 0.0, "tolerance"),
    ("precision", 7, "precision"),
    ("matrix_free", 3, "matrix_free"),
    ("tensor_cores", 2, "tensor_cores"),
])
def test_context_creation_rejects_bad_options_before_touching_the_device(field, value, words):
    """AmgPreconditioner's option checks (src/fem/Multigrid.cpp:907-925;
    tests/test_multigrid.cpp:451-453 asserts strength 1.5 is refused): the
    context is refused with SIMP_BAD_INPUT and the option named, whether or
    not a GPU is present, because the checks come before any CUDA call."""
    lib = _lib.load()
    o = _lib.default_options()
    setattr(o, field, value)
    h = C.c_void_p()
    assert lib.simp_ctx_create(C.byref(o), C.byref(h)) == _lib.SIMP_BAD_INPUT
    assert not h.value
    assert words in lib.simp_last_error(None).decode()


@pytest.mark.parametrize("field,value,words", [
    ("penalty", 0.5, "penalty"),
    ("emin_ratio", 0.0, "emin_ratio"),
    ("emin_ratio", 1.5, "emin_ratio"),
    ("volume_fraction", 0.0, "volume fraction"),
    ("move_limit", 0.0, "move_limit"),
    ("damping", 1.5, "damping"),
    ("warm_start", 4, "warm_start"),
])
def test_problem_creation_rejects_bad_descriptors_before_touching_the_device(field, value, words):
    """SimpOptions::validate (src/topopt/SimpInterpolation.cpp:31-44; tests/
    test_topopt.cpp:146-161 refuses penalty 0.5 and emin_ratio 0 and 1.5) and
    the optimiser's option checks: simp_problem_create refuses the
    descriptor with SIMP_BAD_INPUT and names the field, with or without a
    GPU, because the descriptor is checked before the device is selected."""
    from sparlab_gb300 import problems as P
    from sparlab_gb300.topopt import GpuSimpProblem
    spec = P.hex8_cantilever(4, 2, 2, 0.3, "bad_descriptor")
    setattr(spec, field, value)
    with pytest.raises(_lib.SolverError) as e:
        GpuSimpProblem(spec)
    assert e.value.code == _lib.SIMP_BAD_INPUT
    assert words in str(e.value)


def test_context_creation_reports_cuda_errors_without_a_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load()
    h = C.c_void_p()
    code = lib.simp_ctx_create(None, C.byref(h))
    assert code == _lib.SIMP_CUDA_ERROR
    assert lib.simp_last_error(None)


def header_structs():
    """{typedef name: [(field, type)]} of the plain-C structs include/simp_gpu.h
    declares, in declaration order; type is 'double', 'int32_t', 'int64_t',
    'float', 'ptr', or (element type, length) for an array."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct(?: \w+)? \{(.*?)\} (simp_\w+);", text, flags=re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            typ, names = re.match(r"((?:const\s+)?\w+\s*\**)\s*(.*)", decl).groups()
            for nm in names.split(","):
                nm = nm.strip()
                ptr = "*" in typ or nm.startswith("*")
                arr = re.match(r"(\w+)\[(\d+)\]$", nm.lstrip("*"))
                base = "ptr" if ptr else typ.strip()
                if arr:
                    fields.append((arr.group(1), (base, int(arr.group(2)))))
                else:
                    fields.append((nm.lstrip("*"), base))
        out[m.group(2)] = fields
    return out


MIRRORS = {"simp_solver_options": "SolverOptions", "simp_amg_stats": "AmgStats",
           "simp_problem_desc": "ProblemDesc", "simp_evaluation": "Evaluation",
           "simp_oc_step": "OcStep", "simp_iteration_record": "IterationRecord",
           "simp_robust_record": "RobustRecord", "simp_modal_options": "ModalOptions",
           "simp_modal_info": "ModalInfo", "simp_buckling_options": "BucklingOptions",
           "simp_buckling_info": "BucklingInfo"}


def test_ctypes_mirrors_follow_the_header():
    """Every struct of the C ABI has a ctypes mirror with the same fields, in
    the same order, of the same C types (so the offsets agree)."""
    structs = header_structs()
    assert set(structs) == set(MIRRORS)
    scalar = {"double": C.c_double, "int32_t": C.c_int32, "int64_t": C.c_int64, "float": C.c_float}
    for cname, pyname in MIRRORS.items():
        mirror = getattr(_lib, pyname)._fields_
        python_name = {"lambda": "lam"}  # a Python keyword
        assert [f for f, _ in mirror] == [python_name.get(f, f) for f, _ in structs[cname]], cname
        for (f, ctype), (_, htype) in zip(mirror, structs[cname]):
            if isinstance(htype, tuple):
                assert ctype._type_ is scalar[htype[0]] and ctype._length_ == htype[1], (cname, f)
            elif htype == "ptr":
                assert C.sizeof(ctype) == C.sizeof(C.c_void_p) and ctype not in scalar.values(), (cname, f)
            else:
                assert ctype is scalar[htype], (cname, f, ctype, htype)
