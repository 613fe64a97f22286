"""The C ABI from C: tests/abi_client.c, compiled with gcc -std=c99 against
include/simp_gpu.h and linked with libsimp_gb300.so, drives the LinearSolver
boundary (create, set_layout, factorize, solve, stats, destroy) and reports
failures by status code and simp_last_error text.

CPU: the client compiles warning-free and a bad option set fails with
SIMP_BAD_INPUT and a message before any device call.  GPU: the client's
solution of a Hex8 bench-model system matches the oracle's AMG-PCG to 1e-9,
and an iteration cap of 1 ends with SIMP_MAXITER and the reference's
"did not converge" diagnosis."""
import os
import subprocess

import numpy as np
import pytest

from sparlab_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    lib = B.build()
    exe = str(tmp_path_factory.mktemp("abi") / "abi_client")
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "abi_client.c"), "-o", exe, "-L", os.path.dirname(lib), "-lsimp_gb300",
           "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.check_call(cmd)
    return exe


def test_client_compiles_and_rejects_bad_options(client):
    r = subprocess.run([client, "bad-options"], capture_output=True, text=True)
    assert r.returncode == 1, r.stderr     # SIMP_BAD_INPUT
    assert "status 1:" in r.stdout and len(r.stdout.split(":", 1)[1].strip()) > 0


def _write_system(path, dim, coords, free, ptr, col, val, rhs, rtol):
    with open(path, "wb") as f:
        np.array([dim, len(free), coords.size // dim], np.int32).tofile(f)
        np.array([len(col)], np.int64).tofile(f)
        np.ascontiguousarray(coords, np.float64).tofile(f)     # node-major, dim per node
        np.asarray(free, np.int32).tofile(f)
        np.asarray(ptr, np.int32).tofile(f)
        np.asarray(col, np.int32).tofile(f)
        np.asarray(val, np.float64).tofile(f)
        np.asarray(rhs, np.float64).tofile(f)
        np.array([rtol], np.float64).tofile(f)


def _read_solution(path, n):
    with open(path, "rb") as f:
        status, its, levels = np.fromfile(f, np.int32, 3)
        relres, oc = np.fromfile(f, np.float64, 2)
        x = np.fromfile(f, np.float64, n)
    return int(status), int(its), int(levels), float(relres), float(oc), x


@pytest.mark.gpu
def test_client_solve_matches_oracle_and_reports_maxiter(client, tmp_path):
    import oracle
    from sparlab_gb300 import problems as P
    spec = P.bench_model(3, 16, 8, 4)
    pr = oracle.Problem(spec)
    ptr, col, val = pr.kff(None)
    free = pr.free_dofs()
    coords = pr.coords()
    f = spec.loads[0][free]
    sys_path, out = str(tmp_path / "system.bin"), str(tmp_path / "x.bin")
    _write_system(sys_path, 3, coords, free, ptr, col, val, f, 1e-12)
    r = subprocess.run([client, "solve", sys_path, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    status, its, levels, relres, oc, x = _read_solution(out, len(free))
    ref = oracle.Solver(rtol=1e-12)
    ref.factorize(ptr, col, val, 3, coords, free)
    xr, itr, _ = ref.solve(f)
    assert status == 0 and levels == ref.num_levels() and relres <= 1e-12
    assert abs(its - itr) <= 1
    assert np.linalg.norm(x - xr) <= 1e-9 * np.linalg.norm(xr)
    # an iteration cap of 1 is a ConvergenceError in the reference
    r = subprocess.run([client, "solve", sys_path, out, "1"], capture_output=True, text=True)
    assert r.returncode == 4, r.stderr     # SIMP_MAXITER
    assert "did not converge" in r.stdout
    status, its, *_ = _read_solution(out, len(free))
    assert status == 4 and its == 1
