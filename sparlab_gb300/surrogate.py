"""The displacement surrogate over the C ABI (the learned PCG start).

A 3-D convolutional encoder-decoder on the nodal grid (4 levels, channels
16/32/64/64, 3x3x3 kernels, BF16 weights and activations with FP32
accumulation on the tensor cores) predicts the displacement shape of a load
case from the physical density.  ``GpuSimpProblem(spec)`` with
``spec.warm_start = 3`` and ``problem.set_surrogate(s)`` starts every PCG
solve from the energy-optimal combination of the previous displacements and
the prediction, so the solve converges to the unchanged tolerance whatever
the prediction's error.  The reference has no counterpart: its solves start
from the previous displacement (src/topopt/Sensitivity.cpp:142, 169-176).

Training data: (density, displacement) pairs that the plain FP64 solver
produces along SIMP runs of seeded Hex8 cantilever variants
(:func:`training_variants`).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import List, Optional

import numpy as np

from . import _lib
from . import problems as P

# layer shapes (input channels per segment, output channels), in parameter order
LAYERS = [((16,), 16), ((16,), 16), ((16,), 32), ((32,), 32), ((32,), 64), ((64,), 64),
          ((64,), 64), ((64,), 64), ((64, 64), 64), ((64, 32), 32), ((32, 16), 16), ((16,), 3)]
LAYER_NAMES = ["e0a", "e0b", "e1a", "e1b", "e2a", "e2b", "e3a", "e3b", "d2", "d1", "d0", "head"]


def _raise(code):
    if code:
        _lib.raise_for(code, _lib.load().simp_surrogate_last_error().decode())


class Surrogate:
    def __init__(self, seed: int = 7, device: int = 0):
        self._lib = _lib.load()
        self._h = C.c_void_p()
        _raise(self._lib.simp_surrogate_create(C.c_int32(device), C.c_uint64(seed), C.byref(self._h)))
        n = C.c_int64()
        _raise(self._lib.simp_surrogate_num_params(self._h, C.byref(n)))
        self.num_params = n.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.simp_surrogate_destroy(self._h)
            self._h = None

    __del__ = close

    @property
    def handle(self):
        return self._h

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, np.float32)
        _raise(self._lib.simp_surrogate_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.num_params:
            raise ValueError("parameter vector of the wrong size")
        _raise(self._lib.simp_surrogate_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def layer_params(self, p: Optional[np.ndarray] = None):
        """[(weights [27, cout, cin], bias [cout])] per layer, views of p."""
        p = self.get_params() if p is None else p
        out, off = [], 0
        for cins, cout in LAYERS:
            cin = sum(cins)
            w = p[off: off + 27 * cout * cin].reshape(27, cout, cin)
            off += 27 * cout * cin
            b = p[off: off + cout]
            off += cout
            out.append((w, b))
        return out

    def loss_gradient(self, nx: int, ny: int, nz: int, input_device_ptr: int, target_device_ptr: int,
                      mask_device_ptr: int, count: int):
        """(loss, parameter gradient) of one example on device tensors."""
        loss = C.c_double()
        g = np.zeros(self.num_params, np.float32)
        _raise(self._lib.simp_surrogate_loss_gradient(
            self._h, C.c_int32(nx), C.c_int32(ny), C.c_int32(nz), C.c_void_p(input_device_ptr),
            C.c_void_p(target_device_ptr), C.c_void_p(mask_device_ptr), C.c_int64(count), C.byref(loss),
            g.ctypes.data_as(C.POINTER(C.c_float))))
        return loss.value, g

    def add_sample(self, problem, load_case: int = 0):
        _raise(self._lib.simp_surrogate_add_sample(self._h, problem._h, C.c_int32(load_case)))

    @property
    def num_samples(self) -> int:
        n = C.c_int32()
        _raise(self._lib.simp_surrogate_num_samples(self._h, C.byref(n)))
        return n.value

    def train(self, epochs: int, learning_rate: float = 2e-3, batch: int = 4, seed: int = 11) -> List[float]:
        losses = np.zeros(epochs)
        _raise(self._lib.simp_surrogate_train(self._h, C.c_int32(epochs), C.c_double(learning_rate),
                                              C.c_int32(batch), C.c_uint64(seed), _lib.ptr(losses)))
        return [float(v) for v in losses]

    def predict(self, problem, load_case: int, u_device_ptr: int):
        _raise(self._lib.simp_surrogate_predict(self._h, problem._h, C.c_int32(load_case),
                                                C.c_void_p(u_device_ptr)))

    def forward(self, nx: int, ny: int, nz: int, input_device_ptr: int, output_device_ptr: int):
        _raise(self._lib.simp_surrogate_forward(self._h, C.c_int32(nx), C.c_int32(ny), C.c_int32(nz),
                                                C.c_void_p(input_device_ptr), C.c_void_p(output_device_ptr)))


def training_variants(seeds=range(100, 200)) -> List[P.ProblemSpec]:
    """Seeded variants of the Hex8 cantilever: seeds 100-149 on a 48 x 24 x 24
    grid, 150-199 on 96 x 48 x 48; clamped x = 0 face; a unit total load in
    -z spread over the tip edge {i = nx, k = k0} with k0 the bottom or the
    mid-height edge and the direction tilted by up to 30 degrees about x;
    volume fraction ~ U[0.1, 0.3]."""
    out = []
    for s in seeds:
        rng = P.SplitMix64(s)
        nx, ny, nz = (48, 24, 24) if s < 150 else (96, 48, 48)
        vf = rng.uniform(0.1, 0.3)
        spec = P.hex8_cantilever(nx, ny, nz, vf, f"variant{s}")
        k0 = 0 if rng.uniform() < 0.5 else nz // 2
        t = math.radians(rng.uniform(-30.0, 30.0))
        edge = [spec.node_index(nx, j, k0) for j in range(ny + 1)]
        spec.loads = P.point_load(spec, edge, (0.0, math.sin(t), -math.cos(t)))[None, :]
        out.append(spec)
    return out


def generate_samples(sur: Surrogate, specs, iterations: int = 20, precision: str = "fp64"):
    """Runs `iterations` SIMP iterations of every spec with the plain solver
    and adds each iteration's (density, displacement) pair."""
    from .topopt import GpuSimpProblem
    for spec in specs:
        prob = GpuSimpProblem(spec, precision=precision)
        for _ in range(iterations):
            prob.iterate()
            sur.add_sample(prob, 0)
        prob.close()
