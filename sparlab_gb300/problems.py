"""Structured cantilever problems on Q4 / Hex8 grids.

These builders play the role of the reference's ``FemModel::finalize`` for the
structured decks the SIMP loop runs on (``src/fem/FemModel.cpp:286-385``):
box supports select nodes within ``1e-9 * diagonal`` of the box
(``src/fem/Selector.cpp:12-52``), a point load spread over N nodes puts
``force / N`` on each (``src/fem/BoundaryConditions.cpp:46-52``), and
load-case weights are normalised to sum to one (``FemModel.cpp:412-420``).

The seeded generator is SplitMix64 (Steele, Lea and Flood, 2014) so the CPU
and GPU paths, and every machine, see identical bits.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional

import numpy as np

MASK64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 stream; ``stream`` offsets the state by the golden gamma."""

    def __init__(self, seed: int, stream: int = 0):
        self.state = (seed * 0xD1B54A32D192ED03 + stream * 0x9E3779B97F4A7C15) & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))

    def integers(self, lo: int, hi: int) -> int:
        """Uniform integer in [lo, hi] inclusive."""
        return lo + self.next_u64() % (hi - lo + 1)

    def uniform_array(self, n: int, lo: float, hi: float) -> np.ndarray:
        # vectorised SplitMix64 over a counter: identical to n calls of uniform()
        idx = np.arange(1, n + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            z = (np.uint64(self.state) + idx * np.uint64(0x9E3779B97F4A7C15))
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        self.state = (self.state + n * 0x9E3779B97F4A7C15) & MASK64
        u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
        return lo + (hi - lo) * u


@dataclasses.dataclass
class ProblemSpec:
    dim: int
    nx: int
    ny: int
    nz: int
    lx: float
    ly: float
    lz: float
    young: float = 1.0
    poisson: float = 0.3
    thickness: float = 1.0
    density: float = 1.0                    # material density (modal analysis)
    fixed: Optional[np.ndarray] = None      # uint8 per DOF (node * dim + k)
    loads: Optional[np.ndarray] = None      # (L, ndof)
    weights: Optional[np.ndarray] = None    # (L,) raw weights
    filter_radius: float = 1.5
    volume_fraction: float = 0.5
    initial_density: float = -1.0
    penalty: float = 3.0
    emin_ratio: float = 1e-9
    move_limit: float = 0.2
    damping: float = 0.5
    rtol: float = 1e-8
    max_cg_iterations: int = 0
    warm_start: int = 1  # 0 zero guess, 1 previous displacement, 2 projection on the last 3,
    #                      3 that projection with the surrogate's prediction added
    warm_history: int = 0  # displacements the projected starts combine (1..3; 0: 3)
    # Heaviside projection of the filtered density with beta continuation
    # (ProjectionOptions, include/sparlab/topopt/Projection.hpp:69-96)
    projection: bool = False
    eta: float = 0.5
    beta_start: float = 1.0
    beta_max: float = 32.0
    beta_factor: float = 2.0
    beta_interval: int = 50
    advance_on_convergence: bool = True
    change_tolerance: float = 1e-3  # run_oc's design-change tolerance (beta advance)
    # robust formulation: eroded objective (eta + delta), dilated volume
    # (eta - delta) against a target rescaled every robust_volume_interval
    robust: bool = False
    robust_delta: float = 0.1
    robust_volume_interval: int = 1
    amg: Dict = dataclasses.field(default_factory=dict)
    name: str = ""

    @property
    def nodes_per_axis(self):
        return (self.nx + 1, self.ny + 1, (self.nz + 1) if self.dim == 3 else 1)

    @property
    def num_nodes(self) -> int:
        a, b, c = self.nodes_per_axis
        return a * b * c

    @property
    def num_elements(self) -> int:
        return self.nx * self.ny * (self.nz if self.dim == 3 else 1)

    @property
    def num_dofs(self) -> int:
        return self.num_nodes * self.dim

    def node_index(self, i, j, k=0) -> int:
        nnx, nny, _ = self.nodes_per_axis
        return (k * nny + j) * nnx + i

    def node_coords(self) -> np.ndarray:
        """(num_nodes, dim) coordinates, x0 + i * dx as the mesh generator forms them."""
        nnx, nny, nnz = self.nodes_per_axis
        dx, dy = self.lx / self.nx, self.ly / self.ny
        i = np.arange(nnx) * dx
        j = np.arange(nny) * dy
        if self.dim == 2:
            X, Y = np.meshgrid(i, j, indexing="xy")
            return np.stack([X.ravel(), Y.ravel()], axis=1)
        dz = self.lz / self.nz
        k = np.arange(nnz) * dz
        Z, Y, X = np.meshgrid(k, j, i, indexing="ij")
        return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)

    def free_dofs(self) -> np.ndarray:
        return np.flatnonzero(self.fixed == 0).astype(np.int32)


def _diag(spec: ProblemSpec) -> float:
    if spec.dim == 2:
        return math.hypot(spec.lx, spec.ly)
    return math.sqrt(spec.lx ** 2 + spec.ly ** 2 + spec.lz ** 2)


def clamp_left(spec: ProblemSpec, components=None) -> np.ndarray:
    """Fix every component of the nodes on the x = 0 face (box xmax = 0)."""
    tol = 1e-9 * max(_diag(spec), 1e-30)
    x = spec.node_coords()[:, 0]
    nodes = np.flatnonzero(x <= 0.0 + tol)
    fixed = np.zeros(spec.num_dofs, np.uint8)
    comps = range(spec.dim) if components is None else components
    for k in comps:
        fixed[nodes * spec.dim + k] = 1
    return fixed


def nearest_node(spec: ProblemSpec, point) -> int:
    c = spec.node_coords()
    p = np.zeros(spec.dim)
    p[:] = point[: spec.dim]
    d2 = ((c - p) ** 2).sum(axis=1)
    return int(np.argmin(d2))   # first minimum, as the reference's strict '<' scan


def point_load(spec: ProblemSpec, nodes, force) -> np.ndarray:
    """Load vector with ``force`` spread equally over ``nodes``."""
    f = np.zeros(spec.num_dofs)
    nodes = np.atleast_1d(np.asarray(nodes, np.int64))
    scale = 1.0 / len(nodes)
    for n in nodes:
        for k in range(spec.dim):
            f[n * spec.dim + k] += scale * force[k]
    return f


# ---------------------------------------------------------------------------
# The reference's own benchmark model (apps/sparlab_bench.cpp:87-127)
# ---------------------------------------------------------------------------
def bench_model(dim: int, nx: int, ny: int, nz: int = 0) -> ProblemSpec:
    """lx=2, ly=1, lz=0.5; E=70e9, nu=0.3; t=0.01 in 2-D; x=0 clamped;
    (0, -1000, 0) N at the node nearest (lx, 0, 0); solid density."""
    spec = ProblemSpec(dim=dim, nx=nx, ny=ny, nz=nz if dim == 3 else 0, lx=2.0, ly=1.0,
                       lz=0.5 if dim == 3 else 0.0, young=70.0e9, poisson=0.3,
                       thickness=0.01 if dim == 2 else 1.0, filter_radius=0.0,
                       name=f"bench_{'hex8' if dim == 3 else 'quad4'}_{nx}x{ny}" +
                       (f"x{nz}" if dim == 3 else ""))
    spec.fixed = clamp_left(spec)
    tip = nearest_node(spec, (spec.lx, 0.0, 0.0))
    spec.loads = point_load(spec, [tip], (0.0, -1000.0, 0.0))[None, :]
    spec.weights = np.ones(1)
    return spec


def plane_cantilever(nx: int, ny: int, length: float = 1.0, height: float = 0.1,
                     thickness: float = 0.01, young: float = 70.0e9, poisson: float = 0.0,
                     density: float = 2700.0) -> ProblemSpec:
    """The reference's standard modal / static cantilever (tests/TestSupport.hpp:
    23-86): plane stress, root x = 0 clamped, a -1000 N tip resultant spread
    over the tip edge."""
    spec = ProblemSpec(dim=2, nx=nx, ny=ny, nz=0, lx=length, ly=height, lz=0.0, young=young,
                       poisson=poisson, thickness=thickness, density=density, filter_radius=0.0,
                       rtol=1e-12, name=f"cantilever_{nx}x{ny}")
    spec.fixed = clamp_left(spec)
    tip = [spec.node_index(nx, j) for j in range(ny + 1)]
    spec.loads = point_load(spec, tip, (0.0, -1000.0))[None, :]
    spec.weights = np.ones(1)
    return spec


def column(dim: int, nx: int, ny: int, nz: int = 0, length: float = 1.0, height: float = 0.05,
           width: float = 0.05, thickness: float = 0.02, force: float = -1.0, young: float = 200.0e9,
           poisson: float = 0.3, transverse: float = 0.0) -> ProblemSpec:
    """The reference's buckling column (tests/test_buckling.cpp:41-68): along
    x, root x = 0 clamped, a uniform traction on the face x = length whose
    axial resultant is `force` (negative: compression) plus an optional
    transverse (-y) resultant, as consistent nodal forces of the face cells."""
    spec = ProblemSpec(dim=dim, nx=nx, ny=ny, nz=nz if dim == 3 else 0, lx=length, ly=height,
                       lz=width if dim == 3 else 0.0, young=young, poisson=poisson,
                       thickness=thickness if dim == 2 else 1.0, density=7850.0, filter_radius=0.0,
                       rtol=1e-12, name=f"column_{nx}x{ny}" + (f"x{nz}" if dim == 3 else ""))
    spec.fixed = clamp_left(spec)
    f = np.zeros(spec.num_dofs)
    if dim == 2:
        for j in range(ny):
            for jj in (j, j + 1):
                node = spec.node_index(nx, jj)
                f[node * 2] += force / ny / 2.0
                f[node * 2 + 1] -= transverse / ny / 2.0
    else:
        for k in range(nz):
            for j in range(ny):
                for jj, kk in ((j, k), (j + 1, k), (j + 1, k + 1), (j, k + 1)):
                    node = spec.node_index(nx, jj, kk)
                    f[node * 3] += force / (ny * nz) / 4.0
                    f[node * 3 + 1] -= transverse / (ny * nz) / 4.0
    spec.loads = f[None, :]
    spec.weights = np.ones(1)
    return spec


# ---------------------------------------------------------------------------
# The five workload configurations
# ---------------------------------------------------------------------------
def q4_cantilever_120x40() -> ProblemSpec:
    """Q4 120x40 unit cells, x=0 clamped, unit downward load at (120, 20)."""
    spec = ProblemSpec(dim=2, nx=120, ny=40, nz=0, lx=120.0, ly=40.0, lz=0.0,
                       thickness=1.0, filter_radius=1.5, volume_fraction=0.5,
                       initial_density=0.5, rtol=1e-8, name="q4_120x40")
    spec.fixed = clamp_left(spec)
    spec.loads = point_load(spec, [spec.node_index(120, 20)], (0.0, -1.0))[None, :]
    spec.weights = np.ones(1)
    return spec


def q4_cantilever_600x200(seed: int = 2) -> ProblemSpec:
    """Q4 600x200, r=3, vf=0.35, three unit loads at right-edge nodes j=50,
    100, 150 in directions (sin t, -cos t), t ~ U[-90, 90] deg (stream i)."""
    spec = ProblemSpec(dim=2, nx=600, ny=200, nz=0, lx=600.0, ly=200.0, lz=0.0,
                       thickness=1.0, filter_radius=3.0, volume_fraction=0.35,
                       rtol=1e-8, name="q4_600x200")
    spec.fixed = clamp_left(spec)
    loads = []
    for i, j in enumerate((50, 100, 150)):
        t = math.radians(SplitMix64(seed, i).uniform(-90.0, 90.0))
        loads.append(point_load(spec, [spec.node_index(600, j)], (math.sin(t), -math.cos(t))))
    spec.loads = np.stack(loads)
    spec.weights = np.full(3, 1.0 / 3.0)
    return spec


def hex8_cantilever(nx: int, ny: int, nz: int, volume_fraction: float, name: str) -> ProblemSpec:
    """Hex8 unit cells, x=0 face clamped, unit total load in -z spread over the
    edge {i = nx, k = 0} (ny + 1 nodes)."""
    spec = ProblemSpec(dim=3, nx=nx, ny=ny, nz=nz, lx=float(nx), ly=float(ny), lz=float(nz),
                       filter_radius=1.5, volume_fraction=volume_fraction, rtol=1e-8, name=name)
    spec.fixed = clamp_left(spec)
    edge = [spec.node_index(nx, j, 0) for j in range(ny + 1)]
    spec.loads = point_load(spec, edge, (0.0, 0.0, -1.0))[None, :]
    spec.weights = np.ones(1)
    return spec


def hex8_96x48x48() -> ProblemSpec:
    return hex8_cantilever(96, 48, 48, 0.2, "hex8_96x48x48")


def hex8_192x96x96() -> ProblemSpec:
    return hex8_cantilever(192, 96, 96, 0.15, "hex8_192x96x96")


def seeded_density(spec: ProblemSpec, seed: int = 3, lo: float = 0.01, hi: float = 1.0) -> np.ndarray:
    """i.i.d. U[lo, hi] element densities (seeded SplitMix64)."""
    return SplitMix64(seed).uniform_array(spec.num_elements, lo, hi)


def batched_instances(seed: int = 4, count_q4: int = 48, count_hex: int = 16) -> List[ProblemSpec]:
    """Uneven independent instances: Q4 nx~U{64..256}, ny~U{32..128}; Hex8
    edges ~U{16..40}; clamped left face; 1-4 unit loads at random right-face
    nodes; vf ~ U[0.2, 0.5]; p=3, r=1.5."""
    rng = SplitMix64(seed)
    out = []
    for q in range(count_q4 + count_hex):
        dim = 2 if q < count_q4 else 3
        if dim == 2:
            nx, ny, nz = rng.integers(64, 256), rng.integers(32, 128), 0
        else:
            nx, ny, nz = rng.integers(16, 40), rng.integers(16, 40), rng.integers(16, 40)
        spec = ProblemSpec(dim=dim, nx=nx, ny=ny, nz=nz, lx=float(nx), ly=float(ny),
                           lz=float(nz), filter_radius=1.5,
                           volume_fraction=rng.uniform(0.2, 0.5), rtol=1e-8,
                           name=f"inst{q}")
        spec.fixed = clamp_left(spec)
        loads = []
        for _ in range(rng.integers(1, 4)):
            j = rng.integers(0, ny)
            k = rng.integers(0, nz) if dim == 3 else 0
            if dim == 2:
                t = rng.uniform(-math.pi / 2, math.pi / 2)
                force = (math.sin(t), -math.cos(t))
            else:
                # uniform direction on the sphere
                zc = rng.uniform(-1.0, 1.0)
                ph = rng.uniform(0.0, 2.0 * math.pi)
                s = math.sqrt(max(0.0, 1.0 - zc * zc))
                force = (s * math.cos(ph), s * math.sin(ph), zc)
            loads.append(point_load(spec, [spec.node_index(nx, j, k)], force))
        spec.loads = np.stack(loads)
        spec.weights = np.ones(len(loads))
        out.append(spec)
    return out


# ---------------------------------------------------------------------------
# The reference's published topology benchmarks on structured grids
# (configs/benchmarks/*.json; their first-iteration and full-solid compliances
# are in docs/results/benchmarks.csv)
# ---------------------------------------------------------------------------
def box_nodes(spec: ProblemSpec, xmin=-math.inf, xmax=math.inf, ymin=-math.inf, ymax=math.inf,
              zmin=-math.inf, zmax=math.inf) -> np.ndarray:
    """Nodes inside a box selector, widened by 1e-9 of the mesh diagonal
    (Selector::contains, src/fem/Selector.cpp:12-19, 52-54)."""
    tol = 1e-9 * max(_diag(spec), 1e-30)
    c = spec.node_coords()
    z = c[:, 2] if spec.dim == 3 else np.zeros(len(c))
    inside = ((c[:, 0] >= xmin - tol) & (c[:, 0] <= xmax + tol) & (c[:, 1] >= ymin - tol) &
              (c[:, 1] <= ymax + tol) & (z >= zmin - tol) & (z <= zmax + tol))
    return np.flatnonzero(inside)


def _radius(spec: ProblemSpec, elements: float) -> float:
    """radius_elements x the mean cell side (Configuration::resolved_filter_radius)."""
    cells = [spec.lx / spec.nx, spec.ly / spec.ny] + ([spec.lz / spec.nz] if spec.dim == 3 else [])
    return elements * float(np.prod(cells)) ** (1.0 / spec.dim)


def mbb_beam(projection: bool = False, robust: bool = False) -> ProblemSpec:
    """configs/benchmarks/mbb_beam{,_projected,_robust}.json: the MBB half
    beam, Q4 180 x 60 unit cells, E = 1, nu = 0.3, t = 1; u_x = 0 on x = 0,
    a vertical roller at the node nearest (180, 0); (0, -1) N at the node
    nearest (0, 60); vf 0.5, radius 4.5 cells; the projected variants start
    at beta 1 (eta 0.5; robust: eta 0.5 +- 0.1)."""
    spec = ProblemSpec(dim=2, nx=180, ny=60, nz=0, lx=180.0, ly=60.0, lz=0.0, young=1.0, poisson=0.3,
                       thickness=1.0, volume_fraction=0.5, initial_density=0.5, rtol=1e-10,
                       projection=projection or robust, eta=0.5, beta_start=1.0,
                       beta_max=32.0, beta_factor=2.0, beta_interval=40, robust=robust,
                       robust_delta=0.1, robust_volume_interval=20,
                       name="mbb_beam" + ("_robust" if robust else "_projected" if projection else ""))
    spec.filter_radius = _radius(spec, 4.5)
    fixed = clamp_left(spec, components=[0])
    fixed[nearest_node(spec, (180.0, 0.0)) * 2 + 1] = 1
    spec.fixed = fixed
    spec.loads = point_load(spec, [nearest_node(spec, (0.0, 60.0))], (0.0, -1.0))[None, :]
    spec.weights = np.ones(1)
    return spec


def cantilever_beam() -> ProblemSpec:
    """configs/benchmarks/cantilever_beam.json: Q4 160 x 80 over 0.4 x 0.2 m,
    Al 7075-T6 (E = 71.7 GPa, nu = 0.33), t = 4 mm; x = 0 clamped; 2000 N
    down spread over the tip nodes with y in [0.0975, 0.1025]; vf 0.4,
    radius 2 cells."""
    spec = ProblemSpec(dim=2, nx=160, ny=80, nz=0, lx=0.4, ly=0.2, lz=0.0, young=71.7e9, poisson=0.33,
                       thickness=0.004, density=2810.0, volume_fraction=0.4, initial_density=0.4,
                       rtol=1e-10, name="cantilever_beam")
    spec.filter_radius = _radius(spec, 2.0)
    spec.fixed = clamp_left(spec)
    tip = box_nodes(spec, xmin=0.4, ymin=0.0975, ymax=0.1025)
    spec.loads = point_load(spec, tip, (0.0, -2000.0))[None, :]
    spec.weights = np.ones(1)
    return spec


def bracket_3d(projection: bool = False, large: bool = False) -> ProblemSpec:
    """configs/benchmarks/bracket_3d{,_projected,_large}.json: Hex8 over
    0.24 x 0.12 x 0.06 m (32 x 16 x 8 cells; large: 96 x 48 x 24), Al
    7075-T6; x = 0 clamped; load case 1 (weight 1): 3000 N down spread over
    the tip's bottom edge (x = 0.24, y = 0); load case 2 (weight 0.5): 1200 N
    along z spread over the tip's mid line (y in [0.0555, 0.0645]; large:
    [0.0585, 0.0615]); vf 0.3, radius 1.5 cells; the projected and large
    variants start at beta 1 (eta 0.5)."""
    n = (96, 48, 24) if large else (32, 16, 8)
    spec = ProblemSpec(dim=3, nx=n[0], ny=n[1], nz=n[2], lx=0.24, ly=0.12, lz=0.06, young=71.7e9,
                       poisson=0.33, density=2810.0, volume_fraction=0.3, initial_density=0.3,
                       rtol=1e-10, projection=projection or large, eta=0.5, beta_start=1.0,
                       beta_max=16.0, beta_factor=2.0, beta_interval=40,
                       name="bracket_3d" + ("_large" if large else "_projected" if projection else ""))
    spec.filter_radius = _radius(spec, 1.5)
    spec.fixed = clamp_left(spec)
    edge = box_nodes(spec, xmin=0.24, ymax=0.0)
    mid = box_nodes(spec, xmin=0.24, ymin=0.0585 if large else 0.0555, ymax=0.0615 if large else 0.0645)
    spec.loads = np.stack([point_load(spec, edge, (0.0, -3000.0, 0.0)),
                           point_load(spec, mid, (0.0, 0.0, 1200.0))])
    spec.weights = np.array([1.0, 0.5])
    return spec


# ---------------------------------------------------------------------------
# The reference's cross-validation models on structured grids
# (configs/verification/*.json; SparLab's results are in
# docs/results/cross_validation.csv)
# ---------------------------------------------------------------------------
def face_traction(spec: ProblemSpec, axis: int, at_max: bool, traction) -> np.ndarray:
    """Consistent nodal forces of a uniform traction on a boundary face of
    the box grid: each face cell's traction x area shared equally by its
    corner nodes (exact for bilinear faces)."""
    f = np.zeros(spec.num_dofs)
    n = [spec.nx, spec.ny, spec.nz][: spec.dim]
    h = [spec.lx / spec.nx, spec.ly / spec.ny] + ([spec.lz / spec.nz] if spec.dim == 3 else [])
    others = [a for a in range(spec.dim) if a != axis]
    fixed_index = n[axis] if at_max else 0
    area = float(np.prod([h[a] for a in others])) * (1.0 if spec.dim == 3 else spec.thickness)
    corners = 2 ** len(others)
    shape = [n[a] for a in others]
    for cell in np.ndindex(*shape):
        for corner in np.ndindex(*([2] * len(others))):
            idx = [0, 0, 0]
            idx[axis] = fixed_index
            for a, c, o in zip(others, cell, corner):
                idx[a] = c + o
            node = spec.node_index(idx[0], idx[1], idx[2] if spec.dim == 3 else 0)
            for k in range(spec.dim):
                f[node * spec.dim + k] += traction[k] * area / corners
    return f


def cantilever_analysis() -> ProblemSpec:
    """configs/verification/cantilever_analysis.json: Q4 120 x 12 over
    1.0 x 0.1 m, E = 70 GPa, nu = 0, t = 10 mm; x = 0 clamped; 1000 N down
    spread over the tip edge (box xmin = 1.0)."""
    spec = plane_cantilever(120, 12)
    spec.name = "cantilever_analysis"
    return spec


def block_3d_analysis() -> ProblemSpec:
    """configs/verification/block_3d_analysis.json: Hex8 40 x 8 x 4 over
    0.5 x 0.1 x 0.05 m, E = 68.9 GPa, nu = 0.33; x = 0 clamped; load case
    tip_load: 1000 N along -y spread over the tip face (box xmin = 0.5);
    load case top_pressure: a -2e5 Pa traction along z on the top face
    (box zmin = 0.05)."""
    spec = ProblemSpec(dim=3, nx=40, ny=8, nz=4, lx=0.5, ly=0.1, lz=0.05, young=68.9e9, poisson=0.33,
                       density=2700.0, filter_radius=0.0, rtol=1e-12, name="block_3d_analysis")
    spec.fixed = clamp_left(spec)
    tip = box_nodes(spec, xmin=0.5)
    spec.loads = np.stack([point_load(spec, tip, (0.0, -1000.0, 0.0)),
                           face_traction(spec, 2, True, (0.0, 0.0, -2.0e5))])
    spec.weights = np.ones(2)
    return spec


def column_hex_buckling_analysis() -> ProblemSpec:
    """configs/verification/column_hex_buckling_analysis.json: Hex8 40 x 4 x 4
    over 1.0 x 0.05 x 0.05 m, steel (E = 200 GPa, nu = 0.3); x = 0 clamped;
    a -400 Pa axial traction on the end face x = 1 (1 N of compression)."""
    spec = column(3, 40, 4, 4, length=1.0, height=0.05, width=0.05, force=-400.0 * 0.05 * 0.05,
                  young=200.0e9, poisson=0.3)
    spec.name = "column_hex_buckling_analysis"
    return spec


def column_buckling() -> ProblemSpec:
    """configs/benchmarks/column_buckling.json: Q4 40 x 80 over 0.5 x 1.0 m,
    Al 7075-T6 (E = 71.7 GPa, nu = 0.33), t = 10 mm; the base y = 0 clamped;
    1e5 N down spread over the top nodes with x in [0.2, 0.3]; vf 0.25,
    radius 3 cells."""
    spec = ProblemSpec(dim=2, nx=40, ny=80, nz=0, lx=0.5, ly=1.0, lz=0.0, young=71.7e9, poisson=0.33,
                       thickness=0.01, density=2810.0, volume_fraction=0.25, initial_density=0.25,
                       rtol=1e-10, name="column_buckling")
    spec.filter_radius = _radius(spec, 3.0)
    fixed = np.zeros(spec.num_dofs, np.uint8)
    for node in box_nodes(spec, ymax=0.0):
        fixed[node * 2: node * 2 + 2] = 1
    spec.fixed = fixed
    spec.loads = point_load(spec, box_nodes(spec, ymin=1.0, xmin=0.2, xmax=0.3), (0.0, -1.0e5))[None, :]
    spec.weights = np.ones(1)
    return spec
