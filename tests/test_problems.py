"""Host-side model builders of sparlab_gb300.problems: the selectors and load
distributions that the published benchmark and verification models use
(src/fem/Selector.cpp:12-19, 52-54; src/fem/BoundaryConditions.cpp:27-57)."""
import numpy as np
import pytest

from sparlab_gb300 import problems as P


def test_box_selector_is_inclusive_within_the_diagonal_tolerance():
    spec = P.cantilever_beam()  # 160 x 80 cells over 0.4 x 0.2 m
    tip = P.box_nodes(spec, xmin=0.4, ymin=0.0975, ymax=0.1025)
    c = spec.node_coords()[tip]
    # the bounds are node coordinates: both end nodes are in (j = 39, 40, 41)
    assert len(tip) == 3 and np.allclose(c[:, 0], 0.4) and np.allclose(c[:, 1], [0.0975, 0.1, 0.1025])
    # a bound a hair inside a node still selects it, one cell inside does not
    tol = 1e-9 * np.hypot(spec.lx, spec.ly)
    assert len(P.box_nodes(spec, xmin=0.4 + 0.5 * tol, ymin=0.0975, ymax=0.1025)) == 3
    assert len(P.box_nodes(spec, xmin=0.4, ymin=0.0975 + 0.0025, ymax=0.1025)) == 2
    # unbounded sides take every node on the face
    assert len(P.box_nodes(spec, xmax=0.0)) == spec.ny + 1


def test_total_point_load_keeps_its_resultant():
    spec = P.bracket_3d()
    for f, want in zip(spec.loads, ((0.0, -3000.0, 0.0), (0.0, 0.0, 1200.0))):
        np.testing.assert_allclose(f.reshape(-1, 3).sum(axis=0), want, rtol=1e-14, atol=1e-9)
    # tip bottom edge: the nz + 1 nodes at x = 0.24, y = 0
    edge = np.flatnonzero(spec.loads[0].reshape(-1, 3)[:, 1])
    assert len(edge) == spec.nz + 1


@pytest.mark.parametrize("axis,at_max", [(2, True), (0, True), (1, False)])
def test_face_traction_is_consistent(axis, at_max):
    spec = P.block_3d_analysis()
    t = np.array([0.3, -2.0, 5.0]) * 1e4
    f = P.face_traction(spec, axis, at_max, t).reshape(-1, 3)
    ext = [spec.lx, spec.ly, spec.lz]
    area = np.prod([ext[a] for a in range(3) if a != axis])
    np.testing.assert_allclose(f.sum(axis=0), t * area, rtol=1e-12)
    # only nodes on that face carry force, corners a quarter of an inner node's
    c = spec.node_coords()
    loaded = np.flatnonzero(np.abs(f).sum(axis=1) > 0)
    assert np.allclose(c[loaded, axis], ext[axis] if at_max else 0.0)
    mags = np.abs(f[loaded, 2])
    assert np.isclose(mags.max() / mags.min(), 4.0)


def test_face_traction_in_2d_uses_the_thickness():
    spec = P.cantilever_analysis()  # t = 10 mm
    f = P.face_traction(spec, 0, True, (0.0, -1.0e5)).reshape(-1, 2)
    np.testing.assert_allclose(f.sum(axis=0), [0.0, -1.0e5 * spec.ly * spec.thickness], rtol=1e-12)


def test_benchmark_models_match_their_configs():
    mbb = P.mbb_beam()
    # u_x fixed on x = 0 only, plus the roller's u_y at (180, 0)
    fixed = mbb.fixed.reshape(-1, 2)
    assert fixed[:, 0].sum() == mbb.ny + 1 and fixed[:, 1].sum() == 1
    assert fixed[mbb.node_index(180, 0), 1] == 1
    assert mbb.loads[0].reshape(-1, 2)[mbb.node_index(0, 60), 1] == -1.0
    assert mbb.filter_radius == pytest.approx(4.5)
    col = P.column_buckling()
    assert col.fixed.reshape(-1, 2)[: col.nx + 1].all() and col.fixed.sum() == 2 * (col.nx + 1)
    assert np.count_nonzero(col.loads[0]) == 9  # x = 0.2 .. 0.3 at 0.0125 spacing
    assert col.filter_radius == pytest.approx(3.0 * 0.0125)
    assert P.bracket_3d(large=True).num_dofs == 356475
