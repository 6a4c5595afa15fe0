"""Mesh connectivity and the VTK PolyData writer (host only).

The writer's content follows VtkPolymeshInterface (src/vtk/lpm_vtk_io_impl.hpp):
points = vertices, polygons = leaf faces in slot order, cell array "area",
then lag_crds and the added arrays.  Files are parsed back with the standard
XML parser and every value must read back bit for bit."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from lpm_gb300 import core
from lpm_gb300.vtk import VtkPolymeshInterface


def _arrays(path):
    root = ET.parse(path).getroot()
    piece = root.find("PolyData/Piece")
    out = {}
    for sec in ("PointData", "CellData", "Points", "Polys"):
        for da in piece.find(sec):
            vals = np.array(da.text.split(), dtype=np.float64 if da.get("type") == "Float64"
                            else np.int64)
            out[(sec, da.get("Name"))] = vals.reshape(-1, int(da.get("NumberOfComponents")))
    return piece, out


@pytest.mark.parametrize("kind,level,radius", [(core.MESH_ICOS_TRI, 2, 1.0),
                                               (core.MESH_CUBED_SPHERE, 2, 1.0),
                                               (core.MESH_QUAD_RECT, 3, 4.0)])
def test_face_vertices_orientation_and_centres(kind, level, radius):
    vx, fx, fa, fm = core.build_mesh(kind, level, radius)
    fv = core.mesh_face_vertices(kind, level, radius)
    assert fv.shape == (fx.shape[0], 3 if kind == core.MESH_ICOS_TRI else 4)
    assert fv.min() >= 0 and fv.max() < vx.shape[0]
    p = vx[fv]  # nf x nfv x ndim
    c = p.mean(axis=1)
    if vx.shape[1] == 3:
        c = c / np.linalg.norm(c, axis=1, keepdims=True)
        n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        assert (np.sum(n * fx, 1) > 0).all()  # counter-clockwise seen from outside
    else:
        a = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - \
            (p[:, 1, 1] - p[:, 0, 1]) * (p[:, 2, 0] - p[:, 0, 0])
        assert (a > 0).all()
    assert np.abs(c - fx).max() < 1e-14 * radius


def test_vtp_round_trip(tmp_path):
    kind, level = core.MESH_ICOS_TRI, 2
    vx, fx, fa, fm = core.build_mesh(kind, level)
    fv = core.mesh_face_vertices(kind, level)
    rng = np.random.default_rng(3)
    vort = rng.standard_normal(vx.shape[0])
    vel = rng.standard_normal(fx.shape)
    w = VtkPolymeshInterface(vx, fv, fm, fa, lag_vx=vx, lag_fx=fx)
    w.add_scalar_point_data(vort, "rel_vort")
    w.add_vector_cell_data(vel, "velocity")
    w.add_tracers([vort * 2], [fa * 3], names=["q"])
    path = tmp_path / "mesh.vtp"
    w.write(path)
    piece, A = _arrays(path)
    leaf = fm == 0
    assert int(piece.get("NumberOfPoints")) == vx.shape[0]
    assert int(piece.get("NumberOfPolys")) == int(leaf.sum())
    assert np.array_equal(A[("Points", "Points")], vx)
    assert np.array_equal(A[("Polys", "connectivity")].ravel(), fv[leaf].ravel())
    assert np.array_equal(A[("Polys", "offsets")].ravel(), 3 * np.arange(1, leaf.sum() + 1))
    assert np.array_equal(A[("CellData", "area")].ravel(), fa[leaf])
    assert np.array_equal(A[("CellData", "lag_crds")], fx[leaf])
    assert np.array_equal(A[("PointData", "lag_crds")], vx)
    assert np.array_equal(A[("PointData", "rel_vort")].ravel(), vort)
    assert np.array_equal(A[("CellData", "velocity")], vel[leaf])
    assert np.array_equal(A[("PointData", "q")].ravel(), vort * 2)
    assert np.array_equal(A[("CellData", "q")].ravel(), (fa * 3)[leaf])
    # the cell arrays keep the writer's order: area first
    names = [da.get("Name") for da in piece.find("CellData")]
    assert names[0] == "area"


def test_vtp_height_fields(tmp_path):
    vx, fx, fa, fm = core.build_mesh(core.MESH_QUAD_RECT, 2, 1.0)
    fv = core.mesh_face_vertices(core.MESH_QUAD_RECT, 2, 1.0)
    h = np.sin(vx[:, 0])
    VtkPolymeshInterface(vx, fv, fm, fa, height=h).write(tmp_path / "p.vtp")
    _, A = _arrays(tmp_path / "p.vtp")
    assert np.array_equal(A[("Points", "Points")], np.column_stack([vx, h]))
    assert np.array_equal(A[("Polys", "offsets")].ravel(), 4 * np.arange(1, (fm == 0).sum() + 1))
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, 1)
    fv = core.mesh_face_vertices(core.MESH_ICOS_TRI, 1)
    h = 0.1 * vx[:, 2]
    VtkPolymeshInterface(vx, fv, fm, fa, height=h).write(tmp_path / "s.vtp")
    _, A = _arrays(tmp_path / "s.vtp")
    assert np.array_equal(A[("Points", "Points")], (1 + h)[:, None] * vx)


def test_vtp_errors(tmp_path):
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, 1)
    fv = core.mesh_face_vertices(core.MESH_ICOS_TRI, 1)
    w = VtkPolymeshInterface(vx, fv, fm, fa)
    with pytest.raises(core.LpmError):
        w.write(tmp_path / "no" / "such" / "dir.vtp")
    with pytest.raises(ValueError):
        w.add_scalar_cell_data(np.zeros(3), "short")
    bad = fv.copy()
    bad[np.flatnonzero(fm == 0)[0], 0] = vx.shape[0]
    with pytest.raises(core.LpmError):
        VtkPolymeshInterface(vx, bad, fm, fa).write(tmp_path / "bad.vtp")
