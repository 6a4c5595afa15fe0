"""NetCDF output (lpm_netcdf_write_polymesh / NcPolymeshWriter), read back by
an independent reader (scipy's classic-format NetCDF reader): dimensions,
the global attribute and the time variable of the reference's NcWriter
(src/netcdf/lpm_netcdf_writer.cpp:5-47), and every array bit for bit."""
import math

import numpy as np
import pytest

from lpm_gb300 import core
from lpm_gb300.vtk import NcPolymeshWriter

netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.mark.parametrize("kind,level,radius", [(core.MESH_ICOS_TRI, 2, 1.0),
                                               (core.MESH_QUAD_RECT, 3, 4.0)])
def test_netcdf_round_trip(tmp_path, kind, level, radius):
    vx, fx, fa, fm = core.build_mesh(kind, level, radius)
    fv = core.mesh_face_vertices(kind, level, radius)
    nd = vx.shape[1]
    rng = np.random.default_rng(5)
    zeta_f = rng.standard_normal(fx.shape[0])
    vel_v = rng.standard_normal((vx.shape[0], nd))
    nc = NcPolymeshWriter(vx, fv, fm, fa, fx)
    nc.add_scalar_cell_data(zeta_f, "rel_vort")
    nc.add_vector_point_data(vel_v, "velocity")
    path = tmp_path / "mesh.nc"
    nc.write(path, t=0.25)
    with netcdf(str(path), "r", mmap=False) as f:
        assert f.version_byte == 2
        assert f.LPM == b"Lagrangian Particle Methods"
        assert f.dimensions["time"] is None  # unlimited
        assert f.dimensions["vertices"] == vx.shape[0]
        assert f.dimensions["faces"] == fx.shape[0]
        assert f.dimensions["coord"] == nd
        assert f.dimensions["facekind"] == fv.shape[1]
        v = f.variables
        assert v["time"].units == b"time_units" and v["time"][:].tolist() == [0.25]
        assert np.array_equal(v["vertices.phys_crds"][0], vx)
        assert np.array_equal(v["faces.phys_crds"][0], fx)
        assert np.array_equal(v["faces.vertices"][:], fv)
        assert np.array_equal(v["faces.mask"][:].astype(np.uint8), fm)
        assert np.array_equal(v["faces.area"][:], fa)
        assert np.array_equal(v["rel_vort"][0], zeta_f)
        assert np.array_equal(v["velocity"][0], vel_v)
        assert v["velocity"].dimensions == ("time", "vertices", "coord")
    if kind == core.MESH_ICOS_TRI:
        assert math.isclose(fa.sum(), 4 * math.pi, rel_tol=1e-13)


def test_netcdf_rejects_bad_fields(tmp_path):
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, 1, 1.0)
    fv = core.mesh_face_vertices(core.MESH_ICOS_TRI, 1)
    nc = NcPolymeshWriter(vx, fv, fm, fa, fx)
    nc.add_scalar_point_data(np.zeros((vx.shape[0], 2)), "two_components")
    with pytest.raises(core.LpmError):
        nc.write(tmp_path / "bad.nc")
