"""VTK XML PolyData output of a panel mesh, mirroring the reference's
VtkPolymeshInterface (src/vtk/lpm_vtk_io.hpp:36-76,
src/vtk/lpm_vtk_io_impl.hpp): vertices are points, leaf faces are polygons,
cell array "area", "lag_crds" point and cell arrays, then whatever is added.
The file is written by the library (lpm_vtk_write_polymesh), not by VTK.

    vtk = VtkPolymeshInterface(vx, fverts, fmask, farea, lag_vx=vx0, lag_fx=fx0)
    vtk.add_scalar_point_data(vort_verts, "rel_vort")
    vtk.add_vector_cell_data(vel_faces, "velocity")
    vtk.write("bve_0000.vtp")

Arrays may be numpy arrays or tensors (device tensors are copied to the
host); cell arrays are given per face slot, leaf slots are written.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .core import check, lib


class _Field(C.Structure):
    _fields_ = [("name", C.c_char_p), ("location", C.c_int), ("ncomp", C.c_int),
                ("data", C.c_void_p)]


def _host(a) -> np.ndarray:
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(a, np.float64)


class VtkPolymeshInterface:
    def __init__(self, vx, fverts, fmask, farea, lag_vx=None, lag_fx=None, height=None):
        self.vx = _host(vx)
        self.ndim = self.vx.shape[1]
        self.fverts = np.ascontiguousarray(fverts, np.int32)
        self.fmask = np.ascontiguousarray(
            fmask.detach().cpu().numpy() if hasattr(fmask, "detach") else fmask, np.uint8)
        self.farea = _host(farea)
        self.height = None if height is None else _host(height)
        self._fields: list[tuple[str, int, np.ndarray]] = []
        if lag_vx is not None:
            self.add_vector_point_data(lag_vx, "lag_crds")
        if lag_fx is not None:
            self.add_vector_cell_data(lag_fx, "lag_crds")

    def update_positions(self, vx) -> None:
        self.vx = _host(vx)

    def _add(self, a, name: str, loc: int) -> None:
        a = _host(a)
        n = self.vx.shape[0] if loc == 0 else self.fverts.shape[0]
        if a.shape[0] != n:
            raise ValueError(f"{name}: {a.shape[0]} tuples, expected {n}")
        self._fields.append((name, loc, a.reshape(n, -1)))

    def add_scalar_point_data(self, s, name: str) -> None:
        self._add(s, name, 0)

    def add_vector_point_data(self, v, name: str) -> None:
        self._add(v, name, 0)

    def add_scalar_cell_data(self, s, name: str) -> None:
        self._add(s, name, 1)

    def add_vector_cell_data(self, v, name: str) -> None:
        self._add(v, name, 1)

    def add_tracers(self, point_tracers, cell_tracers, names=None) -> None:
        if len(point_tracers) != len(cell_tracers):
            raise ValueError("point and cell tracer lists differ in length")
        for k, (p, c) in enumerate(zip(point_tracers, cell_tracers)):
            name = names[k] if names else f"tracer{k}"
            self.add_scalar_point_data(p, name)
            self.add_scalar_cell_data(c, name)

    def write(self, path: str) -> None:
        fields = (_Field * max(1, len(self._fields)))()
        names = []
        for k, (name, loc, a) in enumerate(self._fields):
            names.append(name.encode())
            fields[k] = _Field(names[-1], loc, a.shape[1], a.ctypes.data)
        h = self.height
        check(lib().lpm_vtk_write_polymesh(
            str(path).encode(), self.ndim, self.vx.shape[0], self.vx.ctypes.data,
            None if h is None else h.ctypes.data, self.fverts.shape[0], self.fverts.shape[1],
            self.fverts.ctypes.data, self.fmask.ctypes.data, self.farea.ctypes.data,
            len(self._fields), C.addressof(fields)))


class NcPolymeshWriter(VtkPolymeshInterface):
    """NetCDF output of the same content (NcWriter with the reference's mesh
    and field names, src/netcdf/lpm_netcdf_writer.cpp,
    src/netcdf/lpm_netcdf_impl.hpp), written by the library
    (lpm_netcdf_write_polymesh) in the classic format with 64-bit offsets:
    one time record of vertices.phys_crds, faces.phys_crds and the added
    fields (1 or ndim components), and faces.vertices / faces.mask /
    faces.area.  Cell arrays are given per face slot (all slots written).

        nc = NcPolymeshWriter(vx, fverts, fmask, farea, fx)
        nc.add_scalar_cell_data(vort_faces, "rel_vort")
        nc.write("bve_0000.nc", t=0.0)
    """

    def __init__(self, vx, fverts, fmask, farea, fx):
        super().__init__(vx, fverts, fmask, farea)
        self.fx = _host(fx)

    def write(self, path: str, t: float = 0.0) -> None:
        fields = (_Field * max(1, len(self._fields)))()
        names = []
        for k, (name, loc, a) in enumerate(self._fields):
            names.append(name.encode())
            fields[k] = _Field(names[-1], loc, a.shape[1], a.ctypes.data)
        check(lib().lpm_netcdf_write_polymesh(
            str(path).encode(), self.ndim, self.vx.shape[0], self.vx.ctypes.data,
            self.fverts.shape[0], self.fverts.shape[1], self.fverts.ctypes.data,
            self.fmask.ctypes.data, self.farea.ctypes.data, self.fx.ctypes.data, float(t),
            len(self._fields), C.addressof(fields)))
