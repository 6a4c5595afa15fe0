// vtk.cpp -- VTK XML PolyData (.vtp) output of a polygon mesh, written by the
// library itself (no VTK dependency).  Content of the reference's
// VtkPolymeshInterface (src/vtk/lpm_vtk_io_impl.hpp): the vertices are the
// points (z = 0 in the plane, or the height field there), every leaf face
// (no children: mask 0) is a polygon of its vertex list in slot order, cell
// array "area" first, then the caller's point arrays (one tuple per vertex)
// and cell arrays (given per face slot; the leaf slots are written, in slot
// order).  Reference differences: the spherical height-field constructor of
// the reference (make_points(height), :56-76) computes the displaced
// coordinates but never inserts them, leaving the point set empty; here the
// points are (1 + h) x as that code intends.  Values are written in ASCII
// with the shortest representation that reads back to the same double.
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lpm_host.hpp"

namespace lpm {
int fail(int code, const char* msg);  // capi.cu
int handle_exception();               // capi.cu

namespace {

class Out {
 public:
  explicit Out(const char* path) : f_(std::fopen(path, "wb")) {
    if (!f_) throw Error(LPM_ERR_ARG, std::string("cannot open ") + path + " for writing");
    buf_.reserve(1 << 20);
  }
  ~Out() {
    if (f_) std::fclose(f_);
  }
  void str(const char* s) { buf_.append(s); flush_if(); }
  void str(const std::string& s) { buf_.append(s); flush_if(); }
  void num(double v) {
    char t[32];
    auto r = std::to_chars(t, t + sizeof(t), v);
    buf_.append(t, r.ptr);
    buf_.push_back(' ');
    flush_if();
  }
  void num(int64_t v) {
    char t[24];
    auto r = std::to_chars(t, t + sizeof(t), v);
    buf_.append(t, r.ptr);
    buf_.push_back(' ');
    flush_if();
  }
  void close() {
    write_out();
    if (std::fclose(f_) != 0) {
      f_ = nullptr;
      throw Error(LPM_ERR_ARG, "write failed");
    }
    f_ = nullptr;
  }

 private:
  void flush_if() {
    if (buf_.size() > (1u << 20)) write_out();
  }
  void write_out() {
    if (!buf_.empty() && std::fwrite(buf_.data(), 1, buf_.size(), f_) != buf_.size())
      throw Error(LPM_ERR_ARG, "write failed");
    buf_.clear();
  }
  std::FILE* f_;
  std::string buf_;
};

std::string xml_escape(const char* s) {
  std::string o;
  for (; *s; ++s) {
    switch (*s) {
      case '&': o += "&amp;"; break;
      case '<': o += "&lt;"; break;
      case '>': o += "&gt;"; break;
      case '"': o += "&quot;"; break;
      default: o += *s;
    }
  }
  return o;
}

void array_open(Out& o, const char* type, const char* name, int ncomp) {
  o.str("        <DataArray type=\"");
  o.str(type);
  o.str("\"");
  if (name) o.str(" Name=\"" + xml_escape(name) + "\"");
  o.str(" NumberOfComponents=\"" + std::to_string(ncomp) + "\" format=\"ascii\">\n");
}
void array_close(Out& o) { o.str("\n        </DataArray>\n"); }

}  // namespace

void vtk_write_polymesh(const char* path, int ndim, int64_t nv, const double* vx,
                        const double* height, int64_t nf, int nfv, const int32_t* fverts,
                        const uint8_t* fmask, const double* farea, int nfields,
                        const lpm_vtk_field* fields) {
  int64_t nleaf = 0;
  for (int64_t i = 0; i < nf; ++i) nleaf += fmask[i] == 0;
  for (int64_t i = 0; i < nf; ++i) {
    if (fmask[i]) continue;
    for (int k = 0; k < nfv; ++k)
      if (fverts[i * nfv + k] < 0 || fverts[i * nfv + k] >= nv)
        throw Error(LPM_ERR_ARG, "face vertex index out of range");
  }
  Out o(path);
  o.str("<?xml version=\"1.0\"?>\n<VTKFile type=\"PolyData\" version=\"1.0\" "
        "byte_order=\"LittleEndian\" header_type=\"UInt64\">\n  <PolyData>\n");
  o.str("    <Piece NumberOfPoints=\"" + std::to_string(nv) +
        "\" NumberOfVerts=\"0\" NumberOfLines=\"0\" NumberOfStrips=\"0\" NumberOfPolys=\"" +
        std::to_string(nleaf) + "\">\n");
  o.str("      <PointData>\n");
  for (int k = 0; k < nfields; ++k) {
    const lpm_vtk_field& f = fields[k];
    if (f.location != 0) continue;
    array_open(o, "Float64", f.name, f.ncomp);
    for (int64_t i = 0; i < nv * f.ncomp; ++i) o.num(f.data[i]);
    array_close(o);
  }
  o.str("      </PointData>\n      <CellData>\n");
  array_open(o, "Float64", "area", 1);
  for (int64_t i = 0; i < nf; ++i)
    if (!fmask[i]) o.num(farea[i]);
  array_close(o);
  for (int k = 0; k < nfields; ++k) {
    const lpm_vtk_field& f = fields[k];
    if (f.location != 1) continue;
    array_open(o, "Float64", f.name, f.ncomp);
    for (int64_t i = 0; i < nf; ++i)
      if (!fmask[i])
        for (int c = 0; c < f.ncomp; ++c) o.num(f.data[i * f.ncomp + c]);
    array_close(o);
  }
  o.str("      </CellData>\n      <Points>\n");
  array_open(o, "Float64", "Points", 3);
  for (int64_t i = 0; i < nv; ++i) {
    const double* p = vx + i * ndim;
    if (ndim == 3) {
      const double s = height ? 1.0 + height[i] : 1.0;
      o.num(height ? s * p[0] : p[0]);
      o.num(height ? s * p[1] : p[1]);
      o.num(height ? s * p[2] : p[2]);
    } else {
      o.num(p[0]);
      o.num(p[1]);
      o.num(height ? height[i] : 0.0);
    }
  }
  array_close(o);
  o.str("      </Points>\n      <Polys>\n");
  array_open(o, "Int64", "connectivity", 1);
  for (int64_t i = 0; i < nf; ++i)
    if (!fmask[i])
      for (int k = 0; k < nfv; ++k) o.num(int64_t(fverts[i * nfv + k]));
  array_close(o);
  array_open(o, "Int64", "offsets", 1);
  for (int64_t c = 1; c <= nleaf; ++c) o.num(c * nfv);
  array_close(o);
  o.str("      </Polys>\n    </Piece>\n  </PolyData>\n</VTKFile>\n");
  o.close();
}

}  // namespace lpm

extern "C" {

int lpm_mesh_face_vertices(int kind, int level, double radius, int* nfv, int32_t* fverts) {
  try {
    if (!nfv) return lpm::fail(LPM_ERR_ARG, "null nfv");
    *nfv = lpm::mesh_nfv(kind);
    if (!fverts) return LPM_OK;
    if (!(radius > 0) || !std::isfinite(radius)) return lpm::fail(LPM_ERR_ARG, "radius must be > 0");
    int64_t nv, nf;
    lpm::mesh_sizes(kind, level, &nv, &nf);
    const int ndim = kind == LPM_MESH_QUAD_RECT ? 2 : 3;
    std::vector<double> vx(size_t(nv) * ndim), fx(size_t(nf) * ndim), fa(nf);
    std::vector<uint8_t> fm(nf);
    lpm::mesh_build(kind, level, radius, vx.data(), fx.data(), fa.data(), fm.data(), fverts);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

int lpm_vtk_write_polymesh(const char* path, int ndim, int64_t nv, const double* vx,
                           const double* height, int64_t nf, int nfv, const int32_t* fverts,
                           const uint8_t* fmask, const double* farea, int nfields,
                           const lpm_vtk_field* fields) {
  try {
    if (!path) return lpm::fail(LPM_ERR_ARG, "null path");
    if (ndim != 2 && ndim != 3) return lpm::fail(LPM_ERR_ARG, "ndim must be 2 or 3");
    if (nfv < 3 || nfv > 4) return lpm::fail(LPM_ERR_ARG, "nfv must be 3 or 4");
    if (nv < 0 || nf < 0 || nfields < 0) return lpm::fail(LPM_ERR_ARG, "negative count");
    if ((nv > 0 && !vx) || (nf > 0 && (!fverts || !fmask || !farea)) || (nfields > 0 && !fields))
      return lpm::fail(LPM_ERR_ARG, "null array");
    for (int k = 0; k < nfields; ++k) {
      const lpm_vtk_field& f = fields[k];
      if (!f.name || (f.location != 0 && f.location != 1) || f.ncomp < 1 || f.ncomp > 9 ||
          (!f.data && (f.location == 0 ? nv : nf) > 0))
        return lpm::fail(LPM_ERR_ARG, "bad field (name, location 0/1, 1-9 components, data)");
    }
    lpm::vtk_write_polymesh(path, ndim, nv, vx, height, nf, nfv, fverts, fmask, farea, nfields,
                            fields);
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}

}  // extern "C"
