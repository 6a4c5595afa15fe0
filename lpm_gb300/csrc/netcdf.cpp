// netcdf.cpp -- NetCDF output of a polygon mesh and its fields, written by the
// library itself (no netCDF library): the classic format with 64-bit offsets
// (CDF-2), which every netCDF reader opens.
//
// The reference's writer (NcWriter, src/netcdf/lpm_netcdf_writer.cpp:5-47)
// opens a file with the global attribute "LPM" = "Lagrangian Particle
// Methods" and an unlimited "time" dimension with a "time" variable carrying
// a "units" attribute; its mesh and field definitions
// (src/netcdf/lpm_netcdf_impl.hpp) name the arrays "vertices.phys_crds",
// "faces.phys_crds", "faces.vertices", "faces.mask" and "faces.area" over
// the dimensions "vertices", "faces", "coord" and "facekind".  This file
// writes one time record of that content: the coordinates and the fields
// are record variables (time first), the face topology, masks and areas are
// fixed.  Reference difference: the reference creates NetCDF-4 (HDF5)
// files, which need the HDF5 library; the data model is the same.
//
// Layout of the classic format: big-endian; header = magic "CDF\2", record
// count, dimension list, global attribute list, variable list (name,
// dimension ids, attributes, type, size per record, 64-bit start offset);
// then the fixed variables' data, then the records (each record holds every
// record variable's slice in variable order).
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "lpm_host.hpp"

namespace lpm {
int fail(int code, const char* msg);  // capi.cu
int handle_exception();               // capi.cu

namespace {

constexpr uint32_t NC_DIMENSION = 0x0A, NC_VARIABLE = 0x0B, NC_ATTRIBUTE = 0x0C;
constexpr uint32_t T_BYTE = 1, T_CHAR = 2, T_INT = 4, T_DOUBLE = 6;

struct Buf {
  std::vector<unsigned char> b;
  void u32(uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) b.push_back(static_cast<unsigned char>(v >> s));
  }
  void u64(uint64_t v) {
    for (int s = 56; s >= 0; s -= 8) b.push_back(static_cast<unsigned char>(v >> s));
  }
  void f64(double d) {
    uint64_t v;
    std::memcpy(&v, &d, 8);
    u64(v);
  }
  void pad4() {
    while (b.size() % 4) b.push_back(0);
  }
  void name(const std::string& s) {
    u32(uint32_t(s.size()));
    b.insert(b.end(), s.begin(), s.end());
    pad4();
  }
};

struct Var {
  std::string name;
  std::vector<int> dims;  // dimension ids
  uint32_t type;
  bool record;
  uint64_t vsize;  // bytes (per record for record variables), padded to 4
  std::vector<std::pair<std::string, std::string>> text_atts;
  // data writer: appends this variable's bytes (one record) to a buffer
  std::function<void(Buf&)> write;
  uint64_t begin = 0;
};

uint64_t pad4(uint64_t n) { return (n + 3) / 4 * 4; }

}  // namespace
}  // namespace lpm

extern "C" {

int lpm_netcdf_write_polymesh(const char* path, int ndim, int64_t nv, const double* vx,
                              int64_t nf, int nfv, const int32_t* fverts, const uint8_t* fmask,
                              const double* farea, const double* fx, double time, int nfields,
                              const lpm_vtk_field* fields) {
  using namespace lpm;
  try {
    if (!path || !vx || !fverts || !fmask || !farea || !fx || nv <= 0 || nf <= 0)
      return fail(LPM_ERR_ARG, "lpm_netcdf_write_polymesh: null or empty argument");
    if ((ndim != 2 && ndim != 3) || (nfv != 3 && nfv != 4))
      return fail(LPM_ERR_ARG, "lpm_netcdf_write_polymesh: ndim must be 2 or 3, nfv 3 or 4");
    if (nv > (int64_t(1) << 31) - 1 || nf > (int64_t(1) << 31) - 1)
      return fail(LPM_ERR_ARG, "lpm_netcdf_write_polymesh: counts out of range");
    if (nfields < 0 || (nfields > 0 && !fields))
      return fail(LPM_ERR_ARG, "lpm_netcdf_write_polymesh: bad field list");
    enum { D_TIME, D_COORD, D_VERTS, D_FACES, D_KIND };
    const std::vector<std::pair<std::string, uint64_t>> dims = {
        {"time", 0}, {"coord", uint64_t(ndim)}, {"vertices", uint64_t(nv)},
        {"faces", uint64_t(nf)}, {"facekind", uint64_t(nfv)}};
    std::vector<Var> vars;
    auto doubles = [](const double* p, int64_t n) {
      return [p, n](Buf& o) {
        for (int64_t i = 0; i < n; ++i) o.f64(p[i]);
      };
    };
    vars.push_back({"time", {D_TIME}, T_DOUBLE, true, 8, {{"units", "time_units"}},
                    [time](Buf& o) { o.f64(time); }});
    vars.push_back({"vertices.phys_crds", {D_TIME, D_VERTS, D_COORD}, T_DOUBLE, true,
                    uint64_t(8 * nv * ndim), {}, doubles(vx, nv * ndim)});
    vars.push_back({"faces.phys_crds", {D_TIME, D_FACES, D_COORD}, T_DOUBLE, true,
                    uint64_t(8 * nf * ndim), {}, doubles(fx, nf * ndim)});
    for (int k = 0; k < nfields; ++k) {
      const lpm_vtk_field& f = fields[k];
      if (!f.name || !f.data || (f.location != 0 && f.location != 1) ||
          (f.ncomp != 1 && f.ncomp != ndim))
        return fail(LPM_ERR_ARG,
                    "lpm_netcdf_write_polymesh: a field needs a name, data, location 0/1 "
                    "and 1 or ndim components");
      const int64_t n = (f.location == 0 ? nv : nf) * f.ncomp;
      std::vector<int> d = {D_TIME, f.location == 0 ? D_VERTS : D_FACES};
      if (f.ncomp > 1) d.push_back(D_COORD);
      vars.push_back({f.name, d, T_DOUBLE, true, uint64_t(8 * n), {}, doubles(f.data, n)});
    }
    vars.push_back({"faces.vertices", {D_FACES, D_KIND}, T_INT, false, uint64_t(4 * nf * nfv),
                    {}, [fverts, nf, nfv](Buf& o) {
                      for (int64_t i = 0; i < nf * nfv; ++i) o.u32(uint32_t(fverts[i]));
                    }});
    vars.push_back({"faces.mask", {D_FACES}, T_BYTE, false, pad4(uint64_t(nf)), {},
                    [fmask, nf](Buf& o) {
                      for (int64_t i = 0; i < nf; ++i) o.b.push_back(fmask[i] ? 1 : 0);
                      o.pad4();
                    }});
    vars.push_back({"faces.area", {D_FACES}, T_DOUBLE, false, uint64_t(8 * nf), {},
                    doubles(farea, nf)});

    // header with placeholder offsets, to learn its size
    auto header = [&](Buf& h) {
      h.b.clear();
      h.b.insert(h.b.end(), {'C', 'D', 'F', 2});
      h.u32(1);  // one record
      h.u32(NC_DIMENSION);
      h.u32(uint32_t(dims.size()));
      for (const auto& d : dims) {
        h.name(d.first);
        h.u32(uint32_t(d.second));
      }
      const std::string lpm_att = "Lagrangian Particle Methods";
      h.u32(NC_ATTRIBUTE);
      h.u32(1);
      h.name("LPM");
      h.u32(T_CHAR);
      h.u32(uint32_t(lpm_att.size()));
      h.b.insert(h.b.end(), lpm_att.begin(), lpm_att.end());
      h.pad4();
      h.u32(NC_VARIABLE);
      h.u32(uint32_t(vars.size()));
      for (const auto& v : vars) {
        h.name(v.name);
        h.u32(uint32_t(v.dims.size()));
        for (int d : v.dims) h.u32(uint32_t(d));
        if (v.text_atts.empty()) {
          h.u32(0);
          h.u32(0);
        } else {
          h.u32(NC_ATTRIBUTE);
          h.u32(uint32_t(v.text_atts.size()));
          for (const auto& a : v.text_atts) {
            h.name(a.first);
            h.u32(T_CHAR);
            h.u32(uint32_t(a.second.size()));
            h.b.insert(h.b.end(), a.second.begin(), a.second.end());
            h.pad4();
          }
        }
        h.u32(v.type);
        h.u32(v.vsize > 0xFFFFFFFFull ? 0xFFFFFFFFu : uint32_t(v.vsize));
        h.u64(v.begin);
      }
    };
    Buf h;
    header(h);
    uint64_t off = h.b.size();
    for (auto& v : vars)
      if (!v.record) {
        v.begin = off;
        off += v.vsize;
      }
    for (auto& v : vars)
      if (v.record) {
        v.begin = off;
        off += v.vsize;
      }
    header(h);  // the same size, now with the offsets
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(LPM_ERR_ARG, (std::string("cannot open ") + path).c_str());
    bool ok = std::fwrite(h.b.data(), 1, h.b.size(), f) == h.b.size();
    for (int pass = 0; pass < 2 && ok; ++pass)
      for (auto& v : vars) {
        if (v.record != (pass == 1)) continue;
        Buf d;
        d.b.reserve(v.vsize);
        v.write(d);
        ok = ok && d.b.size() == v.vsize && std::fwrite(d.b.data(), 1, d.b.size(), f) == d.b.size();
      }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(LPM_ERR_ARG, "lpm_netcdf_write_polymesh: write failed");
    return LPM_OK;
  } catch (...) {
    return handle_exception();
  }
}

}  // extern "C"
