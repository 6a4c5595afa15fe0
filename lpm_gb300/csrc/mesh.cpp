// mesh.cpp -- host-side uniform panel meshes that feed the direct-sum path.
//
// Restates what PolyMesh2d::tree_init does for a uniform mesh
// (src/mesh/lpm_polymesh2d_impl.hpp:26-42): start from a seed, then divide
// every leaf face level by level in index order, appending four children per
// divided face (src/mesh/lpm_faces_impl.hpp:285-431 triangles, :434-574
// quads).  A divided face keeps its slot with mask = 1 and area = 0
// (:427-430, :569-573), so the face arrays hold every tree level.  Child faces
// take the spherical (or planar) barycentre of their vertices as centre and
// the polygon area as the sum of centre-edge triangle areas
// (src/lpm_geometry.hpp:517-547, 594-642).  Edge midpoints become new
// vertices the first time an edge is divided (src/mesh/lpm_edges.cpp:59-96);
// a divided quad's centre becomes a vertex (src/mesh/lpm_faces_impl.hpp
// :503-517).
//
// The seeds are built here from their geometry (icosahedron, cube, 2x2
// square), not read from the reference's seed files, so vertex numbering may
// differ from the reference's; the point sets, areas and the parent/leaf slot
// structure are the same.

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "lpm_gb300.h"
#include "lpm_host.hpp"

namespace lpm {
namespace {

constexpr double PI = 3.1415926535897932384626433832795;

struct Builder {
  int ndim;
  bool sphere;
  int nfv;  // vertices per face
  std::vector<double> vx;
  std::vector<double> fx;
  std::vector<double> area;
  std::vector<uint8_t> mask;
  std::vector<std::array<int64_t, 4>> fverts;
  std::unordered_map<uint64_t, int64_t> mids;

  const double* v(int64_t i) const { return vx.data() + ndim * i; }

  int64_t add_vertex(const double* p) {
    for (int k = 0; k < ndim; ++k) vx.push_back(p[k]);
    return int64_t(vx.size() / ndim) - 1;
  }

  // SphereGeometry::midpoint (normalised half sum) or PlaneGeometry::midpoint.
  void midpoint(double* m, const double* a, const double* b) const {
    for (int k = 0; k < ndim; ++k) m[k] = 0.5 * (a[k] + b[k]);
    if (sphere) normalize(m);
  }
  static void normalize(double* p) {
    const double r = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    const double s = 1.0 / r;
    p[0] *= s;
    p[1] *= s;
    p[2] *= s;
  }
  // barycenter: sum, scale by 1/n, normalise on the sphere.
  void barycenter(double* c, const int64_t* vs, int n) const {
    for (int k = 0; k < ndim; ++k) c[k] = 0;
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < ndim; ++k) c[k] += v(vs[i])[k];
    const double s = 1.0 / n;
    for (int k = 0; k < ndim; ++k) c[k] *= s;
    if (sphere) normalize(c);
  }
  static double sdistance(const double* a, const double* b) {
    const double cp[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                          a[0] * b[1] - a[1] * b[0]};
    const double dp = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    return std::atan2(std::sqrt(cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2]),
                      dp);
  }
  // Spherical triangle area by L'Huilier's theorem; planar by cross product.
  double tri_area(const double* a, const double* b, const double* c) const {
    if (!sphere) {
      const double ar = (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]);
      return 0.5 * std::fabs(ar);
    }
    const double s1 = sdistance(a, b), s2 = sdistance(b, c),
                 s3 = sdistance(c, a);
    const double hp = 0.5 * (s1 + s2 + s3);
    double zz = std::tan(0.5 * hp) * std::tan(0.5 * (hp - s1)) *
                std::tan(0.5 * (hp - s2)) * std::tan(0.5 * (hp - s3));
    if (std::fabs(zz) < 2.220446049250313e-16) zz = 0;
    return 4 * std::atan(std::sqrt(zz));
  }
  double polygon_area(const double* ctr, const int64_t* vs, int n) const {
    double ar = 0;
    for (int i = 0; i < n; ++i) ar += tri_area(ctr, v(vs[i]), v(vs[(i + 1) % n]));
    return ar;
  }

  void add_face(const int64_t* vs) {
    std::array<int64_t, 4> f{-1, -1, -1, -1};
    for (int i = 0; i < nfv; ++i) f[i] = vs[i];
    double c[3] = {0, 0, 0};
    barycenter(c, vs, nfv);
    for (int k = 0; k < ndim; ++k) fx.push_back(c[k]);
    area.push_back(polygon_area(c, vs, nfv));
    mask.push_back(0);
    fverts.push_back(f);
  }

  int64_t edge_mid(int64_t a, int64_t b) {
    const uint64_t lo = uint64_t(a < b ? a : b), hi = uint64_t(a < b ? b : a);
    const uint64_t key = (hi << 32) | lo;
    auto it = mids.find(key);
    if (it != mids.end()) return it->second;
    double m[3];
    midpoint(m, v(a), v(b));
    const int64_t idx = add_vertex(m);
    mids.emplace(key, idx);
    return idx;
  }

  void divide(int64_t f) {
    const std::array<int64_t, 4> p = fverts[f];
    if (nfv == 3) {
      const int64_t m01 = edge_mid(p[0], p[1]);
      const int64_t m12 = edge_mid(p[1], p[2]);
      const int64_t m20 = edge_mid(p[2], p[0]);
      const int64_t k0[3] = {p[0], m01, m20};
      const int64_t k1[3] = {m01, p[1], m12};
      const int64_t k2[3] = {m20, m12, p[2]};
      const int64_t k3[3] = {m12, m20, m01};
      add_face(k0);
      add_face(k1);
      add_face(k2);
      add_face(k3);
    } else {
      int64_t m[4];
      for (int i = 0; i < 4; ++i) m[i] = edge_mid(p[i], p[(i + 1) % 4]);
      // the parent's centre coordinate becomes the shared inner vertex
      double c[3] = {0, 0, 0};
      for (int k = 0; k < ndim; ++k) c[k] = fx[ndim * f + k];
      const int64_t ci = add_vertex(c);
      for (int i = 0; i < 4; ++i) {
        int64_t kv[4];
        kv[i] = p[i];
        kv[(i + 1) % 4] = m[i];
        kv[(i + 2) % 4] = ci;
        kv[(i + 3) % 4] = m[(i + 3) % 4];
        add_face(kv);
      }
    }
    area[f] = 0.0;
    mask[f] = 1;
  }

  void tree(int levels) {
    int64_t start = 0;
    for (int l = 0; l < levels; ++l) {
      const int64_t stop = int64_t(mask.size());
      for (int64_t j = start; j < stop; ++j)
        if (!mask[j]) divide(j);
      start = stop;
    }
  }

  // Orient a face counter-clockwise as seen from outside (sphere) or from +z.
  void orient(int64_t* vs) const {
    const double* a = v(vs[0]);
    const double* b = v(vs[1]);
    const double* c = v(vs[2]);
    double s;
    if (sphere) {
      const double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      const double ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
      const double n[3] = {ab[1] * ac[2] - ab[2] * ac[1],
                           ab[2] * ac[0] - ab[0] * ac[2],
                           ab[0] * ac[1] - ab[1] * ac[0]};
      s = n[0] * (a[0] + b[0] + c[0]) + n[1] * (a[1] + b[1] + c[1]) +
          n[2] * (a[2] + b[2] + c[2]);
    } else {
      s = (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]);
    }
    if (s < 0) {
      // reverse, keeping vs[0]
      for (int i = 1, j = nfv - 1; i < j; ++i, --j) std::swap(vs[i], vs[j]);
    }
  }
};

void seed_icosahedron(Builder& b) {
  b.ndim = 3;
  b.sphere = true;
  b.nfv = 3;
  const double zr = 1.0 / std::sqrt(5.0), rr = 2.0 / std::sqrt(5.0);
  const double north[3] = {0, 0, 1};
  b.add_vertex(north);
  for (int k = 0; k < 5; ++k) {  // upper ring 1..5
    const double t = 2 * PI * k / 5;
    const double p[3] = {rr * std::cos(t), rr * std::sin(t), zr};
    b.add_vertex(p);
  }
  for (int k = 0; k < 5; ++k) {  // lower ring 6..10
    const double t = 2 * PI * k / 5 + PI / 5;
    const double p[3] = {rr * std::cos(t), rr * std::sin(t), -zr};
    b.add_vertex(p);
  }
  const double south[3] = {0, 0, -1};
  b.add_vertex(south);
  auto U = [](int k) { return int64_t(1 + (k % 5)); };
  auto L = [](int k) { return int64_t(6 + (k % 5)); };
  for (int k = 0; k < 5; ++k) {
    int64_t f[3] = {0, U(k), U(k + 1)};
    b.orient(f);
    b.add_face(f);
  }
  for (int k = 0; k < 5; ++k) {
    int64_t f1[3] = {U(k), L(k), U(k + 1)};
    b.orient(f1);
    b.add_face(f1);
    int64_t f2[3] = {U(k + 1), L(k), L(k + 1)};
    b.orient(f2);
    b.add_face(f2);
  }
  for (int k = 0; k < 5; ++k) {
    int64_t f[3] = {11, L(k + 1), L(k)};
    b.orient(f);
    b.add_face(f);
  }
}

void seed_cube(Builder& b) {
  b.ndim = 3;
  b.sphere = true;
  b.nfv = 4;
  const double s = 1.0 / std::sqrt(3.0);
  // vertex index = 4*(x>0) + 2*(y>0) + (z>0)
  for (int i = 0; i < 8; ++i) {
    const double p[3] = {(i & 4) ? s : -s, (i & 2) ? s : -s, (i & 1) ? s : -s};
    b.add_vertex(p);
  }
  const int64_t faces[6][4] = {{4, 6, 7, 5}, {0, 1, 3, 2}, {2, 3, 7, 6},
                               {0, 4, 5, 1}, {1, 5, 7, 3}, {0, 2, 6, 4}};
  for (int f = 0; f < 6; ++f) {
    int64_t vs[4] = {faces[f][0], faces[f][1], faces[f][2], faces[f][3]};
    b.orient(vs);
    b.add_face(vs);
  }
}

void seed_square(Builder& b, double radius) {
  b.ndim = 2;
  b.sphere = false;
  b.nfv = 4;
  // 3 x 3 grid on [-r, r]^2, index = 3*row + col, row along y
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      const double p[2] = {radius * (c - 1), radius * (r - 1)};
      b.add_vertex(p);
    }
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 2; ++c) {
      int64_t vs[4] = {3 * r + c, 3 * r + c + 1, 3 * (r + 1) + c + 1,
                       3 * (r + 1) + c};
      b.orient(vs);
      b.add_face(vs);
    }
}

int64_t ipow4(int l) {
  int64_t r = 1;
  for (int i = 0; i < l; ++i) r *= 4;
  return r;
}

}  // namespace

void mesh_sizes(int kind, int level, int64_t* nv, int64_t* nf) {
  if (level < 0 || level > 10) throw std::invalid_argument("mesh level out of range [0,10]");
  int64_t nf0;
  switch (kind) {
    case LPM_MESH_ICOS_TRI:
      nf0 = 20;
      *nv = 2 + 10 * ipow4(level);  // IcosTriSphereSeed::n_vertices_at_tree_level
      break;
    case LPM_MESH_CUBED_SPHERE:
      nf0 = 6;
      *nv = 2 + 6 * ipow4(level);
      break;
    case LPM_MESH_QUAD_RECT: {
      nf0 = 4;
      int64_t side = 3;
      for (int i = 1; i <= level; ++i) side += int64_t(1) << i;
      *nv = side * side;  // QuadRectSeed::n_vertices_at_tree_level
      break;
    }
    default:
      throw std::invalid_argument("unknown mesh kind");
  }
  int64_t total = 0;
  for (int i = 0; i <= level; ++i) total += nf0 * ipow4(i);
  *nf = total;
}

void mesh_seed(int kind, double radius, MeshSeed& out) {
  Builder b;
  switch (kind) {
    case LPM_MESH_ICOS_TRI:
      seed_icosahedron(b);
      break;
    case LPM_MESH_CUBED_SPHERE:
      seed_cube(b);
      break;
    case LPM_MESH_QUAD_RECT:
      seed_square(b, radius);
      break;
    default:
      throw std::invalid_argument("unknown mesh kind");
  }
  out.ndim = b.ndim;
  out.nfv = b.nfv;
  out.sphere = b.sphere;
  out.vx = b.vx;
  out.fx = b.fx;
  out.area = b.area;
  out.fverts.clear();
  for (const auto& f : b.fverts)
    for (int i = 0; i < b.nfv; ++i) out.fverts.push_back(int(f[i]));
}

void mesh_build(int kind, int level, double radius, double* vx, double* fx,
                double* farea, uint8_t* fmask, int32_t* fverts) {
  int64_t nv, nf;
  mesh_sizes(kind, level, &nv, &nf);
  Builder b;
  switch (kind) {
    case LPM_MESH_ICOS_TRI:
      seed_icosahedron(b);
      break;
    case LPM_MESH_CUBED_SPHERE:
      seed_cube(b);
      break;
    case LPM_MESH_QUAD_RECT:
      seed_square(b, radius);
      break;
  }
  b.vx.reserve(size_t(nv) * b.ndim);
  b.fx.reserve(size_t(nf) * b.ndim);
  b.mids.reserve(size_t(nv) * 2);
  b.tree(level);
  if (int64_t(b.vx.size()) != nv * b.ndim || int64_t(b.area.size()) != nf)
    throw std::runtime_error("mesh_build: size mismatch with the tree formula");
  std::memcpy(vx, b.vx.data(), sizeof(double) * b.vx.size());
  std::memcpy(fx, b.fx.data(), sizeof(double) * b.fx.size());
  std::memcpy(farea, b.area.data(), sizeof(double) * b.area.size());
  std::memcpy(fmask, b.mask.data(), b.mask.size());
  if (fverts) {
    int64_t k = 0;
    for (const auto& f : b.fverts)
      for (int i = 0; i < b.nfv; ++i) fverts[k++] = int32_t(f[i]);
  }
}

int mesh_nfv(int kind) {
  switch (kind) {
    case LPM_MESH_ICOS_TRI:
      return 3;
    case LPM_MESH_CUBED_SPHERE:
    case LPM_MESH_QUAD_RECT:
      return 4;
    default:
      throw std::invalid_argument("unknown mesh kind");
  }
}

}  // namespace lpm
