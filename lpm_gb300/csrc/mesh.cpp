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
// Seeds.  The reference reads its seeds from mesh_seeds/*.dat
// (MeshSeed::read_file, src/mesh/lpm_mesh_seed.cpp:20-201): vertex
// coordinates, face centres, face vertex lists.  The three seeds of the
// direct-sum path are generated here in the same numbering and with the same
// values bit for bit: the icosahedron's coordinates are the correctly rounded
// values of their closed forms ((5 +- sqrt5)/10, sqrt((5 +- sqrt5)/10),
// 2/sqrt5, 1/sqrt5, evaluated in double-double arithmetic and rounded once)
// and its face centres the seed files' rule c = ((v0 + v1) + v2) / 3,
// c / sqrt((c0^2 + c1^2) + c2^2); the cube's vertices are +-1/sqrt(3) with the
// face centres on the axes; the square's are the 3 x 3 grid of [-1, 1]^2
// scaled by the radius.  A face's edge i joins its vertices i and i + 1 in
// every seed, so dividing edges in face order numbers the new vertices as
// the reference's edge-based dividers do.

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

  // a face with the given centre; its area about that centre
  // (MeshSeed::face_area, src/mesh/lpm_mesh_seed.cpp:281-295)
  void add_face_at(const double* c, const int64_t* vs) {
    std::array<int64_t, 4> f{-1, -1, -1, -1};
    for (int i = 0; i < nfv; ++i) f[i] = vs[i];
    for (int k = 0; k < ndim; ++k) fx.push_back(c[k]);
    area.push_back(polygon_area(c, vs, nfv));
    mask.push_back(0);
    fverts.push_back(f);
  }
  // a child face: centre at the barycentre of its vertices
  void add_face(const int64_t* vs) {
    double c[3] = {0, 0, 0};
    barycenter(c, vs, nfv);
    add_face_at(c, vs);
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

};

// ---- double-double arithmetic for the icosahedron's coordinates ---------
struct DD {
  double hi, lo;
};
DD quick_two_sum(double a, double b) {
  const double s = a + b;
  return {s, b - (s - a)};
}
DD two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
DD dd_add(DD a, DD b) {
  DD s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return quick_two_sum(s.hi, s.lo);
}
DD dd_neg(DD a) { return {-a.hi, -a.lo}; }
// a / b for a double-double a and a double b: quotient plus the exact residual
DD dd_div(DD a, double b) {
  const double q = a.hi / b;
  const double p = q * b;
  const double pe = std::fma(q, b, -p);
  const double r = ((a.hi - p) - pe) + a.lo;
  return quick_two_sum(q, r / b);
}
// b / a for a double b and a double-double a
DD dd_rdiv(double b, DD a) {
  const double q = b / a.hi;
  const double p = q * a.hi;
  const double pe = std::fma(q, a.hi, -p);
  const double r = ((b - p) - pe) - q * a.lo;
  return quick_two_sum(q, r / a.hi);
}
DD dd_sqrt(DD a) {
  const double x = std::sqrt(a.hi);
  const double p = x * x;
  const double pe = std::fma(x, x, -p);
  const double r = ((a.hi - p) - pe) + a.lo;
  return quick_two_sum(x, r / (2.0 * x));
}
double dd_round(DD a) { return a.hi + a.lo; }

// IcosTriSphereSeed: vertex 0 the north pole, 1-5 the upper ring at
// longitudes 36 + 72 k degrees, 6-10 the lower ring at 72 k degrees, 11 the
// south pole; faces: the five around the north pole, then for each k the
// band faces (U(k), L(k), L(k+1)) and (L(k+1), U(k+1), U(k)), then the five
// around the south pole.
void seed_icosahedron(Builder& b) {
  b.ndim = 3;
  b.sphere = true;
  b.nfv = 3;
  const DD s5 = dd_sqrt(DD{5.0, 0.0});
  const DD ap = dd_div(dd_add(DD{5.0, 0.0}, s5), 10.0);          // (5 + sqrt5)/10
  const DD am = dd_div(dd_add(DD{5.0, 0.0}, dd_neg(s5)), 10.0);  // (5 - sqrt5)/10
  const double A = dd_round(ap);            // r cos 36
  const double Bm = dd_round(dd_sqrt(am));  // r sin 36
  const double C = dd_round(am);            // r cos 72
  const double D = dd_round(dd_sqrt(ap));   // r sin 72
  const double E = dd_round(dd_rdiv(2.0, s5));  // r = 2/sqrt5
  const double Z = dd_round(dd_rdiv(1.0, s5));  // z = 1/sqrt5
  const double v[12][3] = {{0, 0, 1},   {A, Bm, Z},   {-C, D, Z},   {-E, 0, Z},
                           {-C, -D, Z}, {A, -Bm, Z},  {E, 0, -Z},   {C, D, -Z},
                           {-A, Bm, -Z}, {-A, -Bm, -Z}, {C, -D, -Z}, {0, 0, -1}};
  for (int i = 0; i < 12; ++i) b.add_vertex(v[i]);
  auto U = [](int k) { return int64_t(1 + (k % 5)); };
  auto L = [](int k) { return int64_t(6 + (k % 5)); };
  std::vector<std::array<int64_t, 3>> f;
  for (int k = 0; k < 5; ++k) f.push_back({0, U(k), U(k + 1)});
  for (int k = 0; k < 5; ++k) {
    f.push_back({U(k), L(k), L(k + 1)});
    f.push_back({L(k + 1), U(k + 1), U(k)});
  }
  for (int k = 0; k < 5; ++k) f.push_back({11, L(k + 1), L(k)});
  for (const auto& t : f) {
    double c[3];
    for (int k = 0; k < 3; ++k) c[k] = ((b.v(t[0])[k] + b.v(t[1])[k]) + b.v(t[2])[k]) / 3.0;
    const double n = std::sqrt((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]);
    for (int k = 0; k < 3; ++k) c[k] /= n;
    b.add_face_at(c, t.data());
  }
}

// CubedSphereSeed: vertices (s,-s,s), (s,-s,-s), (s,s,-s), (s,s,s),
// (-s,s,-s), (-s,s,s), (-s,-s,-s), (-s,-s,s) with s = 1/sqrt3; faces
// +x, +y, -x, -y, +z, -z with their centres on the axes.
void seed_cube(Builder& b) {
  b.ndim = 3;
  b.sphere = true;
  b.nfv = 4;
  const double s = 1.0 / std::sqrt(3.0);
  const double v[8][3] = {{s, -s, s},  {s, -s, -s}, {s, s, -s},  {s, s, s},
                          {-s, s, -s}, {-s, s, s},  {-s, -s, -s}, {-s, -s, s}};
  for (int i = 0; i < 8; ++i) b.add_vertex(v[i]);
  const int64_t faces[6][4] = {{0, 1, 2, 3}, {3, 2, 4, 5}, {5, 4, 6, 7},
                               {7, 6, 1, 0}, {7, 0, 3, 5}, {1, 6, 4, 2}};
  const double ctr[6][3] = {{1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  for (int f = 0; f < 6; ++f) b.add_face_at(ctr[f], faces[f]);
}

// QuadRectSeed on [-r, r]^2: the boundary vertices counter-clockwise from
// (-r, r) down the left side, then the centre; four faces with centres
// (+-r/2, +-r/2).
void seed_square(Builder& b, double radius) {
  b.ndim = 2;
  b.sphere = false;
  b.nfv = 4;
  const double v[9][2] = {{-1, 1}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1},
                          {1, 0},  {1, 1},  {0, 1},   {0, 0}};
  for (int i = 0; i < 9; ++i) {
    const double p[2] = {v[i][0] * radius, v[i][1] * radius};
    b.add_vertex(p);
  }
  const int64_t faces[4][4] = {{0, 1, 8, 7}, {1, 2, 3, 8}, {8, 3, 4, 5}, {7, 8, 5, 6}};
  const double ctr[4][2] = {{-0.5, 0.5}, {-0.5, -0.5}, {0.5, -0.5}, {0.5, 0.5}};
  for (int f = 0; f < 4; ++f) {
    const double c[2] = {ctr[f][0] * radius, ctr[f][1] * radius};
    b.add_face_at(c, faces[f]);
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
