// lpm_oracle_mesh.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of how the reference builds the inputs of the direct-sum
// path: the uniform panel mesh grown from a mesh seed and the initial
// vorticity fields.  The tests, the golden-fixture scripts and the
// reference arm of the benchmark build their meshes and vorticity with this
// file, so the oracle's side of every comparison uses no code of the product
// library.  The seed itself (coordinates, edges, faces) is passed in by the
// caller: it comes from the reference's own seed files
// (mesh_seeds/*.dat, stored as tests/golden/mesh_seeds.npz).
//
// Mesh: PolyMesh2d::tree_init (src/mesh/lpm_polymesh2d_impl.hpp:26-42) with
// the seed copied in by Vertices/Edges/Faces::init_from_seed
// (src/mesh/lpm_vertices_impl.hpp:34, src/mesh/lpm_edges.cpp:43-56,
// src/mesh/lpm_faces_impl.hpp:180-201), Edges::divide
// (src/mesh/lpm_edges.cpp:59-96) and the triangle and quadrilateral face
// dividers (src/mesh/lpm_faces_impl.hpp:285-432, 434-575): the edge list with
// origin/destination/left/right/kids is kept, edges are divided when a face
// first needs them, and the vertex, edge and face numbering follows from the
// same insertion order.  Geometry: SphereGeometry / PlaneGeometry
// (src/lpm_geometry.hpp:30-160, 340-640) in the same operation order.
//
// Initial conditions: SolidBodyRotation, GaussianVortexSphere,
// RossbyHaurwitz54 and CollidingDipolePairPlane (src/lpm_vorticity_gallery.hpp
// :31-259) with atan4 and the Numerical Recipes Bessel approximations
// (src/util/lpm_math.hpp:70-100, 310-418).
//
// Compiled with -ffp-contract=off, like the rest of the oracle.

#include <cmath>
#include <cstdint>
#include <vector>

namespace {

constexpr double PI = 3.1415926535897932384626433832795;
constexpr double ZERO_TOL = 2.220446049250313e-16;  // FloatingPoint<Real>::zero_tol
constexpr int64_t NONE = -1;

// ---- geometry (src/lpm_geometry.hpp) --------------------------------------
struct Geom {
  int ndim;
  bool sphere;

  double dot(const double* a, const double* b) const {
    return sphere ? a[0] * b[0] + a[1] * b[1] + a[2] * b[2] : a[0] * b[0] + a[1] * b[1];
  }
  double mag(const double* v) const { return std::sqrt(dot(v, v)); }
  void scale(double a, double* v) const {
    for (int k = 0; k < ndim; ++k) v[k] *= a;
  }
  void normalize(double* v) const { scale(1.0 / mag(v), v); }
  void midpoint(double* m, const double* a, const double* b) const {
    for (int k = 0; k < ndim; ++k) m[k] = 0.5 * (a[k] + b[k]);
    if (sphere) normalize(m);
  }
  // barycenter of n points pts[idx[i]]
  void barycenter(double* c, const double* const* p, int n) const {
    for (int k = 0; k < ndim; ++k) c[k] = 0.0;
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < ndim; ++k) c[k] += p[i][k];
    scale(1.0 / n, c);
    if (sphere) normalize(c);
  }
  static void cross(double* c, const double* a, const double* b) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  }
  // great-circle distance atan2(|a x b|, a.b)
  double distance(const double* a, const double* b) const {
    double cp[3];
    cross(cp, a, b);
    return std::atan2(std::sqrt(cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2]), dot(a, b));
  }
  double tri_area(const double* a, const double* b, const double* c) const {
    if (!sphere) {
      const double bma[2] = {b[0] - a[0], b[1] - a[1]};
      const double cma[2] = {c[0] - a[0], c[1] - a[1]};
      const double ar = bma[0] * cma[1] - bma[1] * cma[0];
      return 0.5 * std::abs(ar);
    }
    // L'Huilier
    const double s1 = distance(a, b);
    const double s2 = distance(b, c);
    const double s3 = distance(c, a);
    const double hp = 0.5 * (s1 + s2 + s3);
    double zz = std::tan(0.5 * hp) * std::tan(0.5 * (hp - s1)) * std::tan(0.5 * (hp - s2)) *
                std::tan(0.5 * (hp - s3));
    if (std::abs(zz) < ZERO_TOL) zz = 0;
    return 4 * std::atan(std::sqrt(zz));
  }
  double polygon_area(const double* ctr, const double* const* v, int n) const {
    double ar = 0.0;
    for (int i = 0; i < n; ++i) ar += tri_area(ctr, v[i], v[(i + 1) % n]);
    return ar;
  }
};

// ---- mesh ----------------------------------------------------------------
struct Mesh {
  Geom g;
  int nfv;
  std::vector<double> vx;  // vertex coordinates
  // edges
  std::vector<int64_t> eo, ed, el, er, ek;  // ek: 2 kids per edge
  // faces
  std::vector<int64_t> fv, fe, fk;  // nfv vertices, nfv edges, 4 kids per face
  std::vector<double> fx, farea;
  std::vector<uint8_t> fmask;

  const double* vert(int64_t i) const { return vx.data() + g.ndim * i; }
  int64_t nverts() const { return int64_t(vx.size()) / g.ndim; }
  int64_t nedges() const { return int64_t(eo.size()); }
  int64_t nfaces() const { return int64_t(farea.size()); }

  int64_t add_vertex(const double* p) {
    for (int k = 0; k < g.ndim; ++k) vx.push_back(p[k]);
    return nverts() - 1;
  }
  void add_edge(int64_t o, int64_t d, int64_t l, int64_t r) {
    eo.push_back(o);
    ed.push_back(d);
    el.push_back(l);
    er.push_back(r);
    ek.push_back(NONE);
    ek.push_back(NONE);
  }
  void add_face(const double* c, const int64_t* v, const int64_t* e, double area) {
    for (int k = 0; k < g.ndim; ++k) fx.push_back(c[k]);
    for (int i = 0; i < nfv; ++i) {
      fv.push_back(v[i]);
      fe.push_back(e[i]);
    }
    for (int i = 0; i < 4; ++i) fk.push_back(NONE);
    farea.push_back(area);
    fmask.push_back(0);
  }
  bool edge_has_kids(int64_t e) const { return ek[2 * e] != NONE; }
  // Faces::edge_is_positive: the face is the edge's left face
  bool edge_is_positive(int64_t f, int i) const { return el[fe[nfv * f + i]] == f; }

  // Edges::divide: midpoint vertex, kids (origin, mid) and (mid, destination)
  void divide_edge(int64_t e) {
    const int64_t vi = nverts();
    const int64_t ei = nedges();
    double m[3];
    g.midpoint(m, vert(eo[e]), vert(ed[e]));
    add_vertex(m);
    add_edge(eo[e], vi, el[e], er[e]);
    add_edge(vi, ed[e], el[e], er[e]);
    ek[2 * e] = ei;
    ek[2 * e + 1] = ei + 1;
  }

  // the child edges that replace edge i of face f, their faces recorded
  void child_edges(int64_t f, int i, int64_t* nfe, const int64_t* kids, int64_t* nfvi) {
    const int n = nfv;
    const int64_t pe = fe[n * f + i];
    int64_t k0, k1;
    if (edge_has_kids(pe)) {
      k0 = ek[2 * pe];
      k1 = ek[2 * pe + 1];
    } else {
      k0 = nedges();
      k1 = nedges() + 1;
      divide_edge(pe);
    }
    if (edge_is_positive(f, i)) {
      nfe[n * i + i] = k0;
      el[k0] = kids[i];
      nfe[n * ((i + 1) % n) + i] = k1;
      el[k1] = kids[(i + 1) % n];
    } else {
      nfe[n * i + i] = k1;
      er[k1] = kids[i];
      nfe[n * ((i + 1) % n) + i] = k0;
      er[k0] = kids[(i + 1) % n];
    }
    *nfvi = ed[k0];  // the midpoint vertex
  }

  void finish_children(int64_t f, const int64_t* nfvtx, const int64_t* nfe) {
    const int n = nfv;
    double ctr[4][3];
    double ar[4];
    for (int c = 0; c < 4; ++c) {
      const double* p[4];
      for (int j = 0; j < n; ++j) p[j] = vert(nfvtx[n * c + j]);
      g.barycenter(ctr[c], p, n);
      ar[c] = g.polygon_area(ctr[c], p, n);
    }
    const int64_t first = nfaces();
    for (int c = 0; c < 4; ++c) add_face(ctr[c], nfvtx + n * c, nfe + n * c, ar[c]);
    for (int c = 0; c < 4; ++c) fk[4 * f + c] = first + c;
    farea[f] = 0.0;
    fmask[f] = 1;
  }

  // FaceDivider<Geo, TriFace>::divide
  void divide_tri(int64_t f) {
    int64_t kids[4], nfvtx[12], nfe[12];
    for (int c = 0; c < 4; ++c) kids[c] = nfaces() + c;
    for (int i = 0; i < 12; ++i) nfvtx[i] = nfe[i] = NONE;
    for (int i = 0; i < 3; ++i) nfvtx[3 * i + i] = fv[3 * f + i];
    for (int i = 0; i < 3; ++i) {
      int64_t mid;
      child_edges(f, i, nfe, kids, &mid);
      if (i == 0) {
        nfvtx[0 * 3 + 1] = mid;
        nfvtx[1 * 3 + 0] = mid;
        nfvtx[3 * 3 + 2] = mid;
      } else if (i == 1) {
        nfvtx[1 * 3 + 2] = mid;
        nfvtx[2 * 3 + 1] = mid;
        nfvtx[3 * 3 + 0] = mid;
      } else {
        nfvtx[2 * 3 + 0] = mid;
        nfvtx[0 * 3 + 2] = mid;
        nfvtx[3 * 3 + 1] = mid;
      }
    }
    const int64_t e0 = nedges();
    for (int i = 0; i < 3; ++i) nfe[3 * 3 + i] = e0 + i;
    nfe[0 * 3 + 1] = e0 + 1;
    nfe[1 * 3 + 2] = e0 + 2;
    nfe[2 * 3 + 0] = e0;
    add_edge(nfvtx[2 * 3 + 1], nfvtx[2 * 3 + 0], kids[3], kids[2]);
    add_edge(nfvtx[0 * 3 + 2], nfvtx[0 * 3 + 1], kids[3], kids[0]);
    add_edge(nfvtx[1 * 3 + 0], nfvtx[1 * 3 + 2], kids[3], kids[1]);
    finish_children(f, nfvtx, nfe);
  }

  // FaceDivider<Geo, QuadFace>::divide
  void divide_quad(int64_t f) {
    int64_t kids[4], nfvtx[16], nfe[16];
    for (int c = 0; c < 4; ++c) kids[c] = nfaces() + c;
    for (int i = 0; i < 16; ++i) nfvtx[i] = nfe[i] = NONE;
    for (int i = 0; i < 4; ++i) nfvtx[4 * i + i] = fv[4 * f + i];
    for (int i = 0; i < 4; ++i) {
      int64_t mid;
      child_edges(f, i, nfe, kids, &mid);
      nfvtx[4 * i + (i + 1) % 4] = mid;
      nfvtx[4 * ((i + 1) % 4) + i] = mid;
    }
    // the parent's centre becomes the shared vertex
    double c[3] = {0, 0, 0};
    for (int k = 0; k < g.ndim; ++k) c[k] = fx[g.ndim * f + k];
    const int64_t cv = add_vertex(c);
    for (int i = 0; i < 4; ++i) nfvtx[4 * i + (i + 2) % 4] = cv;
    const int64_t e0 = nedges();
    add_edge(nfvtx[0 * 4 + 1], nfvtx[0 * 4 + 2], kids[0], kids[1]);
    nfe[0 * 4 + 1] = e0;
    nfe[1 * 4 + 3] = e0;
    add_edge(nfvtx[2 * 4 + 0], nfvtx[2 * 4 + 3], kids[3], kids[2]);
    nfe[2 * 4 + 3] = e0 + 1;
    nfe[3 * 4 + 1] = e0 + 1;
    add_edge(nfvtx[2 * 4 + 1], nfvtx[2 * 4 + 0], kids[1], kids[2]);
    nfe[1 * 4 + 2] = e0 + 2;
    nfe[2 * 4 + 0] = e0 + 2;
    add_edge(nfvtx[3 * 4 + 1], nfvtx[3 * 4 + 0], kids[0], kids[3]);
    nfe[0 * 4 + 2] = e0 + 3;
    nfe[3 * 4 + 0] = e0 + 3;
    finish_children(f, nfvtx, nfe);
  }

  // PolyMesh2d::tree_init: divide every leaf, level by level, in index order
  void tree_init(int depth) {
    int64_t start = 0;
    for (int l = 0; l < depth; ++l) {
      const int64_t stop = nfaces();
      for (int64_t j = start; j < stop; ++j) {
        if (fk[4 * j] != NONE) continue;
        if (nfv == 3)
          divide_tri(j);
        else
          divide_quad(j);
      }
      start = stop - 1;
    }
  }
};

// ---- initial conditions (src/lpm_vorticity_gallery.hpp) ------------------
double atan4(double y, double x) {
  double result = 0.0;
  if (std::abs(x) < ZERO_TOL) {
    if (y > 0.0)
      result = 0.5 * PI;
    else if (y < 0.0)
      result = 1.5 * PI;
  } else if (std::abs(y) < ZERO_TOL) {
    if (x < 0.0) result = PI;
  } else {
    const double theta = std::atan2(std::abs(y), std::abs(x));
    if (x > 0.0 && y > 0.0)
      result = theta;
    else if (x < 0.0 && y > 0.0)
      result = PI - theta;
    else if (x < 0.0 && y < 0.0)
      result = PI + theta;
    else if (x > 0.0 && y < 0.0)
      result = 2.0 * PI - theta;
  }
  return result;
}

// Numerical Recipes (Press et al., 2nd ed., sec. 6.5) bessj0 / bessj1.
double nr_bessj0(double x) {
  const double ax = std::abs(x);
  if (ax < 8.0) {
    const double y = x * x;
    const double a1 = 57568490574.0 +
                      y * (-13362590354.0 +
                           y * (651619640.7 + y * (-11214424.18 + y * (77392.33017 + y * (-184.9052456)))));
    const double a2 =
        57568490411.0 + y * (1029532985.0 + y * (9494680.718 + y * (59272.64853 + y * (267.8532712 + y * 1.0))));
    return a1 / a2;
  }
  const double z = 8.0 / ax, y = z * z, xx = ax - 0.785398164;
  const double a1 = 1.0 + y * (-0.1098628627e-2 + y * (0.2734510407e-4 + y * (-0.2073370639e-5 + y * 0.2093887211e-6)));
  const double a2 = -0.1562499995e-1 + y * (0.1430488765e-3 + y * (-0.6911147651e-5 + y * (0.7621095161e-6 - y * 0.934935152e-7)));
  return std::sqrt(0.636619772 / ax) * (std::cos(xx) * a1 - z * std::sin(xx) * a2);
}

double nr_bessj1(double x) {
  const double ax = std::abs(x);
  if (ax < 8.0) {
    const double y = x * x;
    const double a1 = x * (72362614232.0 +
                           y * (-7895059235.0 +
                                y * (242396853.1 + y * (-2972611.439 + y * (15704.48260 + y * (-30.16036606))))));
    const double a2 = 144725228442.0 +
                      y * (2300535178.0 + y * (18583304.74 + y * (99447.43394 + y * (376.9991397 + y * 1.0))));
    return a1 / a2;
  }
  const double z = 8.0 / ax, y = z * z, xx = ax - 2.356194491;
  const double a1 = 1.0 + y * (0.183105e-2 + y * (-0.3516396496e-4 + y * (0.2457520174e-5 + y * (-0.240337019e-6))));
  const double a2 = 0.04687499995 + y * (-0.2002690873e-3 + y * (0.8449199096e-5 + y * (-0.88228987e-6 + y * 0.105787412e-6)));
  const double r = std::sqrt(0.636619772 / ax) * (std::cos(xx) * a1 - z * std::sin(xx) * a2);
  return x < 0.0 ? -r : r;
}

double lamb_dipole_vorticity(double x, double y, double xctr, double yctr, double radius,
                             double strength) {
  const double K0 = 3.8317;
  const double r = std::sqrt((x - xctr) * (x - xctr) + (y - yctr) * (y - yctr));
  double result = 0;
  if (r < radius && !(std::abs(r) < ZERO_TOL)) {
    const double k = K0 / radius;
    const double sintheta = y / r;
    const double denom = nr_bessj0(K0);
    result = -2 * strength * k * nr_bessj1(k * r) * sintheta / denom;
  }
  return result;
}

// GaussianVortexSphere(str, b, lon, lat) at p, minus gauss_const
double gaussian_vortex(const double* p, double str, double b, double lon, double lat,
                       double gauss_const) {
  const double c[3] = {std::cos(lon) * std::cos(lat), std::sin(lon) * std::cos(lat),
                       std::sin(lat)};
  const double distsq = 1.0 - p[0] * c[0] - p[1] * c[1] - p[2] * c[2];
  return str * std::exp(-(b * b) * distsq) - gauss_const;
}

}  // namespace

extern "C" {

// Builds the uniform mesh of `depth` levels from a seed: seed_crds holds
// nverts0 vertex rows then nfaces0 face-centre rows (ndim columns), scaled by
// radius like MeshSeed(maxr); seed_edges (origin, destination, left, right),
// seed_faceverts / seed_faceedges nfv columns.  Outputs (sized by the caller
// from the tree formulas, see oracle_mesh_sizes): vertex coordinates, face
// centres, areas, masks (1 = divided) and face vertex lists.  Returns 0, or
// -1 if the output counts disagree with the caller's.
int oracle_mesh_build(int ndim, int sphere, int nfv, long nverts0, long nedges0, long nfaces0,
                      const double* seed_crds, const long* seed_edges,
                      const long* seed_faceverts, const long* seed_faceedges, double radius,
                      int depth, long nv_out, long nf_out, double* vx, double* fx,
                      double* farea, unsigned char* fmask, long* fverts) {
  Mesh m;
  m.g = Geom{ndim, sphere != 0};
  m.nfv = nfv;
  auto crd = [&](long i, double* out) {
    for (int k = 0; k < ndim; ++k) out[k] = seed_crds[ndim * i + k] * radius;
  };
  for (long i = 0; i < nverts0; ++i) {
    double p[3];
    crd(i, p);
    m.add_vertex(p);
  }
  for (long e = 0; e < nedges0; ++e)
    m.add_edge(seed_edges[4 * e], seed_edges[4 * e + 1], seed_edges[4 * e + 2],
               seed_edges[4 * e + 3]);
  for (long f = 0; f < nfaces0; ++f) {
    double c[3];
    crd(nverts0 + f, c);
    int64_t v[4], e[4];
    const double* p[4];
    for (int i = 0; i < nfv; ++i) {
      v[i] = seed_faceverts[nfv * f + i];
      e[i] = seed_faceedges[nfv * f + i];
      p[i] = m.vert(v[i]);
    }
    // MeshSeed::face_area: polygon area about the seed's face centre
    m.add_face(c, v, e, m.g.polygon_area(c, p, nfv));
  }
  m.tree_init(depth);
  if (m.nverts() != nv_out || m.nfaces() != nf_out) return -1;
  for (size_t i = 0; i < m.vx.size(); ++i) vx[i] = m.vx[i];
  for (size_t i = 0; i < m.fx.size(); ++i) fx[i] = m.fx[i];
  for (long f = 0; f < nf_out; ++f) {
    farea[f] = m.farea[f];
    fmask[f] = m.fmask[f];
    for (int i = 0; i < nfv; ++i) fverts[nfv * f + i] = m.fv[nfv * f + i];
  }
  return 0;
}

// Initial relative vorticity at n points x (ndim columns).
//   kind 1 SolidBodyRotation: 2 (2 pi) z
//   kind 2 GaussianVortexSphere + background: prm = (strength, b, lon, lat,
//          gauss_const, Omega_bg): gaussian - gauss_const + 2 Omega_bg z
//   kind 3 RossbyHaurwitz54: prm = (u0, amplitude)
//   kind 4 CollidingDipolePairPlane: prm = (strA, rA, xA, yA, strB, rB, xB, yB)
//   kind 5 sum of k Gaussian vortices: prm = (k, then (str, b, lon, lat) x k)
// Returns 0, or -1 for an unknown kind or too few parameters.
int oracle_ic_eval(int kind, const double* prm, int np, int ndim, long n, const double* x,
                   double* zeta) {
  switch (kind) {
    case 1:
      if (ndim != 3) return -1;
      for (long i = 0; i < n; ++i) zeta[i] = 2 * (2 * PI) * x[3 * i + 2];
      return 0;
    case 2:
      if (ndim != 3 || np < 6) return -1;
      for (long i = 0; i < n; ++i) {
        const double* p = x + 3 * i;
        zeta[i] = gaussian_vortex(p, prm[0], prm[1], prm[2], prm[3], prm[4]) + 2 * prm[5] * p[2];
      }
      return 0;
    case 3:
      if (ndim != 3 || np < 2) return -1;
      for (long i = 0; i < n; ++i) {
        const double* p = x + 3 * i;
        const double lon = atan4(p[1], p[0]);
        const double z = p[2];
        const double p54 = z * ((z * z - 1) * (z * z - 1));  // legendreP54
        zeta[i] = 2 * prm[0] * z + 30 * prm[1] * std::cos(4 * lon) * p54;
      }
      return 0;
    case 4:
      if (ndim != 2 || np < 8) return -1;
      for (long i = 0; i < n; ++i) {
        const double px = x[2 * i], py = x[2 * i + 1];
        zeta[i] = lamb_dipole_vorticity(px, py, prm[2], prm[3], prm[1], prm[0]) +
                  lamb_dipole_vorticity(px, py, prm[6], prm[7], prm[5], prm[4]);
      }
      return 0;
    case 5: {
      if (ndim != 3 || np < 1) return -1;
      const int k = int(prm[0]);
      if (np < 1 + 4 * k) return -1;
      for (long i = 0; i < n; ++i) {
        double s = 0;
        for (int v = 0; v < k; ++v) {
          const double* q = prm + 1 + 4 * v;
          s += gaussian_vortex(x + 3 * i, q[0], q[1], q[2], q[3], 0.0);
        }
        zeta[i] = s;
      }
      return 0;
    }
    default:
      return -1;
  }
}

}  // extern "C"
