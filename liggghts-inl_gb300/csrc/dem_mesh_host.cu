// Host-side preparation of a triangle-mesh wall (setup, not on the step path):
//   element geometry   SurfaceMesh::calcSurfPropertiesOfNewElement,
//                      calcEdgeVecLen/calcSurfaceNorm/calcEdgeNormals/calcObtuseAngleIndex
//                      src/surface_mesh_I.h:301-471; MultiNodeMesh::updateCenterRbound
//                      src/multi_node_mesh_I.h:716-740
//   topology           SurfaceMesh::buildNeighbours/shareEdge/handleSharedEdge/
//                      handleCorner/checkNodeRecursive src/surface_mesh_I.h:473-1236
//   coplanar neighbours SurfaceMesh::areCoplanarNodeNeighs src/surface_mesh_I.h:921-962
// Compiled without FMA contraction (-ffp-contract=off), so every value equals
// the reference's on x86-64 and aarch64 hosts.  Candidate element pairs come
// from a hash grid of element centres; the results do not depend on the
// order in which pairs are visited.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "../../include/liggghts_gb300.h"
#include "dem_device.cuh"
#include "dem_mesh_host.h"

namespace gb300 {

namespace {

constexpr double kPrecision = 1e-8;           // EPSILON_PRECISION
constexpr double kCurvature = 1. - 0.00001;   // 1 - EPSILON_CURVATURE

inline void sub(const double *a, const double *b, double *r) {
  r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2];
}
inline double dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline double mag(const double *v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
inline void cross(const double *a, const double *b, double *r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
inline void sdiv(double *v, double s) {
  const double sinv = 1. / s;
  v[0] = sinv * v[0]; v[1] = sinv * v[1]; v[2] = sinv * v[2];
}
inline bool comp(double a, double b) {
  if (a == b) return true;
  if (b == 0) return a < kPrecision && a > -kPrecision;
  const double x = a - b;
  return x < kPrecision && x > -kPrecision;
}
inline bool nodes_equal(const double *a, const double *b) {
  return comp(a[0], b[0]) && comp(a[1], b[1]) && comp(a[2], b[2]);
}

struct Geo {
  int n;
  const double *node;  // [t][3][3]
  std::vector<double> ev, en, el, sn, c, rb;
  std::vector<int> obtuse;
  const double *N(int t, int q) const { return node + 9 * (size_t)t + 3 * q; }
  const double *EV(int t, int q) const { return &ev[9 * (size_t)t + 3 * q]; }
  const double *EN(int t, int q) const { return &en[9 * (size_t)t + 3 * q]; }
};

void geometry(Geo &g) {
  const int n = g.n;
  g.ev.assign(9 * (size_t)n, 0.);
  g.en.assign(9 * (size_t)n, 0.);
  g.el.assign(3 * (size_t)n, 0.);
  g.sn.assign(3 * (size_t)n, 0.);
  g.c.assign(3 * (size_t)n, 0.);
  g.rb.assign(n, 0.);
  g.obtuse.assign(n, -1);
  for (int t = 0; t < n; t++) {
    for (int i = 0; i < 3; i++) {
      double *v = &g.ev[9 * (size_t)t + 3 * i];
      sub(g.N(t, (i + 1) % 3), g.N(t, i), v);
      g.el[3 * t + i] = mag(v);
      sdiv(v, g.el[3 * t + i]);
    }
    double *s = &g.sn[3 * t];
    cross(g.EV(t, 0), g.EV(t, 1), s);
    if (mag(s) < 1e-15) {
      cross(g.EV(t, 1), g.EV(t, 2), s);
      if (mag(s) < 1e-15) cross(g.EV(t, 2), g.EV(t, 0), s);
    }
    sdiv(s, mag(s));
    for (int i = 0; i < 3; i++) {
      double *e = &g.en[9 * (size_t)t + 3 * i];
      cross(g.EV(t, i), s, e);
      if (mag(e) < 1e-15) {
        const double *o = g.EV(t, (i + 1) % 3);
        e[0] = o[0]; e[1] = o[1]; e[2] = o[2];
      } else {
        sdiv(e, mag(e));
      }
    }
    // calcObtuseAngleIndex runs for nodes 0,1,2 and each call overwrites the
    // stored index: the value that survives is node 2's
    for (int i = 0; i < 3; i++) g.obtuse[t] = dot(g.EV(t, i), g.EV(t, (i + 2) % 3)) > 0. ? i : -1;
    double *c = &g.c[3 * t];
    for (int j = 0; j < 3; j++) {
      const double *q = g.N(t, j);
      c[0] = q[0] + c[0]; c[1] = q[1] + c[1]; c[2] = q[2] + c[2];
    }
    sdiv(c, 3.0);
    double r = 0.;
    for (int j = 0; j < 3; j++) {
      double v[3];
      sub(c, g.N(t, j), v);
      r = std::max(r, mag(v));
    }
    g.rb[t] = r;
  }
}

// candidate pairs (a, b), b != a, whose bounding spheres may touch
std::vector<std::vector<int>> near_pairs(const Geo &g) {
  const int n = g.n;
  double rbmax = 0.;
  for (int t = 0; t < n; t++) rbmax = std::max(rbmax, g.rb[t]);
  const double h = std::max(2. * rbmax, 1e-300);
  auto key = [&](int t, int dx, int dy, int dz) -> long long {
    const long long ix = (long long)std::floor(g.c[3 * t] / h) + dx;
    const long long iy = (long long)std::floor(g.c[3 * t + 1] / h) + dy;
    const long long iz = (long long)std::floor(g.c[3 * t + 2] / h) + dz;
    return (ix * 73856093LL) ^ (iy * 19349663LL) ^ (iz * 83492791LL);
  };
  std::unordered_map<long long, std::vector<int>> grid;
  for (int t = 0; t < n; t++) grid[key(t, 0, 0, 0)].push_back(t);
  std::vector<std::vector<int>> out(n);
  for (int a = 0; a < n; a++) {
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          auto it = grid.find(key(a, dx, dy, dz));
          if (it == grid.end()) continue;
          for (int b : it->second) {
            if (b == a) continue;
            double d[3];
            sub(&g.c[3 * a], &g.c[3 * b], d);
            const double rs = g.rb[a] + g.rb[b];
            if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] > rs * rs) continue;
            out[a].push_back(b);
          }
        }
    std::sort(out[a].begin(), out[a].end());
    out[a].erase(std::unique(out[a].begin(), out[a].end()), out[a].end());
  }
  return out;
}

bool share2nodes(const Geo &g, int a, int b, int &a1, int &b1, int &a2, int &b2) {
  int ns = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      if (nodes_equal(g.N(a, i), g.N(b, j))) {
        if (ns == 0) { a1 = i; b1 = j; }
        else { a2 = i; b2 = j; return true; }
        ns++;
      }
  return false;
}

int n_shared(const Geo &g, int a, int b) {
  int ns = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      if (nodes_equal(g.N(a, i), g.N(b, j))) ns++;
  return ns;
}

struct Topo {
  std::vector<uint8_t> ea, ca;
  std::vector<int> nNeighs, neigh;  // [t][5]
};

int contains_node(const Geo &g, int t, const double *p) {
  for (int q = 0; q < 3; q++)
    if (nodes_equal(g.N(t, q), p)) return q;
  return -1;
}

struct Corner {
  std::vector<int> visited, has;
  std::vector<double> edges, ends;
  bool anyActive;
};

void check_node(const Geo &g, const Topo &tp, int t, const double *p, Corner &c) {
  for (int v : c.visited)
    if (v == t) return;
  c.visited.push_back(t);
  const int q = contains_node(g, t, p);
  if (q < 0) return;
  c.has.push_back(t);
  const double *e0 = g.EV(t, q), *e1 = g.EV(t, (q + 2) % 3);
  const double *p0 = g.N(t, (q + 1) % 3), *p1 = g.N(t, (q + 2) % 3);
  c.edges.insert(c.edges.end(), e0, e0 + 3);
  c.edges.insert(c.edges.end(), e1, e1 + 3);
  c.ends.insert(c.ends.end(), p0, p0 + 3);
  c.ends.insert(c.ends.end(), p1, p1 + 3);
  if (tp.ea[3 * t + q]) c.anyActive = true;
  else if (tp.ea[3 * t + (q + 2) % 3]) c.anyActive = true;
  for (int k = 0; k < std::min(tp.nNeighs[t], 5); k++) {
    const int nb = tp.neigh[5 * t + k];
    if (nb < 0) return;
    check_node(g, tp, nb, p, c);
  }
}

Topo topology(const Geo &g, const std::vector<std::vector<int>> &near) {
  const int n = g.n;
  Topo tp;
  tp.ea.assign(3 * (size_t)n, 1);
  tp.ca.assign(3 * (size_t)n, 1);
  tp.nNeighs.assign(n, 0);
  tp.neigh.assign(5 * (size_t)n, -1);
  for (int i = 0; i < n; i++)
    for (int j : near[i]) {
      if (j >= i) continue;
      int a1 = 0, b1 = 0, a2 = 0, b2 = 0;
      if (!share2nodes(g, i, j, a1, b1, a2, b2)) continue;
      const int iE = (2 == a1 + a2) ? 2 : std::min(a1, a2);
      const int jE = (2 == b1 + b2) ? 2 : std::min(b1, b2);
      const bool coplanar = std::fabs(dot(&g.sn[3 * i], &g.sn[3 * j])) >= kCurvature;
      if (tp.nNeighs[i] < 5) tp.neigh[5 * i + tp.nNeighs[i]] = j;
      if (tp.nNeighs[j] < 5) tp.neigh[5 * j + tp.nNeighs[j]] = i;
      tp.nNeighs[i]++;
      tp.nNeighs[j]++;
      bool overlap = false;
      if (coplanar) {  // coplanarNeighsOverlap
        double vI[3], vJ[3];
        const double *pRef = g.N(i, iE), *eN = g.EN(i, iE);
        sub(g.N(i, (iE + 2) % 3), pRef, vI);
        sub(g.N(j, (jE + 2) % 3), pRef, vJ);
        overlap = dot(vI, eN) * dot(vJ, eN) > 0.;
      }
      if (!coplanar || overlap) {
        if (i < j) { tp.ea[3 * i + iE] = 0; tp.ea[3 * j + jE] = 1; }
        else { tp.ea[3 * i + iE] = 1; tp.ea[3 * j + jE] = 0; }
      } else {
        tp.ea[3 * i + iE] = 0;
        tp.ea[3 * j + jE] = 0;
      }
    }
  Corner c;
  for (int t = 0; t < n; t++)
    for (int q = 0; q < 3; q++) {
      const double *p = g.N(t, q);
      c.visited.clear(); c.has.clear(); c.edges.clear(); c.ends.clear();
      c.anyActive = false;
      check_node(g, tp, t, p, c);
      int maxId = -1;
      for (int h : c.has) maxId = std::max(maxId, h);
      const int nE = (int)c.edges.size() / 3;
      bool colinear = false;
      for (int a = 0; a < nE; a++)
        for (int b = a + 1; b < nE; b++)
          if (std::fabs(dot(&c.edges[3 * a], &c.edges[3 * b])) > kCurvature &&
              !nodes_equal(&c.ends[3 * a], &c.ends[3 * b]))
            colinear = true;
      if (colinear || !c.anyActive) tp.ca[3 * t + q] = 0;
      else tp.ca[3 * t + q] = (t == maxId) ? 1 : 0;
    }
  return tp;
}

}  // namespace

int mesh_prepare(int ntri, const double *nodes, const uint8_t *ea_in, const uint8_t *ca_in,
                 MeshHost &out) {
  if (ntri < 1 || !nodes) return DEM_ERR_BAD_ARG;
  Geo g;
  g.n = ntri;
  g.node = nodes;
  geometry(g);
  for (int t = 0; t < ntri; t++)
    if (!(g.el[3 * t] > 0.) || !(g.el[3 * t + 1] > 0.) || !(g.el[3 * t + 2] > 0.)) return DEM_ERR_BAD_ARG;
  const auto near = near_pairs(g);
  Topo tp = topology(g, near);
  if (ea_in) std::copy(ea_in, ea_in + 3 * (size_t)ntri, tp.ea.begin());
  if (ca_in) std::copy(ca_in, ca_in + 3 * (size_t)ntri, tp.ca.begin());
  out.ntri = ntri;
  out.tri.assign((size_t)ntri * kTriStride, 0.0);
  out.meta.assign(ntri, 0);
  out.edge_active = tp.ea;
  out.corner_active = tp.ca;
  for (int t = 0; t < ntri; t++) {
    double *d = &out.tri[(size_t)t * kTriStride];
    std::copy(g.N(t, 0), g.N(t, 0) + 9, d);
    std::copy(&g.ev[9 * (size_t)t], &g.ev[9 * (size_t)t] + 9, d + 9);
    std::copy(&g.en[9 * (size_t)t], &g.en[9 * (size_t)t] + 9, d + 18);
    std::copy(&g.el[3 * (size_t)t], &g.el[3 * (size_t)t] + 3, d + 27);
    std::copy(&g.sn[3 * (size_t)t], &g.sn[3 * (size_t)t] + 3, d + 30);
    std::copy(&g.c[3 * (size_t)t], &g.c[3 * (size_t)t] + 3, d + 33);
    d[36] = g.rb[t];
    int m = g.obtuse[t] + 1;
    for (int q = 0; q < 3; q++) {
      if (tp.ea[3 * t + q]) m |= 1 << (2 + q);
      if (tp.ca[3 * t + q]) m |= 1 << (5 + q);
    }
    out.meta[t] = m;
  }
  // areCoplanarNodeNeighs: edge neighbours or elements sharing a node, with
  // |n_a . n_b| > curvature (sharing a node implies the bounding spheres touch)
  out.cn_start.assign(ntri + 1, 0);
  out.cn_list.clear();
  for (int a = 0; a < ntri; a++) {
    out.cn_start[a] = (int)out.cn_list.size();
    for (int b : near[a]) {
      bool neigh = false;
      for (int k = 0; k < std::min(tp.nNeighs[a], 5); k++)
        if (tp.neigh[5 * a + k] == b) neigh = true;
      if (!neigh && n_shared(g, a, b) == 0) continue;
      if (std::fabs(dot(&g.sn[3 * a], &g.sn[3 * b])) > kCurvature) out.cn_list.push_back(b);
    }
  }
  out.cn_start[ntri] = (int)out.cn_list.size();
  return DEM_OK;
}

}  // namespace gb300

extern "C" int dem_mesh_topology(int ntri, const double *nodes, unsigned char *edge_active,
                                 unsigned char *corner_active) {
  gb300::MeshHost m;
  const int rc = gb300::mesh_prepare(ntri, nodes, nullptr, nullptr, m);
  if (rc) return rc;
  if (edge_active) std::copy(m.edge_active.begin(), m.edge_active.end(), edge_active);
  if (corner_active) std::copy(m.corner_active.begin(), m.corner_active.end(), corner_active);
  return DEM_OK;
}
