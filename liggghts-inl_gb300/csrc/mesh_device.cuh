// Sphere-triangle geometry of LIGGGHTS-INL's mesh walls, as device code.
//
//   TriMesh::resolveTriSphereContactBary and its edge/corner/face resolvers
//   src/tri_mesh_I.h:65-271; MathExtraLiggghts::calcBaryTriCoords
//   src/math_extra_liggghts.h:583-594; TriMesh::resolveTriSphereNeighbuild
//   src/tri_mesh_I.h:275-305.
//
// Every operation is an explicit round-to-nearest add/mul (no contraction),
// so the region decisions (barycentric sign pattern, active feature) and the
// overlap that decides contact are the reference's bit for bit.
#pragma once
#include "dem_device.cuh"

namespace gb300 {

constexpr double kTriSmall = 1.e-10;    // SMALL_TRIMESH
constexpr double kTriLarge = 1000000;   // LARGE_TRIMESH
constexpr double kMeshPrecision = 1e-8; // EPSILON_PRECISION

__device__ __forceinline__ double dot3_rn(const double *a, const double *b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}
__device__ __forceinline__ void sub3_rn(const double *a, const double *b, double *r) {
  r[0] = __dadd_rn(a[0], -b[0]);
  r[1] = __dadd_rn(a[1], -b[1]);
  r[2] = __dadd_rn(a[2], -b[2]);
}

__device__ __forceinline__ const double *tri_node(const double *g, int q) { return g + 3 * q; }
__device__ __forceinline__ const double *tri_ev(const double *g, int q) { return g + 9 + 3 * q; }
__device__ __forceinline__ const double *tri_en(const double *g, int q) { return g + 18 + 3 * q; }
__device__ __forceinline__ double tri_el(const double *g, int q) { return g[27 + q]; }
__device__ __forceinline__ const double *tri_sn(const double *g) { return g + 30; }
__device__ __forceinline__ const double *tri_c(const double *g) { return g + 33; }
__device__ __forceinline__ double tri_rb(const double *g) { return g[36]; }
__device__ __forceinline__ bool edge_active(int meta, int q) { return (meta >> (2 + q)) & 1; }
__device__ __forceinline__ bool corner_active(int meta, int q) { return (meta >> (5 + q)) & 1; }
__device__ __forceinline__ int obtuse_index(int meta) { return (meta & 3) - 1; }

// TriMesh::calcDist: delta = closest - p, returns |p - closest|
__device__ __forceinline__ double calc_dist_rn(const double *p, const double *cp, double *delta) {
  sub3_rn(cp, p, delta);
  double d[3];
  sub3_rn(p, cp, d);
  return sqrt(dot3_rn(d, d));
}

__device__ __forceinline__ void closest_on_edge(const double *n, double dist, const double *e, double *cp) {
  cp[0] = __dadd_rn(n[0], __dmul_rn(dist, e[0]));
  cp[1] = __dadd_rn(n[1], __dmul_rn(dist, e[1]));
  cp[2] = __dadd_rn(n[2], __dmul_rn(dist, e[2]));
}

__device__ inline double resolve_edge(const double *g, int meta, int iE, const double *p, double *delta,
                                      double *bary) {
  const int ip = (iE + 1) % 3, ipp = (iE + 2) % 3;
  double nodeToP[3];
  sub3_rn(p, tri_node(g, iE), nodeToP);
  const double distFromNode = dot3_rn(nodeToP, tri_ev(g, iE));
  if (distFromNode < -kTriSmall) {
    if (!corner_active(meta, iE)) return kTriLarge;
    bary[iE] = 1.; bary[ip] = 0.; bary[ipp] = 0.;
    return calc_dist_rn(p, tri_node(g, iE), delta);
  } else if (distFromNode > __dadd_rn(tri_el(g, iE), kTriSmall)) {
    if (!corner_active(meta, ip)) return kTriLarge;
    bary[iE] = 0.; bary[ip] = 1.; bary[ipp] = 0.;
    return calc_dist_rn(p, tri_node(g, ip), delta);
  } else {
    if (!edge_active(meta, iE)) return kTriLarge;
    double cp[3];
    closest_on_edge(tri_node(g, iE), distFromNode, tri_ev(g, iE), cp);
    const double d = calc_dist_rn(p, cp, delta);
    bary[ipp] = 0.;
    bary[iE] = __dadd_rn(1., -(distFromNode / tri_el(g, iE)));
    bary[ip] = __dadd_rn(1., -bary[iE]);
    return d;
  }
}

__device__ inline double resolve_corner(const double *g, int meta, int iN, bool obtuse, const double *p,
                                        double *delta, double *bary) {
  const int ip = (iN + 1) % 3, ipp = (iN + 2) % 3;
  const double *n = tri_node(g, iN);
  if (obtuse) {
    double nodeToP[3], cp[3];
    sub3_rn(p, n, nodeToP);
    double distFromNode = dot3_rn(nodeToP, tri_ev(g, ipp));
    if (distFromNode < kTriSmall) {
      if (distFromNode > -tri_el(g, ipp)) {
        if (!edge_active(meta, ipp)) return kTriLarge;
        closest_on_edge(n, distFromNode, tri_ev(g, ipp), cp);
        bary[ip] = 0.;
        bary[iN] = __dadd_rn(1., distFromNode / tri_el(g, ipp));
        bary[ipp] = __dadd_rn(1., -bary[iN]);
        return calc_dist_rn(p, cp, delta);
      } else {
        if (!corner_active(meta, ipp)) return kTriLarge;
        bary[ipp] = 1.; bary[iN] = bary[ip] = 0.;
        return calc_dist_rn(p, tri_node(g, ipp), delta);
      }
    }
    distFromNode = dot3_rn(nodeToP, tri_ev(g, iN));
    if (distFromNode > -kTriSmall) {
      if (distFromNode < tri_el(g, iN)) {
        if (!edge_active(meta, iN)) return kTriLarge;
        closest_on_edge(n, distFromNode, tri_ev(g, iN), cp);
        bary[ipp] = 0.;
        bary[iN] = __dadd_rn(1., -(distFromNode / tri_el(g, iN)));
        bary[ip] = __dadd_rn(1., -bary[iN]);
        return calc_dist_rn(p, cp, delta);
      } else {
        if (!corner_active(meta, ip)) return kTriLarge;
        bary[ip] = 1.; bary[iN] = bary[ipp] = 0.;
        return calc_dist_rn(p, tri_node(g, ip), delta);
      }
    }
  }
  if (!corner_active(meta, iN)) return kTriLarge;
  bary[iN] = 1.; bary[ip] = bary[ipp] = 0.;
  return calc_dist_rn(p, n, delta);
}

// distance minus radius; barySign 1..7 as the reference
__device__ inline double resolve_tri_sphere(const double *g, int meta, double rS, const double *cS,
                                            double *delta, double *bary, int &barySign) {
  double ap[3];
  bary[0] = bary[1] = bary[2] = 0.;
  sub3_rn(cS, tri_node(g, 0), ap);
  const double *e0 = tri_ev(g, 0), *e2 = tri_ev(g, 2);
  const double a = dot3_rn(ap, e0), b = dot3_rn(ap, e2), c = dot3_rn(e0, e2);
  const double oneMinCSqr = __dadd_rn(1., -__dmul_rn(c, c));
  bary[1] = __dadd_rn(a, -__dmul_rn(b, c)) / __dmul_rn(tri_el(g, 0), oneMinCSqr);
  bary[2] = __dadd_rn(__dmul_rn(a, c), -b) / __dmul_rn(tri_el(g, 2), oneMinCSqr);
  bary[0] = __dadd_rn(__dadd_rn(1., -bary[1]), -bary[2]);
  const double invlen = 1. / __dmul_rn(2., tri_rb(g));
  const double lim = __dmul_rn(-kMeshPrecision, invlen);
  const int bs = (bary[0] > lim) + 2 * (bary[1] > lim) + 4 * (bary[2] > lim);
  barySign = bs;
  const int ob = obtuse_index(meta);
  double d;
  switch (bs) {
    case 1: d = resolve_corner(g, meta, 0, ob == 0, cS, delta, bary); break;
    case 2: d = resolve_corner(g, meta, 1, ob == 1, cS, delta, bary); break;
    case 3: d = resolve_edge(g, meta, 0, cS, delta, bary); break;
    case 4: d = resolve_corner(g, meta, 2, ob == 2, cS, delta, bary); break;
    case 5: d = resolve_edge(g, meta, 2, cS, delta, bary); break;
    case 6: d = resolve_edge(g, meta, 1, cS, delta, bary); break;
    case 7: {
      const double *sn = tri_sn(g);
      const double dNorm = dot3_rn(sn, ap);
      double csPlane[3];
      csPlane[0] = __dadd_rn(cS[0], -__dmul_rn(sn[0], dNorm));
      csPlane[1] = __dadd_rn(cS[1], -__dmul_rn(sn[1], dNorm));
      csPlane[2] = __dadd_rn(cS[2], -__dmul_rn(sn[2], dNorm));
      d = calc_dist_rn(cS, csPlane, delta);
      break;
    }
    default: d = kTriLarge; break;
  }
  return __dadd_rn(d, -rS);
}

// TriMesh::resolveTriSphereNeighbuild
__device__ inline bool tri_sphere_neighbuild(const double *g, double rS, const double *cS, double treshold) {
  const double maxDist = __dadd_rn(rS, treshold);
  double v[3];
  sub3_rn(cS, tri_c(g), v);
  const double dNorm = fabs(dot3_rn(tri_sn(g), v));
  if (dNorm > maxDist) return false;
  const double dParaMax = __dmul_rn(maxDist, maxDist);
  for (int i = 0; i < 3; i++) {
    sub3_rn(cS, tri_node(g, i), v);
    const double d = dot3_rn(tri_en(g, i), v);
    if (d > 0 && __dmul_rn(d, d) > dParaMax) return false;
  }
  return true;
}

}  // namespace gb300
