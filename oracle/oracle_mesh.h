/* ORACLE — TEST INFRASTRUCTURE ONLY.  Included by dem_oracle.c.
 *
 * Triangle-mesh granular walls of LIGGGHTS-INL restated in C:
 *   element geometry  SurfaceMesh::calcSurfPropertiesOfNewElement,
 *                     calcEdgeVecLen/calcSurfaceNorm/calcEdgeNormals/
 *                     calcObtuseAngleIndex  src/surface_mesh_I.h:301-471,
 *                     MultiNodeMesh::updateCenterRbound src/multi_node_mesh_I.h:716-740
 *   topology          SurfaceMesh::buildNeighbours, shareEdge, handleSharedEdge,
 *                     handleCorner, checkNodeRecursive src/surface_mesh_I.h:473-1236
 *   neighbour list    FixNeighlistMesh::pre_force/handleTriangle/checkBin
 *                     src/fix_neighlist_mesh.cpp:230-407, TriMesh::resolveTriSphereNeighbuild
 *                     src/tri_mesh_I.h:275-305
 *   closest feature   TriMesh::resolveTriSphereContactBary, resolveEdgeContactBary,
 *                     resolveCornerContactBary, resolveFaceContactBary src/tri_mesh_I.h:65-271,
 *                     MathExtraLiggghts::calcBaryTriCoords src/math_extra_liggghts.h:583-594
 *   contact history   FixContactHistoryMesh handleContact/haveContact/coplanarContactAlready/
 *                     checkCoplanarContactHistory/addNewTriContactToExistingParticle
 *                     src/fix_contact_history_mesh_I.h:51-216, markAllContacts/cleanUpContacts/
 *                     cleanUpContactJumps/sort_contacts/pre_force
 *                     src/fix_contact_history_mesh.cpp:304-500
 *   wall force        FixWallGran::post_force_mesh src/fix_wall_gran.cpp:803-982
 * The bin geometry of the candidate search is not restated: candidates are the
 * atoms inside the triangle's bounding box grown by distmax that pass
 * resolveTriSphereNeighbuild; atoms the reference's coarser bins add on top
 * can never touch the triangle.
 */

#define TRI_SMALL (1.e-10)
#define TRI_LARGE 1000000
#define MESH_PRECISION 1e-8        /* EPSILON_PRECISION */
#define MESH_CURVATURE (1. - 0.00001) /* 1 - EPSILON_CURVATURE */
#define MESH_MAXSLOT 128

typedef struct {
  int ntri;
  double *node;        /* [t][3][3] */
  double *nodev;       /* node velocities [t][3][3] (moving mesh) or NULL */
  double *edgeVec, *edgeLen, *edgeNorm, *surfNorm, *center, *rBound;
  int *obtuse;
  unsigned char *edgeActive, *cornerActive; /* [t][3] */
  int *nNeighs, *neighFaces;                /* [t][5] edge neighbours (ids = index) */
  int wall_type, rolling;
  /* fix move/mesh ... linear vx vy vz (moving = 1) or
   * rotate origin ox oy oz axis ax ay az period T (moving = 2) */
  int moving;
  double vel[3];
  double rot_origin[3], rot_omega[3], rot_dq[4];
  double *nodeLast;    /* node positions at the last neighbour build [t][3][3] */
  /* per-triangle candidate lists (rebuild) */
  int *cstart, *cand;
  /* per-atom slots (FixContactHistoryMesh), capacity MESH_MAXSLOT */
  int *nslot, *npartner, *partner; /* partner[i*MAXSLOT+s] */
  unsigned char *keep, *inter;
  double *hist;                    /* [i][s][3] */
  int natom_cap;
} orc_mesh;

static inline void v3sub(const double *a, const double *b, double *r) {
  r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2];
}
static inline double v3dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double v3mag(const double *v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
static inline void v3cross(const double *a, const double *b, double *r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
static inline void v3sdiv(double *v, double s) {
  const double sinv = 1. / s;
  v[0] = sinv * v[0]; v[1] = sinv * v[1]; v[2] = sinv * v[2];
}
static inline int comp_double(double a, double b, double prec) {
  if (a == b) return 1;
  if (b == 0) return a < prec && a > -prec;
  double x = (a - b);
  return x < prec && x > -prec;
}

#define MN(m, t, q) (&(m)->node[9 * (size_t)(t) + 3 * (q)])
#define MEV(m, t, q) (&(m)->edgeVec[9 * (size_t)(t) + 3 * (q)])
#define MEN(m, t, q) (&(m)->edgeNorm[9 * (size_t)(t) + 3 * (q)])

static void mesh_geometry(orc_mesh *m) {
  for (int t = 0; t < m->ntri; t++) {
    for (int i = 0; i < 3; i++) {
      double *vec = MEV(m, t, i);
      v3sub(MN(m, t, (i + 1) % 3), MN(m, t, i), vec);
      m->edgeLen[3 * t + i] = v3mag(vec);
      v3sdiv(vec, m->edgeLen[3 * t + i]);
    }
    double *sn = &m->surfNorm[3 * t];
    v3cross(MEV(m, t, 0), MEV(m, t, 1), sn);
    if (v3mag(sn) < 1e-15) {
      v3cross(MEV(m, t, 1), MEV(m, t, 2), sn);
      if (v3mag(sn) < 1e-15) v3cross(MEV(m, t, 2), MEV(m, t, 0), sn);
    }
    v3sdiv(sn, v3mag(sn));
    for (int i = 0; i < 3; i++) {
      double *en = MEN(m, t, i);
      v3cross(MEV(m, t, i), sn, en);
      if (v3mag(en) < 1e-15) {
        const double *o = MEV(m, t, (i + 1) % 3);
        en[0] = o[0]; en[1] = o[1]; en[2] = o[2];
      } else
        v3sdiv(en, v3mag(en));
    }
    /* calcObtuseAngleIndex is called for nodes 0,1,2 and each call sets or
     * clears the index: only node 2 decides the stored value */
    m->obtuse[t] = -1;
    for (int i = 0; i < 3; i++) {
      const double dot = v3dot(MEV(m, t, i), MEV(m, t, (i - 1 + 3) % 3));
      m->obtuse[t] = dot > 0. ? i : -1;
    }
    double *c = &m->center[3 * t];
    c[0] = c[1] = c[2] = 0.0;
    for (int j = 0; j < 3; j++) {
      const double *n = MN(m, t, j);
      c[0] = n[0] + c[0]; c[1] = n[1] + c[1]; c[2] = n[2] + c[2];
    }
    v3sdiv(c, 3.0);
    double rb = 0.;
    for (int j = 0; j < 3; j++) {
      double vec[3];
      v3sub(c, MN(m, t, j), vec);
      const double d = v3mag(vec);
      rb = rb > d ? rb : d;
    }
    m->rBound[t] = rb;
  }
}

static int nodes_equal(const double *a, const double *b) {
  for (int i = 0; i < 3; i++)
    if (!comp_double(a[i], b[i], MESH_PRECISION)) return 0;
  return 1;
}

static int share2nodes(const orc_mesh *m, int a, int b, int *ia1, int *ib1, int *ia2, int *ib2) {
  double dist[3];
  v3sub(&m->center[3 * a], &m->center[3 * b], dist);
  const double radsum = m->rBound[a] + m->rBound[b];
  if (dist[0] * dist[0] + dist[1] * dist[1] + dist[2] * dist[2] > radsum * radsum) return 0;
  int nShared = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      if (nodes_equal(MN(m, a, i), MN(m, b, j))) {
        if (nShared == 0) { *ia1 = i; *ib1 = j; }
        else { *ia2 = i; *ib2 = j; return 1; }
        nShared++;
      }
  return 0;
}

static int n_shared_nodes(const orc_mesh *m, int a, int b) {
  double dist[3];
  v3sub(&m->center[3 * a], &m->center[3 * b], dist);
  const double radsum = m->rBound[a] + m->rBound[b];
  if (dist[0] * dist[0] + dist[1] * dist[1] + dist[2] * dist[2] > radsum * radsum) return 0;
  int n = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      if (nodes_equal(MN(m, a, i), MN(m, b, j))) n++;
  return n;
}

static int are_coplanar(const orc_mesh *m, int a, int b) {
  const double dot = v3dot(&m->surfNorm[3 * a], &m->surfNorm[3 * b]);
  return fabs(dot) >= MESH_CURVATURE;
}

static int coplanar_neighs_overlap(const orc_mesh *m, int iS, int iE, int jS, int jE) {
  double vI[3], vJ[3];
  const double *pRef = MN(m, iS, iE), *edgeN = MEN(m, iS, iE);
  v3sub(MN(m, iS, (iE + 2) % 3), pRef, vI);
  v3sub(MN(m, jS, (jE + 2) % 3), pRef, vJ);
  return v3dot(vI, edgeN) * v3dot(vJ, edgeN) > 0.;
}

static void handle_shared_edge(orc_mesh *m, int iS, int iE, int jS, int jE, int coplanar) {
  if (m->nNeighs[iS] < 5) m->neighFaces[5 * iS + m->nNeighs[iS]] = jS;
  if (m->nNeighs[jS] < 5) m->neighFaces[5 * jS + m->nNeighs[jS]] = iS;
  m->nNeighs[iS]++;
  m->nNeighs[jS]++;
  if (!coplanar || coplanar_neighs_overlap(m, iS, iE, jS, jE)) {
    if (iS < jS) { m->edgeActive[3 * iS + iE] = 0; m->edgeActive[3 * jS + jE] = 1; }
    else { m->edgeActive[3 * iS + iE] = 1; m->edgeActive[3 * jS + jE] = 0; }
  } else {
    m->edgeActive[3 * iS + iE] = 0;
    m->edgeActive[3 * jS + jE] = 0;
  }
}

static int contains_node(const orc_mesh *m, int t, const double *p) {
  for (int q = 0; q < 3; q++) {
    const double *n = MN(m, t, q);
    if (comp_double(n[0], p[0], MESH_PRECISION) && comp_double(n[1], p[1], MESH_PRECISION) &&
        comp_double(n[2], p[2], MESH_PRECISION))
      return q;
  }
  return -1;
}

typedef struct {
  int *visited, nvisited, *has, nhas;
  double *edgeList, *edgeEnd;
  int anyActive;
} corner_ctx;

static void check_node_recursive(const orc_mesh *m, int t, const double *p, corner_ctx *c) {
  for (int i = 0; i < c->nvisited; i++)
    if (c->visited[i] == t) return;
  c->visited[c->nvisited++] = t;
  const int q = contains_node(m, t, p);
  if (q < 0) return;
  const int ne = 2 * c->nhas;
  c->has[c->nhas++] = t;
  const double *e0 = MEV(m, t, q), *e1 = MEV(m, t, (q + 2) % 3);
  const double *p0 = MN(m, t, (q + 1) % 3), *p1 = MN(m, t, (q + 2) % 3);
  for (int d = 0; d < 3; d++) {
    c->edgeList[3 * ne + d] = e0[d];
    c->edgeList[3 * (ne + 1) + d] = e1[d];
    c->edgeEnd[3 * ne + d] = p0[d];
    c->edgeEnd[3 * (ne + 1) + d] = p1[d];
  }
  if (m->edgeActive[3 * t + q]) c->anyActive = 1;
  else if (m->edgeActive[3 * t + (q + 2) % 3]) c->anyActive = 1;
  for (int k = 0; k < m->nNeighs[t] && k < 5; k++) {
    const int nb = m->neighFaces[5 * t + k];
    if (nb < 0) return;
    check_node_recursive(m, nb, p, c);
  }
}

static void mesh_topology(orc_mesh *m) {
  const int n = m->ntri;
  for (int t = 0; t < n; t++) {
    m->nNeighs[t] = 0;
    for (int k = 0; k < 5; k++) m->neighFaces[5 * t + k] = -1;
    for (int q = 0; q < 3; q++) { m->edgeActive[3 * t + q] = 1; m->cornerActive[3 * t + q] = 1; }
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < i; j++) {
      int a1 = 0, b1 = 0, a2, b2;
      if (share2nodes(m, i, j, &a1, &b1, &a2, &b2)) {
        const int iE = (2 == a1 + a2) ? 2 : (a1 < a2 ? a1 : a2);
        const int jE = (2 == b1 + b2) ? 2 : (b1 < b2 ? b1 : b2);
        handle_shared_edge(m, i, iE, j, jE, are_coplanar(m, i, j));
      }
    }
  corner_ctx c;
  c.visited = (int *)malloc(n * sizeof(int));
  c.has = (int *)malloc(n * sizeof(int));
  c.edgeList = (double *)malloc(6 * (size_t)n * sizeof(double));
  c.edgeEnd = (double *)malloc(6 * (size_t)n * sizeof(double));
  for (int t = 0; t < n; t++)
    for (int q = 0; q < 3; q++) {
      double p[3] = {MN(m, t, q)[0], MN(m, t, q)[1], MN(m, t, q)[2]};
      c.nvisited = c.nhas = 0;
      c.anyActive = 0;
      check_node_recursive(m, t, p, &c);
      int maxId = -1;
      for (int k = 0; k < c.nhas; k++) maxId = maxId > c.has[k] ? maxId : c.has[k];
      const int nE = 2 * c.nhas;
      int colinear = 0;
      for (int a = 0; a < nE; a++)
        for (int b = a + 1; b < nE; b++) {
          const double dot = v3dot(&c.edgeList[3 * a], &c.edgeList[3 * b]);
          if (fabs(dot) > MESH_CURVATURE && !nodes_equal(&c.edgeEnd[3 * a], &c.edgeEnd[3 * b])) colinear = 1;
        }
      if (colinear || !c.anyActive) m->cornerActive[3 * t + q] = 0;
      else if (t == maxId) m->cornerActive[3 * t + q] = 1;
      else m->cornerActive[3 * t + q] = 0;
    }
  free(c.visited); free(c.has); free(c.edgeList); free(c.edgeEnd);
}

/* SurfaceMesh::areCoplanarNodeNeighs */
static int coplanar_node_neighs(const orc_mesh *m, int a, int b) {
  int neigh = 0;
  for (int k = 0; k < m->nNeighs[a] && k < 5; k++)
    if (m->neighFaces[5 * a + k] == b) neigh = 1;
  if (!neigh && n_shared_nodes(m, a, b) == 0) return 0;
  const double dot = v3dot(&m->surfNorm[3 * a], &m->surfNorm[3 * b]);
  return fabs(dot) > MESH_CURVATURE;
}

/* TriMesh::resolveTriSphereNeighbuild */
static int tri_sphere_neighbuild(const orc_mesh *m, int t, double rS, const double *cS, double treshold) {
  const double maxDist = rS + treshold;
  double v[3];
  v3sub(cS, &m->center[3 * t], v);
  const double dNorm = fabs(v3dot(&m->surfNorm[3 * t], v));
  if (dNorm > maxDist) return 0;
  const double dParaMax = maxDist * maxDist;
  for (int i = 0; i < 3; i++) {
    v3sub(cS, MN(m, t, i), v);
    const double d = v3dot(MEN(m, t, i), v);
    if (d > 0 && d * d > dParaMax) return 0;
  }
  return 1;
}

static double calc_dist(const double *cs, const double *cp, double *delta) {
  v3sub(cp, cs, delta);
  const double dx = cs[0] - cp[0], dy = cs[1] - cp[1], dz = cs[2] - cp[2];
  return sqrt(dx * dx + dy * dy + dz * dz);
}

static double resolve_edge(const orc_mesh *m, int t, int iE, const double *p, double *delta, double *bary) {
  const int ip = (iE + 1) % 3, ipp = (iE + 2) % 3;
  double nodeToP[3];
  v3sub(p, MN(m, t, iE), nodeToP);
  const double distFromNode = v3dot(nodeToP, MEV(m, t, iE));
  if (distFromNode < -TRI_SMALL) {
    if (!m->cornerActive[3 * t + iE]) return TRI_LARGE;
    bary[iE] = 1.; bary[ip] = 0.; bary[ipp] = 0.;
    return calc_dist(p, MN(m, t, iE), delta);
  } else if (distFromNode > m->edgeLen[3 * t + iE] + TRI_SMALL) {
    if (!m->cornerActive[3 * t + ip]) return TRI_LARGE;
    bary[iE] = 0.; bary[ip] = 1.; bary[ipp] = 0.;
    return calc_dist(p, MN(m, t, ip), delta);
  } else {
    if (!m->edgeActive[3 * t + iE]) return TRI_LARGE;
    double cp[3];
    const double *n = MN(m, t, iE), *e = MEV(m, t, iE);
    cp[0] = n[0] + distFromNode * e[0];
    cp[1] = n[1] + distFromNode * e[1];
    cp[2] = n[2] + distFromNode * e[2];
    const double d = calc_dist(p, cp, delta);
    bary[ipp] = 0.;
    bary[iE] = 1. - distFromNode / m->edgeLen[3 * t + iE];
    bary[ip] = 1. - bary[iE];
    return d;
  }
}

static double resolve_corner(const orc_mesh *m, int t, int iN, int obtuse, const double *p, double *delta,
                             double *bary) {
  const int ip = (iN + 1) % 3, ipp = (iN + 2) % 3;
  const double *n = MN(m, t, iN);
  if (obtuse) {
    double nodeToP[3], cp[3];
    v3sub(p, n, nodeToP);
    double distFromNode = v3dot(nodeToP, MEV(m, t, ipp));
    if (distFromNode < TRI_SMALL) {
      if (distFromNode > -m->edgeLen[3 * t + ipp]) {
        if (!m->edgeActive[3 * t + ipp]) return TRI_LARGE;
        const double *e = MEV(m, t, ipp);
        cp[0] = n[0] + distFromNode * e[0]; cp[1] = n[1] + distFromNode * e[1]; cp[2] = n[2] + distFromNode * e[2];
        bary[ip] = 0.;
        bary[iN] = 1. + distFromNode / m->edgeLen[3 * t + ipp];
        bary[ipp] = 1. - bary[iN];
        return calc_dist(p, cp, delta);
      } else {
        if (!m->cornerActive[3 * t + ipp]) return TRI_LARGE;
        bary[ipp] = 1.; bary[iN] = bary[ip] = 0.;
        return calc_dist(p, MN(m, t, ipp), delta);
      }
    }
    distFromNode = v3dot(nodeToP, MEV(m, t, iN));
    if (distFromNode > -TRI_SMALL) {
      if (distFromNode < m->edgeLen[3 * t + iN]) {
        if (!m->edgeActive[3 * t + iN]) return TRI_LARGE;
        const double *e = MEV(m, t, iN);
        cp[0] = n[0] + distFromNode * e[0]; cp[1] = n[1] + distFromNode * e[1]; cp[2] = n[2] + distFromNode * e[2];
        bary[ipp] = 0.;
        bary[iN] = 1. - distFromNode / m->edgeLen[3 * t + iN];
        bary[ip] = 1. - bary[iN];
        return calc_dist(p, cp, delta);
      } else {
        if (!m->cornerActive[3 * t + ip]) return TRI_LARGE;
        bary[ip] = 1.; bary[iN] = bary[ipp] = 0.;
        return calc_dist(p, MN(m, t, ip), delta);
      }
    }
  }
  if (!m->cornerActive[3 * t + iN]) return TRI_LARGE;
  bary[iN] = 1.; bary[ip] = bary[ipp] = 0.;
  return calc_dist(p, n, delta);
}

/* returns distance - radius; barySign as the reference */
static double resolve_tri_sphere(const orc_mesh *m, int t, double rS, const double *cS, double *delta,
                                 double *bary, int *barySign) {
  double ap[3];
  bary[0] = bary[1] = bary[2] = 0.;
  v3sub(cS, MN(m, t, 0), ap);
  const double *e0 = MEV(m, t, 0), *e2 = MEV(m, t, 2);
  const double a = v3dot(ap, e0), b = v3dot(ap, e2), c = v3dot(e0, e2);
  const double oneMinCSqr = 1 - c * c;
  bary[1] = (a - b * c) / (m->edgeLen[3 * t] * oneMinCSqr);
  bary[2] = (a * c - b) / (m->edgeLen[3 * t + 2] * oneMinCSqr);
  bary[0] = 1. - bary[1] - bary[2];
  const double invlen = 1. / (2. * m->rBound[t]);
  const double prec = MESH_PRECISION;
  const int bs = (bary[0] > -prec * invlen) + 2 * (bary[1] > -prec * invlen) + 4 * (bary[2] > -prec * invlen);
  *barySign = bs;
  const int ob = m->obtuse[t];
  double d = 1.;
  switch (bs) {
    case 1: d = resolve_corner(m, t, 0, ob == 0, cS, delta, bary); break;
    case 2: d = resolve_corner(m, t, 1, ob == 1, cS, delta, bary); break;
    case 3: d = resolve_edge(m, t, 0, cS, delta, bary); break;
    case 4: d = resolve_corner(m, t, 2, ob == 2, cS, delta, bary); break;
    case 5: d = resolve_edge(m, t, 2, cS, delta, bary); break;
    case 6: d = resolve_edge(m, t, 1, cS, delta, bary); break;
    case 7: {
      const double *sn = &m->surfNorm[3 * t];
      const double dNorm = v3dot(sn, ap);
      double tmp[3], csPlane[3];
      tmp[0] = dNorm * sn[0]; tmp[1] = dNorm * sn[1]; tmp[2] = dNorm * sn[2];
      v3sub(cS, tmp, csPlane);
      d = calc_dist(cS, csPlane, delta);
      break;
    }
    default: d = TRI_LARGE; break;
  }
  return d - rS;
}
