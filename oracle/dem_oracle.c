/* ORACLE — TEST INFRASTRUCTURE ONLY (see dem_oracle.h).
 *
 * Single-threaded C restatement of the LIGGGHTS-INL timestep for spheres:
 *   Verlet::setup / Verlet::run          src/verlet.cpp:264-431
 *   FixNVESphere initial/final_integrate src/fix_nve_sphere.cpp:134-244
 *   Neighbor::decide / check_distance    src/neighbor.cpp:1362-1466
 *   Domain::pbc, CommBrick::exchange     src/domain.cpp:550-650, src/comm_brick.cpp:732-808
 *   ghost images x_j + pbc*prd           src/atom_vec_sphere.cpp:203-225
 *   Neighbor::granular_bin_no_newton     src/neigh_gran.cpp:485-644
 *   FixContactHistory::pre_exchange      src/fix_contact_history.cpp:305-425
 *   Granular<CM>::compute_force          src/pair_gran_base.h:187-503
 *   SurfaceModel<SURFACE_DEFAULT>        src/surface_model_default.h:146-211
 *   NormalModel<HERTZ>                   src/normal_model_hertz.h:205-408
 *   NormalModel<HOOKE>                   src/normal_model_hooke.h:230-400
 *   TangentialModel<TANGENTIAL_HISTORY>  src/tangential_model_history.h:135-439
 *   RollingModel<ROLLING_CDT>            src/rolling_model_cdt.h:89-167
 *   CohesionModel<BOND_NONLINEAR>        src/cohesion_model_bond_nonlinear.h:330-992
 *   FixGravity::post_force               src/fix_gravity.cpp:301-352
 *   FixWallGran::post_force_primitive    src/fix_wall_gran.cpp:988-1119
 *   Walls::Granular::compute_force       src/fix_wall_gran_base.h:159-372
 *   PrimitiveWall plane contact/neighbour src/primitive_wall_definitions.h:123-150
 * Every arithmetic expression keeps the reference's operand order, and the
 * file must be compiled with -ffp-contract=off so that no FMA is formed
 * (the reference is x86-64 SSE2 code without contraction).
 *
 * Not restated: the reference's bin geometry, so the ORDER of j inside one
 * atom's neighbour list (and hence the summation order of forces) differs;
 * the pair SET and every per-pair value are the reference's.
 */
#include "dem_oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAXTYPE_ERR "type out of range"
#define CONTACT_NORMAL_MODEL (1 << 0)
#define CONTACT_TANGENTIAL_MODEL (1 << 2)

#include "oracle_mesh.h"

typedef struct {
  int axis;
  double pos;        /* plane: position on the axis; cylinder: radius */
  int kind;          /* 0: plane, 1: cylinder about the axis through (c1, c2) */
  double c1, c2;     /* cylinder centre: coordinates (axis+1)%3 and (axis+2)%3 */
  int wall_type;
  int rolling_model;
  int *nlist;        /* PrimitiveWall neighbour list (atom indices) */
  int nn, nncap;
  double *hist;      /* 3 doubles per atom: shearx, sheary, shearz */
} orc_plane;

struct orc_sys {
  orc_config cfg;
  /* atoms staged by orc_insert_atoms: they join at the next step after its
   * initial integration, with a rebuild at that step (FixInsert) */
  int npend;
  int *pend_tag, *pend_type;
  double *pend_x, *pend_v, *pend_w, *pend_r, *pend_m;
  /* diagnostics of the last force pass: entries with a contact force, and
   * the total force of each wall (planes, then meshes) on the atoms */
  long long ncontacts;
  double wall_f[3 * ORC_DIAG_MAX_WALLS];
  double *cur_wall_f;
  char err[256];
  int ntypes;
  double *Yeff, *Geff, *betaeff, *frict, *rollfrict, *restlog;
  double charVel;

  int n, nmax;
  int *tag, *type;
  double *x, *v, *omega, *f, *torque, *radius, *rmass, *xhold;
  int *prow; /* row of this atom in the partner table */

  /* half neighbour list, CSR by owner i */
  int *nstart, *nj, *nshift, *nflag;
  double *nhist;
  int np, npcap;
  int dnum;
  int list_valid;
  int list_n;      /* atoms the current list was built for (later insertions have no rows) */

  /* partner table (FixContactHistory npartner_/partner_/contacthistory_) */
  int *pstart, *ptag;
  double *phist;
  int prows;

  orc_plane planes[8];
  int nplanes;
  orc_mesh meshes[4];
  int nmeshes;

  /* cohesion bond/nonlinear: ORC_BOND_NTABLES tables of (ntypes+1)^2 */
  int bond_on;
  double *bond;
  orc_bond_settings bset;
  int shear_off;     /* offset of shear[3] inside a pair's history */

  double cutneighmax;
  long ntimestep, nrebuilds;
  long next_reneighbor;  /* FixMesh::next_reneighbor (mesh moved > skin/2) */
  int ago;
  int computeflag;   /* FixContactHistory computeflag_: a pair compute ran */
};

static void *xrealloc(void *p, size_t n) {
  void *q = realloc(p, n ? n : 1);
  if (!q) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
  return q;
}

orc_sys *orc_create(const orc_config *cfg) {
  orc_sys *s = (orc_sys *)calloc(1, sizeof(orc_sys));
  s->cfg = *cfg;
  /* history values in the order the models register them (normal, cohesion,
   * tangential, rolling: src/contact_models.h:142-157): the bond's 28
   * (src/cohesion_model_bond_nonlinear.h:198-226) before the shear's 3
   * (src/tangential_model_history.h:79-81) */
  s->bond_on = cfg->cohesion_model == ORC_COHESION_BOND_NONLINEAR;
  s->dnum = s->bond_on ? 31 : 3;
  s->shear_off = s->bond_on ? 28 : 0;
  s->next_reneighbor = -1;
  return s;
}

void orc_destroy(orc_sys *s) {
  if (!s) return;
  free(s->Yeff); free(s->Geff); free(s->betaeff); free(s->frict); free(s->rollfrict);
  free(s->restlog); free(s->bond);
  free(s->tag); free(s->type); free(s->x); free(s->v); free(s->omega); free(s->f);
  free(s->torque); free(s->radius); free(s->rmass); free(s->xhold); free(s->prow);
  free(s->pend_tag); free(s->pend_type); free(s->pend_x); free(s->pend_v); free(s->pend_w);
  free(s->pend_r); free(s->pend_m);
  free(s->nstart); free(s->nj); free(s->nshift); free(s->nflag); free(s->nhist);
  free(s->pstart); free(s->ptag); free(s->phist);
  for (int w = 0; w < s->nplanes; w++) { free(s->planes[w].nlist); free(s->planes[w].hist); }
  for (int k = 0; k < s->nmeshes; k++) {
    orc_mesh *m = &s->meshes[k];
    free(m->node); free(m->nodev); free(m->edgeVec); free(m->edgeLen); free(m->edgeNorm);
    free(m->surfNorm); free(m->center); free(m->rBound); free(m->obtuse); free(m->edgeActive);
    free(m->cornerActive); free(m->nNeighs); free(m->nodeLast); free(m->neighFaces); free(m->cstart); free(m->cand);
    free(m->nslot); free(m->npartner); free(m->partner); free(m->keep); free(m->inter); free(m->hist);
  }
  free(s);
}

const char *orc_last_error(const orc_sys *s) { return s->err; }

static double *dupm(const double *a, int nt) {
  if (!a) return NULL;
  size_t m = (size_t)(nt + 1) * (nt + 1);
  double *b = (double *)xrealloc(NULL, m * sizeof(double));
  memcpy(b, a, m * sizeof(double));
  return b;
}

int orc_set_pair_params(orc_sys *s, int ntypes, const double *Yeff, const double *Geff,
                        const double *betaeff, const double *coeffFrict,
                        const double *coeffRollFrict, const double *coeffRestLog,
                        double charVel) {
  s->ntypes = ntypes;
  s->Yeff = dupm(Yeff, ntypes);
  s->Geff = dupm(Geff, ntypes);
  s->betaeff = dupm(betaeff, ntypes);
  s->frict = dupm(coeffFrict, ntypes);
  s->rollfrict = dupm(coeffRollFrict, ntypes);
  s->restlog = dupm(coeffRestLog, ntypes);
  s->charVel = charVel;
  return 0;
}

int orc_set_bond_params(orc_sys *s, const double *tables, const orc_bond_settings *st) {
  if (!s->bond_on || s->ntypes < 1) {
    snprintf(s->err, sizeof s->err, "bond parameters need cohesion bond/nonlinear and pair params");
    return -1;
  }
  const size_t m = (size_t)(s->ntypes + 1) * (s->ntypes + 1) * ORC_BOND_NTABLES;
  s->bond = (double *)xrealloc(s->bond, m * sizeof(double));
  memcpy(s->bond, tables, m * sizeof(double));
  s->bset = *st;
  /* CohesionModel::connectToProperties: dampingBondSmooth implies dampingBond */
  if (s->bset.dampingBondSmooth) s->bset.dampingBond = 1;
  return 0;
}

int orc_add_plane(orc_sys *s, int axis, double pos, int wall_type, int rolling_model) {
  if (s->nplanes >= 8) { snprintf(s->err, sizeof s->err, "too many planes"); return -1; }
  orc_plane *w = &s->planes[s->nplanes++];
  memset(w, 0, sizeof *w);
  w->axis = axis; w->pos = pos; w->wall_type = wall_type; w->rolling_model = rolling_model;
  return 0;
}

/* FixWallGran primitive xcylinder/ycylinder/zcylinder R c1 c2
   (src/primitive_wall_definitions.h:69-71,155-200: param[0] radius,
   param[1], param[2] the centre's coordinates along (axis+1)%3, (axis+2)%3) */
int orc_add_cylinder(orc_sys *s, int axis, double radius, double c1, double c2, int wall_type, int rolling_model) {
  if (s->nplanes >= 8) { snprintf(s->err, sizeof s->err, "too many primitive walls"); return -1; }
  orc_plane *w = &s->planes[s->nplanes++];
  memset(w, 0, sizeof *w);
  w->axis = axis; w->pos = radius; w->kind = 1; w->c1 = c1; w->c2 = c2;
  w->wall_type = wall_type; w->rolling_model = rolling_model;
  return 0;
}

static void grow_atoms(orc_sys *s, int n) {
  if (n <= s->nmax) return;
  s->nmax = n;
  size_t n3 = 3 * (size_t)n * sizeof(double), n1 = (size_t)n * sizeof(double);
  s->tag = (int *)xrealloc(s->tag, n * sizeof(int));
  s->type = (int *)xrealloc(s->type, n * sizeof(int));
  s->prow = (int *)xrealloc(s->prow, n * sizeof(int));
  s->x = (double *)xrealloc(s->x, n3); s->v = (double *)xrealloc(s->v, n3);
  s->omega = (double *)xrealloc(s->omega, n3); s->f = (double *)xrealloc(s->f, n3);
  s->torque = (double *)xrealloc(s->torque, n3); s->xhold = (double *)xrealloc(s->xhold, n3);
  s->radius = (double *)xrealloc(s->radius, n1); s->rmass = (double *)xrealloc(s->rmass, n1);
  for (int w = 0; w < s->nplanes; w++) s->planes[w].hist = (double *)xrealloc(s->planes[w].hist, n3);
  for (int k = 0; k < s->nmeshes; k++) {
    orc_mesh *m = &s->meshes[k];
    const size_t ns = (size_t)n * MESH_MAXSLOT;
    m->nslot = (int *)xrealloc(m->nslot, n * sizeof(int));
    m->npartner = (int *)xrealloc(m->npartner, n * sizeof(int));
    m->partner = (int *)xrealloc(m->partner, ns * sizeof(int));
    m->keep = (unsigned char *)xrealloc(m->keep, ns);
    m->inter = (unsigned char *)xrealloc(m->inter, ns);
    m->hist = (double *)xrealloc(m->hist, 3 * ns * sizeof(double));
  }
}

/* fix mesh/surface + fix wall/gran ... mesh: nodes[ntri][3][3] in element
 * order (element id = index).  edge/corner activity: given (the reference's
 * own flags) or NULL to derive them as SurfaceMesh::buildNeighbours does. */
int orc_add_mesh(orc_sys *s, int ntri, const double *nodes, int wall_type, int rolling_model,
                 const unsigned char *edge_active, const unsigned char *corner_active) {
  if (s->nmeshes >= 4 || s->n > 0) { snprintf(s->err, sizeof s->err, "add meshes before atoms (max 4)"); return -1; }
  orc_mesh *m = &s->meshes[s->nmeshes++];
  memset(m, 0, sizeof *m);
  m->ntri = ntri;
  m->wall_type = wall_type;
  m->rolling = rolling_model;
  const size_t t9 = 9 * (size_t)ntri, t3 = 3 * (size_t)ntri;
  m->node = (double *)xrealloc(NULL, t9 * sizeof(double));
  memcpy(m->node, nodes, t9 * sizeof(double));
  m->edgeVec = (double *)xrealloc(NULL, t9 * sizeof(double));
  m->edgeNorm = (double *)xrealloc(NULL, t9 * sizeof(double));
  m->edgeLen = (double *)xrealloc(NULL, t3 * sizeof(double));
  m->surfNorm = (double *)xrealloc(NULL, t3 * sizeof(double));
  m->center = (double *)xrealloc(NULL, t3 * sizeof(double));
  m->rBound = (double *)xrealloc(NULL, ntri * sizeof(double));
  m->obtuse = (int *)xrealloc(NULL, ntri * sizeof(int));
  m->edgeActive = (unsigned char *)xrealloc(NULL, t3);
  m->cornerActive = (unsigned char *)xrealloc(NULL, t3);
  m->nNeighs = (int *)xrealloc(NULL, ntri * sizeof(int));
  m->neighFaces = (int *)xrealloc(NULL, 5 * (size_t)ntri * sizeof(int));
  mesh_geometry(m);
  mesh_topology(m);
  if (edge_active) memcpy(m->edgeActive, edge_active, t3);
  if (corner_active) memcpy(m->cornerActive, corner_active, t3);
  return 0;
}

int orc_set_mesh_motion(orc_sys *s, int k, double vx, double vy, double vz) {
  if (k < 0 || k >= s->nmeshes || s->n > 0) { snprintf(s->err, sizeof s->err, "set mesh motion before atoms"); return -1; }
  orc_mesh *m = &s->meshes[k];
  m->moving = 1;
  m->vel[0] = vx; m->vel[1] = vy; m->vel[2] = vz;
  const size_t t9 = 9 * (size_t)m->ntri;
  m->nodev = (double *)xrealloc(m->nodev, t9 * sizeof(double));
  memset(m->nodev, 0, t9 * sizeof(double));
  m->nodeLast = (double *)xrealloc(m->nodeLast, t9 * sizeof(double));
  memcpy(m->nodeLast, m->node, t9 * sizeof(double));
  return 0;
}

/* fix move/mesh mesh ID rotate origin O axis A period T (MeshMoverRotate,
 * src/mesh_mover_rotation.cpp:66-131): axis normalised
 * (vectorNormalize3D), omega = 2 pi / T; every step the mesh turns by
 * omega*dt through the quaternion of MultiNodeMesh::rotate(dAngle, axis, p)
 * (src/multi_node_mesh_I.h:620-640) */
int orc_set_mesh_rotation(orc_sys *s, int k, const double *origin, const double *axis, double period) {
  if (k < 0 || k >= s->nmeshes || s->n > 0) { snprintf(s->err, sizeof s->err, "set mesh motion before atoms"); return -1; }
  if (!(period != 0.0)) { snprintf(s->err, sizeof s->err, "rotation period is zero"); return -1; }
  orc_mesh *m = &s->meshes[k];
  double ax[3] = {axis[0], axis[1], axis[2]};
  const double norm = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
  const double invnorm = (norm == 0.) ? 0. : 1. / norm;
  for (int d = 0; d < 3; d++) ax[d] *= invnorm;
  const double omega = 2. * M_PI / period;
  const double dangle = omega * s->cfg.dt;
  /* MultiNodeMesh::rotate(dAngle, axis, p): axisNorm = axis / |axis| */
  double an[3] = {ax[0], ax[1], ax[2]};
  const double mag = sqrt(an[0] * an[0] + an[1] * an[1] + an[2] * an[2]);
  const double sinv = 1. / mag;
  for (int d = 0; d < 3; d++) an[d] = sinv * an[d];
  m->rot_dq[0] = cos(dangle * 0.5);
  for (int d = 0; d < 3; d++) m->rot_dq[d + 1] = an[d] * sin(dangle * 0.5);
  for (int d = 0; d < 3; d++) {
    m->rot_origin[d] = origin[d];
    m->rot_omega[d] = ax[d] * omega; /* vectorScalarMult3D(axis_, omega_, omegaVec) */
  }
  m->moving = 2;
  const size_t t9 = 9 * (size_t)m->ntri;
  m->nodev = (double *)xrealloc(m->nodev, t9 * sizeof(double));
  memset(m->nodev, 0, t9 * sizeof(double));
  m->nodeLast = (double *)xrealloc(m->nodeLast, t9 * sizeof(double));
  memcpy(m->nodeLast, m->node, t9 * sizeof(double));
  return 0;
}

int orc_get_mesh_nodes(const orc_sys *s, int k, double *nodes) {
  if (k < 0 || k >= s->nmeshes) return -1;
  memcpy(nodes, s->meshes[k].node, 9 * (size_t)s->meshes[k].ntri * sizeof(double));
  return s->meshes[k].ntri;
}

/* MeshMoverLinear::initial_integrate: v := 0 then += vel; nodes and centres
 * move by dx = dt*vel (MultiNodeMesh::move, src/multi_node_mesh_I.h:502-520) */
static void mesh_move(orc_sys *s, orc_mesh *m) {
  double dx[3];
  for (int d = 0; d < 3; d++) dx[d] = s->cfg.dt * m->vel[d];
  for (int t = 0; t < m->ntri; t++) {
    for (int q = 0; q < 3; q++)
      for (int d = 0; d < 3; d++) {
        m->node[9 * (size_t)t + 3 * q + d] = m->node[9 * (size_t)t + 3 * q + d] + dx[d];
        m->nodev[9 * (size_t)t + 3 * q + d] = 0.0 + m->vel[d];
      }
    for (int d = 0; d < 3; d++) m->center[3 * (size_t)t + d] = m->center[3 * (size_t)t + d] + dx[d];
  }
}

/* MathExtra::quatquat (src/math_extra.h:596-602) */
static void quatquat(const double *a, const double *b, double *c) {
  c[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  c[1] = a[0] * b[1] + b[0] * a[1] + a[2] * b[3] - a[3] * b[2];
  c[2] = a[0] * b[2] + b[0] * a[2] + a[3] * b[1] - a[1] * b[3];
  c[3] = a[0] * b[3] + b[0] * a[3] + a[1] * b[2] - a[2] * b[1];
}

/* MathExtraLiggghts::vec_quat_rotate, in place (src/math_extra_liggghts.h:455-471):
 * (0, v) -> q (0, v) q* */
static void vec_quat_rotate(double *v, const double *q) {
  const double vq[4] = {0., v[0], v[1], v[2]};
  const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
  double t[4], r[4];
  quatquat(q, vq, t);
  quatquat(t, qc, r);
  v[0] = r[1]; v[1] = r[2]; v[2] = r[3];
}

/* MeshMoverRotate::initial_integrate (src/mesh_mover_rotation.cpp:105-131):
 * MultiNodeMesh::rotate(dQ, origin) on nodes and centres
 * (src/multi_node_mesh_I.h:643-668), the rotating element vectors (edgeVec,
 * edgeNorm, surfaceNorm; TrackingMesh::rotate -> CustomValueTracker), then
 * node velocities v = 0 + omega x (node - origin) */
static void mesh_rotate(orc_sys *s, orc_mesh *m) {
  (void)s;
  const double *o = m->rot_origin, *q = m->rot_dq, *w = m->rot_omega;
  const int trans = (o[0] * o[0] + o[1] * o[1] + o[2] * o[2]) > 0.;
  for (int t = 0; t < m->ntri; t++) {
    double *c = &m->center[3 * (size_t)t];
    c[0] = c[1] = c[2] = 0.0;
    for (int j = 0; j < 3; j++) {
      double *nd = &m->node[9 * (size_t)t + 3 * j];
      if (trans) for (int d = 0; d < 3; d++) nd[d] = nd[d] - o[d];
      vec_quat_rotate(nd, q);
      if (trans) for (int d = 0; d < 3; d++) nd[d] = nd[d] + o[d];
      for (int d = 0; d < 3; d++) c[d] = nd[d] + c[d];
    }
    const double sinv = 1. / 3.;
    for (int d = 0; d < 3; d++) c[d] = sinv * c[d];
  }
  for (int t = 0; t < m->ntri; t++) {
    for (int j = 0; j < 3; j++) vec_quat_rotate(&m->edgeVec[9 * (size_t)t + 3 * j], q);
    for (int j = 0; j < 3; j++) vec_quat_rotate(&m->edgeNorm[9 * (size_t)t + 3 * j], q);
    vec_quat_rotate(&m->surfNorm[3 * (size_t)t], q);
  }
  for (int t = 0; t < m->ntri; t++)
    for (int j = 0; j < 3; j++) {
      const double *nd = &m->node[9 * (size_t)t + 3 * j];
      const double r[3] = {nd[0] - o[0], nd[1] - o[1], nd[2] - o[2]};
      double *v = &m->nodev[9 * (size_t)t + 3 * j];
      v[0] = 0.0 + (w[1] * r[2] - w[2] * r[1]);
      v[1] = 0.0 + (w[2] * r[0] - w[0] * r[2]);
      v[2] = 0.0 + (w[0] * r[1] - w[1] * r[0]);
    }
}

/* MultiNodeMesh::decideRebuild, src/multi_node_mesh_I.h:792-823 */
static int mesh_moved(const orc_sys *s, const orc_mesh *m) {
  const double triggersq = 0.25 * s->cfg.skin * s->cfg.skin;
  for (size_t k = 0; k < (size_t)m->ntri * 3; k++) {
    const double *a = &m->node[3 * k], *b = &m->nodeLast[3 * k];
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    if (dx * dx + dy * dy + dz * dz > triggersq) return 1;
  }
  return 0;
}

int orc_get_mesh_flags(const orc_sys *s, int k, unsigned char *edge_active, unsigned char *corner_active) {
  if (k < 0 || k >= s->nmeshes) return -1;
  const orc_mesh *m = &s->meshes[k];
  memcpy(edge_active, m->edgeActive, 3 * (size_t)m->ntri);
  memcpy(corner_active, m->cornerActive, 3 * (size_t)m->ntri);
  return m->ntri;
}

/* Mesh contacts: (atom tag, triangle index, slot, history[3]) per occupied slot */
int orc_get_mesh_contacts(const orc_sys *s, int k, int *tag, int *tri, int *slot, double *hist) {
  if (k < 0 || k >= s->nmeshes) return -1;
  const orc_mesh *m = &s->meshes[k];
  int c = 0;
  for (int i = 0; i < s->n; i++)
    for (int q = 0; q < m->nslot[i]; q++) {
      const int p = m->partner[(size_t)i * MESH_MAXSLOT + q];
      if (p < 0) continue;
      if (tag) tag[c] = s->tag[i];
      if (tri) tri[c] = p;
      if (slot) slot[c] = q;
      if (hist) for (int d = 0; d < 3; d++) hist[3 * c + d] = m->hist[3 * ((size_t)i * MESH_MAXSLOT + q) + d];
      c++;
    }
  return c;
}

/* FixInsert::pre_exchange (src/fix_insert.cpp): new atoms staged between
 * runs join at the next step after initial_integrate, and that step rebuilds
 * (next_reneighbor = the insertion step) */
int orc_insert_atoms(orc_sys *s, int k, const int *tag, const int *type, const double *x, const double *v,
                     const double *omega, const double *radius, const double *rmass) {
  if (k <= 0) return 0;
  const int m = s->npend + k;
  s->pend_tag = (int *)xrealloc(s->pend_tag, m * sizeof(int));
  s->pend_type = (int *)xrealloc(s->pend_type, m * sizeof(int));
  s->pend_x = (double *)xrealloc(s->pend_x, 3 * (size_t)m * sizeof(double));
  s->pend_v = (double *)xrealloc(s->pend_v, 3 * (size_t)m * sizeof(double));
  s->pend_w = (double *)xrealloc(s->pend_w, 3 * (size_t)m * sizeof(double));
  s->pend_r = (double *)xrealloc(s->pend_r, (size_t)m * sizeof(double));
  s->pend_m = (double *)xrealloc(s->pend_m, (size_t)m * sizeof(double));
  const int o = s->npend;
  memcpy(s->pend_tag + o, tag, k * sizeof(int));
  memcpy(s->pend_type + o, type, k * sizeof(int));
  memcpy(s->pend_x + 3 * o, x, 3 * (size_t)k * sizeof(double));
  memcpy(s->pend_v + 3 * o, v, 3 * (size_t)k * sizeof(double));
  memcpy(s->pend_w + 3 * o, omega, 3 * (size_t)k * sizeof(double));
  memcpy(s->pend_r + o, radius, (size_t)k * sizeof(double));
  memcpy(s->pend_m + o, rmass, (size_t)k * sizeof(double));
  s->npend = m;
  return 0;
}

static void commit_insert(orc_sys *s) {
  const int n0 = s->n, k = s->npend;
  grow_atoms(s, n0 + k);
  for (int q = 0; q < k; q++) {
    const int i = n0 + q;
    s->tag[i] = s->pend_tag[q];
    s->type[i] = s->pend_type[q];
    for (int d = 0; d < 3; d++) {
      s->x[3 * i + d] = s->pend_x[3 * q + d];
      s->v[3 * i + d] = s->pend_v[3 * q + d];
      s->omega[3 * i + d] = s->pend_w[3 * q + d];
      s->f[3 * i + d] = 0.0;
      s->torque[3 * i + d] = 0.0;
      for (int w = 0; w < s->nplanes; w++) s->planes[w].hist[3 * i + d] = 0.0;
    }
    s->radius[i] = s->pend_r[q];
    s->rmass[i] = s->pend_m[q];
    s->prow[i] = -1;
    for (int mm = 0; mm < s->nmeshes; mm++) {
      orc_mesh *m = &s->meshes[mm];
      m->nslot[i] = 0;
      m->npartner[i] = 0;
      for (int u = 0; u < MESH_MAXSLOT; u++) {
        m->partner[(size_t)i * MESH_MAXSLOT + u] = -1;
        m->keep[(size_t)i * MESH_MAXSLOT + u] = 0;
        m->inter[(size_t)i * MESH_MAXSLOT + u] = 0;
        for (int d = 0; d < 3; d++) m->hist[3 * ((size_t)i * MESH_MAXSLOT + u) + d] = 0.0;
      }
    }
  }
  s->n = n0 + k;
  s->npend = 0;
  s->next_reneighbor = s->ntimestep;
}

int orc_set_atoms(orc_sys *s, int n, const int *tag, const int *type, const double *x,
                  const double *v, const double *omega, const double *radius,
                  const double *rmass) {
  grow_atoms(s, n);
  s->n = n;
  memcpy(s->tag, tag, n * sizeof(int));
  memcpy(s->type, type, n * sizeof(int));
  memcpy(s->x, x, 3 * (size_t)n * sizeof(double));
  memcpy(s->v, v, 3 * (size_t)n * sizeof(double));
  memcpy(s->omega, omega, 3 * (size_t)n * sizeof(double));
  memcpy(s->radius, radius, (size_t)n * sizeof(double));
  memcpy(s->rmass, rmass, (size_t)n * sizeof(double));
  memset(s->f, 0, 3 * (size_t)n * sizeof(double));
  memset(s->torque, 0, 3 * (size_t)n * sizeof(double));
  for (int w = 0; w < s->nplanes; w++) memset(s->planes[w].hist, 0, 3 * (size_t)n * sizeof(double));
  for (int k = 0; k < s->nmeshes; k++) {
    orc_mesh *m = &s->meshes[k];
    for (int i = 0; i < n; i++) { m->nslot[i] = 0; m->npartner[i] = 0; }
    for (size_t q = 0; q < (size_t)n * MESH_MAXSLOT; q++) { m->partner[q] = -1; m->keep[q] = 0; m->inter[q] = 0; }
    memset(m->hist, 0, 3 * (size_t)n * MESH_MAXSLOT * sizeof(double));
  }
  for (int i = 0; i < n; i++) s->prow[i] = -1;
  s->list_valid = 0;
  s->computeflag = 0;
  s->prows = 0;
  return 0;
}

/* Restart data: per-atom partner lists as FixContactHistory::unpack_restart
 * leaves them (src/fix_contact_history.cpp:554-659).  Entries are directed
 * (owner tag, partner tag, owner's history). */
int orc_set_contact_history(orc_sys *s, int ne, const int *towner, const int *tpartner,
                            const double *hist) {
  const int n = s->n, dnum = s->dnum;
  int *cnt = (int *)calloc(n + 1, sizeof(int));
  int *own = (int *)malloc((ne + 1) * sizeof(int));
  for (int k = 0; k < ne; k++) {
    own[k] = -1;
    for (int i = 0; i < n; i++) if (s->tag[i] == towner[k]) { own[k] = i; break; }
    if (own[k] < 0) { free(cnt); free(own); snprintf(s->err, sizeof s->err, "unknown tag"); return -1; }
    cnt[own[k]]++;
  }
  s->pstart = (int *)xrealloc(s->pstart, (n + 1) * sizeof(int));
  s->pstart[0] = 0;
  for (int i = 0; i < n; i++) s->pstart[i + 1] = s->pstart[i] + cnt[i];
  s->ptag = (int *)xrealloc(s->ptag, (ne + 1) * sizeof(int));
  s->phist = (double *)xrealloc(s->phist, ((size_t)ne * dnum + 1) * sizeof(double));
  memset(cnt, 0, (n + 1) * sizeof(int));
  for (int k = 0; k < ne; k++) {
    int m = s->pstart[own[k]] + cnt[own[k]]++;
    s->ptag[m] = tpartner[k];
    for (int d = 0; d < dnum; d++) s->phist[(size_t)m * dnum + d] = hist[(size_t)k * dnum + d];
  }
  for (int i = 0; i < n; i++) s->prow[i] = i;
  s->prows = n;
  free(cnt);
  free(own);
  return 0;
}

int orc_set_wall_history(orc_sys *s, int wall, const double *hist) {
  if (wall < 0 || wall >= s->nplanes) return -1;
  memcpy(s->planes[wall].hist, hist, 3 * (size_t)s->n * sizeof(double));
  return 0;
}

/* ------------------------------------------------------------------ */
/* Parameters                                                          */
/* ------------------------------------------------------------------ */

static inline double M(const orc_sys *s, const double *m, int i, int j) {
  return m[(size_t)i * (s->ntypes + 1) + j];
}

/* cutneighmax = max over type pairs of (maxrad_i + maxrad_j)*cdf + skin,
 * src/pair_gran.cpp:591-602, src/neighbor.cpp:316-337 */
static void compute_cutneighmax(orc_sys *s) {
  double maxrad = 0.0;
  for (int i = 0; i < s->n; i++) if (s->radius[i] > maxrad) maxrad = s->radius[i];
  double cutoff = (maxrad + maxrad) * s->cfg.contact_distance_factor;
  double cutsq = cutoff * cutoff;
  s->cutneighmax = sqrt(cutsq) + s->cfg.skin;
}

/* ------------------------------------------------------------------ */
/* Domain::pbc + CommBrick::exchange (atom deletion in non-periodic dims) */
/* ------------------------------------------------------------------ */

static void copy_atom(orc_sys *s, int from, int to) {
  s->tag[to] = s->tag[from]; s->type[to] = s->type[from]; s->prow[to] = s->prow[from];
  for (int d = 0; d < 3; d++) {
    s->x[3 * to + d] = s->x[3 * from + d]; s->v[3 * to + d] = s->v[3 * from + d];
    s->omega[3 * to + d] = s->omega[3 * from + d]; s->f[3 * to + d] = s->f[3 * from + d];
    s->torque[3 * to + d] = s->torque[3 * from + d];
    for (int w = 0; w < s->nplanes; w++) s->planes[w].hist[3 * to + d] = s->planes[w].hist[3 * from + d];
  }
  for (int k = 0; k < s->nmeshes; k++) {
    orc_mesh *m = &s->meshes[k];
    m->nslot[to] = m->nslot[from];
    m->npartner[to] = m->npartner[from];
    for (int q = 0; q < MESH_MAXSLOT; q++) {
      m->partner[(size_t)to * MESH_MAXSLOT + q] = m->partner[(size_t)from * MESH_MAXSLOT + q];
      m->keep[(size_t)to * MESH_MAXSLOT + q] = m->keep[(size_t)from * MESH_MAXSLOT + q];
      m->inter[(size_t)to * MESH_MAXSLOT + q] = m->inter[(size_t)from * MESH_MAXSLOT + q];
      for (int d = 0; d < 3; d++)
        m->hist[3 * ((size_t)to * MESH_MAXSLOT + q) + d] = m->hist[3 * ((size_t)from * MESH_MAXSLOT + q) + d];
    }
  }
  s->radius[to] = s->radius[from]; s->rmass[to] = s->rmass[from];
}

static void pbc_and_exchange(orc_sys *s) {
  const double *lo = s->cfg.boxlo, *hi = s->cfg.boxhi;
  for (int i = 0; i < s->n; i++) {
    for (int d = 0; d < 3; d++) {
      if (!s->cfg.periodic[d]) continue;
      double prd = hi[d] - lo[d];
      double *xd = &s->x[3 * i + d];
      if (*xd < lo[d]) *xd += prd;
      if (*xd >= hi[d]) { *xd -= prd; if (*xd < lo[d]) *xd = lo[d]; }
    }
  }
  for (int dim = 0; dim < 3; dim++) {
    int i = 0;
    while (i < s->n) {
      double xd = s->x[3 * i + dim];
      if (xd < lo[dim] || xd >= hi[dim]) { copy_atom(s, s->n - 1, i); s->n--; }
      else i++;
    }
  }
}

/* ------------------------------------------------------------------ */
/* FixContactHistory::pre_exchange: neighbour list -> per-atom partners  */
/* ------------------------------------------------------------------ */

/* newtonflag of history value d (add_history_value's second argument) */
static inline int hist_newton(const orc_sys *s, int d) {
  if (!s->bond_on) return 1;
  return (d >= 5 && d <= 13) || d >= 28;
}

static void pre_exchange(orc_sys *s) {
  const int n = s->n, dnum = s->dnum;
  /* atoms inserted since the last build (FixInsert) are not in the list */
  const int nl = s->list_valid ? (s->list_n < n ? s->list_n : n) : 0;
  int *cnt = (int *)calloc(n + 1, sizeof(int));
  if (s->list_valid) {
    for (int i = 0; i < nl; i++)
      for (int p = s->nstart[i]; p < s->nstart[i + 1]; p++)
        if (s->nflag[p]) {
          cnt[i]++;
          int sh = s->nshift[p];
          if (sh == 0) cnt[s->nj[p]]++;  /* j < nlocal_neigh */
        }
  }
  s->pstart = (int *)xrealloc(s->pstart, (n + 1) * sizeof(int));
  s->pstart[0] = 0;
  for (int i = 0; i < n; i++) s->pstart[i + 1] = s->pstart[i] + cnt[i];
  int tot = s->pstart[n];
  s->ptag = (int *)xrealloc(s->ptag, (tot + 1) * sizeof(int));
  s->phist = (double *)xrealloc(s->phist, ((size_t)tot * dnum + 1) * sizeof(double));
  memset(cnt, 0, (n + 1) * sizeof(int));
  if (s->list_valid) {
    for (int i = 0; i < nl; i++)
      for (int p = s->nstart[i]; p < s->nstart[i + 1]; p++)
        if (s->nflag[p]) {
          const double *hist = &s->nhist[(size_t)p * dnum];
          int j = s->nj[p];
          int m = s->pstart[i] + cnt[i]++;
          s->ptag[m] = s->tag[j];
          for (int d = 0; d < dnum; d++) s->phist[(size_t)m * dnum + d] = hist[d];
          if (s->nshift[p] == 0) {
            m = s->pstart[j] + cnt[j]++;
            s->ptag[m] = s->tag[i];
            /* j's copy: values registered with newtonflag 1 change sign —
             * all of shear[3]; of the bond's, ft[3], thetan[3], thetat[3] */
            for (int d = 0; d < dnum; d++)
              s->phist[(size_t)m * dnum + d] = hist_newton(s, d) ? -hist[d] : hist[d];
          }
        }
  }
  for (int i = 0; i < n; i++) s->prow[i] = i;
  s->prows = n;
  free(cnt);
  s->computeflag = 0;
}

/* ------------------------------------------------------------------ */
/* Neighbour build                                                     */
/* ------------------------------------------------------------------ */

static inline int shift_code(int sx, int sy, int sz) { return (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1) - 13; }
static inline void shift_decode(int c, int *sx, int *sy, int *sz) {
  c += 13; *sx = c % 3 - 1; *sy = (c / 3) % 3 - 1; *sz = c / 9 - 1;
}

typedef struct { int j, sh; } cand_t;
static int cand_cmp(const void *a, const void *b) {
  const cand_t *p = (const cand_t *)a, *q = (const cand_t *)b;
  if (p->j != q->j) return p->j < q->j ? -1 : 1;
  return (p->sh > q->sh) - (p->sh < q->sh);
}

/* ghost coordinate x_j + pbc*prd exactly as CommBrick::borders/forward_comm */
static inline void image_x(const orc_sys *s, int j, int sh, double *xj) {
  int sx, sy, sz; shift_decode(sh, &sx, &sy, &sz);
  int sv[3] = {sx, sy, sz};
  for (int d = 0; d < 3; d++) {
    double dx = sv[d] * (s->cfg.boxhi[d] - s->cfg.boxlo[d]);
    xj[d] = sv[d] ? s->x[3 * j + d] + dx : s->x[3 * j + d];
  }
}

/* Whether the periodic image of j with shift sh exists as a ghost atom.
 * CommBrick::borders sends an atom across a periodic boundary when it lies
 * within slab_offset + its radius of that boundary (the granular criterion
 * of CommBrick::decide, src/comm_brick.cpp:443,1613-1624, with
 * slab_offset = cutghost/2 + skin/2 and cutghost = cutneighmax).  With a
 * contact distance factor above 1 this band is narrower than the pair
 * cutoff, so the reference misses some periodic pairs near the cutoff;
 * they are left out here as well. */
static int ghost_exists(const orc_sys *s, int j, int sh) {
  int sv[3];
  shift_decode(sh, &sv[0], &sv[1], &sv[2]);
  const double slab_offset = s->cutneighmax / 2. + s->cfg.skin / 2.;
  const double rad = s->radius[j];
  for (int d = 0; d < 3; d++) {
    const double pos = s->x[3 * j + d];
    if (sv[d] > 0 && !(pos <= (s->cfg.boxlo[d] + slab_offset) + rad)) return 0;
    if (sv[d] < 0 && !(pos >= (s->cfg.boxhi[d] - slab_offset) - rad)) return 0;
  }
  return 1;
}

static int neighbor_build(orc_sys *s) {
  const int n = s->n, dnum = s->dnum;
  const double cdf = s->cfg.contact_distance_factor, skin = s->cfg.skin;
  compute_cutneighmax(s);
  int nc[3];
  double csz[3];
  for (int d = 0; d < 3; d++) {
    double L = s->cfg.boxhi[d] - s->cfg.boxlo[d];
    nc[d] = (int)floor(L / s->cutneighmax);
    if (nc[d] < 1) nc[d] = 1;
    if (s->cfg.periodic[d] && nc[d] < 3) {
      snprintf(s->err, sizeof s->err, "periodic box dimension %d shorter than 3 neighbour cutoffs", d);
      return -1;
    }
    if (nc[d] > 1024) nc[d] = 1024;
    csz[d] = L / nc[d];
  }
  size_t ncell = (size_t)nc[0] * nc[1] * nc[2];
  int *head = (int *)malloc(ncell * sizeof(int));
  int *next = (int *)malloc((n + 1) * sizeof(int));
  int *cell = (int *)malloc((n + 1) * sizeof(int));
  for (size_t c = 0; c < ncell; c++) head[c] = -1;
  for (int i = n - 1; i >= 0; i--) {
    int ci[3];
    for (int d = 0; d < 3; d++) {
      int c = (int)((s->x[3 * i + d] - s->cfg.boxlo[d]) / csz[d]);
      if (c < 0) c = 0;
      if (c >= nc[d]) c = nc[d] - 1;
      ci[d] = c;
    }
    int c = ci[0] + nc[0] * (ci[1] + nc[1] * ci[2]);
    cell[i] = c;
    next[i] = head[c];
    head[c] = i;
  }

  /* new list */
  int *nstart = (int *)malloc((n + 1) * sizeof(int));
  int cap = s->npcap > 16 ? s->npcap : 16 * (n + 1);
  int *nj = (int *)malloc(cap * sizeof(int));
  int *nsh = (int *)malloc(cap * sizeof(int));
  int *nfl = (int *)malloc(cap * sizeof(int));
  double *nh = (double *)malloc((size_t)cap * dnum * sizeof(double));
  int np = 0;
  cand_t *cand = (cand_t *)malloc(4096 * sizeof(cand_t));
  int candcap = 4096;

  for (int i = 0; i < n; i++) {
    nstart[i] = np;
    const double xtmp = s->x[3 * i], ytmp = s->x[3 * i + 1], ztmp = s->x[3 * i + 2];
    const double radi = s->radius[i];
    int c = cell[i];
    int ci[3] = {c % nc[0], (c / nc[0]) % nc[1], c / (nc[0] * nc[1])};
    int nca = 0;
    for (int oz = -1; oz <= 1; oz++)
      for (int oy = -1; oy <= 1; oy++)
        for (int ox = -1; ox <= 1; ox++) {
          int o[3] = {ox, oy, oz}, cc[3], sv[3] = {0, 0, 0}, skip = 0;
          for (int d = 0; d < 3; d++) {
            cc[d] = ci[d] + o[d];
            if (nc[d] == 1 && o[d] != 0) { skip = 1; break; }
            if (cc[d] < 0) { if (!s->cfg.periodic[d]) { skip = 1; break; } cc[d] += nc[d]; sv[d] = -1; }
            if (cc[d] >= nc[d]) { if (!s->cfg.periodic[d]) { skip = 1; break; } cc[d] -= nc[d]; sv[d] = 1; }
          }
          if (skip) continue;
          int sh = shift_code(sv[0], sv[1], sv[2]);
          for (int j = head[cc[0] + nc[0] * (cc[1] + nc[1] * cc[2])]; j >= 0; j = next[j]) {
            if (sh == 0 && j <= i) continue;
            if (sh != 0 && !ghost_exists(s, j, sh)) continue;
            double xj[3];
            image_x(s, j, sh, xj);
            const double delx = xtmp - xj[0];
            const double dely = ytmp - xj[1];
            const double delz = ztmp - xj[2];
            const double rsq = delx * delx + dely * dely + delz * delz;
            const double radsum = (radi + s->radius[j]) * cdf;
            const double cutsq = (radsum + skin) * (radsum + skin);
            if (rsq <= cutsq) {
              if (nca == candcap) { candcap *= 2; cand = (cand_t *)xrealloc(cand, candcap * sizeof(cand_t)); }
              cand[nca].j = j; cand[nca].sh = sh; nca++;
            }
          }
        }
    qsort(cand, nca, sizeof(cand_t), cand_cmp);
    for (int k = 0; k < nca; k++) {
      if (np == cap) {
        cap *= 2;
        nj = (int *)xrealloc(nj, cap * sizeof(int)); nsh = (int *)xrealloc(nsh, cap * sizeof(int));
        nfl = (int *)xrealloc(nfl, cap * sizeof(int));
        nh = (double *)xrealloc(nh, (size_t)cap * dnum * sizeof(double));
      }
      int j = cand[k].j, sh = cand[k].sh;
      double xj[3];
      image_x(s, j, sh, xj);
      const double delx = xtmp - xj[0];
      const double dely = ytmp - xj[1];
      const double delz = ztmp - xj[2];
      const double rsq = delx * delx + dely * dely + delz * delz;
      const double radsum = (radi + s->radius[j]) * cdf;
      nj[np] = j; nsh[np] = sh;
      double *h = &nh[(size_t)np * dnum];
      int found = -1;
      if (rsq < radsum * radsum && s->prow[i] >= 0) {
        int r = s->prow[i];
        for (int m = s->pstart[r]; m < s->pstart[r + 1]; m++)
          if (s->ptag[m] == s->tag[j]) { found = m; break; }
      }
      if (found >= 0) {
        nfl[np] = 1;
        for (int d = 0; d < dnum; d++) h[d] = s->phist[(size_t)found * dnum + d];
      } else {
        nfl[np] = 0;
        for (int d = 0; d < dnum; d++) h[d] = 0.0;
      }
      np++;
    }
  }
  nstart[n] = np;
  free(cand); free(head); free(next); free(cell);
  free(s->nstart); free(s->nj); free(s->nshift); free(s->nflag); free(s->nhist);
  s->nstart = nstart; s->nj = nj; s->nshift = nsh; s->nflag = nfl; s->nhist = nh;
  s->np = np; s->npcap = cap;
  s->list_valid = 1;
  s->list_n = n;
  memcpy(s->xhold, s->x, 3 * (size_t)n * sizeof(double));
  s->ago = 0;
  s->nrebuilds++;
  /* partner rows are stale once the list owns the history */
  for (int i = 0; i < n; i++) s->prow[i] = -1;
  return 0;
}

/* PrimitiveWall::buildNeighList, src/primitive_wall.h:129-138, threshold = skin */
static void plane_neighbors(orc_sys *s) {
  for (int w = 0; w < s->nplanes; w++) {
    orc_plane *pl = &s->planes[w];
    if (pl->nncap < s->n) { pl->nncap = s->n; pl->nlist = (int *)xrealloc(pl->nlist, s->n * sizeof(int)); }
    pl->nn = 0;
    const int ay = (pl->axis + 1) % 3, az = (pl->axis + 2) % 3;
    for (int i = 0; i < s->n; i++) {
      double dMax = s->radius[i] + s->cfg.skin;
      if (pl->kind == 1) {
        /* Cylinder<dim>::resolveNeighlist (src/primitive_wall_definitions.h:192-198) */
        double dy = s->x[3 * i + ay] - pl->c1, dz = s->x[3 * i + az] - pl->c2;
        double dist = sqrt(dy * dy + dz * dz) - pl->pos;
        if (dMax < dist || -dMax < dist) pl->nlist[pl->nn++] = i;
        continue;
      }
      double dist = s->x[3 * i + pl->axis] - pl->pos;
      double absdist = (dist > 0.0) ? dist : -dist;
      if (absdist <= dMax) pl->nlist[pl->nn++] = i;
    }
  }
}

/* ------------------------------------------------------------------ */
/* Contact law                                                         */
/* ------------------------------------------------------------------ */

typedef struct {
  double dF[3], dT[3];
} fdata;

typedef struct {
  int is_wall, itype, jtype, update_history;
  double radi, radj, radsum, r, rinv, rsq, meff;
  double en[3], delta[3];
  const double *v_i, *v_j, *omega_i, *omega_j;
  double vn, deltan, cri, crj, wr1, wr2, wr3, vtr1, vtr2, vtr3;
  double Fn, kn, kt, gamman, gammat;
  double *shear;
  int *contact_flags;
  double *bondhist;        /* the bond's 28 history values, NULL without the model */
  const double *x_i;
  int has_force_update;
} sidata_t;

static void surface_default(sidata_t *sd) {
  const double enx = sd->en[0], eny = sd->en[1], enz = sd->en[2];
  const double vr1 = sd->v_i[0] - sd->v_j[0];
  const double vr2 = sd->v_i[1] - sd->v_j[1];
  const double vr3 = sd->v_i[2] - sd->v_j[2];
  const double vn = vr1 * enx + vr2 * eny + vr3 * enz;
  const double vn1 = vn * enx, vn2 = vn * eny, vn3 = vn * enz;
  const double vt1 = vr1 - vn1, vt2 = vr2 - vn2, vt3 = vr3 - vn3;
  const double deltan = sd->radsum - sd->r;
  const double dx = sd->delta[0], dy = sd->delta[1], dz = sd->delta[2];
  const double rinv = sd->rinv;
  double wr1, wr2, wr3;
  if (sd->is_wall) {
    const double cr = sd->radi - 0.5 * sd->deltan;
    wr1 = cr * sd->omega_i[0] * rinv;
    wr2 = cr * sd->omega_i[1] * rinv;
    wr3 = cr * sd->omega_i[2] * rinv;
    sd->cri = cr;
  } else {
    const double cri = sd->radi - 0.5 * deltan;
    const double crj = sd->radj - 0.5 * deltan;
    wr1 = (cri * sd->omega_i[0] + crj * sd->omega_j[0]) * rinv;
    wr2 = (cri * sd->omega_i[1] + crj * sd->omega_j[1]) * rinv;
    wr3 = (cri * sd->omega_i[2] + crj * sd->omega_j[2]) * rinv;
    sd->cri = cri;
    sd->crj = crj;
  }
  sd->vtr1 = vt1 - (dz * wr2 - dy * wr3);
  sd->vtr2 = vt2 - (dx * wr3 - dz * wr1);
  sd->vtr3 = vt3 - (dy * wr1 - dx * wr2);
  sd->vn = vn;
  sd->deltan = deltan;
  sd->wr1 = wr1; sd->wr2 = wr2; sd->wr3 = wr3;
}

static void normal_hertz(const orc_sys *s, sidata_t *sd, fdata *fi, fdata *fj) {
  if (sd->contact_flags) *sd->contact_flags |= CONTACT_NORMAL_MODEL;
  const int it = sd->itype, jt = sd->jtype;
  const double radi = sd->radi, radj = sd->radj;
  double reff = sd->is_wall ? radi : (radi * radj / (radi + radj));
  const double meff = sd->meff;
  const double sqrtval = sqrt(reff * sd->deltan);
  const double deltan = sd->deltan;
  const double Y = M(s, s->Yeff, it, jt), G = M(s, s->Geff, it, jt), be = M(s, s->betaeff, it, jt);
  const double Sn = 2. * Y * sqrtval;
  const double St = 8. * G * sqrtval;
  double kn = 4. / 3. * Y * sqrtval;
  double kt = St;
  const double sqrtFiveOverSix = 0.91287092917527685576161630466800355658790782499663875;
  const double gamman = -2. * sqrtFiveOverSix * be * sqrt(Sn * meff);
  const double gammat = s->cfg.tangential_damping ? -2. * sqrtFiveOverSix * be * sqrt(St * meff) : 0.0;
  kn /= 1.0; /* force->nktv2p, 1 in SI */
  kt /= 1.0;
  const double Fn_damping = -gamman * sd->vn;
  const double Fn_contact = kn * deltan;
  double Fn = Fn_damping + Fn_contact;
  if (s->cfg.limit_force && Fn < 0.0) Fn = 0.0;
  sd->Fn = Fn; sd->kn = kn; sd->kt = kt; sd->gamman = gamman; sd->gammat = gammat;
  if (sd->is_wall) {
    const double Fn_ = Fn * 1.0; /* area_ratio */
    fi->dF[0] += Fn_ * sd->en[0]; fi->dF[1] += Fn_ * sd->en[1]; fi->dF[2] += Fn_ * sd->en[2];
  } else {
    fi->dF[0] += sd->Fn * sd->en[0]; fi->dF[1] += sd->Fn * sd->en[1]; fi->dF[2] += sd->Fn * sd->en[2];
    fj->dF[0] += -fi->dF[0]; fj->dF[1] += -fi->dF[1]; fj->dF[2] += -fi->dF[2];
  }
}

static void normal_hooke(const orc_sys *s, sidata_t *sd, fdata *fi, fdata *fj) {
  if (sd->contact_flags) *sd->contact_flags |= CONTACT_NORMAL_MODEL;
  const int it = sd->itype, jt = sd->jtype;
  const double radi = sd->radi, radj = sd->radj;
  double reff = sd->is_wall ? radi : (radi * radj / (radi + radj));
  const double meff = sd->meff;
  const double sqrtval = sqrt(reff);
  const double Y = M(s, s->Yeff, it, jt);
  const double coeffRestLogChosen = M(s, s->restlog, it, jt);
  const double charVel = s->charVel;
  double kn = 16. / 15. * sqrtval * (Y) * pow(15. * meff * charVel * charVel / (16. * sqrtval * Y), 0.2);
  double kt = kn;
  const double coeffRestLogChosenSq = coeffRestLogChosen * coeffRestLogChosen;
  const double gamman = sqrt(4. * meff * kn * coeffRestLogChosenSq / (coeffRestLogChosenSq + M_PI * M_PI));
  const double gammat = s->cfg.tangential_damping ? gamman : 0.0;
  kn /= 1.0;
  kt /= 1.0;
  const double Fn_damping = -gamman * sd->vn;
  const double deltan = sd->deltan;
  const double Fn_contact = kn * deltan;
  double Fn = Fn_damping + Fn_contact;
  if (s->cfg.limit_force && Fn < 0.0) Fn = 0.0;
  sd->Fn = Fn; sd->kn = kn; sd->kt = kt; sd->gamman = gamman; sd->gammat = gammat;
  if (sd->is_wall) {
    const double Fn_ = Fn * 1.0;
    fi->dF[0] += Fn_ * sd->en[0]; fi->dF[1] += Fn_ * sd->en[1]; fi->dF[2] += Fn_ * sd->en[2];
  } else {
    fi->dF[0] += sd->Fn * sd->en[0]; fi->dF[1] += sd->Fn * sd->en[1]; fi->dF[2] += sd->Fn * sd->en[2];
    fj->dF[0] += -fi->dF[0]; fj->dF[1] += -fi->dF[1]; fj->dF[2] += -fi->dF[2];
  }
}

static void tangential_history(const orc_sys *s, sidata_t *sd, fdata *fi, fdata *fj) {
  const double enx = sd->en[0], eny = sd->en[1], enz = sd->en[2];
  if (sd->contact_flags) *sd->contact_flags |= CONTACT_TANGENTIAL_MODEL;
  double *const shear = sd->shear;
  if (sd->update_history) {
    const double dt = s->cfg.dt;
    shear[0] += sd->vtr1 * dt;
    shear[1] += sd->vtr2 * dt;
    shear[2] += sd->vtr3 * dt;
    double rsht = shear[0] * enx + shear[1] * eny + shear[2] * enz;
    shear[0] -= rsht * enx;
    shear[1] -= rsht * eny;
    shear[2] -= rsht * enz;
  }
  const double shrmag = sqrt(shear[0] * shear[0] + shear[1] * shear[1] + shear[2] * shear[2]);
  const double kt = sd->kt;
  const double xmu = M(s, s->frict, sd->itype, sd->jtype);
  double Ft1 = -(kt * shear[0]);
  double Ft2 = -(kt * shear[1]);
  double Ft3 = -(kt * shear[2]);
  const double Ft_shear = kt * shrmag;
  const double Ft_friction = xmu * fabs(sd->Fn);
  if (Ft_shear > Ft_friction) {
    if (shrmag != 0.0) {
      const double ratio = Ft_friction / Ft_shear;
      Ft1 *= ratio; Ft2 *= ratio; Ft3 *= ratio;
      if (sd->update_history) {
        shear[0] = -Ft1 / kt;
        shear[1] = -Ft2 / kt;
        shear[2] = -Ft3 / kt;
      }
    } else
      Ft1 = Ft2 = Ft3 = 0.0;
  } else {
    const double gammat = sd->gammat;
    Ft1 -= (gammat * sd->vtr1);
    Ft2 -= (gammat * sd->vtr2);
    Ft3 -= (gammat * sd->vtr3);
  }
  const double Tn_shear = 0.;
  const double tor1 = eny * Ft3 - enz * Ft2;
  const double tor2 = enz * Ft1 - enx * Ft3;
  const double tor3 = enx * Ft2 - eny * Ft1;
  double torque_i[3], torque_j[3] = {0., 0., 0.};
  torque_i[0] = -sd->cri * tor1 + Tn_shear * enx;
  torque_i[1] = -sd->cri * tor2 + Tn_shear * eny;
  torque_i[2] = -sd->cri * tor3 + Tn_shear * enz;
  if (!sd->is_wall) {
    torque_j[0] = -sd->crj * tor1 - Tn_shear * enx;
    torque_j[1] = -sd->crj * tor2 - Tn_shear * eny;
    torque_j[2] = -sd->crj * tor3 - Tn_shear * enz;
  }
  if (sd->is_wall) {
    const double area_ratio = 1.0;
    fi->dF[0] += Ft1 * area_ratio; fi->dF[1] += Ft2 * area_ratio; fi->dF[2] += Ft3 * area_ratio;
    fi->dT[0] += torque_i[0] * area_ratio; fi->dT[1] += torque_i[1] * area_ratio;
    fi->dT[2] += torque_i[2] * area_ratio;
  } else {
    fi->dF[0] += Ft1; fi->dF[1] += Ft2; fi->dF[2] += Ft3;
    fj->dF[0] += -Ft1; fj->dF[1] += -Ft2; fj->dF[2] += -Ft3;
    fi->dT[0] += torque_i[0]; fi->dT[1] += torque_i[1]; fi->dT[2] += torque_i[2];
    fj->dT[0] += torque_j[0]; fj->dT[1] += torque_j[1]; fj->dT[2] += torque_j[2];
  }
}

static void rolling_cdt(const orc_sys *s, sidata_t *sd, fdata *fi, fdata *fj) {
  const double rmu = M(s, s->rollfrict, sd->itype, sd->jtype);
  double r_torque[3] = {0., 0., 0.}, wr_roll[3];
  const double radi = sd->radi, radj = sd->radj;
  double reff = sd->is_wall ? radi : (radi * radj / (radi + radj));
  if (sd->is_wall) {
    const double wr1 = sd->wr1, wr2 = sd->wr2, wr3 = sd->wr3;
    const double wrmag = sqrt(wr1 * wr1 + wr2 * wr2 + wr3 * wr3);
    if (wrmag > 0.) {
      const double kn = sd->kn;
      const double enx = sd->en[0], eny = sd->en[1], enz = sd->en[2];
      const double Fn = sd->deltan * kn;
      r_torque[0] = rmu * Fn * wr1 / wrmag * reff;
      r_torque[1] = rmu * Fn * wr2 / wrmag * reff;
      r_torque[2] = rmu * Fn * wr3 / wrmag * reff;
      double rtd = r_torque[0] * enx + r_torque[1] * eny + r_torque[2] * enz;
      double rn[3] = {enx * rtd, eny * rtd, enz * rtd};
      r_torque[0] = r_torque[0] - rn[0];
      r_torque[1] = r_torque[1] - rn[1];
      r_torque[2] = r_torque[2] - rn[2];
    }
  } else {
    wr_roll[0] = sd->omega_i[0] - sd->omega_j[0];
    wr_roll[1] = sd->omega_i[1] - sd->omega_j[1];
    wr_roll[2] = sd->omega_i[2] - sd->omega_j[2];
    const double wr_rollmag = sqrt(wr_roll[0] * wr_roll[0] + wr_roll[1] * wr_roll[1] + wr_roll[2] * wr_roll[2]);
    if (wr_rollmag > 0.) {
      const double enx = sd->en[0], eny = sd->en[1], enz = sd->en[2];
      const double fac = rmu * sd->kn * sd->deltan * reff / wr_rollmag;
      r_torque[0] = fac * wr_roll[0];
      r_torque[1] = fac * wr_roll[1];
      r_torque[2] = fac * wr_roll[2];
      const double rtd = r_torque[0] * enx + r_torque[1] * eny + r_torque[2] * enz;
      double rn[3] = {enx * rtd, eny * rtd, enz * rtd};
      r_torque[0] = r_torque[0] - rn[0];
      r_torque[1] = r_torque[1] - rn[1];
      r_torque[2] = r_torque[2] - rn[2];
    }
  }
  fi->dT[0] -= r_torque[0]; fi->dT[1] -= r_torque[1]; fi->dT[2] -= r_torque[2];
  fj->dT[0] += r_torque[0]; fj->dT[1] += r_torque[1]; fj->dT[2] += r_torque[2];
}

/* ------------------------------------------------------------------ */
/* CohesionModel<COHESION_BOND_NONLINEAR>                              */
/* src/cohesion_model_bond_nonlinear.h:394-992 (particle pairs)        */
/* ------------------------------------------------------------------ */

#define CONTACT_COHESION_MODEL (1 << 1)

static inline double BT(const orc_sys *s, int table, int i, int j) {
  const size_t m = (size_t)(s->ntypes + 1) * (s->ntypes + 1);
  return s->bond[table * m + (size_t)i * (s->ntypes + 1) + j];
}

/* MathExtraLiggghts::sgn, src/math_extra_liggghts.h:120-123 */
static inline int sgn_d(double v) { return (0.0 < v) - (v < 0.0); }

/* vectorProject3D with vectorNormalize3D, src/vector_liggghts.h:63-70,437-442 */
static void project3(const double *v, const double *on, double *res) {
  double nrm[3] = {on[0], on[1], on[2]};
  const double norm = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  const double invnorm = (norm == 0.) ? 0. : 1. / norm;
  nrm[0] *= invnorm; nrm[1] *= invnorm; nrm[2] *= invnorm;
  const double dot = v[0] * nrm[0] + v[1] * nrm[1] + v[2] * nrm[2];
  res[0] = dot * nrm[0]; res[1] = dot * nrm[1]; res[2] = dot * nrm[2];
}

/* one component of the hysteretic twisting/bending torque,
 * src/cohesion_model_bond_nonlinear.h:677-761 (normal), :792-866 (tangential):
 * sign-driven reset of the opposite extreme, piecewise law, new extremes */
static double bond_hyst(double th, double *hmax, double *hmin, double k, double ku, double kc,
                        double JI) {
  if (th > 0.0) *hmin = 0.0;
  else if (th < 0.0) *hmax = 0.0;
  const double c1 = (ku - k) / (ku + kc) * *hmax;
  const double c2 = (ku - k) / (ku + kc) * *hmin;
  double t;
  if ((th >= *hmax) || (th <= *hmin)) t = -k * JI * th;
  else if (th > c1) t = -ku * JI * th + (ku - k) * JI * *hmax;
  else if (th >= c2) t = kc * JI * th;
  else t = -ku * JI * th + (ku - k) * JI * *hmin;
  if (th > *hmax) *hmax = th;
  if (th < *hmin) *hmin = th;
  return t;
}

/* breakBondnonlinear, :980-992 */
static void bond_break(sidata_t *sd) {
  if (sd->contact_flags) *sd->contact_flags &= ~CONTACT_COHESION_MODEL;
  sd->bondhist[0] = 0.;
  sd->bondhist[1] = 0.;
}

/* surfacesClose (also reached from surfacesIntersect once lambda > 0) for a
 * particle pair; ASSIGNS i/j forces and torques when the pair is bonded
 * (the override of :917-939). */
static void bond_nonlinear(const orc_sys *s, sidata_t *sd, fdata *fi, fdata *fj) {
  const orc_bond_settings *bs = &s->bset;
  const int it = sd->itype, jt = sd->jtype;
  const double radi = sd->radi, radj = sd->radj;
  const double lambda = BT(s, ORC_BOND_RADIUS_MULTIPLIER, it, jt);
  if (lambda < 1.e-15) return;
  double *const h = sd->bondhist;
  const int update_history = sd->update_history;
  const double r_centers = 1.0 * sqrt(sd->rsq);
  const double r = r_centers;
  if (update_history) {
    if (h[0] < 1.e-15) {
      const int create = (bs->createBondAlways || s->ntimestep == (long)(int)bs->tsCreate) &&
                         (r_centers < BT(s, ORC_BOND_CREATE_DIST, it, jt));
      if (!create) return;
      /* createBondnonlinear, :961-978 */
      if (sd->contact_flags) *sd->contact_flags |= CONTACT_COHESION_MODEL;
      h[0] = 1.0;
      h[1] = r;
      for (int d = 0; d < 3; d++) h[2 + d] = sd->x_i[d] - sd->delta[d];
      for (int d = 5; d < 14; d++) h[d] = 0.0;
    }
  } else if (h[0] < 1.e-15) {
    return;
  }
  double delta[3] = {sd->delta[0], sd->delta[1], sd->delta[2]};
  double force_tang[3] = {h[5], h[6], h[7]};
  double theta_normal[3] = {h[8], h[9], h[10]};
  double theta_tang[3] = {h[11], h[12], h[13]};
  if (!bs->stressBreak && r > BT(s, ORC_BOND_MAX_DIST, it, jt) && update_history) {
    bond_break(sd);
    return;
  }
  if (sd->contact_flags) *sd->contact_flags |= CONTACT_COHESION_MODEL;
  const double rinv = 1. / r;
  const double en[3] = {rinv * delta[0], rinv * delta[1], rinv * delta[2]};
  const double *vi = sd->v_i, *vj = sd->v_j, *omegai = sd->omega_i, *omegaj = sd->omega_j;
  const double k_fn1 = BT(s, ORC_BOND_K_FN1, it, jt), ku_fn1 = BT(s, ORC_BOND_KU_FN1, it, jt);
  const double kc_fn1 = BT(s, ORC_BOND_KC_FN1, it, jt), k_fn2 = BT(s, ORC_BOND_K_FN2, it, jt);
  const double ku_fn2 = BT(s, ORC_BOND_KU_FN2, it, jt), kc_fn2 = BT(s, ORC_BOND_KC_FN2, it, jt);
  const double k_ft = BT(s, ORC_BOND_K_FT, it, jt);
  const double k_tn = BT(s, ORC_BOND_K_TN, it, jt), ku_tn = BT(s, ORC_BOND_KU_TN, it, jt);
  const double kc_tn = BT(s, ORC_BOND_KC_TN, it, jt);
  const double k_tt = BT(s, ORC_BOND_K_TT, it, jt), ku_tt = BT(s, ORC_BOND_KU_TT, it, jt);
  const double kc_tt = BT(s, ORC_BOND_KC_TT, it, jt);
  const double rb = lambda * (radi < radj ? radi : radj);
  const double A = M_PI * rb * rb;
  const double J = 0.5 * A * rb * rb;
  const double I = 0.5 * J;
  const double dt = s->cfg.dt;
  const double radsuminv = 1. / (radi + radj);
  const double cri = r * radi * radsuminv;
  const double crj = r * radj * radsuminv;
  double tmp1[3], tmp2[3];
  double vr[3] = {vi[0] - vj[0], vi[1] - vj[1], vi[2] - vj[2]};
  double vn[3], vt[3], wr[3], vtr[3], wn[3], wt[3];
  project3(vr, en, vn);
  for (int d = 0; d < 3; d++) vt[d] = vr[d] - vn[d];
  for (int d = 0; d < 3; d++) {
    tmp1[d] = (radi * radsuminv) * omegai[d];
    tmp2[d] = (radj * radsuminv) * omegaj[d];
    wr[d] = tmp1[d] + tmp2[d];
  }
  tmp1[0] = delta[1] * wr[2] - delta[2] * wr[1];
  tmp1[1] = delta[2] * wr[0] - delta[0] * wr[2];
  tmp1[2] = delta[0] * wr[1] - delta[1] * wr[0];
  for (int d = 0; d < 3; d++) vtr[d] = vt[d] + tmp1[d];
  for (int d = 0; d < 3; d++) wr[d] = omegai[d] - omegaj[d];
  project3(wr, en, wn);
  for (int d = 0; d < 3; d++) wt[d] = wr[d] - wn[d];

  /* normal force, :582-636 */
  double nforce[3] = {0., 0., 0.}, dtforce[3] = {0., 0., 0.};
  double nfd[3] = {0., 0., 0.}, tfd[3] = {0., 0., 0.}, ntd[3] = {0., 0., 0.}, ttd[3] = {0., 0., 0.};
  const double displacement = (h[1] - r);
  double dmax, dmin;
  if (displacement > h[14]) { h[14] = displacement; dmax = displacement; }
  else dmax = h[14];
  if (displacement < h[27]) { h[27] = displacement; dmin = displacement; }
  else dmin = h[27];
  if (displacement < 0.0) h[14] = 0.0;
  if (displacement > 0.0) h[27] = 0.0;
  const double minvel = 1e-5 * (radi < radj ? radi : radj) / dt;
  if (bs->tensionStress || bs->compressionStress) {
    if ((bs->tensionStress && displacement < -1.e-15) ||
        (bs->compressionStress && displacement > 1.e-15)) {
      const double dc1 = pow((ku_fn1 - k_fn1) / (ku_fn1 + kc_fn1), 2.0) * dmax;
      const double dc2 = pow((ku_fn2 - k_fn2) / (ku_fn2 + kc_fn2), 1.0) * dmin;
      double frcmag;
      if (displacement < dmin) frcmag = k_fn2 * A * displacement;
      else if (displacement < dc2) frcmag = ku_fn2 * A * displacement + (k_fn2 - ku_fn2) * A * dmin;
      else if (displacement < 0.0) frcmag = -kc_fn2 * A * displacement;
      else if (displacement < dc1) frcmag = -kc_fn1 * pow(fabs(displacement), 0.5);
      else if (displacement < dmax)
        frcmag = ku_fn1 * pow(fabs(displacement), 0.5) + (k_fn1 - ku_fn1) * pow(fabs(dmax), 0.5);
      else frcmag = k_fn1 * pow(fabs(displacement), 0.5);
      for (int d = 0; d < 3; d++) nforce[d] = frcmag * en[d];
      if (bs->dampingBond) {
        const double dfn = BT(s, ORC_BOND_DAMP_FN, it, jt);
        for (int d = 0; d < 3; d++) {
          const double dv = 0.01 * nforce[d] * dt;
          const double mult = bs->dampingBondSmooth ? fmin(1.0, fmax(-1.0, vn[d] / fmax(minvel, dv)))
                                                    : (double)sgn_d(vn[d]);
          nfd[d] = nforce[d] - dfn * fabs(nforce[d]) * mult;
        }
      } else {
        for (int d = 0; d < 3; d++) nfd[d] = nforce[d];
      }
    }
  }
  /* shear force, :639-664 */
  if (bs->shearStress) {
    const double sc = -k_ft * A * dt;
    for (int d = 0; d < 3; d++) dtforce[d] = sc * vtr[d];
    project3(force_tang, en, tmp1);
    for (int d = 0; d < 3; d++) force_tang[d] = force_tang[d] - tmp1[d];
    for (int d = 0; d < 3; d++) force_tang[d] = force_tang[d] + dtforce[d];
    if (bs->dampingBond) {
      const double dft = BT(s, ORC_BOND_DAMP_FT, it, jt);
      for (int d = 0; d < 3; d++) {
        const double dv = 0.01 * force_tang[d] * dt;
        const double mult = bs->dampingBondSmooth ? fmin(1.0, fmax(-1.0, vtr[d] / fmax(minvel, dv)))
                                                  : (double)sgn_d(vtr[d]);
        tfd[d] = force_tang[d] - dft * fabs(force_tang[d]) * mult;
      }
    } else {
      for (int d = 0; d < 3; d++) tfd[d] = force_tang[d];
    }
  }
  /* twisting torque, :666-771 (the projected elastic torque formed first at
   * :673-674 is overwritten component-wise below and is not restated) */
  double torque_normal[3] = {0., 0., 0.}, torque_tang[3] = {0., 0., 0.};
  if (bs->normalTorqueStress) {
    for (int d = 0; d < 3; d++) theta_normal[d] = theta_normal[d] + dt * wn[d];
    for (int d = 0; d < 3; d++)
      torque_normal[d] = bond_hyst(theta_normal[d], &h[15 + d], &h[21 + d], k_tn, ku_tn, kc_tn, J);
    if (bs->dampingBond) {
      const double dtn = BT(s, ORC_BOND_DAMP_TN, it, jt);
      for (int d = 0; d < 3; d++)
        ntd[d] = torque_normal[d] - dtn * fabs(torque_normal[d]) * (double)sgn_d(wn[d]);
    } else {
      for (int d = 0; d < 3; d++) ntd[d] = torque_normal[d];
    }
  }
  /* bending torque, :774-873 */
  if (bs->shearTorqueStress) {
    for (int d = 0; d < 3; d++) theta_tang[d] = theta_tang[d] + dt * wt[d];
    for (int d = 0; d < 3; d++)
      torque_tang[d] = bond_hyst(theta_tang[d], &h[18 + d], &h[24 + d], k_tt, ku_tt, kc_tt, I);
    if (bs->dampingBond) {
      const double dtt = BT(s, ORC_BOND_DAMP_TT, it, jt);
      for (int d = 0; d < 3; d++)
        ttd[d] = torque_tang[d] - dtt * fabs(torque_tang[d]) * (double)sgn_d(wt[d]);
    } else {
      for (int d = 0; d < 3; d++) ttd[d] = torque_tang[d];
    }
  }
  /* stress breakage on undamped values, :876-891 */
  if (bs->stressBreak) {
    const double nfm = sqrt(nforce[0] * nforce[0] + nforce[1] * nforce[1] + nforce[2] * nforce[2]);
    const double tfm = sqrt(force_tang[0] * force_tang[0] + force_tang[1] * force_tang[1] +
                            force_tang[2] * force_tang[2]);
    const double ntm = sqrt(torque_normal[0] * torque_normal[0] + torque_normal[1] * torque_normal[1] +
                            torque_normal[2] * torque_normal[2]);
    const double ttm = sqrt(torque_tang[0] * torque_tang[0] + torque_tang[1] * torque_tang[1] +
                            torque_tang[2] * torque_tang[2]);
    const double maxSigma = BT(s, ORC_BOND_MAX_SIGMA, it, jt) *
                            ((bs->ratioTCBond && displacement < -1.e-15) ? BT(s, ORC_BOND_RATIO_TC, it, jt) : 1.0);
    const int nstress = maxSigma < (nfm / A + ttm * rb / I);
    const double maxTau = BT(s, ORC_BOND_MAX_TAU, it, jt);
    const int tstress = maxTau < (tfm / A + ntm * rb / J);
    if ((nstress || tstress) && update_history) {
      bond_break(sd);
      return;
    }
  }
  double tor[3];
  tor[0] = tfd[1] * en[2] - tfd[2] * en[1];
  tor[1] = tfd[2] * en[0] - tfd[0] * en[2];
  tor[2] = tfd[0] * en[1] - tfd[1] * en[0];
  sd->has_force_update = 1;
  if (update_history) {
    for (int d = 0; d < 3; d++) {
      h[5 + d] = force_tang[d];
      h[8 + d] = theta_normal[d];
      h[11 + d] = theta_tang[d];
    }
  }
  for (int d = 0; d < 3; d++) {
    const double F = nfd[d] + tfd[d];
    fi->dF[d] = F;
    fi->dT[d] = cri * tor[d] + ntd[d] + ttd[d];
    fj->dF[d] = -F;
    fj->dT[d] = crj * tor[d] - ntd[d] - ttd[d];
  }
}

/* the cohesion bond/nonlinear cutoff: neighbor->register_contact_dist_factor
 * from connectToProperties, :330-380 (minimum radius over the atoms) */
static int bond_contact_distance_factor(orc_sys *s) {
  if (!s->bond_on) return 0;
  if (!s->bond) { snprintf(s->err, sizeof s->err, "bond parameters not set"); return -1; }
  double minrad = 1e99;
  for (int i = 0; i < s->n; i++) minrad = fmin(minrad, s->radius[i]);
  double cdf_all = 1.;
  const int nt = s->ntypes;
  for (int i = 1; i < nt + 1; i++)
    for (int j = 1; j < nt + 1; j++) {
      double cdf_one;
      if (!s->bset.stressBreak) {
        cdf_one = 1.1 * 0.5 * BT(s, ORC_BOND_MAX_DIST, i, j) / minrad;
      } else {
        double stress = BT(s, ORC_BOND_MAX_SIGMA, i, j);
        if (s->bset.ratioTCBond) stress = fmax(stress, stress * BT(s, ORC_BOND_RATIO_TC, i, j));
        if (BT(s, ORC_BOND_K_FN2, i, j) <= 1e-15) {
          snprintf(s->err, sizeof s->err, "stress breakage needs stiffnessPerUnitAreaK_fn2 > 0");
          return -1;
        }
        cdf_one = 0.5 * 1.1 * BT(s, ORC_BOND_CREATE_DIST, i, j) / minrad +
                  0.5 * 1.1 * stress / (BT(s, ORC_BOND_K_FN2, i, j) * minrad);
      }
      cdf_all = cdf_one > cdf_all ? cdf_one : cdf_all;
    }
  if (cdf_all > 10.) { snprintf(s->err, sizeof s->err, "bond distance above 10 diameters"); return -1; }
  if (cdf_all > s->cfg.contact_distance_factor) s->cfg.contact_distance_factor = cdf_all;
  return 0;
}

static void surfaces_intersect(const orc_sys *s, sidata_t *sd, fdata *fi, fdata *fj, int rolling) {
  surface_default(sd);
  if (s->cfg.normal_model == ORC_NORMAL_HOOKE) normal_hooke(s, sd, fi, fj);
  else normal_hertz(s, sd, fi, fj);
  if (sd->bondhist) bond_nonlinear(s, sd, fi, fj);
  tangential_history(s, sd, fi, fj);
  if (rolling == ORC_ROLLING_CDT) rolling_cdt(s, sd, fi, fj);
}

/* TangentialModel<TANGENTIAL_HISTORY>::surfacesClose */
static void surfaces_close(sidata_t *sd) {
  if (sd->contact_flags) *sd->contact_flags &= ~CONTACT_TANGENTIAL_MODEL;
  if (!sd->shear) return;
  sd->shear[0] = 0.0; sd->shear[1] = 0.0; sd->shear[2] = 0.0;
}

/* Granular<CM>::compute_force, half list, newton off */
static void pair_compute(orc_sys *s, int shearupdate) {
  const double cdm = s->cfg.contact_distance_factor * s->cfg.contact_distance_factor;
  for (int i = 0; i < s->n; i++) {
    const double xtmp = s->x[3 * i], ytmp = s->x[3 * i + 1], ztmp = s->x[3 * i + 2];
    const double radi = s->radius[i];
    for (int p = s->nstart[i]; p < s->nstart[i + 1]; p++) {
      const int j = s->nj[p], sh = s->nshift[p];
      double xj[3];
      image_x(s, j, sh, xj);
      const double delx = xtmp - xj[0];
      const double dely = ytmp - xj[1];
      const double delz = ztmp - xj[2];
      const double rsq = delx * delx + dely * dely + delz * delz;
      const double radj = s->radius[j];
      const double radsum = radi + radj;
      sidata_t sd;
      memset(&sd, 0, sizeof sd);
      sd.is_wall = 0;
      sd.update_history = shearupdate;
      sd.radi = radi; sd.radj = radj; sd.radsum = radsum; sd.rsq = rsq;
      sd.delta[0] = delx; sd.delta[1] = dely; sd.delta[2] = delz;
      sd.contact_flags = &s->nflag[p];
      sd.shear = &s->nhist[(size_t)p * s->dnum + s->shear_off];
      sd.bondhist = s->bond_on ? &s->nhist[(size_t)p * s->dnum] : NULL;
      sd.x_i = &s->x[3 * i];
      sd.v_i = &s->v[3 * i]; sd.v_j = &s->v[3 * j];
      sd.omega_i = &s->omega[3 * i]; sd.omega_j = &s->omega[3 * j];
      sd.itype = s->type[i]; sd.jtype = s->type[j];
      fdata fi, fj;
      memset(&fi, 0, sizeof fi); memset(&fj, 0, sizeof fj);
      int has_force = 0;
      if (rsq < radsum * radsum) {
        const double r = sqrt(rsq);
        const double rinv = 1.0 / r;
        const double mi = s->rmass[i], mj = s->rmass[j];
        const double meff = mi * mj / (mi + mj);
        sd.r = r; sd.rinv = rinv; sd.meff = meff;
        sd.en[0] = delx * rinv; sd.en[1] = dely * rinv; sd.en[2] = delz * rinv;
        surfaces_intersect(s, &sd, &fi, &fj, s->cfg.rolling_model);
        has_force = 1;
      } else if (rsq < cdm * radsum * radsum) {
        /* ContactModel::surfacesClose: normal (no-op), cohesion, tangential */
        if (sd.bondhist) bond_nonlinear(s, &sd, &fi, &fj);
        surfaces_close(&sd);
        has_force = sd.has_force_update;
      }
      if (has_force) {
        s->ncontacts++;
        for (int d = 0; d < 3; d++) {
          s->f[3 * i + d] += 1.0 * fi.dF[d];
          s->torque[3 * i + d] += 1.0 * fi.dT[d];
        }
        if (sh == 0) {
          for (int d = 0; d < 3; d++) {
            s->f[3 * j + d] += 1.0 * fj.dF[d];
            s->torque[3 * j + d] += 1.0 * fj.dT[d];
          }
        }
      }
    }
  }
  s->computeflag = 1;
}

static void gravity_post_force(orc_sys *s) {
  if (!s->cfg.gravity_on) return;
  for (int i = 0; i < s->n; i++) {
    const double massone = s->rmass[i] * 1.;
    s->f[3 * i] += massone * s->cfg.gravity[0];
    s->f[3 * i + 1] += massone * s->cfg.gravity[1];
    s->f[3 * i + 2] += massone * s->cfg.gravity[2];
  }
}

/* Walls::Granular::compute_force for one wall contact with overlap -deltan,
 * wall-to-particle vector -delta (src/fix_wall_gran_base.h:159-372) */
static void wall_contact(orc_sys *s, int ip, double deltan, const double *delta, double *hist,
                         const double *vwall, int wall_type, int rolling, int shearupdate) {
  sidata_t sd;
  memset(&sd, 0, sizeof sd);
  sd.is_wall = 1;
  sd.radi = s->radius[ip];
  const int intersectflag = (deltan <= 0);
  sd.deltan = -deltan;
  sd.delta[0] = -delta[0]; sd.delta[1] = -delta[1]; sd.delta[2] = -delta[2];
  sd.shear = hist;
  sd.v_i = &s->v[3 * ip]; sd.v_j = vwall; sd.omega_i = &s->omega[3 * ip];
  sd.r = sd.radi - sd.deltan;
  sd.rsq = sd.r * sd.r;
  const double rinv = 1.0 / sd.r;
  sd.rinv = rinv;
  sd.contact_flags = NULL;
  sd.itype = s->type[ip];
  sd.meff = s->rmass[ip];
  sd.update_history = shearupdate;
  sd.jtype = wall_type;
  sd.en[0] = sd.delta[0] * rinv; sd.en[1] = sd.delta[1] * rinv; sd.en[2] = sd.delta[2] * rinv;
  sd.radsum = sd.radi;
  fdata fi, fj;
  memset(&fi, 0, sizeof fi); memset(&fj, 0, sizeof fj);
  if (intersectflag) {
    surfaces_intersect(s, &sd, &fi, &fj, rolling);
    for (int d = 0; d < 3; d++) {
      s->f[3 * ip + d] += fi.dF[d];
      s->torque[3 * ip + d] += fi.dT[d];
      if (s->cur_wall_f) s->cur_wall_f[d] += fi.dF[d];
    }
  } else {
    surfaces_close(&sd);
  }
}

static void plane_post_force(orc_sys *s, orc_plane *pl, int shearupdate) {
  const double cdm1 = s->cfg.contact_distance_factor - 1.0;
  const double vwall[3] = {0., 0., 0.};
  for (int k = 0; k < pl->nn; k++) {
    const int ip = pl->nlist[k];
    sidata_t sd;
    memset(&sd, 0, sizeof sd);
    sd.is_wall = 1;
    sd.radi = s->radius[ip];
    /* Plane<dim>::resolveContact */
    double delta[3];
    double deltan;
    const double *pos = &s->x[3 * ip];
    const int ax = pl->axis, ay = (ax + 1) % 3, az = (ax + 2) % 3;
    if (pl->kind == 1) {
      /* Cylinder<dim>::resolveContact (src/primitive_wall_definitions.h:170-190) */
      const double dy = pos[ay] - pl->c1, dz = pos[az] - pl->c2;
      const double dist = sqrt(dy * dy + dz * dz);
      if (dist < 1e-13 && dist > -1e-13) { /* compDouble(dist, 0.0) */
        delta[0] = delta[1] = delta[2] = 0.;
        deltan = 0.0;
      } else if (dist > pl->pos) {
        deltan = dist - pl->pos - sd.radi;
        const double fact = (dist - pl->pos) / dist;
        delta[ax] = 0.; delta[ay] = -dy * fact; delta[az] = -dz * fact;
      } else {
        deltan = pl->pos - dist - sd.radi;
        const double fact = (pl->pos - dist) / dist;
        delta[ax] = 0.; delta[ay] = +dy * fact; delta[az] = +dz * fact;
      }
    } else if (pos[ax] > pl->pos) {
      delta[ax] = pl->pos - pos[ax]; delta[ay] = 0.; delta[az] = 0.;
      deltan = pos[ax] - pl->pos - sd.radi;
    } else {
      delta[ax] = pl->pos - pos[ax]; delta[ay] = 0.; delta[az] = 0.;
      deltan = pl->pos - pos[ax] - sd.radi;
    }
    if (deltan > s->cutneighmax) continue;
    double *hist = &pl->hist[3 * ip];
    if (deltan <= 0 || deltan < cdm1 * s->radius[ip]) {
      wall_contact(s, ip, deltan, delta, hist, vwall, pl->wall_type, pl->rolling_model, shearupdate);
    } else {
      hist[0] = 0.; hist[1] = 0.; hist[2] = 0.;
    }
  }
}

/* ------------------------------------------------------------------ */
/* mesh walls                                                           */
/* ------------------------------------------------------------------ */

#define SLOT(m, i, q) ((size_t)(i) * MESH_MAXSLOT + (q))

static void mesh_swap(orc_mesh *m, int i, int a, int b, int keepflag) {
  int t = m->partner[SLOT(m, i, a)];
  m->partner[SLOT(m, i, a)] = m->partner[SLOT(m, i, b)];
  m->partner[SLOT(m, i, b)] = t;
  for (int d = 0; d < 3; d++) {
    double h = m->hist[3 * SLOT(m, i, a) + d];
    m->hist[3 * SLOT(m, i, a) + d] = m->hist[3 * SLOT(m, i, b) + d];
    m->hist[3 * SLOT(m, i, b) + d] = h;
  }
  if (keepflag) {
    unsigned char k = m->keep[SLOT(m, i, a)];
    m->keep[SLOT(m, i, a)] = m->keep[SLOT(m, i, b)];
    m->keep[SLOT(m, i, b)] = k;
    k = m->inter[SLOT(m, i, a)];
    m->inter[SLOT(m, i, a)] = m->inter[SLOT(m, i, b)];
    m->inter[SLOT(m, i, b)] = k;
  }
}

/* FixContactHistoryMesh::sort_contacts (pre_exchange) */
static void mesh_sort_contacts(orc_sys *s, orc_mesh *m) {
  for (int i = 0; i < s->n; i++) {
    const int nn = m->nslot[i];
    if (nn == 0) continue;
    int fe, lf;
    do {
      fe = lf = -1;
      for (int j = 0; j < nn; j++) {
        if (fe == -1 && m->partner[SLOT(m, i, j)] == -1) fe = j;
        if (m->partner[SLOT(m, i, j)] >= 0) lf = j;
      }
      if (fe > -1 && lf > -1 && fe < lf) mesh_swap(m, i, fe, lf, 1);
    } while (fe > -1 && lf > -1 && fe < lf);
  }
}

static int in_candidates(const orc_mesh *m, int t, int i) {
  for (int k = m->cstart[t]; k < m->cstart[t + 1]; k++)
    if (m->cand[k] == i) return 1;
  return 0;
}

/* FixNeighlistMesh::pre_force then FixContactHistoryMesh::pre_force */
static int mesh_neighbors(orc_sys *s, orc_mesh *m) {
  const int moving = m->nodev != NULL;
  const double cnm = s->cutneighmax, skin = s->cfg.skin;
  const double rmax = 0.5 * (cnm - skin);
  const double small_delta = skin / (70. * M_PI);
  const double tskin = moving ? skin : 0.5 * skin;
  const double distmax = moving ? cnm + small_delta : cnm - rmax + small_delta;
  const double cdf = s->cfg.contact_distance_factor;
  int *cnt = (int *)calloc(s->n + 1, sizeof(int));
  free(m->cstart);
  m->cstart = (int *)malloc((m->ntri + 1) * sizeof(int));
  int cap = 1024, np = 0;
  int *cand = (int *)malloc(cap * sizeof(int));
  for (int t = 0; t < m->ntri; t++) {
    m->cstart[t] = np;
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      lo[d] = hi[d] = MN(m, t, 0)[d];
      for (int q = 1; q < 3; q++) {
        const double v = MN(m, t, q)[d];
        lo[d] = v < lo[d] ? v : lo[d];
        hi[d] = v > hi[d] ? v : hi[d];
      }
      lo[d] -= distmax;
      hi[d] += distmax;
    }
    for (int i = 0; i < s->n; i++) {
      const double *x = &s->x[3 * i];
      if (x[0] < lo[0] || x[0] > hi[0] || x[1] < lo[1] || x[1] > hi[1] || x[2] < lo[2] || x[2] > hi[2])
        continue;
      if (!tri_sphere_neighbuild(m, t, s->radius[i] * cdf, x, tskin)) continue;
      if (np == cap) { cap *= 2; cand = (int *)xrealloc(cand, cap * sizeof(int)); }
      cand[np++] = i;
      cnt[i]++;
    }
  }
  m->cstart[m->ntri] = np;
  free(m->cand);
  m->cand = cand;
  for (int i = 0; i < s->n; i++) {
    if (cnt[i] > MESH_MAXSLOT) {
      snprintf(s->err, sizeof s->err, "mesh slot overflow");
      free(cnt);
      return -1;
    }
    /* cleanUpContactJumps */
    int ip = 0;
    while (ip < m->npartner[i]) {
      const int t = m->partner[SLOT(m, i, ip)];
      if (!in_candidates(m, t, i)) {
        m->partner[SLOT(m, i, ip)] = -1;
        for (int d = 0; d < 3; d++) m->hist[3 * SLOT(m, i, ip) + d] = 0.0;
        mesh_swap(m, i, ip, m->npartner[i] - 1, 0);
        m->npartner[i]--;
      } else
        ip++;
    }
    /* new pages: partners keep their slots, the rest is empty */
    for (int q = m->npartner[i]; q < MESH_MAXSLOT; q++) {
      m->partner[SLOT(m, i, q)] = -1;
      for (int d = 0; d < 3; d++) m->hist[3 * SLOT(m, i, q) + d] = 0.0;
    }
    m->nslot[i] = cnt[i];
  }
  free(cnt);
  return 0;
}

static int mesh_coplanar_already(const orc_mesh *m, int i, int t) {
  for (int q = 0; q < m->nslot[i]; q++) {
    const int p = m->partner[SLOT(m, i, q)];
    if (p >= 0 && p != t && coplanar_node_neighs(m, p, t) && m->keep[SLOT(m, i, q)]) return 1;
  }
  return 0;
}

/* FixContactHistoryMesh::handleContact; returns the slot or -1 (no contact) */
static int mesh_handle_contact(orc_sys *s, orc_mesh *m, int i, int t, int intersect, int faceflag) {
  for (int q = 0; q < m->nslot[i]; q++)
    if (m->partner[SLOT(m, i, q)] == t) {
      m->keep[SLOT(m, i, q)] = 1;
      m->inter[SLOT(m, i, q)] = (unsigned char)intersect;
      return q;
    }
  if (faceflag && mesh_coplanar_already(m, i, t)) return -1;
  if (m->npartner[i] >= m->nslot[i]) {
    snprintf(s->err, sizeof s->err, "mesh contact slots exhausted");
    return -1;
  }
  int slot = -1;
  for (int q = 0; q < m->nslot[i]; q++)
    if (m->partner[SLOT(m, i, q)] == -1) { slot = q; break; }
  m->partner[SLOT(m, i, slot)] = t;
  m->keep[SLOT(m, i, slot)] = 1;
  m->inter[SLOT(m, i, slot)] = (unsigned char)intersect;
  for (int d = 0; d < 3; d++) m->hist[3 * SLOT(m, i, slot) + d] = 0.0;
  m->npartner[i]++;
  if (faceflag)
    for (int q = 0; q < m->nslot[i]; q++) {
      const int p = m->partner[SLOT(m, i, q)];
      if (p >= 0 && p != t && coplanar_node_neighs(m, p, t))
        for (int d = 0; d < 3; d++) m->hist[3 * SLOT(m, i, slot) + d] = m->hist[3 * SLOT(m, i, q) + d];
    }
  return slot;
}

/* FixWallGran::post_force_mesh */
static void mesh_post_force(orc_sys *s, orc_mesh *m, int shearupdate) {
  const double cdm1 = s->cfg.contact_distance_factor - 1.0;
  for (int i = 0; i < s->n; i++)
    for (int q = 0; q < m->nslot[i]; q++) {
      m->keep[SLOT(m, i, q)] = 0;
      m->inter[SLOT(m, i, q)] = 0;
    }
  for (int t = 0; t < m->ntri; t++) {
    for (int k = m->cstart[t]; k < m->cstart[t + 1]; k++) {
      const int ip = m->cand[k];
      double delta[3], bary[3];
      int bs;
      const double deltan = resolve_tri_sphere(m, t, s->radius[ip], &s->x[3 * ip], delta, bary, &bs);
      if (deltan > s->cutneighmax) continue;
      const int intersect = deltan <= 0;
      if (deltan <= 0 || deltan < cdm1 * s->radius[ip]) {
        const int slot = mesh_handle_contact(s, m, ip, t, intersect, bs == 7);
        if (slot < 0) continue;
        double vwall[3] = {0., 0., 0.};
        if (m->nodev) {
          const double *vn = &m->nodev[9 * (size_t)t];
          for (int d = 0; d < 3; d++)
            vwall[d] = (bary[0] * vn[d] + bary[1] * vn[3 + d] + bary[2] * vn[6 + d]);
        }
        wall_contact(s, ip, deltan, delta, &m->hist[3 * SLOT(m, ip, slot)], vwall, m->wall_type,
                     m->rolling, shearupdate);
      }
    }
  }
  /* cleanUpContacts */
  for (int i = 0; i < s->n; i++)
    for (int q = 0; q < m->nslot[i]; q++)
      if (!m->keep[SLOT(m, i, q)]) {
        if (m->partner[SLOT(m, i, q)] > -1) m->npartner[i]--;
        m->partner[SLOT(m, i, q)] = -1;
        m->inter[SLOT(m, i, q)] = 0;
        for (int d = 0; d < 3; d++) m->hist[3 * SLOT(m, i, q) + d] = 0.0;
      }
}

static void force_clear(orc_sys *s) {
  memset(s->f, 0, 3 * (size_t)s->n * sizeof(double));
  memset(s->torque, 0, 3 * (size_t)s->n * sizeof(double));
  s->ncontacts = 0;
  memset(s->wall_f, 0, sizeof s->wall_f);
}

static void initial_integrate(orc_sys *s) {
  const double dtf = 0.5 * s->cfg.dt * 1.0; /* force->ftm2v = 1 in SI */
  const double dtv = s->cfg.dt;
  const double dtfrotate = dtf / 0.4;
  for (int i = 0; i < s->n; i++) {
    const double dtfm = dtf / (s->rmass[i] * (1. + 0.0));
    double *v = &s->v[3 * i], *x = &s->x[3 * i], *w = &s->omega[3 * i];
    const double *f = &s->f[3 * i], *t = &s->torque[3 * i];
    v[0] += dtfm * f[0]; v[1] += dtfm * f[1]; v[2] += dtfm * f[2];
    x[0] += dtv * v[0]; x[1] += dtv * v[1]; x[2] += dtv * v[2];
    const double dtirotate = dtfrotate / (s->radius[i] * s->radius[i] * s->rmass[i]);
    w[0] += dtirotate * t[0]; w[1] += dtirotate * t[1]; w[2] += dtirotate * t[2];
  }
}

static void final_integrate(orc_sys *s) {
  const double dtf = 0.5 * s->cfg.dt * 1.0;
  const double dtfrotate = dtf / 0.4;
  for (int i = 0; i < s->n; i++) {
    const double dtfm = dtf / (s->rmass[i] * (1. + 0.0));
    double *v = &s->v[3 * i], *w = &s->omega[3 * i];
    const double *f = &s->f[3 * i], *t = &s->torque[3 * i];
    v[0] += dtfm * f[0]; v[1] += dtfm * f[1]; v[2] += dtfm * f[2];
    const double dtirotate = dtfrotate / (s->radius[i] * s->radius[i] * s->rmass[i]);
    w[0] += dtirotate * t[0]; w[1] += dtirotate * t[1]; w[2] += dtirotate * t[2];
  }
}

static int check_distance(orc_sys *s) {
  const double skin = s->cfg.skin;
  const double deltasq = 0.25 * skin * skin;
  int flag = 0;
  for (int i = 0; i < s->n; i++) {
    const double delx = s->x[3 * i] - s->xhold[3 * i];
    const double dely = s->x[3 * i + 1] - s->xhold[3 * i + 1];
    const double delz = s->x[3 * i + 2] - s->xhold[3 * i + 2];
    const double rsq = delx * delx + dely * dely + delz * delz;
    if (rsq > deltasq) flag = 1;
  }
  return flag;
}

static int decide(orc_sys *s) {
  /* fixes that force a rebuild (FixMesh::next_reneighbor) come first */
  if (s->ntimestep == s->next_reneighbor) return 1;
  s->ago++;
  if (s->ago >= s->cfg.neigh_delay && s->ago % s->cfg.neigh_every == 0) {
    if (s->cfg.neigh_check == 0) return 1;
    return check_distance(s);
  }
  return 0;
}

static int rebuild(orc_sys *s) {
  /* FixMesh::pre_force on a rebuild step: node positions of this build
   * (refreshOwned -> storeNodePosRebuild) */
  for (int k = 0; k < s->nmeshes; k++)
    if (s->meshes[k].moving)
      memcpy(s->meshes[k].nodeLast, s->meshes[k].node, 9 * (size_t)s->meshes[k].ntri * sizeof(double));
  if (s->computeflag) pre_exchange(s);
  for (int k = 0; k < s->nmeshes; k++) mesh_sort_contacts(s, &s->meshes[k]);
  pbc_and_exchange(s);
  if (neighbor_build(s)) return -1;
  plane_neighbors(s);
  for (int k = 0; k < s->nmeshes; k++)
    if (mesh_neighbors(s, &s->meshes[k])) return -1;
  return 0;
}

static void compute_forces(orc_sys *s, int shearupdate) {
  force_clear(s);
  pair_compute(s, shearupdate);
  gravity_post_force(s);
  for (int w = 0; w < s->nplanes; w++) {
    s->cur_wall_f = w < ORC_DIAG_MAX_WALLS ? &s->wall_f[3 * w] : NULL;
    plane_post_force(s, &s->planes[w], shearupdate);
  }
  for (int k = 0; k < s->nmeshes; k++) {
    const int w = s->nplanes + k;
    s->cur_wall_f = w < ORC_DIAG_MAX_WALLS ? &s->wall_f[3 * w] : NULL;
    mesh_post_force(s, &s->meshes[k], shearupdate);
  }
  s->cur_wall_f = NULL;
}

int orc_setup(orc_sys *s) {
  if (!s->Yeff) { snprintf(s->err, sizeof s->err, "pair parameters not set"); return -1; }
  if (bond_contact_distance_factor(s)) return -1;
  if (rebuild(s)) return -1;
  compute_forces(s, 0);
  return 0;
}

int orc_run(orc_sys *s, int nsteps) {
  for (int k = 0; k < nsteps; k++) {
    s->ntimestep++;
    initial_integrate(s);
    for (int k = 0; k < s->nmeshes; k++)
      if (s->meshes[k].moving == 1) mesh_move(s, &s->meshes[k]);
      else if (s->meshes[k].moving == 2) mesh_rotate(s, &s->meshes[k]);
    if (s->npend > 0) commit_insert(s);
    if (decide(s)) {
      if (rebuild(s)) return -1;
    } else {
      /* FixMesh::pre_force on a regular step */
      for (int k = 0; k < s->nmeshes; k++)
        if (s->meshes[k].moving && mesh_moved(s, &s->meshes[k])) s->next_reneighbor = s->ntimestep + 1;
    }
    compute_forces(s, 1);
    final_integrate(s);
  }
  return 0;
}

/* diagnostics of the last force pass (see dem_get_diagnostics) */
long long orc_ncontacts(const orc_sys *s) { return s->ncontacts; }
int orc_get_wall_forces(const orc_sys *s, double *out) {
  const int nw = s->nplanes + s->nmeshes;
  for (int w = 0; w < nw && w < ORC_DIAG_MAX_WALLS; w++)
    for (int d = 0; d < 3; d++) out[3 * w + d] = s->wall_f[3 * w + d];
  return nw;
}

int orc_natoms(const orc_sys *s) { return s->n; }
int orc_npairs(const orc_sys *s) { return s->list_valid ? s->np : 0; }
int orc_dnum(const orc_sys *s) { return s->dnum; }
long orc_nrebuilds(const orc_sys *s) { return s->nrebuilds; }
long orc_ntimestep(const orc_sys *s) { return s->ntimestep; }

int orc_get_atoms(const orc_sys *s, int *tag, int *type, double *x, double *v, double *omega,
                  double *f, double *torque, double *radius, double *rmass) {
  const int n = s->n;
  size_t n3 = 3 * (size_t)n * sizeof(double);
  if (tag) memcpy(tag, s->tag, n * sizeof(int));
  if (type) memcpy(type, s->type, n * sizeof(int));
  if (x) memcpy(x, s->x, n3);
  if (v) memcpy(v, s->v, n3);
  if (omega) memcpy(omega, s->omega, n3);
  if (f) memcpy(f, s->f, n3);
  if (torque) memcpy(torque, s->torque, n3);
  if (radius) memcpy(radius, s->radius, n * sizeof(double));
  if (rmass) memcpy(rmass, s->rmass, n * sizeof(double));
  return n;
}

int orc_get_pairs(const orc_sys *s, int *tag_i, int *tag_j, int *shift, int *flag, double *hist) {
  if (!s->list_valid) return 0;
  for (int i = 0; i < s->n; i++)
    for (int p = s->nstart[i]; p < s->nstart[i + 1]; p++) {
      int sx, sy, sz;
      shift_decode(s->nshift[p], &sx, &sy, &sz);
      if (tag_i) tag_i[p] = s->tag[i];
      if (tag_j) tag_j[p] = s->tag[s->nj[p]];
      if (shift) { shift[3 * p] = sx; shift[3 * p + 1] = sy; shift[3 * p + 2] = sz; }
      if (flag) flag[p] = s->nflag[p];
      if (hist) for (int d = 0; d < s->dnum; d++) hist[(size_t)p * s->dnum + d] = s->nhist[(size_t)p * s->dnum + d];
    }
  return s->np;
}

int orc_get_wall_history(const orc_sys *s, int wall, double *hist) {
  if (wall < 0 || wall >= s->nplanes) return -1;
  memcpy(hist, s->planes[wall].hist, 3 * (size_t)s->n * sizeof(double));
  return s->n;
}
