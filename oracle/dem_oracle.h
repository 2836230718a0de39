/* ORACLE — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, single-threaded restatement of LIGGGHTS-INL's per-timestep DEM
 * path for spheres.  It exists to check the GPU product: only tests/, the
 * smoke check and the CPU-baseline leg of bench.py may load it.  The product
 * never links or calls it.
 *
 * Parity pin: tests/golden/ holds snapshots of the reference binary itself
 * (built from the reference sources by oracle/ref/Makefile) on seeded inputs;
 * tests/test_oracle_golden.py checks this restatement against them.
 *
 * Arrays follow the reference's per-atom layout: x[3*i+d] is atom->x[i][d].
 * Per-type-pair matrices are (ntypes+1)*(ntypes+1), row-major, index [i][j]
 * with types starting at 1, as MatrixProperty in src/global_properties.cpp.
 */
#ifndef DEM_ORACLE_H
#define DEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_NORMAL_HERTZ = 0, ORC_NORMAL_HOOKE = 1 };
enum { ORC_ROLLING_OFF = 0, ORC_ROLLING_CDT = 1 };
enum { ORC_COHESION_OFF = 0, ORC_COHESION_BOND_NONLINEAR = 1 };

typedef struct orc_config {
  double boxlo[3], boxhi[3];
  int periodic[3];
  double dt;
  double skin;                 /* neighbor SKIN bin */
  double contact_distance_factor; /* neigh_modify contact_distance_factor */
  int neigh_every, neigh_delay, neigh_check; /* neigh_modify every/delay/check */
  int normal_model;            /* ORC_NORMAL_* */
  int rolling_model;           /* ORC_ROLLING_* */
  int cohesion_model;          /* ORC_COHESION_* */
  int tangential_damping;      /* model option, default 1 */
  int limit_force;             /* model option limitForce, default 0 */
  int gravity_on;
  double gravity[3];           /* xacc, yacc, zacc of fix gravity */
} orc_config;

typedef struct orc_sys orc_sys;

orc_sys *orc_create(const orc_config *cfg);
void orc_destroy(orc_sys *s);

/* Per-type-pair tables, (ntypes+1)^2 each.  coeffRestLog and charVel are only
 * read by the Hooke law, coeffRollFrict only with CDT rolling. */
int orc_set_pair_params(orc_sys *s, int ntypes, const double *Yeff, const double *Geff,
                        const double *betaeff, const double *coeffFrict,
                        const double *coeffRollFrict, const double *coeffRestLog,
                        double charVel);

/* cohesion bond/nonlinear (src/cohesion_model_bond_nonlinear.h): the 23
 * per-type-pair property/global tables, each (ntypes+1)^2, stacked in this
 * order into one array; unused tables (e.g. maxSigma without stressBreak)
 * may hold zeros. */
enum {
  ORC_BOND_RADIUS_MULTIPLIER, ORC_BOND_K_FN1, ORC_BOND_KU_FN1, ORC_BOND_KC_FN1, ORC_BOND_K_FN2,
  ORC_BOND_KU_FN2, ORC_BOND_KC_FN2, ORC_BOND_K_FT, ORC_BOND_K_TN, ORC_BOND_KU_TN, ORC_BOND_KC_TN,
  ORC_BOND_K_TT, ORC_BOND_KU_TT, ORC_BOND_KC_TT, ORC_BOND_DAMP_FN, ORC_BOND_DAMP_FT,
  ORC_BOND_DAMP_TN, ORC_BOND_DAMP_TT, ORC_BOND_MAX_DIST, ORC_BOND_MAX_SIGMA, ORC_BOND_MAX_TAU,
  ORC_BOND_RATIO_TC, ORC_BOND_CREATE_DIST, ORC_BOND_NTABLES
};
/* The model's on/off settings (registerSettings, :231-243) and the scalar
 * tsCreateBondnonlinear. */
typedef struct orc_bond_settings {
  double tsCreate;
  int stressBreak, tensionStress, compressionStress, shearStress, normalTorqueStress,
      shearTorqueStress, createBondAlways, dampingBond, dampingBondSmooth, ratioTCBond;
} orc_bond_settings;
/* After orc_set_pair_params; cfg.cohesion_model must be ORC_COHESION_BOND_NONLINEAR.
 * The granular list then carries dnum = 31 history doubles per pair in the
 * reference's order: 28 bond values (bondFlag, initial_dist, contactPos[3],
 * ft[3], thetan[3], thetat[3], deltan_max, thetan_max[3], thetat_max[3],
 * thetan_min[3], thetat_min[3], deltan_min), then shear[3]. */
int orc_set_bond_params(orc_sys *s, const double *tables, const orc_bond_settings *st);

/* fix wall/gran ... primitive type WTYPE {x,y,z}plane POS (axis 0/1/2). */
int orc_add_plane(orc_sys *s, int axis, double pos, int wall_type, int rolling_model);
int orc_add_cylinder(orc_sys *s, int axis, double radius, double c1, double c2, int wall_type, int rolling_model);

/* fix mesh/surface + fix wall/gran mesh: nodes[ntri*9], element id = index.
 * edge_active/corner_active[ntri*3]: the reference's flags, or NULL to derive
 * them as SurfaceMesh::buildNeighbours does.  Add meshes before atoms. */
int orc_add_mesh(orc_sys *s, int ntri, const double *nodes, int wall_type, int rolling_model,
                 const unsigned char *edge_active, const unsigned char *corner_active);
/* fix move/mesh mesh ID linear vx vy vz (FixMoveMesh + MeshMoverLinear,
 * src/fix_move_mesh.cpp:194-240, src/mesh_mover_linear.cpp:95-112); add
 * before atoms. */
int orc_set_mesh_motion(orc_sys *s, int mesh, double vx, double vy, double vz);
int orc_set_mesh_rotation(orc_sys *s, int mesh, const double *origin, const double *axis, double period);
int orc_get_mesh_nodes(const orc_sys *s, int mesh, double *nodes);
int orc_get_mesh_flags(const orc_sys *s, int mesh, unsigned char *edge_active,
                       unsigned char *corner_active);
int orc_get_mesh_contacts(const orc_sys *s, int mesh, int *tag, int *tri, int *slot, double *hist);

int orc_set_atoms(orc_sys *s, int n, const int *tag, const int *type, const double *x,
                  const double *v, const double *omega, const double *radius,
                  const double *rmass);

/* Restart data (between orc_set_atoms and orc_setup): directed contact
 * history entries and per-atom wall history, as after read_restart. */
int orc_set_contact_history(orc_sys *s, int nentries, const int *tag_owner,
                            const int *tag_partner, const double *hist);
int orc_set_wall_history(orc_sys *s, int wall, const double *hist);

/* atoms that join at the next step after its initial integration, with a
 * rebuild at that step (FixInsert::pre_exchange) */
int orc_insert_atoms(orc_sys *s, int k, const int *tag, const int *type, const double *x, const double *v,
                     const double *omega, const double *radius, const double *rmass);
int orc_setup(orc_sys *s);            /* Verlet::setup */
int orc_run(orc_sys *s, int nsteps);  /* nsteps iterations of Verlet::run */

#define ORC_DIAG_MAX_WALLS 16
/* entries with a contact force, and the total force of each wall (planes,
 * then meshes; 3 doubles each) in the last force pass */
long long orc_ncontacts(const orc_sys *s);
int orc_get_wall_forces(const orc_sys *s, double *out);
int orc_natoms(const orc_sys *s);
int orc_get_atoms(const orc_sys *s, int *tag, int *type, double *x, double *v, double *omega,
                  double *f, double *torque, double *radius, double *rmass);
int orc_npairs(const orc_sys *s);
int orc_dnum(const orc_sys *s);
/* shift[3*p+d] is the periodic image of j: j's coordinate is x_j + shift*L. */
int orc_get_pairs(const orc_sys *s, int *tag_i, int *tag_j, int *shift, int *flag,
                  double *hist);
int orc_get_wall_history(const orc_sys *s, int wall, double *hist);
long orc_nrebuilds(const orc_sys *s);
long orc_ntimestep(const orc_sys *s);
const char *orc_last_error(const orc_sys *s);

#ifdef __cplusplus
}
#endif
#endif
