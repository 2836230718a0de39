/* liggghts_gb300.h — C ABI of the GB300 sphere-DEM timestep (libdemgpu.so).
 *
 * One handle holds one granular system resident on the GPU: particle state,
 * the granular half neighbour list with its contact history, primitive-wall
 * histories.  Every call returns a dem_status code; no exception crosses the
 * ABI.  One handle per host thread; each handle owns one CUDA stream.
 *
 * Reference interfaces each entry point replaces (LIGGGHTS-INL source paths):
 *   dem_create            PairGran::settings/init_style + Neighbor::init
 *                         (src/pair_gran_proxy.cpp:63-79, src/pair_gran.cpp:229-330,
 *                          src/neighbor.cpp:258-337)
 *   dem_set_pair_params   ContactModel::connectToProperties -> PropertyRegistry
 *                         matrices Yeff/Geff/betaeff/coeffFrict/coeffRollFrict/
 *                         coeffRestLog/charVel (src/global_properties.cpp:428-561,
 *                         src/normal_model_hertz.h:172-183, src/rolling_model_cdt.h:83-86)
 *   dem_set_bond_params   CohesionModel<COHESION_BOND_NONLINEAR>::registerSettings +
 *                         connectToProperties (src/cohesion_model_bond_nonlinear.h:231-381)
 *   dem_add_plane         FixWallGran "primitive type T {x,y,z}plane P"
 *                         (src/fix_wall_gran.cpp:176-215, src/primitive_wall_definitions.h:123-150)
 *   dem_upload_atoms      Atom arrays x v omega radius rmass type tag
 *                         (src/atom_vec_sphere.cpp:1060-1090, src/library.h:59-74)
 *   dem_setup             Verlet::setup (src/verlet.cpp setup(); src/pair_gran.cpp:633-635)
 *   dem_step              Verlet::run loop body (src/verlet.cpp:281-389): nve/sphere
 *                         initial/final_integrate, Neighbor::decide/build with history
 *                         carry-over, PairGran::compute, FixGravity and FixWallGran post_force
 *   dem_download_atoms    lammps_gather_atoms / Atom::extract (src/library.h:59-74)
 *   dem_download_contacts compute pair/gran/local id force history (src/compute_pair_gran_local.cpp:100-116)
 *   dem_download_wall_history  fix property/atom history_<wallid> (src/fix_wall_gran.cpp:477-500)
 *   dem_get_stats         Timer / Finish breakdown, Neighbor::ncalls (src/timer.h:51-52)
 */
#ifndef LIGGGHTS_GB300_H
#define LIGGGHTS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum dem_status {
  DEM_OK = 0,
  DEM_ERR_BAD_ARG = 1,        /* invalid argument or call order */
  DEM_ERR_CUDA = 2,           /* a CUDA runtime call failed; see dem_last_error */
  DEM_ERR_NEIGH_OVERFLOW = 3, /* neighbour list capacity could not be grown */
  DEM_ERR_NAN = 4,            /* non-finite particle state detected */
  DEM_ERR_TIMEOUT = 5,        /* a bounded device wait gave up */
  DEM_ERR_BOX = 6,            /* periodic box shorter than 3 neighbour cutoffs */
  DEM_ERR_UNSUPPORTED = 7,    /* contact-model combination not on the GPU path */
  DEM_ERR_NO_DEVICE = 8,      /* no CUDA device / kernel image */
  DEM_ERR_CAPACITY = 9        /* a fixed capacity was exceeded (mesh candidates per atom) */
} dem_status;

enum { DEM_NORMAL_HERTZ = 0, DEM_NORMAL_HOOKE = 1 };
enum { DEM_ROLLING_OFF = 0, DEM_ROLLING_CDT = 1 };
enum { DEM_COHESION_OFF = 0, DEM_COHESION_BOND_NONLINEAR = 1 };

/* Same meaning as the input-script settings of the reference. */
typedef struct dem_config {
  double boxlo[3], boxhi[3];
  int periodic[3];             /* boundary p (1) or f (0) per dimension */
  double dt;                   /* timestep */
  double skin;                 /* neighbor SKIN bin */
  double contact_distance_factor; /* neigh_modify contact_distance_factor (1.0) */
  int neigh_every, neigh_delay, neigh_check; /* neigh_modify every/delay/check */
  int normal_model;            /* DEM_NORMAL_* of pair_style gran model ... */
  int rolling_model;           /* DEM_ROLLING_* (rolling_friction cdt) */
  int cohesion_model;          /* DEM_COHESION_* */
  int tangential_damping;      /* model option tangential_damping (default 1) */
  int limit_force;             /* model option limitForce (default 0) */
  int gravity_on;              /* fix gravity present */
  double gravity[3];           /* xacc, yacc, zacc as FixGravity::set_acceleration */
} dem_config;

typedef struct dem_stats {
  long long ntimestep;         /* update->ntimestep */
  long long nrebuilds;         /* neighbour list builds (Neighbor::ncalls) */
  long long npairs;            /* entries in the granular half list */
  long long nlost;             /* atoms removed at non-periodic boundaries */
  long long natoms;
  int device;                  /* CUDA ordinal */
  int pair_capacity;
  double last_step_ms;         /* device time of the last dem_step call */
  int host_direct;             /* 1: dem_upload_atoms / dem_download_atoms kernels read and write the
                                  caller's arrays in place (the device reaches pageable host memory
                                  through the host's page tables); 0: through device staging copies */
  int mesh_slot_capacity;      /* history slots per atom of the widest mesh (grows on demand, as the
                                  reference's FixContactHistoryMesh pages do) */
  int ens_inplace_builds;      /* ensembles: builds that rebuilt only the rebuilding systems' atoms and
                                  list segments, every other system left in place */
  int ens_relayout_builds;     /* ensembles: builds in place for the atoms whose list was laid out anew
                                  (a rebuilding system outgrew its segment) */
} dem_stats;

typedef struct dem_handle dem_handle;

int dem_create(const dem_config *cfg, dem_handle **out);
int dem_destroy(dem_handle *h);

/* Matrices are (ntypes+1)^2, row-major, types start at 1 (row/col 0 unused),
 * the layout of the reference's MatrixProperty.  coeffRollFrict may be NULL
 * without rolling friction; coeffRestLog/charVel are read by the Hooke law. */
int dem_set_pair_params(dem_handle *h, int ntypes, const double *Yeff, const double *Geff,
                        const double *betaeff, const double *coeffFrict,
                        const double *coeffRollFrict, const double *coeffRestLog,
                        double charVel);

/* Helper: the reference's derivations of Yeff, Geff, betaeff, coeffRestLog from
 * youngsModulus/poissonsRatio (per type) and coefficientRestitution (per type
 * pair), src/global_properties.cpp:428-561.  Host-only arithmetic. */
int dem_derive_hertz_tables(int ntypes, const double *youngs, const double *poisson,
                            const double *restitution, double *Yeff, double *Geff,
                            double *betaeff, double *coeffRestLog);

/* cohesion bond/nonlinear (pair_style gran ... cohesion bond/nonlinear;
 * CohesionModel<COHESION_BOND_NONLINEAR>::connectToProperties,
 * src/cohesion_model_bond_nonlinear.h:246-381).  tables stacks the 23
 * per-type-pair property/global matrices, each (ntypes+1)^2 as in
 * dem_set_pair_params, in this order: */
enum {
  DEM_BOND_RADIUS_MULTIPLIER = 0, /* radiusMultiplierBondnonlinear */
  DEM_BOND_K_FN1, DEM_BOND_KU_FN1, DEM_BOND_KC_FN1, /* stiffnessPerUnitAreaK/Ku/Kc_fn1 (compression) */
  DEM_BOND_K_FN2, DEM_BOND_KU_FN2, DEM_BOND_KC_FN2, /* stiffnessPerUnitAreaK/Ku/Kc_fn2 (tension) */
  DEM_BOND_K_FT,                                    /* stiffnessPerUnitAreaK_ft */
  DEM_BOND_K_TN, DEM_BOND_KU_TN, DEM_BOND_KC_TN,    /* stiffnessPerUnitAreaK/Ku/Kc_tn (twisting) */
  DEM_BOND_K_TT, DEM_BOND_KU_TT, DEM_BOND_KC_TT,    /* stiffnessPerUnitAreaK/Ku/Kc_tt (bending) */
  DEM_BOND_DAMP_FN, DEM_BOND_DAMP_FT, DEM_BOND_DAMP_TN, DEM_BOND_DAMP_TT, /* damping*Bondnonlinear */
  DEM_BOND_MAX_DIST,                                /* maxDistanceBondnonlinear */
  DEM_BOND_MAX_SIGMA, DEM_BOND_MAX_TAU,             /* maxSigma/maxTauBondnonlinear */
  DEM_BOND_RATIO_TC,                                /* ratioTensionCompressionBondnonlinear */
  DEM_BOND_CREATE_DIST,                             /* createDistanceBondnonlinear */
  DEM_BOND_NTABLES
};
/* The model's on/off settings (registerSettings, :231-243; defaults: all
 * *Stress and dampingBond on, the others off) and the scalar
 * tsCreateBondnonlinear. */
typedef struct dem_bond_settings {
  double tsCreate;
  int stressBreak, tensionStress, compressionStress, shearStress, normalTorqueStress,
      shearTorqueStress, createBondAlways, dampingBond, dampingBondSmooth, ratioTCBond;
} dem_bond_settings;
/* After dem_set_pair_params and before dem_upload_atoms, with
 * cfg.cohesion_model = DEM_COHESION_BOND_NONLINEAR.  Pairs then carry dnum = 31
 * history values in the reference's order (28 bond values, then shear[3]);
 * the contact distance factor grows as the model registers it.  Wall
 * contacts use their own model without cohesion (fix wall/gran model hertz
 * tangential history ...). */
int dem_set_bond_params(dem_handle *h, const double *tables, const dem_bond_settings *st);

/* axis 0/1/2 = xplane/yplane/zplane, rolling_model = DEM_ROLLING_* for this wall.
 * Returns the wall id through *wall_id (may be NULL). */
int dem_add_plane(dem_handle *h, int axis, double pos, int wall_type, int rolling_model,
                  int *wall_id);

/* fix wall/gran ... primitive type T xcylinder|ycylinder|zcylinder R C1 C2
 * (FixWallGran with PrimitiveWall Cylinder<dim>, src/primitive_wall_definitions.h:
 * 69-71,155-200): a cylinder of radius R about the axis 0/1/2 through the point
 * whose coordinates along (axis+1)%3 and (axis+2)%3 are C1, C2.  Contact from
 * inside and from outside, the reference's neighbour rule and history.  Walls
 * share one id sequence (planes and cylinders in the order they are added,
 * then meshes).  Returns the wall id through *wall_id (may be NULL). */
int dem_add_cylinder(dem_handle *h, int axis, double radius, double center1, double center2, int wall_type,
                     int rolling_model, int *wall_id);

/* A primitive plane whose position depends on the atom's type (pos_by_type,
 * ntypes+1 entries, entry 0 unused) and whose wall type is the atom's own
 * type: the floors of independent systems stacked into one handle (the
 * batched ensemble), each system with its own atom type and material.  No
 * reference counterpart (the reference runs one process per system). */
int dem_add_plane_per_type(dem_handle *h, int axis, const double *pos_by_type, int rolling_model,
                           int *wall_id);

/* Batched ensemble: the handle holds nsys independent systems that share the
 * box (boundaries, size) and the model; system k is made of the atoms of
 * type k+1 (each system one material, the type-pair tables' diagonal), its
 * walls are per-type planes (dem_add_plane_per_type).  Every system keeps
 * its own coordinates; its neighbour cells form their own block, so no pair
 * crosses systems.  All systems advance together in one step loop; each
 * system takes its own neighbour decision (Neighbor::decide with the
 * every/delay/check settings, src/neighbor.cpp:1362-1378), as it would
 * running alone: a system that does not rebuild keeps its atom order, list
 * and histories while others rebuild.  The list is laid out in one segment
 * per system with unused entries at its end, so that a build touches only
 * the rebuilding systems (dem_stats.ens_inplace_builds); dem_npairs and
 * dem_download_contacts leave the unused entries out.  After
 * dem_set_pair_params (ntypes == nsys), before dem_upload_atoms; no meshes,
 * no insertion. */
int dem_set_ensemble(dem_handle *h, int nsys);
/* Neighbour list builds of each ensemble system (Neighbor::ncalls of that
 * system run alone, including the setup build): counts[nsys]. */
int dem_ensemble_rebuilds(dem_handle *h, int *counts);

/* Launch shape and neighbour-cell size, set before dem_upload_atoms:
 * grid-stride kernels use at most blocks_per_sm blocks per SM (default 8);
 * cell edges are cell_scale x the neighbour cutoff (default 1, range 1..4).
 * Neither changes the pair set; the cell size changes the order in which a
 * list is built, hence summation order (rounding only).  Used by the
 * ensemble autotuner. */
int dem_set_tuning(dem_handle *h, int blocks_per_sm, double cell_scale);
/* Threads per block of the per-particle kernel (force gather, gravity,
 * primitive walls, nve/sphere; one particle per thread): 64, 128 or 256
 * (default).  Results do not depend on it.  Used by the ensemble autotuner. */
int dem_set_particle_threads(dem_handle *h, int threads);

/* fix mesh/surface FILE type WALL_TYPE + fix wall/gran ... mesh n_meshes 1
 * meshes ID (src/fix_mesh_surface.cpp, src/fix_wall_gran.cpp:803-982):
 * nodes is ntri*9 (triangle t, node q, coordinate d at 9*t+3*q+d) in element
 * order, element id = index.  edge_active/corner_active (ntri*3, may be NULL)
 * are the mesh topology flags the reference's SurfaceMesh::buildNeighbours
 * produces; NULL derives them the same way (see dem_mesh_topology).
 * Returns the mesh id through *mesh_id (may be NULL).  Add before atoms. */
int dem_add_mesh(dem_handle *h, int ntri, const double *nodes, int wall_type, int rolling_model,
                 const unsigned char *edge_active, const unsigned char *corner_active,
                 int *mesh_id);

/* fix move/mesh mesh ID linear vx vy vz (FixMoveMesh + MeshMoverLinear,
 * src/fix_move_mesh.cpp:194-240, src/mesh_mover_linear.cpp:95-112): every
 * step the mesh moves by dt*vel after the particles' drift; node velocities
 * are vel (0 in the dem_setup force pass); a node that travelled more than
 * skin/2 since the last neighbour build forces a build at the next step
 * (FixMesh::pre_force, MultiNodeMesh::decideRebuild).  Before dem_upload_atoms. */
int dem_set_mesh_motion(dem_handle *h, int mesh_id, const double *vel);
/* fix move/mesh mesh ID rotate origin O axis A period T (MeshMoverRotate,
 * src/mesh_mover_rotation.cpp:66-131): every step after the particles' drift
 * the mesh turns by 2 pi dt / T about the axis through O (nodes, centres and
 * the element vectors, in the reference's quaternion arithmetic, so nodes
 * match bit for bit); node velocities are w x (node - O) (0 in the dem_setup
 * force pass); node travel beyond skin/2 forces a rebuild as with linear
 * motion.  One mover per mesh; before dem_upload_atoms. */
int dem_set_mesh_rotation(dem_handle *h, int mesh_id, const double *origin, const double *axis, double period);
/* Current node positions of a mesh, ntri*9 in element order. */
int dem_download_mesh_nodes(dem_handle *h, int mesh_id, double *nodes);

/* Host-only: edge/corner activity of a triangle mesh as SurfaceMesh::buildNeighbours
 * computes it (src/surface_mesh_I.h:473-1236), ntri*3 flags each. */
int dem_mesh_topology(int ntri, const double *nodes, unsigned char *edge_active,
                      unsigned char *corner_active);

/* Mesh contact history as FixContactHistoryMesh keeps it: one entry per
 * occupied slot (atom tag, triangle id, slot index, 3 history doubles). */
int dem_mesh_ncontacts(dem_handle *h, int mesh_id, int *ncontacts);
int dem_download_mesh_contacts(dem_handle *h, int mesh_id, int *tag, int *tri, int *slot,
                               double *hist);

/* x, v, omega are n*3 (x[3*i+d] == atom->x[i][d]). Resets contact history. */
int dem_upload_atoms(dem_handle *h, int n, const int *tag, const int *type, const double *x,
                     const double *v, const double *omega, const double *radius,
                     const double *rmass);

/* Insertion (fix insert/pack, insert/stream, insert/rate/region: the
 * reference's FixInsert::pre_exchange, src/fix_insert.cpp).  Before
 * dem_upload_atoms, dem_set_capacity reserves room for natoms_max atoms and
 * declares the radius range [rmin, rmax] inserted atoms may take (0: the
 * uploaded atoms' range); the neighbour cutoff is sized for it, as
 * PairGran::init_one sizes it for the insertion templates.  Between
 * dem_step calls, dem_insert_atoms stages k new atoms (host arrays as in
 * dem_upload_atoms); they join at the next step after its initial
 * integration, and that step rebuilds the neighbour list, which is when and
 * how FixInsert adds atoms in the reference (pre_exchange of the insertion
 * step, next_reneighbor = that step).  DEM_ERR_CAPACITY when the capacity
 * would be exceeded.  Not with an ensemble. */
int dem_set_capacity(dem_handle *h, int natoms_max, double rmin, double rmax);
int dem_insert_atoms(dem_handle *h, int k, const int *tag, const int *type, const double *x, const double *v,
                     const double *omega, const double *radius, const double *rmass);

/* Restart data, valid between dem_upload_atoms and dem_setup (atoms indexed in
 * upload order).  Contact history as the reference keeps it per atom
 * (FixContactHistory npartner/partner/contacthistory, restored by
 * FixContactHistory::unpack_restart, src/fix_contact_history.cpp:554-659):
 * one entry per (owner atom, partner atom) with the owner's dnum history
 * doubles; a contact between two atoms has one entry per side.  The next
 * neighbour build carries an entry over when the pair touches at that time,
 * exactly as after read_restart.  Wall history: 3 doubles per atom, the
 * fix property/atom history_<wallid> restart data. */
int dem_upload_contact_history(dem_handle *h, int nentries, const int *tag_owner,
                               const int *tag_partner, const double *hist);
int dem_upload_wall_history(dem_handle *h, int wall_id, const double *hist);

int dem_setup(dem_handle *h);
int dem_step(dem_handle *h, int nsteps);

/* Atoms come back in the device's current (cell-sorted) order with their tags.
 * Any array pointer may be NULL: that array is not written.  Page-locked
 * arrays transfer at a steady rate; pageable ones through the host page
 * tables, at a rate that depends on the pages' history. */
int dem_natoms(dem_handle *h, int *n);
int dem_download_atoms(dem_handle *h, int *tag, int *type, double *x, double *v, double *omega,
                       double *f, double *torque, double *radius, double *rmass);

/* Granular half list: owner tag, partner tag, periodic image of the partner
 * (shift[3*p+d] in {-1,0,1}), contact flags (reference bit layout) and the
 * dnum history doubles per pair (dnum = 3: shear x,y,z). */
int dem_npairs(dem_handle *h, int *npairs, int *dnum);
int dem_download_contacts(dem_handle *h, int *tag_i, int *tag_j, int *shift, int *flag,
                          double *hist);
/* 3 doubles per atom in dem_download_atoms order. */
int dem_download_wall_history(dem_handle *h, int wall_id, double *hist);

int dem_get_stats(dem_handle *h, dem_stats *out);

/* Per-kernel device timing with CUDA events on the handle's stream (the
 * reference's Timer buckets, src/timer.h:51-52).  Enabling resets counters.
 * kernel_launches counts every kernel the library launched since the reset. */
typedef struct dem_kernel_times {
  double pair_ms;              /* pair force kernel (PairGran::compute) */
  long long pair_launches;
  double particle_ms;          /* gather + walls + gravity + nve/sphere kernel */
  long long particle_launches;
  double neigh_ms;             /* decide + rebuild stage (Neighbor::decide/build) */
  long long neigh_stages;
  long long kernel_launches;
  double wall_ms;              /* wall kernel: primitive planes and meshes (FixWallGran::post_force) */
  long long wall_launches;
} dem_kernel_times;
/* On-device diagnostics of the current state, without downloading the atoms
 * (long-run acceptance metrics; the reference's ComputeKE and
 * ComputeERotateSphere, src/compute_ke.cpp, src/compute_erotate_sphere.cpp,
 * and the total force of each wall as fix mesh/surface/stress and
 * wall/gran store_force report it).  After dem_setup or dem_step:
 *   ke_translational = 1/2 sum m v^2, ke_rotational = 1/2 sum 0.4 m r^2 w^2;
 *   ncontacts = list entries with a contact force in the last force pass;
 *   solid_volume = sum 4/3 pi r^3 over the atoms whose centre lies in the
 *   region [lo, hi) (NULL: the box), packing_fraction = solid_volume over
 *   the region's volume;
 *   wall_force[w] = total force of wall w on the atoms in the last force
 *   pass, walls numbered in the order they were added, planes first, then
 *   meshes (nwalls of them, at most DEM_DIAG_MAX_WALLS).
 * Sums are deterministic (fixed block order). */
#define DEM_DIAG_MAX_WALLS 16
typedef struct dem_diagnostics {
  double ke_translational, ke_rotational;
  long long ncontacts;
  double solid_volume, packing_fraction;
  int nwalls;
  double wall_force[DEM_DIAG_MAX_WALLS][3];
} dem_diagnostics;
int dem_get_diagnostics(dem_handle *h, const double *region_lo, const double *region_hi, dem_diagnostics *out);

int dem_profile(dem_handle *h, int enable);
int dem_get_kernel_times(dem_handle *h, dem_kernel_times *out);

/* No counterpart in the reference.  Contact forces and torques of one setup
 * force pass (history read, not updated) for a caller-supplied neighbour list,
 * allocating nothing on the device: for callers that cannot call cudaMalloc
 * while they run (GPU memory owned by another allocator or pool, loops that
 * must not allocate after start-up).  All array arguments except the material
 * tables are DEVICE pointers owned by the caller: x, v, omega n*3; radius,
 * rmass, type n; pair_i, pair_j npairs (pair_i non-decreasing, as
 * dem_download_contacts returns the list); shift, hist npairs*3; f, torque
 * n*3 (written).  The material tables are host arrays as in
 * dem_set_pair_params; cfg supplies the box, model and option switches.
 * stream is a cudaStream_t (NULL: legacy default stream); the call
 * synchronises it before returning.
 * Scratch lives in one fixed static device array (about 11 MB per GPU that
 * loads the library, kept until exit); limits: n <= 32768 atoms,
 * npairs <= 131072, ntypes <= 15, else DEM_ERR_BAD_ARG; so is an entry of an
 * atom with itself without an image shift.  CUDA loads a module's static
 * arrays lazily by default (CUDA_MODULE_LOADING=LAZY): the first call on a
 * device is when the ~11 MB is taken, so a caller that must not allocate
 * mid-run makes one call at start-up (npairs = 0 suffices) or sets
 * CUDA_MODULE_LOADING=EAGER; that first call should also come before any
 * stream capture on the device.  Calls share the array: calls that overlap
 * on the GPU race and must be serialised by the caller. */
int dem_contact_forces_noalloc(int n, const double *x, const double *v, const double *omega,
                               const double *radius, const double *rmass, const int *type,
                               int npairs, const int *pair_i, const int *pair_j, const int *shift,
                               const double *hist, const dem_config *cfg, int ntypes,
                               const double *Yeff, const double *Geff, const double *betaeff,
                               const double *coeffFrict, const double *coeffRollFrict,
                               const double *coeffRestLog, double charVel, double *f,
                               double *torque, void *stream);

/* Diagnostic without a reference counterpart: FP64 FMA throughput of the
 * current device in TFLOP/s (dependent-chain-free DFMA loop), used as the
 * FP64 roofline denominator. */
int dem_measure_fp64_peak(double *tflops);
const char *dem_last_error(dem_handle *h);
const char *dem_version(void);

/* ------------------------------------------------------------------------
 * Discrete adjoint (no counterpart in the reference, which has no
 * derivatives).  Gradients of a scalar loss of the final state of an
 * N-step run with respect to Young's modulus, restitution, friction and
 * every particle radius, by reverse-mode differentiation of the exact
 * discrete timestep: Verlet::setup + N Verlet steps (src/verlet.cpp:281-389)
 * of FixNVESphere, PairGran Hertz + tangential history (CDT rolling friction
 * when dem_adjoint_set_rolling is called; cohesion bond/nonlinear when
 * dem_adjoint_set_bonds is called, else contact
 * distance factor 1), FixGravity and FixWallGran primitive planes and static
 * triangle meshes (dem_adjoint_add_mesh), one atom type
 * and one material (Yeff/Geff/betaeff of the material against itself,
 * src/global_properties.cpp).  Masses follow the radii: m = 4/3 pi r^3 rho.
 * The neighbour list is rebuilt every `segment` steps, after the drift of
 * steps segment, 2*segment, ... (neigh_modify every segment delay 0 check
 * no); each rebuild is a checkpoint, so memory grows as N/segment states
 * plus one segment of tape (segment ~ sqrt(N) minimises it).  Within a
 * segment no atom may move more than skin/2 from its position at the build
 * (DEM_ERR_BAD_ARG otherwise, with a message).  The loss:
 *   w_ke * (translational + rotational kinetic energy)
 * + w_height * (mean z - height_target)^2
 * + w_wallforce * (force of wall wall_id on the atoms, summed over atoms at
 *                  the last step - wallforce_target)^2: a plane's normal
 *                  component, a mesh's component wall_axis
 * Gradients are exact for this piecewise-smooth map away from switch
 * points (contacts opening or closing, stick/slip transitions).
 * ------------------------------------------------------------------------ */
typedef struct dem_adjoint_config {
  double boxlo[3], boxhi[3];
  int periodic[3];
  double dt, skin;
  double density;       /* FixDensity / set density: rmass = 4/3 pi r^3 rho */
  double poisson;       /* property/global poissonsRatio */
  int gravity_on;
  double gravity[3];    /* acceleration vector (fix gravity magnitude * direction) */
  int nplanes;          /* <= 8 primitive planes (wall/gran ... primitive type 1 [xyz]plane) */
  int plane_axis[8];
  double plane_pos[8];
} dem_adjoint_config;

typedef struct dem_adjoint_loss {
  double w_ke;
  double w_height, height_target;
  double w_wallforce, wallforce_target;
  int wall_id;          /* wall of the wall-force term, -1 none: planes 0..nplanes-1
                         * (their normal component), then meshes nplanes.. */
  int wall_axis;        /* for a mesh: the component (0/1/2) of its total force */
} dem_adjoint_loss;

typedef struct dem_adjoint dem_adjoint;
int dem_adjoint_create(const dem_adjoint_config *cfg, dem_adjoint **out);
int dem_adjoint_destroy(dem_adjoint *h);
/* cohesion bond/nonlinear in the forward model (pair_style gran ... cohesion
 * bond/nonlinear; CohesionModel<COHESION_BOND_NONLINEAR>, src/
 * cohesion_model_bond_nonlinear.h:394-992): values holds the 23 properties of
 * the one type pair in DEM_BOND_* order, st the model's settings (as in
 * dem_set_bond_params); bonds are created at step tsCreate of the run (the
 * setup pass is step 0) or always.  Call before dem_adjoint_set_state, which
 * derives the contact distance factor from the smallest radius.  The
 * gradients then include the bonds' forces, created, evolved and carried
 * across rebuilds as the main path does. */
int dem_adjoint_set_bonds(dem_adjoint *h, const double *values, const dem_bond_settings *st);
/* a static triangle-mesh wall (fix mesh/surface + fix wall/gran ... mesh) of
 * the atoms' material, nodes[ntri][3][3] as dem_add_mesh; edge/corner
 * activity NULL = derived from the topology.  At most 4, before
 * dem_adjoint_set_state.  Contacts follow the reference's sphere-triangle
 * resolution and FixContactHistoryMesh's history slots
 * (src/tri_mesh_I.h:65-271, src/fix_contact_history_mesh_I.h:51-216); the
 * gradients include them. */
int dem_adjoint_add_mesh(dem_adjoint *h, int ntri, const double *nodes, const unsigned char *edge_active,
                         const unsigned char *corner_active);
/* fix move/mesh ... linear vx vy vz for mesh mesh_id of the adjoint: the
 * nodes translate by dt*vel per step and contacts see the wall velocity
 * (MeshMoverLinear, src/mesh_mover_linear.cpp:95-112); before
 * dem_adjoint_set_state.  The mesh may not move more than skin/2 between two
 * list builds (the reference would then force a rebuild). */
int dem_adjoint_set_mesh_motion(dem_adjoint *h, int mesh_id, const double *vel);
/* CDT rolling friction (rolling_friction cdt, RollingModel<ROLLING_CDT>,
 * src/rolling_model_cdt.h:89-167) with coefficientRollingFriction mur on
 * pairs and on every wall; before dem_adjoint_set_state. */
int dem_adjoint_set_rolling(dem_adjoint *h, double mur);
/* d(loss)/d(coefficientRollingFriction) of the last dem_adjoint_gradient
 * call (0 without rolling friction) */
int dem_adjoint_rolling_gradient(dem_adjoint *h, double *grad_mur);
/* initial state (host arrays): x, v, omega n*3, radius n (the radii define the
 * neighbour cells; runs may use radii up to 1 % larger) */
int dem_adjoint_set_state(dem_adjoint *h, int n, const double *x, const double *v, const double *omega,
                          const double *radius);
/* forward only: loss of the final state; radius NULL = the initial radii */
int dem_adjoint_forward(dem_adjoint *h, double E, double restitution, double friction, const double *radius,
                        int nsteps, int segment, const dem_adjoint_loss *loss, double *loss_out);
/* forward + backward: loss and its gradients (grad_radius n entries) */
int dem_adjoint_gradient(dem_adjoint *h, double E, double restitution, double friction, const double *radius,
                         int nsteps, int segment, const dem_adjoint_loss *loss, double *loss_out,
                         double *grad_E, double *grad_restitution, double *grad_friction, double *grad_radius);
/* final state of the last run (host arrays, n*3 each, NULL to skip) */
int dem_adjoint_download(dem_adjoint *h, double *x, double *v, double *omega);
/* device time of the last run's forward and backward passes, its segment
 * count and largest list */
int dem_adjoint_times(dem_adjoint *h, double *forward_ms, double *backward_ms, int *segments, int *max_pairs);
/* where the backward pass takes each step's record (positions, half-step
 * velocities, history and forces the step's force evaluation saw):
 *   mode 0: replayed from the segment's checkpoint (memory: one checkpoint
 *           per segment plus one segment of record, O(sqrt(N)) states);
 *   mode 1: recorded during the forward pass, no replay (memory: every step);
 *   mode 2 (default): mode 1 when the whole record fits max_bytes (0: half of
 *           the device memory free at the run's start), else mode 0.
 * Both give the same gradients bit for bit; mode 1 saves the replay, about
 * one forward pass of time. */
int dem_adjoint_set_tape(dem_adjoint *h, int mode, double max_bytes);
/* whether the last run recorded its steps in the forward pass (1) or replayed
 * them (0) */
int dem_adjoint_tape_recorded(dem_adjoint *h, int *recorded);
const char *dem_adjoint_last_error(dem_adjoint *h);

#ifdef __cplusplus
}
#endif
#endif
