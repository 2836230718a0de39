// Device-side data layout of one granular system (shared by host and kernels).
//
// HBM layout (all SoA, FP64 unless noted; nmax = atom capacity, pcap = pair
// capacity):
//   atoms[2]   per-atom arrays; a rebuild gathers the cell-sorted order into
//              atoms[1] and copies it back into atoms[0].
//   pairs[2]   granular half list (CSR by owner) with contact flags, history
//              hist[d*pcap + p] and per-pair constants (reff and the two
//              contact constants of contact_consts()); pairs[1] is where a
//              rebuild builds the new list while the history remap still
//              reads the old one in pairs[0].
//   scratch    cell counts/starts, sort permutation, per-pair force results.
//   ctrl       device control block: atom/pair counts, rebuild decision,
//              halt/status words.  Kernels read it, so no host round trip is
//              needed to decide a rebuild.
#pragma once
#include <stdint.h>
#include <vector_types.h>

namespace gb300 {

constexpr int kMaxPlanes = 8;
constexpr int kDnumShear = 3;
constexpr int kContactNormal = 1 << 0;      // CONTACT_NORMAL_MODEL
constexpr int kContactCohesion = 1 << 1;    // CONTACT_COHESION_MODEL
constexpr int kContactTangential = 1 << 2;  // CONTACT_TANGENTIAL_MODEL
constexpr int kNoShift = 13;                // shift code of (0,0,0)

// cohesion bond/nonlinear.  A pair then carries kDnumBond history values; on
// the device the shear comes first (d = 0..2) and the bond's 28 values follow
// (d = 3 + b, b in the reference's order: bondFlag, initial_dist,
// contactPos[3], ft[3], thetan[3], thetat[3], deltan_max, thetan_max[3],
// thetat_max[3], thetan_min[3], thetat_min[3], deltan_min).  The C ABI uses
// the reference's order (bond values first).
constexpr int kBondValues = 28;
constexpr int kDnumBond = kDnumShear + kBondValues;
constexpr int kBondTables = 23;  // per-type-pair tables, DEM_BOND_* order
// Sys::bondp also holds, after those, per-type-pair ratios of the hysteresis
// laws that the model forms from the stiffnesses on every evaluation
// (computed on the host once; IEEE division gives the same bits):
// (Ku-K)/(Ku+Kc) of twisting, of bending, of compression, of tension
constexpr int kBondDerived = 4;
enum { kBondRatioTn = kBondTables, kBondRatioTt, kBondRatioFn1, kBondRatioFn2 };
enum {
  kBondLambda = 0, kBondKfn1, kBondKufn1, kBondKcfn1, kBondKfn2, kBondKufn2, kBondKcfn2, kBondKft,
  kBondKtn, kBondKutn, kBondKctn, kBondKtt, kBondKutt, kBondKctt, kBondDampFn, kBondDampFt,
  kBondDampTn, kBondDampTt, kBondMaxDist, kBondMaxSigma, kBondMaxTau, kBondRatioTC, kBondCreateDist
};
// Sys::bond_flags bits (the model's on/off settings)
enum {
  kBondStressBreak = 1 << 0, kBondTension = 1 << 1, kBondCompression = 1 << 2, kBondShear = 1 << 3,
  kBondNormalTorque = 1 << 4, kBondShearTorque = 1 << 5, kBondCreateAlways = 1 << 6,
  kBondDamping = 1 << 7, kBondDampingSmooth = 1 << 8, kBondUseRatioTC = 1 << 9
};
// The shear history is kept in the list's own orientation (owner = lower
// cell-sorted index; it changes sign when that orientation flips).  The bond
// values are kept in the reference's orientation, owner = lower lidx (the
// reference's local index order), because its twisting/bending extremes and
// smooth damping are not symmetric under a flip; the bond law is evaluated
// in that orientation.

// status words in Ctrl::status
constexpr int kStatOk = 0;
constexpr int kStatPairOverflow = 3;
constexpr int kStatNan = 4;

struct AtomArrays {
  double *x, *y, *z;
  double *vx, *vy, *vz;
  double *wx, *wy, *wz;
  double *fx, *fy, *fz;
  double *tx, *ty, *tz;
  double *r, *m, *dtfm, *dtir;
  double *xh, *yh, *zh;     // xhold
  int *type, *tag;
  int *lidx;                // the atom's index in the caller's (reference's) local order
  double *whist;            // [(w*3+d)*nmax + i]
  uint8_t *wbits;           // bit w: atom in primitive wall w's neighbour list;
                            // bit 7: atom has candidate mesh triangles
  double *fmx, *fmy, *fmz, *tmx, *tmy, *tmz;  // mesh wall force/torque of the step (bit 7 atoms)
};

struct PairArrays {
  int *i, *j;
  uint8_t *sh;              // periodic image code of j, 13 = none
  int *flag;                // contact flags (reference bits)
  double *hist;             // [d*pcap + p]
  double *reff;             // ri*rj/(ri+rj)
  double *c0, *c1;          // contact constants, see contact_consts()
  int *row;                 // [nmax+1] CSR offsets by owner
  int *rev_start;           // [nmax+1] offsets of pairs where the atom is partner
  int *rev;                 // pair ids, ascending per partner
  // ensembles: per-atom ends of the owner row and of the partner list
  // [nmax+1] (each system's entries lie in its own segment, followed by
  // unused entries, so row[i+1] is not the end of a system's last atom)
  int *rowe, *reve;
};

// shift code of an unused list entry inside an ensemble system's segment
// (i = j = -1, flag 0; the pair kernels skip it, no row covers it)
constexpr int kHole = 255;

struct Ctrl {
  int n;            // atoms
  int np;           // pairs in the current list
  int cur_a, cur_p;
  int rebuild;      // decision for the current step
  int moved;        // skin check tripped (any atom moved > skin/2)
  int ago;
  int halt;         // nonzero: all kernels are no-ops until the host resumes
  int status;
  int n_new, np_new, nrev_new;
  int lost_step;    // atoms lost at the last rebuild
  long long lost;
  long long ntimestep, nrebuilds;
  int halt_step;
  int loop_left;    // steps left for the device-side step loop (graph WHILE node)
  int mesh_moved;   // a moving mesh node travelled > skin/2 since the last build
  int force_rebuild;  // rebuild at the next decide (FixMesh next_reneighbor)
  int nmlist;         // atoms with candidate mesh triangles (Sys::mlist)
  int mesh_need;      // most candidate triangles an atom had beyond its mesh's capacity
  // ensemble rebuilds (see k_ens_plan): pmode 1 rebuilds only the rebuilding
  // systems' atoms in place; lmode 1 also keeps every other system's list
  // segment where it is; nR systems rebuild, with nra atoms and ncr entries
  // of segment capacity between them
  int pmode, lmode, nR, nra, ncr;
  int seg_ok;         // the list is laid out in per-system segments
  int np_live;        // entries in use (ensembles: np less the unused entries)
  int ens_inplace;    // ensemble builds in place (atoms and list)
  int ens_relayout;   // ensemble builds in place for the atoms, list re-laid
  int pdone;          // blocks of k_particle done (the last one decides; graph steps)
};

// Primitive wall of fix wall/gran (src/primitive_wall_definitions.h): a
// plane normal to `axis` at pos, or a cylinder about `axis` of radius pos
// through (c1, c2) in the coordinates (axis+1)%3, (axis+2)%3.
struct Plane {
  int axis;
  double pos;
  int kind;           // 0: plane, 1: cylinder
  double c1, c2;
  int wall_type;      // 0: the wall takes each atom's own type (per-type planes)
  int rolling;
  const double *pos_t;  // per-atom-type position [ntypes+1] (stacked ensembles) or nullptr
};

__device__ __forceinline__ double plane_pos(const Plane &pl, int type) {
  return pl.pos_t ? pl.pos_t[type] : pl.pos;
}

// Triangle-mesh wall (fix mesh/surface + fix wall/gran mesh).
constexpr int kMaxMeshes = 4;
// Candidate triangles (= history slots) per atom and mesh: the main path
// starts at kMeshCandInit and doubles MeshDev::ccap when an atom has more
// (k_mesh_cand halts the rebuild, the host grows the slot arrays and resumes
// it), as FixContactHistoryMesh grows its per-atom pages without a bound;
// the adjoint keeps the fixed kMeshMaxCand.
constexpr int kMeshCandInit = 24;
constexpr int kMeshMaxCand = 24;
constexpr int kMeshFastCand = 32;  // k_wall_force's tiled path (32-bit masks); more take the sequential path
constexpr int kSlotKept = 1 << 30; // mesh_contacts: marks a slot touched in this evaluation
constexpr int kTriStride = 40;     // doubles of geometry per triangle, see below
constexpr int kStatMeshSlots = 5;  // Ctrl::status: a mesh contact found no free slot (inconsistent slots)
constexpr int kStatMeshReg = 6;    // Ctrl::status: triangle-cell registrations overflowed (halted, grown, resumed)
constexpr int kStatMeshCand = 7;   // Ctrl::status: an atom has more candidate triangles than ccap (halted, grown,
                                   // resumed)
// geometry layout per triangle: node[9] | edgeVec[9] | edgeNorm[9] |
// edgeLen[3] | surfaceNorm[3] | center[3] | rBound | pad[3]
// meta per triangle: bits 0-1 obtuse node+1 (0 none), bits 2-4 edge active,
// bits 5-7 corner active
struct MeshDev {
  int ntri, wall_type, rolling, moving;
  double distmax, tskin;  // FixNeighlistMesh: bounding-box growth and neighbuild threshold
  double *tri;        // [t*kTriStride]
  float4 *trif;       // [2t]: node 0, [2t+1]: unit normal, FP32 copies (plane-distance prefilter)
  int *meta;          // [t]
  // fix move/mesh ... linear: every step nodes and centres move by dx =
  // dt*vel; node velocities are vel (0 during the setup force pass)
  double vel[3], dx[3];
  int vel_on;
  // fix move/mesh ... rotate origin O axis A period T: per-step quaternion
  // (MultiNodeMesh::rotate), origin, angular velocity vector, node
  // velocities w x (node - O) [t*9]
  int rotating;
  double rq[4], rorig[3], romega[3];
  double *nodev;
  double *node_last;  // node positions at the last neighbour build [t*9]
  int *cn_start, *cn_list;          // coplanar node-neighbours (areCoplanarNodeNeighs)
  int *tc_count, *tc_start, *tc_fill, *tc_list;  // triangles registered per atom cell
  int tc_cap;
  int ccap;                         // candidate triangles (= history slots) per atom
  int *cand_n, *cand;               // per atom: count, [c*nmax + a] ascending
  int *nslot[2], *npart[2];         // per atom (buffer 0 live, 1 permute scratch)
  int *slot_tri[2];                 // [s*nmax + a], -1 empty
  double *slot_hist[2];             // [(s*3+d)*nmax + a]
};

constexpr int kResStride = 12;  // doubles per pair-result record
// list entries per atom that the neighbour count pass keeps for the fill
// pass (Sys::stash): partner | image code << 24 (atom indices stay below 2^24)
constexpr int kStash = 16;

struct Sys {
  AtomArrays atoms[2];
  PairArrays pairs[2];
  Ctrl *ctrl;
  // scratch
  int *cell_count, *cell_start, *cell_fill;  // [ncell+2]
  int *perm;        // new -> old
  int *order;       // slot -> old (before the per-cell sort)
  int *pcount;      // per-atom pair counts [nmax+1]
  int *rev_count, *rev_fill;  // [nmax+1]
  // pair results, one 96-byte record per list entry (three whole 32-byte
  // sectors): F[3], Ti[3], Tj[3], 3 doubles of padding; [kResStride*pcap]
  double *res;
  uint8_t *active;  // [pcap]
  int *scan_tmp;
  float4 *xf;       // FP32 copy (x, y, z, r) of the atoms, refreshed by every drift
  float4 *xhf;      // FP32 copy of x at the last neighbour build (displacement prefilter)
  int *mlist;       // atoms with candidate mesh triangles [nmax]
  int *stash;       // [kStash*nmax]: entries found by the count pass, see kStash
  double *wforce;   // [(w*3+d)*nmax + i]: force of wall w (planes, then meshes) on listed
                    // atom i at the last force evaluation (diagnostics)
  // parameters
  double *params;   // 6 matrices of (nt+1)^2: Y, G, beta, mu, mur, restlog
  int ntypes;
  int nmax, pcap;
  int ncell, nc[3];
  // batched ensemble: independent systems, system k = atom type k+1, each
  // with its own block of ens_ncell neighbour cells (0: one system)
  int ens_ncell;
  // per-system neighbour decisions of an ensemble (system k alone runs its
  // own Neighbor::decide): nsys systems, [nsys] each, sys_start [nsys+1]
  int nsys;          // 0: one system
  int *sys_moved;    // an atom of system k moved more than skin/2 (this step)
  int *sys_reb;      // system k rebuilds at this step
  int *sys_ago;      // steps since system k's last build
  int *sys_start;    // first atom of system k (atoms are grouped by system after every build)
  int *sys_nreb;     // builds of system k
  // list segments: system k's entries lie in [seg_start[k], seg_start[k+1]),
  // the first seg_used[k] in use; a rebuild that keeps the other systems in
  // place compacts the rebuilding ones into rlist (rpre/cpre: their prefix
  // sums of atoms and of segment capacity) [nsys+1] each
  int *seg_start, *seg_used, *rlist, *rpre, *cpre;
  int ens_full;      // 1: every ensemble rebuild takes the whole-list path
  int ens_slack;     // unused entries a segment gets, percent of its entries (plus 64; 0: none)
  double csz[3];
  double icsz[3];     // 1/csz: an atom's cell is floor((x - boxlo) * icsz)
  double boxlo[3], boxhi[3], prd[3];
  // FP32 copies for the prefilters (a double-to-float conversion issues on
  // the FP64 pipe, so none is made inside a loop)
  float prdf[3], cdff, skinf;
  int periodic[3];
  double dt, skin, cdf, cutneighmax;
  double ghost_slab;  // cutneighmax/2 + skin/2: CommBrick slab_offset of the ghost band
  float pf_margin;    // relative margin of the FP32 neighbour prefilter (see k_pairs)
  float pf_margin_touch;  // the same for the touching test of k_pair (radsum^2)
  // FP32 prefilter of the displacement test |x - xhold|^2 > skin^2/4: below
  // skin_lo2 no atom can have moved, above skin_hi2 it has; in between the
  // exact FP64 test decides
  float skin_lo2, skin_hi2;
  // cohesion bond/nonlinear (bond = 0: off, dnum = 3)
  int bond, dnum;
  double *bondp;      // kBondTables + kBondDerived matrices of (nt+1)^2
  int bond_flags;
  long long bond_ts_create;  // static_cast<int>(tsCreateBondnonlinear)
  int neigh_every, neigh_delay, neigh_check;
  int normal, rolling, tdamp, limitf;
  int gravity_on;
  double g[3];
  double charVel;
  int nplanes;
  Plane planes[kMaxPlanes];
  int nmeshes;
  MeshDev meshes[kMaxMeshes];
};

}  // namespace gb300
