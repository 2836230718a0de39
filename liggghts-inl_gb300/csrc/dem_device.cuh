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

namespace gb300 {

constexpr int kMaxPlanes = 8;
constexpr int kDnumShear = 3;
constexpr int kContactNormal = 1 << 0;      // CONTACT_NORMAL_MODEL
constexpr int kContactTangential = 1 << 2;  // CONTACT_TANGENTIAL_MODEL
constexpr int kNoShift = 13;                // shift code of (0,0,0)

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
  double *whist;            // [(w*3+d)*nmax + i]
  uint8_t *wbits;           // bit w: atom in primitive wall w's neighbour list
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
};

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
};

struct Plane {
  int axis;
  double pos;
  int wall_type;
  int rolling;
};

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
  double *resF, *resTi, *resTj;  // [3*pcap]
  uint8_t *active;  // [pcap]
  int *scan_tmp;
  // parameters
  double *params;   // 6 matrices of (nt+1)^2: Y, G, beta, mu, mur, restlog
  int ntypes;
  int nmax, pcap;
  int ncell, nc[3];
  double csz[3];
  double boxlo[3], boxhi[3], prd[3];
  int periodic[3];
  double dt, skin, cdf, cutneighmax;
  int neigh_every, neigh_delay, neigh_check;
  int normal, rolling, tdamp, limitf;
  int gravity_on;
  double g[3];
  double charVel;
  int nplanes;
  Plane planes[kMaxPlanes];
};

}  // namespace gb300
