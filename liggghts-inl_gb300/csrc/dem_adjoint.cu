// Discrete adjoint of the sphere-DEM timestep (Hertz + tangential history,
// cohesion bond/nonlinear, primitive planes, static triangle-mesh walls,
// gravity, nve/sphere) with sqrt(N) checkpointing.
//
// Forward model: the reference's Verlet step (src/verlet.cpp:281-389) with
// FixNVESphere (src/fix_nve_sphere.cpp:120-215), PairGran with the Hertz +
// tangential-history contact model, FixWallGran primitive planes and
// FixGravity:
//   vh = v + a F, wh = w + b T, x' = x + dt vh        initial_integrate
//   [rebuild: pbc wrap, neighbour list, history carried to the new list]
//   F', T', shear' = forces(x', vh, wh, shear)        pair + gravity + walls
//   v' = vh + a F', w' = wh + b T'                    final_integrate
// with a = dt/2/m, b = dt/2/(0.4 r^2 m), m = 4/3 pi r^3 rho; Verlet::setup
// evaluates the forces of the initial state without history update.  The
// neighbour list is rebuilt every L steps, at steps L, 2L, ... after the
// drift (neigh_modify every L delay 0 check no): the same schedule the
// reference runs with those settings.  Atoms keep their input order (no
// spatial sort), so the adjoint state indexes the same atoms over the whole
// horizon.
//
// The steps that share one list form a segment.  The forward pass stores one
// checkpoint per segment: the state before the segment's first drift, the
// segment's neighbour list and its history as carried at the build.  The
// backward pass replays each segment from its checkpoint, recording the
// per-step tape (positions and half-step velocities the forces saw, the
// history before each force evaluation, the forces), then runs the reverse
// kernels over the tape.  Memory: one checkpoint per segment plus one
// segment of tape, O(sqrt(N)) states for L ~ sqrt(N).  The forward pass
// checks that no atom moves more than skin/2 away from its position at the
// build within a segment (the list then holds every touching pair).
//
// History carry-over follows FixContactHistory (src/fix_contact_history.cpp
// pre_exchange/post_neighbor): a new entry (owner i, partner j) takes the
// history of i's old entry with partner j, else (negated) that of j's old
// local entry with partner i, when the pair touches at the build and that
// old entry carries history.  The backward pass maps the history adjoints
// back through the same map.
//
// With cohesion bond/nonlinear (dem_adjoint_set_bonds) each entry also
// carries the bond's 28 history values, created, evolved, broken and carried
// as the main path does (bond_law.cuh, k_pair<..., BOND>): the list cutoff
// and the carry distance grow by the contact distance factor, pairs within
// that distance but not touching clear their tangential history and
// evaluate a bond they hold (or may create), and the bond's force replaces
// the normal model's force of a touching bonded pair.  Bond values with
// newtonflag 1 (ft, thetan, thetat) change sign in a flipped carry, as in
// FixContactHistory::pre_exchange (src/fix_contact_history.cpp:400-410).
// The backward pass carries their adjoints through the same steps
// (adjoint_bond.cuh).
//
// Reverse-mode arithmetic is deterministic: pair results are gathered per
// atom in list order (own row, then reverse list), parameter gradients are
// reduced per block and then summed in block order.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/liggghts_gb300.h"
#include "adjoint_bond.cuh"
#include "adjoint_law.cuh"
#include "dem_device.cuh"
#include "dem_kernels.h"
#include "dem_mesh_host.h"
#include "mesh_device.cuh"

using namespace gb300;

namespace {

// threads per block: small blocks spread a 10^4-atom system over every SM
constexpr int kAB = 128;
constexpr int kMaxGrid = 152 * 16;

// parameter adjoints per entry / atom: Y, G, beta, mu, rolling coefficient
constexpr int kTh = 5;
constexpr int kAMC = kMeshMaxCand;  // candidate triangles (= history slots) per atom and mesh
constexpr int kAMeshes = 4;

// one static triangle-mesh wall on the device (geometry of MeshHost)
struct AMesh {
  int ntri;
  const double *tri;  // [t*kTriStride], node positions at step 0
  const int *meta, *cn_start, *cn_list;
  // fix move/mesh ... linear: the nodes translate by dt*vel per step (step t
  // sees them t*dt*vel away), contacts see the wall velocity vel
  int moving;
  double vel[3];
};

struct AList {
  int np = 0;
  int *pi = nullptr, *pj = nullptr, *row = nullptr, *rev_start = nullptr, *rev = nullptr;
  int *carry = nullptr;     // old entry e (>= 0), -(e + 2) for a flipped copy, -1 none
  uint8_t *sh = nullptr;    // image code of the partner
  uint8_t *flag = nullptr;  // kContact* bits; nonzero: the entry's history is carried
  double *shear = nullptr;  // [3*p+k], evolving
  double *bond = nullptr;   // [kBondValues*p+k], evolving (bonds only)
  // mesh walls: candidates per (mesh, atom) at this build, ascending, and the
  // slot each slot came from at the build (-1: emptied)
  int *mcn = nullptr, *mcand = nullptr, *mmap = nullptr;
};

struct ADev {
  int n;
  double dt, skin, lo[3], hi[3], prd[3];
  int per[3];
  double g[3];
  int gravity_on;
  int nplanes;
  int pax[8];
  double ppos[8];
  double Y, G, beta, mu;
  double mur;   // CDT rolling friction coefficient (rolling: on for pairs and walls)
  int rolling;
  double dtf, dtfrot;
  // cohesion bond/nonlinear: on/off, contact distance factor, parameters of
  // the one type pair, tsCreateBondnonlinear
  int bonds;
  double cdf;
  BondPar bp;
  long long ts_create;
  double *x, *v, *w, *F, *T, *r, *m, *ws;  // ws [(w*n + i)*3 + k]
  // FP32 mirror of the positions and radii (x, y, z, r) for the candidate
  // tests; fm: the distance margin that covers its rounding
  float4 *xf;
  float fm, prdf[3];
  // per-atom kick constants of the run: ka = dtf/m, kb = dtfrot/(r^2 m) and
  // the factors of their derivatives ka/m, kb/m, 2 kb/r
  double *ka, *kb, *kam, *kbm, *kbr;
  // list in use
  int np;
  const int *pi, *pj, *row, *rev_start, *rev;
  const uint8_t *sh;
  uint8_t *flag;
  double *shear;
  double *bh;  // bond history of the list in use
  // pair outputs of the current force evaluation
  double *pF, *pTi, *pTj;
  uint8_t *active;  // touching or bonded: the entry's outputs count
  // cells
  int nc[3];
  double csz[3];
  int ncell;
  int *cell_of, *cell_count, *cell_start, *cell_fill, *order, *pcount;
  int *err;  // [0]: an atom moved more than skin/2 from its build position; [1]: mesh slots exceeded
  // mesh walls: meshes; FixNeighlistMesh's neighbour threshold (static: skin/2)
  int nmeshes;
  AMesh mesh[kAMeshes];
  double cutneighmax, mtskin;
  // slot state per (mesh m, atom i), index b = m*n + i: triangle of each slot
  // (-1 empty), slot histories, occupied slots, slots in use (candidates at
  // the last build); candidates of the list in use
  int *mst;     // [b*kAMC + u]
  double *msh;  // [(b*kAMC + u)*3 + d]
  int *mnp, *mns;
  const int *mcn, *mcand;
};

__device__ __forceinline__ int a_cell_coord(const ADev &s, double x, int d) {
  int c = (int)((x - s.lo[d]) / s.csz[d]);
  c = c < 0 ? 0 : c;
  c = c >= s.nc[d] ? s.nc[d] - 1 : c;
  return c;
}

__device__ __forceinline__ void a_image(const ADev &s, int code, double xj[3]) {
  if (code == kNoShift) return;
  const int sv[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
  for (int d = 0; d < 3; d++)
    if (sv[d]) xj[d] = __dadd_rn(xj[d], sv[d] * s.prd[d]);
}

// FP32 candidate test of entry p against the contact distance (ri + rj) cdf:
// false only when the exact FP64 distance is beyond it (fm bounds the
// rounding of the FP32 mirror and of this arithmetic)
__device__ __forceinline__ bool pair_candidate(const ADev &s, const float4 *xf, int p) {
  const float4 a = xf[s.pi[p]], b = xf[s.pj[p]];
  float bx = b.x, by = b.y, bz = b.z;
  const int code = s.sh[p];
  if (code != kNoShift) {
    bx += (float)(code % 3 - 1) * s.prdf[0];
    by += (float)((code / 3) % 3 - 1) * s.prdf[1];
    bz += (float)(code / 9 - 1) * s.prdf[2];
  }
  const float dx = a.x - bx, dy = a.y - by, dz = a.z - bz;
  const float R = (a.w + b.w) * (float)s.cdf + s.fm;
  return dx * dx + dy * dy + dz * dz <= R * R;
}

#define AGRID(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)
// block-stride loop with the same trip count for every thread of a block (the
// queue kernels synchronise inside it); blockDim.x == kAB
#define ABLOCKS(base, n) for (int base = blockIdx.x * kAB; base < (n); base += gridDim.x * kAB)

// Dense work queue of one block.  The FP64 pipe issues per warp, so a warp in
// which a few lanes run the contact law costs as much as a full one; the
// threads whose `want` is set place their item in consecutive slots of q (in
// thread order) and the first `count` threads then run the expensive part on
// dense warps.  Contains two barriers; the caller synchronises again after
// consuming q.
__device__ __forceinline__ int block_queue(bool want, int item, int *q, int *wcnt) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (lane == 0) wcnt[warp] = __popc(m);
  __syncthreads();
  int off = 0, tot = 0;
#pragma unroll
  for (int k = 0; k < kAB / 32; k++) {
    const int v = wcnt[k];
    off += (k < warp) ? v : 0;
    tot += v;
  }
  if (want) q[off + __popc(m & ((1u << lane) - 1u))] = item;
  __syncthreads();
  return tot;
}

// ---------------------------------------------------------------- list build
// per-atom kick constants of FixNVESphere (src/fix_nve_sphere.cpp:134-244)
// for the run's radii and masses
__global__ void ka_consts(ADev s) {
  AGRID(i, s.n) {
    const double m = s.m[i], r = s.r[i];
    const double a = s.dtf / m, b = s.dtfrot / (r * r * m);
    s.ka[i] = a;
    s.kb[i] = b;
    s.kam[i] = a / m;
    s.kbm[i] = b / m;
    s.kbr[i] = 2.0 * b / r;
  }
}

// Domain::pbc (src/domain.cpp:550-650) for periodic dimensions
__global__ void ka_wrap(ADev s) {
  AGRID(i, s.n) {
    for (int d = 0; d < 3; d++) {
      if (!s.per[d]) continue;
      double x = s.x[3 * i + d];
      if (x < s.lo[d]) x += s.prd[d];
      if (x >= s.hi[d]) {
        x -= s.prd[d];
        if (x < s.lo[d]) x = s.lo[d];
      }
      s.x[3 * i + d] = x;
    }
    s.xf[i] = make_float4((float)s.x[3 * i], (float)s.x[3 * i + 1], (float)s.x[3 * i + 2], (float)s.r[i]);
  }
}
__global__ void ka_cell(ADev s) {
  AGRID(i, s.n) {
    int c[3];
    for (int d = 0; d < 3; d++) c[d] = a_cell_coord(s, s.x[3 * i + d], d);
    const int cell = c[0] + s.nc[0] * (c[1] + s.nc[1] * c[2]);
    s.cell_of[i] = cell;
    atomicAdd(&s.cell_count[cell], 1);
  }
}
__global__ void ka_scatter(ADev s) {
  AGRID(i, s.n) {
    const int c = s.cell_of[i];
    s.order[s.cell_start[c] + atomicAdd(&s.cell_fill[c], 1)] = i;
  }
}
// ascending atom index within a cell: the list order does not depend on
// the order of the atomics above
__global__ void ka_cellsort(ADev s) {
  AGRID(c, s.ncell) {
    const int b = s.cell_start[c], e = s.cell_start[c + 1];
    for (int k = b + 1; k < e; k++) {
      const int v = s.order[k];
      int m = k - 1;
      while (m >= b && s.order[m] > v) {
        s.order[m + 1] = s.order[m];
        m--;
      }
      s.order[m + 1] = v;
    }
  }
}

// granular half list in input order: local pairs once (owner = lower index),
// periodic images as directed entries of each owner; cutoff
// (ri + rj) cdf + skin (src/neigh_gran.cpp:580-586)
// candidates [qb, qe) of the cell-sorted order (s.order), all with image
// code `code`
// A candidate farther in FP32 (the mirror xf, refreshed by every drift and
// wrap) than the cutoff plus fm, the bound of the mirror's rounding and of
// this arithmetic, is beyond the exact cutoff too: it skips the FP64 test.
template <bool FILL>
__device__ __forceinline__ void ka_scan(const ADev &s, int i, const double xi[3], double ri, float4 fi,
                                        float cdff, float skinm, int qb, int qe, int code, int &cnt, int &out,
                                        int out_end, int *pi, int *pj, uint8_t *shc) {
  float sxf = 0.f, syf = 0.f, szf = 0.f;
  if (code != kNoShift) {
    const int sx = code % 3 - 1, sy = (code / 3) % 3 - 1, sz = code / 9 - 1;
    sxf = sx == 0 ? 0.f : (sx > 0 ? s.prdf[0] : -s.prdf[0]);
    syf = sy == 0 ? 0.f : (sy > 0 ? s.prdf[1] : -s.prdf[1]);
    szf = sz == 0 ? 0.f : (sz > 0 ? s.prdf[2] : -s.prdf[2]);
  }
  for (int q = qb; q < qe; q++) {
    const int j = s.order[q];
    if (code == kNoShift && j <= i) continue;
    const float4 b = s.xf[j];
    const float fx = fi.x - (b.x + sxf), fy = fi.y - (b.y + syf), fz = fi.z - (b.z + szf);
    const float rf = (fi.w + b.w) * cdff + skinm;
    if (fx * fx + fy * fy + fz * fz > rf * rf) continue;
    double xj[3] = {s.x[3 * j], s.x[3 * j + 1], s.x[3 * j + 2]};
    a_image(s, code, xj);
    const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
    const double cs = (ri + s.r[j]) * s.cdf + s.skin;
    if (dx * dx + dy * dy + dz * dz > cs * cs) continue;
    if (!FILL) {
      cnt++;
      continue;
    }
    if (out >= out_end) continue;
    pi[out] = i;
    pj[out] = j;
    shc[out] = (uint8_t)code;
    out++;
  }
}

// The 27 cells in the stencil's order (z, then y, then x offsets); along x
// the unwrapped cells of a row are consecutive cells, whose atoms form one
// contiguous run of the cell-sorted order, scanned in one loop (the same
// candidates in the same order as cell by cell); a cell that wraps around a
// periodic x boundary is scanned alone, with its image shift.
template <bool FILL>
__global__ void ka_pairs(ADev s, int *pi, int *pj, uint8_t *shc, const int *row) {
  const float cdff = (float)s.cdf, skinm = (float)s.skin + s.fm;
  AGRID(i, s.n) {
    const double xi[3] = {s.x[3 * i], s.x[3 * i + 1], s.x[3 * i + 2]};
    const double ri = s.r[i];
    const float4 fi = s.xf[i];
    int ci[3];
    for (int d = 0; d < 3; d++) ci[d] = a_cell_coord(s, xi[d], d);
    int cnt = 0, out = FILL ? row[i] : 0;
    const int out_end = FILL ? row[i + 1] : 0;
    int nb[3][3], sv3[3][3];
    bool ok3[3][3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        int cc = ci[d] + k - 1, sv = 0;
        bool ok = true;
        if (cc < 0) {
          ok = s.per[d] != 0;
          cc += s.nc[d];
          sv = -1;
        } else if (cc >= s.nc[d]) {
          ok = s.per[d] != 0;
          cc -= s.nc[d];
          sv = 1;
        }
        nb[d][k] = cc;
        sv3[d][k] = sv;
        ok3[d][k] = ok;
      }
    }
    const bool lwrap = ok3[0][0] && sv3[0][0] != 0, rwrap = ok3[0][2] && sv3[0][2] != 0;
    const int x0 = (ok3[0][0] && !lwrap) ? nb[0][0] : nb[0][1];
    const int x1 = (ok3[0][2] && !rwrap) ? nb[0][2] : nb[0][1];
#pragma unroll
    for (int kz = 0; kz < 3; kz++) {
#pragma unroll
      for (int ky = 0; ky < 3; ky++) {
        if (!ok3[2][kz] || !ok3[1][ky]) continue;
        const int rowb = s.nc[0] * (nb[1][ky] + s.nc[1] * nb[2][kz]);
        const int syz = 3 * (sv3[1][ky] + 1) + 9 * (sv3[2][kz] + 1);
        if (lwrap)
          ka_scan<FILL>(s, i, xi, ri, fi, cdff, skinm, s.cell_start[rowb + nb[0][0]],
                        s.cell_start[rowb + nb[0][0] + 1], syz, cnt, out, out_end, pi, pj, shc);
        ka_scan<FILL>(s, i, xi, ri, fi, cdff, skinm, s.cell_start[rowb + x0], s.cell_start[rowb + x1 + 1],
                      1 + syz, cnt, out, out_end, pi, pj, shc);
        if (rwrap)
          ka_scan<FILL>(s, i, xi, ri, fi, cdff, skinm, s.cell_start[rowb + nb[0][2]],
                        s.cell_start[rowb + nb[0][2] + 1], 2 + syz, cnt, out, out_end, pi, pj, shc);
      }
    }
    if (!FILL) s.pcount[i] = cnt;
  }
}

// reverse lists over all entries (periodic included), ascending per partner
__global__ void ka_rev_count(int np, const int *pj, int *cnt) {
  AGRID(p, np) atomicAdd(&cnt[pj[p]], 1);
}
__global__ void ka_rev_fill(int np, const int *pj, const int *start, int *fill, int *rev) {
  AGRID(p, np) rev[start[pj[p]] + atomicAdd(&fill[pj[p]], 1)] = p;
}
__global__ void ka_rev_sort(int n, const int *start, int *rev) {
  AGRID(i, n) {
    const int b = start[i], e = start[i + 1];
    for (int k = b + 1; k < e; k++) {
      const int v = rev[k];
      int m = k - 1;
      while (m >= b && rev[m] > v) {
        rev[m + 1] = rev[m];
        m--;
      }
      rev[m + 1] = v;
    }
  }
}

// history carried from the previous list (see the file comment): pairs within
// (ri + rj) cdf at the build (src/neigh_gran.cpp:590-620); also sets the new
// entries' flags
__global__ void ka_carry(ADev s, AList nw, AList old) {
  AGRID(p, nw.np) {
    const int i = nw.pi[p], j = nw.pj[p], code = nw.sh[p];
    int e = -1;
    double sgn = 1.0;
    double xj[3] = {s.x[3 * j], s.x[3 * j + 1], s.x[3 * j + 2]};
    a_image(s, code, xj);
    const double dx = s.x[3 * i] - xj[0], dy = s.x[3 * i + 1] - xj[1], dz = s.x[3 * i + 2] - xj[2];
    const double rs = (s.r[i] + s.r[j]) * s.cdf;
    if (old.np > 0 && dx * dx + dy * dy + dz * dz < rs * rs) {
      for (int q = old.row[i]; q < old.row[i + 1]; q++)
        if (old.pj[q] == j && old.flag[q]) {
          e = q;
          break;
        }
      if (e < 0)
        for (int q = old.rev_start[i]; q < old.rev_start[i + 1]; q++) {
          const int o = old.rev[q];
          if (old.pi[o] == j && old.sh[o] == kNoShift && old.flag[o]) {
            e = o;
            sgn = -1.0;
            break;
          }
        }
    }
    nw.carry[p] = e < 0 ? -1 : (sgn > 0 ? e : -(e + 2));
    nw.flag[p] = e >= 0 ? 1 : 0;
    for (int k = 0; k < 3; k++) nw.shear[3 * p + k] = e >= 0 ? sgn * old.shear[3 * e + k] : 0.0;
    if (s.bonds)
      for (int k = 0; k < kBondValues; k++) {
        const double f = (sgn < 0 && k >= 5 && k <= 13) ? -1.0 : 1.0;  // newtonflag 1: ft, thetan, thetat
        nw.bond[(size_t)kBondValues * p + k] = e >= 0 ? f * old.bond[(size_t)kBondValues * e + k] : 0.0;
      }
  }
}

// ------------------------------------------------------------------- forward
__device__ __forceinline__ VjpIn pair_in(const ADev &s, const double *x, int p, const double *vh,
                                         const double *wh, const double *shear) {
  VjpIn a;
  const int i = s.pi[p], j = s.pj[p];
  double xj[3] = {x[3 * j], x[3 * j + 1], x[3 * j + 2]};
  a_image(s, s.sh[p], xj);
  for (int k = 0; k < 3; k++) {
    a.d[k] = x[3 * i + k] - xj[k];
    a.vr[k] = vh[3 * i + k] - vh[3 * j + k];
    a.wi[k] = wh[3 * i + k];
    a.wj[k] = wh[3 * j + k];
    a.sh[k] = shear[3 * p + k];
  }
  a.ri = s.r[i];
  a.rj = s.r[j];
  a.mi = s.m[i];
  a.mj = s.m[j];
  a.Y = s.Y;
  a.G = s.G;
  a.beta = s.beta;
  a.mu = s.mu;
  a.dt = s.dt;
  a.wall = false;
  a.bonded = false;
  a.rolling = s.rolling != 0;
  a.mur = s.mur;
  return a;
}

__device__ __forceinline__ bool pair_touch(const VjpIn &a) {
  const double rs = a.ri + a.rj;
  return dot3(a.d, a.d) < rs * rs;
}

// within the contact distance (ri + rj) cdf (surfacesClose)
__device__ __forceinline__ bool pair_band(const ADev &s, const VjpIn &a) {
  const double rs = a.ri + a.rj;
  return dot3(a.d, a.d) < s.cdf * s.cdf * rs * rs;
}

__device__ __forceinline__ BondArgs bond_in(const ADev &s, const VjpIn &a, const double *x, int i,
                                            long long ntimestep) {
  BondArgs b;
  for (int k = 0; k < 3; k++) {
    b.d[k] = a.d[k];
    b.vr[k] = a.vr[k];
    b.wi[k] = a.wi[k];
    b.wj[k] = a.wj[k];
    b.xi[k] = x[3 * i + k];
  }
  b.ri = a.ri;
  b.rj = a.rj;
  b.dt = a.dt;
  b.upd = a.upd;
  b.may_create = a.upd && ((s.bp.flags & kBondCreateAlways) || ntimestep == s.ts_create);
  return b;
}

// plane w against atom i (FixWallGran primitive: overlap when the distance
// to the plane is at most the radius); false when not touching
__device__ __forceinline__ bool wall_in(const ADev &s, const double *x, int w, int i, const double *vh,
                                        const double *wh, const double *ws, VjpIn &a) {
  const int ax = s.pax[w];
  const double pos = s.ppos[w];
  const double xa = x[3 * i + ax];
  const double dist = xa > pos ? xa - pos : pos - xa;
  if (!(dist - s.r[i] <= 0)) return false;
  for (int k = 0; k < 3; k++) {
    a.d[k] = k == ax ? xa - pos : 0.0;
    a.vr[k] = vh[3 * i + k];
    a.wi[k] = wh[3 * i + k];
    a.wj[k] = 0.0;
    a.sh[k] = ws[((size_t)w * s.n + i) * 3 + k];
  }
  a.ri = s.r[i];
  a.rj = 0.0;
  a.mi = s.m[i];
  a.mj = 0.0;
  a.Y = s.Y;
  a.G = s.G;
  a.beta = s.beta;
  a.mu = s.mu;
  a.dt = s.dt;
  a.wall = true;
  a.bonded = false;
  a.rolling = s.rolling != 0;
  a.mur = s.mur;
  return true;
}

// adjoints of the run's state (the mesh reverse below and the reverse kernels)
struct ABar {
  double *xb, *vb, *wb, *Fb, *Tb, *rb, *mb, *sb, *wsb;
  // per-entry VJP outputs of the pair law
  double *pd, *pv, *pwi, *pwj, *pri, *prj, *pmi, *pmj, *pth;  // pth [kTh*p]: Y, G, beta, mu, mur
  double *bb;   // [kBondValues*p] adjoint of the bond history (bonds only)
  double *wth;  // [kTh*i] wall parameter adjoints per atom
  double *th;   // [4] accumulated parameter adjoints
  double *msb;  // [(b*kAMC + u)*3 + d] adjoints of the mesh slot histories
};

// ------------------------------------------------------------- mesh walls
// Static triangle-mesh walls (fix mesh/surface + wall/gran ... mesh): the
// contact of one atom with its candidate triangles as the main path's
// sequential mesh_contacts does it (FixWallGran::post_force_mesh,
// src/fix_wall_gran.cpp:803-982; TriMesh::resolveTriSphereContactBary,
// src/tri_mesh_I.h:65-271; FixContactHistoryMesh::handleContact,
// coplanarContactAlready, cleanUpContacts, src/fix_contact_history_mesh_I.h:
// 51-216), with the slot state per atom and mesh: the triangle of each
// history slot (-1 empty), the slot histories and the count of occupied
// slots; the slots in use are the first mcn (the candidate count).

__device__ __forceinline__ bool amesh_coplanar(const AMesh &M, int a, int b) {
  for (int q = M.cn_start[a]; q < M.cn_start[a + 1]; q++)
    if (M.cn_list[q] == b) return true;
  return false;
}

// the closest feature of a resolved contact, from resolve_tri_sphere's
// outputs: face (barySign 7), corner (one barycentric weight 1) or edge (the
// edge between the two nodes with weight); ax: the face normal or the edge's
// unit vector.  d = centre - closest point then moves with the centre as
// J = ax ax^T (face), I - ax ax^T (edge), I (corner).
__device__ __forceinline__ int amesh_feature(const double *g, int bs, const double bary[3], double ax[3]) {
  if (bs == 7) {
    for (int k = 0; k < 3; k++) ax[k] = tri_sn(g)[k];
    return 0;
  }
  for (int k = 0; k < 3; k++)
    if (bary[k] == 1.0 && bary[(k + 1) % 3] == 0.0 && bary[(k + 2) % 3] == 0.0) {
      ax[0] = ax[1] = ax[2] = 0.0;
      return 2;
    }
  int e = 0;
  for (int k = 0; k < 3; k++)
    if (bary[(k + 2) % 3] == 0.0) e = k;  // nodes k and k+1 carry the weight
  for (int k = 0; k < 3; k++) ax[k] = tri_ev(g, e)[k];
  return 1;
}

// vw: the wall velocity at the contact (a translating mesh's velocity; 0
// for a static mesh and in the setup force pass)
__device__ __forceinline__ void amesh_contact_in(const ADev &s, int i, const double *vh, const double *wh,
                                                 const double delta[3], const double hin[3], int upd,
                                                 const double vw[3], VjpIn &a) {
  for (int k = 0; k < 3; k++) {
    a.d[k] = -delta[k];
    a.vr[k] = vh[3 * i + k] - vw[k];
    a.wi[k] = wh[3 * i + k];
    a.wj[k] = 0.0;
    a.sh[k] = hin[k];
  }
  a.ri = s.r[i];
  a.rj = 0.0;
  a.mi = s.m[i];
  a.mj = 0.0;
  a.Y = s.Y;
  a.G = s.G;
  a.beta = s.beta;
  a.mu = s.mu;
  a.dt = s.dt;
  a.upd = upd != 0;
  a.wall = true;
  a.bonded = false;
  a.rolling = s.rolling != 0;
  a.mur = s.mur;
}

// one evaluation of the slot logic and contact law for atom i and mesh m on
// the slot state st/sh/np (updated in place); adds the forces to f/t.  rec
// (if set) receives, per evaluated contact, what the reverse needs.
struct AMeshRec {
  int slot, copy, kind, fresh, band;
  double hin[3], delta[3], ax[3];
};

// the atom's position relative to mesh m at step `step` (a translating
// mesh's geometry is its step-0 geometry shifted by step*dt*vel)
__device__ __forceinline__ void amesh_rel(const ADev &s, const AMesh &M, long long step, const double *x, int i,
                                          double xr[3]) {
  for (int k = 0; k < 3; k++) xr[k] = M.moving ? x[3 * i + k] - (double)step * (s.dt * M.vel[k]) : x[3 * i + k];
}

template <bool ROLL>
__device__ inline int amesh_eval(const ADev &s, int m, int i, const double *x, const double *vh, const double *wh,
                                 int upd, long long step, int *st, double *sh, int &np, double f[3], double t[3],
                                 AMeshRec *rec, unsigned &keep, bool &bad) {
  const AMesh &M = s.mesh[m];
  const size_t base = (size_t)m * s.n + i;
  const int nc = s.mcn[base];
  const int *cand = s.mcand + base * kAMC;
  double xi[3];
  amesh_rel(s, M, step, x, i, xi);
  const double vw[3] = {M.moving && upd ? M.vel[0] : 0.0, M.moving && upd ? M.vel[1] : 0.0,
                        M.moving && upd ? M.vel[2] : 0.0};
  const double radi = s.r[i];
  const double cdm1 = s.cdf - 1.0;
  int nr = 0;
  keep = 0u;
  for (int q = 0; q < nc; q++) {
    const int tr = cand[q];
    const double *g = M.tri + (size_t)tr * kTriStride;
    double delta[3], bary[3];
    int bs;
    const double deltan = resolve_tri_sphere(g, M.meta[tr], radi, xi, delta, bary, bs);
    if (deltan > s.cutneighmax) continue;
    if (!(deltan <= 0 || deltan < cdm1 * radi)) continue;
    int slot = -1, copy = -1;
    bool fresh = false;
    for (int u = 0; u < nc; u++)
      if (st[u] == tr) {
        slot = u;
        break;
      }
    if (slot >= 0) {
      keep |= 1u << slot;
    } else {
      const bool face = bs == 7;
      if (face) {  // coplanarContactAlready
        bool already = false;
        for (int u = 0; u < nc; u++) {
          const int p = st[u];
          if (p >= 0 && p != tr && ((keep >> u) & 1u) && amesh_coplanar(M, p, tr)) already = true;
        }
        if (already) continue;
      }
      if (np >= nc) {
        bad = true;
        continue;
      }
      for (int u = 0; u < nc; u++)
        if (st[u] == -1) {
          slot = u;
          break;
        }
      st[slot] = tr;
      keep |= 1u << slot;
      for (int d = 0; d < 3; d++) sh[3 * slot + d] = 0.0;
      np++;
      fresh = true;
      if (face)  // checkCoplanarContactHistory: the last coplanar partner's history
        for (int u = 0; u < nc; u++) {
          const int p = st[u];
          if (p >= 0 && p != tr && amesh_coplanar(M, p, tr)) {
            copy = u;
            for (int d = 0; d < 3; d++) sh[3 * slot + d] = sh[3 * u + d];
          }
        }
    }
    if (rec) {
      AMeshRec &R = rec[nr];
      R.slot = slot;
      R.copy = copy;
      R.fresh = fresh ? 1 : 0;
      R.band = deltan > 0 ? 1 : 0;
      R.kind = amesh_feature(g, bs, bary, R.ax);
      for (int d = 0; d < 3; d++) {
        R.hin[d] = sh[3 * slot + d];
        R.delta[d] = delta[d];
      }
    }
    nr++;
    if (deltan > 0) {  // within the contact distance, apart: surfacesClose
      for (int d = 0; d < 3; d++) sh[3 * slot + d] = 0.0;
      continue;
    }
    VjpIn a;
    amesh_contact_in(s, i, vh, wh, delta, sh + 3 * slot, upd, vw, a);
    LawState S;
    double F[3], Ti[3], Tj[3], s3[3];
    law_forward<ROLL>(a, S, F, Ti, Tj, s3);
    for (int d = 0; d < 3; d++) {
      f[d] += F[d];
      t[d] += Ti[d];
      if (upd) sh[3 * slot + d] = s3[d];
    }
  }
  for (int u = 0; u < nc; u++)  // cleanUpContacts
    if (!((keep >> u) & 1u)) {
      if (st[u] > -1) np--;
      st[u] = -1;
      for (int d = 0; d < 3; d++) sh[3 * u + d] = 0.0;
    }
  return nr;
}

// forward of atom i against every mesh: forces into f/t; the slot state
// before the evaluation goes to the tape (if set)
template <bool ROLL>
__device__ inline void amesh_forward(const ADev &s, int i, const double *x, const double *vh, const double *wh,
                                     int upd, long long step, double f[3], double t[3], int *tst, double *tsh,
                                     int *tnp, double *wallF) {
  for (int m = 0; m < s.nmeshes; m++) {
    const size_t base = (size_t)m * s.n + i;
    int *st = s.mst + base * kAMC;
    double *sh = s.msh + base * kAMC * 3;
    int np = s.mnp[base];
    if (tst) {
      for (int u = 0; u < kAMC; u++) tst[base * kAMC + u] = st[u];
      for (int u = 0; u < 3 * kAMC; u++) tsh[base * kAMC * 3 + u] = sh[u];
      tnp[base] = np;
    }
    if (s.mcn[base] == 0) {
      if (wallF)
        for (int k = 0; k < 3; k++) wallF[(((size_t)s.nplanes + m) * s.n + i) * 3 + k] = 0.0;
      continue;
    }
    unsigned keep;
    bool bad = false;
    double fm[3] = {0., 0., 0.};
    amesh_eval<ROLL>(s, m, i, x, vh, wh, upd, step, st, sh, np, fm, t, nullptr, keep, bad);
    for (int k = 0; k < 3; k++) f[k] += fm[k];
    if (wallF)  // meshes after the planes
      for (int k = 0; k < 3; k++) wallF[(((size_t)s.nplanes + m) * s.n + i) * 3 + k] = fm[k];
    if (bad) s.err[1] = 1;
    s.mnp[base] = np;
  }
}

// reverse of amesh_forward for atom i: Fb/Tb the adjoints of the atom's total
// force and torque; the slot-history adjoints B.msb (of the state after the
// evaluation) become those of the state before it (the tape's)
template <bool ROLL>
__device__ inline void amesh_vjp(const ADev &s, const ABar &B, int i, const double *x, const double *vh,
                                 const double *wh, int upd, long long step, int seed_m, int seed_axis, double seed,
                                 const int *tst, const double *tsh, const int *tnp,
                                 const double Fb[3], const double Tb[3], double xb[3], double vb[3], double wb[3],
                                 double &rb, double &mb, double th[kTh]) {
  for (int m = 0; m < s.nmeshes; m++) {
    const size_t base = (size_t)m * s.n + i;
    const int nc = s.mcn[base];
    if (nc == 0) continue;
    int st[kAMC];
    double sh[3 * kAMC];
    for (int u = 0; u < kAMC; u++) st[u] = tst[base * kAMC + u];
    for (int u = 0; u < 3 * kAMC; u++) sh[u] = tsh[base * kAMC * 3 + u];
    int np = tnp[base];
    AMeshRec rec[kAMC];
    unsigned keep;
    bool bad = false;
    double f[3] = {0., 0., 0.}, t[3] = {0., 0., 0.};
    const int nr = amesh_eval<ROLL>(s, m, i, x, vh, wh, upd, step, st, sh, np, f, t, rec, keep, bad);
    const AMesh &M = s.mesh[m];
    const double vw[3] = {M.moving && upd ? M.vel[0] : 0.0, M.moving && upd ? M.vel[1] : 0.0,
                          M.moving && upd ? M.vel[2] : 0.0};
    double *hb = B.msb + base * kAMC * 3;
    for (int u = 0; u < nc; u++)
      if (!((keep >> u) & 1u))
        for (int d = 0; d < 3; d++) hb[3 * u + d] = 0.0;  // cleared: no dependence on the value before
    for (int r = nr - 1; r >= 0; r--) {
      const AMeshRec &R = rec[r];
      const int u = R.slot;
      if (R.band) {
        for (int d = 0; d < 3; d++) hb[3 * u + d] = 0.0;
      } else {
        VjpIn a;
        amesh_contact_in(s, i, vh, wh, R.delta, R.hin, upd, vw, a);
        VjpBar bb;
        for (int d = 0; d < 3; d++) {
          bb.F[d] = Fb[d] + (m == seed_m && d == seed_axis ? seed : 0.0);
          bb.Ti[d] = Tb[d];
          bb.Tj[d] = 0.0;
          bb.s3[d] = upd ? hb[3 * u + d] : 0.0;
        }
        law_vjp<ROLL>(a, bb);
        for (int d = 0; d < 3; d++) hb[3 * u + d] = bb.sh[d] + (upd ? 0.0 : hb[3 * u + d]);
        // d = centre - closest point
        if (R.kind == 2) {
          for (int d = 0; d < 3; d++) xb[d] += bb.d[d];
        } else {
          const double pr = R.ax[0] * bb.d[0] + R.ax[1] * bb.d[1] + R.ax[2] * bb.d[2];
          for (int d = 0; d < 3; d++) xb[d] += R.kind == 0 ? pr * R.ax[d] : bb.d[d] - pr * R.ax[d];
        }
        for (int d = 0; d < 3; d++) {
          vb[d] += bb.vr[d];
          wb[d] += bb.wi[d];
        }
        rb += bb.ri;
        mb += bb.mi;
        th[0] += bb.Y;
        th[1] += bb.G;
        th[2] += bb.beta;
        th[3] += bb.mu;
        th[4] += bb.mur;
      }
      if (R.fresh) {  // the slot was set to zero, or to a coplanar partner's history
        if (R.copy >= 0)
          for (int d = 0; d < 3; d++) hb[3 * R.copy + d] += hb[3 * u + d];
        for (int d = 0; d < 3; d++) hb[3 * u + d] = 0.0;
      }
    }
  }
}

// FixContactHistoryMesh::sort_contacts (pre_exchange), then the candidates of
// FixNeighlistMesh::pre_force (TriMesh::resolveTriSphereNeighbuild, every
// triangle in ascending order), cleanUpContactJumps and the re-paging of the
// slots, at the positions of a build.  map[s'] receives the slot each new
// slot came from (-1: emptied), for the reverse pass.
__device__ __forceinline__ void amesh_swap(int *st, double *sh, int *orig, int a, int b) {
  const int t = st[a];
  st[a] = st[b];
  st[b] = t;
  const int o = orig[a];
  orig[a] = orig[b];
  orig[b] = o;
  for (int d = 0; d < 3; d++) {
    const double h = sh[3 * a + d];
    sh[3 * a + d] = sh[3 * b + d];
    sh[3 * b + d] = h;
  }
}

__global__ void ka_mesh_build(ADev s, long long step, int *mcn, int *mcand, int *map) {
  AGRID(i, s.n) {
    const double rS = s.r[i] * s.cdf;
    for (int m = 0; m < s.nmeshes; m++) {
      const AMesh &M = s.mesh[m];
      double xi[3];
      amesh_rel(s, M, step, s.x, i, xi);
      // FixNeighlistMesh: a moving mesh takes candidates within r cdf + skin
      const double tskin = M.moving ? s.skin : s.mtskin;
      const size_t base = (size_t)m * s.n + i;
      int *st = s.mst + base * kAMC;
      double *sh = s.msh + base * kAMC * 3;
      int np = s.mnp[base];
      const int nn = s.mns[base];
      int orig[kAMC];
      for (int u = 0; u < kAMC; u++) orig[u] = u;
      int fe, lf;
      do {  // sort_contacts
        fe = lf = -1;
        for (int j = 0; j < nn; j++) {
          if (fe == -1 && st[j] == -1) fe = j;
          if (st[j] >= 0) lf = j;
        }
        if (fe > -1 && lf > -1 && fe < lf) amesh_swap(st, sh, orig, fe, lf);
      } while (fe > -1 && lf > -1 && fe < lf);
      int nc = 0;
      int *cand = mcand + base * kAMC;
      for (int tr = 0; tr < M.ntri; tr++) {
        if (!tri_sphere_neighbuild(M.tri + (size_t)tr * kTriStride, rS, xi, tskin)) continue;
        if (nc == kAMC) {
          s.err[1] = 1;
          break;
        }
        cand[nc++] = tr;
      }
      int ip = 0;  // cleanUpContactJumps
      while (ip < np) {
        const int tr = st[ip];
        bool listed = false;
        for (int q = 0; q < nc; q++) listed |= (cand[q] == tr);
        if (!listed) {
          st[ip] = -1;
          orig[ip] = -1;
          for (int d = 0; d < 3; d++) sh[3 * ip + d] = 0.0;
          amesh_swap(st, sh, orig, ip, np - 1);
          np--;
        } else {
          ip++;
        }
      }
      for (int q = np; q < nc; q++) {
        st[q] = -1;
        orig[q] = -1;
        for (int d = 0; d < 3; d++) sh[3 * q + d] = 0.0;
      }
      s.mnp[base] = np;
      s.mns[base] = nc;
      mcn[base] = nc;
      for (int u = 0; u < kAMC; u++) map[base * kAMC + u] = u < nc ? orig[u] : -1;
    }
  }
}

// slot-history adjoints back through a build: old[orig] += new[s']
__global__ void kb_mesh_uncarry(int cnt, const int *map, const double *hb_new, double *hb_old) {
  AGRID(b, cnt) {  // one (mesh, atom) each
    for (int u = 0; u < kAMC; u++) {
      const int o = map[(size_t)b * kAMC + u];
      if (o >= 0)
        for (int d = 0; d < 3; d++) hb_old[((size_t)b * kAMC + o) * 3 + d] += hb_new[((size_t)b * kAMC + u) * 3 + d];
    }
  }
}

// pair forces of the current state (vh, wh: the velocities the forces see)
// at step ntimestep; tape_sh/tape_bh receive the history before the update.
// The pass follows k_pair<..., BOND> of the main path: touching entries run
// the contact law (with a bond's force in place of the normal force),
// entries within the contact distance but apart clear their tangential
// history and evaluate a bond they hold or may create.
// BONDS: the system has cohesion bond/nonlinear (a separate instance keeps
// the registers of the plain contact path low)
template <bool BONDS, bool ROLL>
__global__ void __launch_bounds__(kAB) ka_pair_force(ADev s, const double *vh, const double *wh, int upd,
                                                     long long ntimestep, double *tape_sh, double *tape_bh) {
  __shared__ int q[kAB];
  __shared__ int wcnt[kAB / 32];
  ABLOCKS(base, s.np) {
    const int p0 = base + threadIdx.x;
    bool work = false;
    if (p0 < s.np) {  // tape and the FP32 candidate test; the rest runs queued
      if (tape_sh)
        for (int k = 0; k < 3; k++) tape_sh[3 * p0 + k] = s.shear[3 * p0 + k];
      if (BONDS && tape_bh)
        for (int k = 0; k < kBondValues; k++)
          tape_bh[(size_t)kBondValues * p0 + k] = s.bh[(size_t)kBondValues * p0 + k];
      work = pair_candidate(s, s.xf, p0);
      if (!work) s.active[p0] = 0;  // beyond the contact distance: nothing changes
    }
    const int tot = block_queue(work, p0, q, wcnt);
    if (threadIdx.x < tot) {
      const int p = q[threadIdx.x];
      VjpIn a = pair_in(s, s.x, p, vh, wh, s.shear);
      a.upd = upd != 0;
      const bool touch = pair_touch(a), band = pair_band(s, a);
      if (!touch && band) {  // TangentialModel<TANGENTIAL_HISTORY>::surfacesClose
        for (int k = 0; k < 3; k++) s.shear[3 * p + k] = 0.0;
        s.flag[p] &= ~kContactTangential;
      }
      int st = kBondNone;
      double bF[3] = {0., 0., 0.}, bTi[3] = {0., 0., 0.}, bTj[3] = {0., 0., 0.};
      if (BONDS && (touch || band)) {
        double *bh = s.bh + (size_t)kBondValues * p;
        const BondArgs b = bond_in(s, a, s.x, s.pi[p], ntimestep);
        double hin[kBondValues], hout[kBondValues];
        for (int k = 0; k < kBondValues; k++) hin[k] = bh[k];
        BondTape T;
        st = bond_fwd(b, s.bp, hin, hout, bF, bTi, bTj, T);
        for (int k = 0; k < kBondValues; k++) bh[k] = hout[k];
        if (st == kBondActive) s.flag[p] |= kContactCohesion;
        if (st == kBondBroken) s.flag[p] &= ~kContactCohesion;
      }
      const bool bonded = st == kBondActive;
      if (touch) {
        a.bonded = bonded;
        LawState S;
        double F[3], Ti[3], Tj[3], s3[3];
        law_forward<ROLL>(a, S, F, Ti, Tj, s3);
        for (int k = 0; k < 3; k++) {
          s.pF[3 * p + k] = F[k] + bF[k];
          s.pTi[3 * p + k] = Ti[k] + bTi[k];
          s.pTj[3 * p + k] = Tj[k] + bTj[k];
          if (upd) s.shear[3 * p + k] = s3[k];
        }
        s.flag[p] |= kContactNormal | kContactTangential;
      } else if (bonded) {
        for (int k = 0; k < 3; k++) {
          s.pF[3 * p + k] = bF[k];
          s.pTi[3 * p + k] = bTi[k];
          s.pTj[3 * p + k] = bTj[k];
        }
      }
      s.active[p] = (touch || bonded) ? 1 : 0;
    }
    __syncthreads();
  }
}

// total force/torque per atom: own row, reverse list (local entries), gravity,
// planes; with final_kick the second half-kick v = vh + a F, w = wh + b T.
// tape_ws receives the wall history before the update, wallF the wall forces,
// tape_F/tape_T (if set) a copy of the forces and torques.
// The next step's first half-kick and drift (ka_kick_drift without a wrap),
// fused into the gather of a step when both lie in one segment: xref and the
// t* records as there, nk = 1 to do it.
struct NextKick {
  const double *xref;
  double *tx, *tv, *tw;
  float4 *txf;
  int on;
};

template <bool ROLL, bool MESH>
__global__ void __launch_bounds__(kAB) ka_gather(ADev s, const double *vh, const double *wh, int upd,
                                                 int final_kick, double *tape_ws, double *wallF, double *tape_F,
                                                 double *tape_T, int *tape_mst, double *tape_msh, int *tape_mnp,
                                                 long long ntimestep, NextKick nk) {
  __shared__ int q[kAB];
  __shared__ int wcnt[kAB / 32];
  __shared__ double sF[3][kAB], sT[3][kAB];
  ABLOCKS(base, s.n) {
    const int i = base + threadIdx.x;
    const bool valid = i < s.n;
    double f[3] = {0., 0., 0.}, t[3] = {0., 0., 0.};
    if (valid) {
      // own row, then the local partner entries, each in ascending order; the
      // active entries of lists of up to 32 are collected as bit masks first,
      // so that the FP64 additions issue once per contact of the warp's
      // busiest atom rather than once per entry of its longest list
      const int pb = s.row[i], pe = s.row[i + 1], rb = s.rev_start[i], re = s.rev_start[i + 1];
      if (pe - pb <= 32 && re - rb <= 32) {
        unsigned mo = 0u, mr = 0u;
        for (int k = 0; k < pe - pb; k++) mo |= (s.active[pb + k] ? 1u : 0u) << k;
        for (int k = 0; k < re - rb; k++) {
          const int p = s.rev[rb + k];
          mr |= ((s.active[p] && s.sh[p] == kNoShift) ? 1u : 0u) << k;
        }
        while (mo) {
          const int p = pb + __ffs(mo) - 1;
          mo &= mo - 1u;
          for (int k = 0; k < 3; k++) {
            f[k] += s.pF[3 * p + k];
            t[k] += s.pTi[3 * p + k];
          }
        }
        while (mr) {
          const int p = s.rev[rb + __ffs(mr) - 1];
          mr &= mr - 1u;
          for (int k = 0; k < 3; k++) {
            f[k] -= s.pF[3 * p + k];
            t[k] += s.pTj[3 * p + k];
          }
        }
      } else {
        for (int p = pb; p < pe; p++)
          if (s.active[p])
            for (int k = 0; k < 3; k++) {
              f[k] += s.pF[3 * p + k];
              t[k] += s.pTi[3 * p + k];
            }
        for (int qq = rb; qq < re; qq++) {
          const int p = s.rev[qq];
          if (!s.active[p] || s.sh[p] != kNoShift) continue;
          for (int k = 0; k < 3; k++) {
            f[k] -= s.pF[3 * p + k];
            t[k] += s.pTj[3 * p + k];
          }
        }
      }
      if (s.gravity_on)
        for (int k = 0; k < 3; k++) f[k] += s.m[i] * s.g[k];
    }
    // planes in order; the atoms touching plane w run the law on dense warps
    for (int w = 0; w < s.nplanes; w++) {
      bool touch = false;
      if (valid) {
        double *hw = s.ws + ((size_t)w * s.n + i) * 3;
        if (tape_ws)
          for (int k = 0; k < 3; k++) tape_ws[((size_t)w * s.n + i) * 3 + k] = hw[k];
        VjpIn a;
        touch = wall_in(s, s.x, w, i, vh, wh, s.ws, a);
        if (!touch) {
          for (int k = 0; k < 3; k++) hw[k] = 0.0;  // surfacesClose
          if (wallF)
            for (int k = 0; k < 3; k++) wallF[((size_t)w * s.n + i) * 3 + k] = 0.0;
        }
      }
      const int tot = block_queue(touch, threadIdx.x, q, wcnt);
      if (threadIdx.x < tot) {
        const int li = q[threadIdx.x], ii = base + li;
        VjpIn a;
        wall_in(s, s.x, w, ii, vh, wh, s.ws, a);
        a.upd = upd != 0;
        LawState S;
        double F[3], Ti[3], Tj[3], s3[3];
        law_forward<ROLL>(a, S, F, Ti, Tj, s3);
        double *hw = s.ws + ((size_t)w * s.n + ii) * 3;
        for (int k = 0; k < 3; k++) {
          sF[k][li] = F[k];
          sT[k][li] = Ti[k];
          if (upd) hw[k] = s3[k];
          if (wallF) wallF[((size_t)w * s.n + ii) * 3 + k] = F[k];
        }
      }
      __syncthreads();
      if (touch)
        for (int k = 0; k < 3; k++) {
          f[k] += sF[k][threadIdx.x];
          t[k] += sT[k][threadIdx.x];
        }
      __syncthreads();
    }
    if (valid) {
      if (MESH) amesh_forward<ROLL>(s, i, s.x, vh, wh, upd, ntimestep, f, t, tape_mst, tape_msh, tape_mnp, wallF);
      const double a = s.ka[i], b = s.kb[i];
      for (int k = 0; k < 3; k++) {
        s.F[3 * i + k] = f[k];
        s.T[3 * i + k] = t[k];
        if (tape_F) {
          tape_F[3 * i + k] = f[k];
          tape_T[3 * i + k] = t[k];
        }
        if (final_kick) {
          s.v[3 * i + k] = vh[3 * i + k] + a * f[k];
          s.w[3 * i + k] = wh[3 * i + k] + b * t[k];
        }
      }
      if (nk.on) {  // the next step's first half-kick and drift, as ka_kick_drift
        double dsq = 0.0;
        for (int k = 0; k < 3; k++) {
          const double v = s.v[3 * i + k] + a * f[k];
          const double w = s.w[3 * i + k] + b * t[k];
          const double x = s.x[3 * i + k] + s.dt * v;
          if (nk.xref) {
            const double e = x - nk.xref[3 * i + k];
            dsq += e * e;
          }
          s.v[3 * i + k] = v;
          s.w[3 * i + k] = w;
          s.x[3 * i + k] = x;
          if (nk.tx) {
            nk.tx[3 * i + k] = x;
            nk.tv[3 * i + k] = v;
            nk.tw[3 * i + k] = w;
          }
        }
        const float4 f4 = make_float4((float)s.x[3 * i], (float)s.x[3 * i + 1], (float)s.x[3 * i + 2], (float)s.r[i]);
        s.xf[i] = f4;
        if (nk.txf) nk.txf[i] = f4;
        if (dsq > 0.25 * s.skin * s.skin) s.err[0] = 1;
      }
    }
  }
}

// first half-kick and drift (v, w then hold vh, wh); xref: positions at the
// list build to check the displacement against, or null; wrap: the periodic
// wrap of a rebuild step (Domain::pbc, as ka_wrap); tx/tv/tw (if set)
// receive a copy of the new x, vh, wh
__global__ void ka_kick_drift(ADev s, const double *xref, int wrap, double *tx, double *tv, double *tw,
                              float4 *txf) {
  AGRID(i, s.n) {
    const double a = s.ka[i], b = s.kb[i];
    double dsq = 0.0;
    for (int k = 0; k < 3; k++) {
      const double v = s.v[3 * i + k] + a * s.F[3 * i + k];
      const double w = s.w[3 * i + k] + b * s.T[3 * i + k];
      double x = s.x[3 * i + k] + s.dt * v;
      if (xref) {
        const double e = x - xref[3 * i + k];
        dsq += e * e;
      }
      if (wrap && s.per[k]) {
        if (x < s.lo[k]) x += s.prd[k];
        if (x >= s.hi[k]) {
          x -= s.prd[k];
          if (x < s.lo[k]) x = s.lo[k];
        }
      }
      s.v[3 * i + k] = v;
      s.w[3 * i + k] = w;
      s.x[3 * i + k] = x;
      if (tx) {
        tx[3 * i + k] = x;
        tv[3 * i + k] = v;
        tw[3 * i + k] = w;
      }
    }
    const float4 f4 = make_float4((float)s.x[3 * i], (float)s.x[3 * i + 1], (float)s.x[3 * i + 2], (float)s.r[i]);
    s.xf[i] = f4;
    if (txf) txf[i] = f4;
    if (dsq > 0.25 * s.skin * s.skin) s.err[0] = 1;
  }
}

// ------------------------------------------------------------------ backward

// gravity and walls of one force evaluation at positions x; vh/wh the
// velocities the forces saw, ws_before the wall history before it; seed adds
// d(loss)/d(normal wall force) on plane seed_w.  Fn1/Tn1 (if set): the
// forces of this evaluation, whose second half-kick v' = vh + a F',
// w' = wh + b T' is reversed first.  The wall parameter adjoints add to
// B.wth.
template <bool ROLL, bool MESH>
__global__ void __launch_bounds__(kAB) kb_walls(ADev s, ABar B, const double *x, const double *vh,
                                                const double *wh, const double *ws_before, int upd, int seed_w,
                                                double seed, const double *Fn1, const double *Tn1,
                                                const int *tmst, const double *tmsh, const int *tmnp,
                                                long long ntimestep, int seed_axis) {
  __shared__ int q[kAB];
  __shared__ int wcnt[kAB / 32];
  ABLOCKS(base, s.n) {
    const int i = base + threadIdx.x;
    const bool valid = i < s.n;
    if (valid) {
      if (Fn1) {
        const double a = s.ka[i], b = s.kb[i];
        double fv = 0.0, tw = 0.0;
        for (int k = 0; k < 3; k++) {
          B.Fb[3 * i + k] += a * B.vb[3 * i + k];
          B.Tb[3 * i + k] += b * B.wb[3 * i + k];
          fv += Fn1[3 * i + k] * B.vb[3 * i + k];
          tw += Tn1[3 * i + k] * B.wb[3 * i + k];
        }
        B.mb[i] += -s.kam[i] * fv - s.kbm[i] * tw;
        B.rb[i] += -s.kbr[i] * tw;
      }
      if (s.gravity_on)
        B.mb[i] += s.g[0] * B.Fb[3 * i] + s.g[1] * B.Fb[3 * i + 1] + s.g[2] * B.Fb[3 * i + 2];
    }
    // planes in order; the atoms touching plane w run the VJP on dense warps
    for (int w = 0; w < s.nplanes; w++) {
      bool touch = false;
      if (valid) {
        VjpIn a;
        touch = wall_in(s, x, w, i, vh, wh, ws_before, a);
        if (!touch && upd)
          for (int k = 0; k < 3; k++) B.wsb[((size_t)w * s.n + i) * 3 + k] = 0.0;  // history zeroed
      }
      const int tot = block_queue(touch, threadIdx.x, q, wcnt);
      if (threadIdx.x < tot) {
        const int ii = base + q[threadIdx.x];
        double *wsb = B.wsb + ((size_t)w * s.n + ii) * 3;
        VjpIn a;
        wall_in(s, x, w, ii, vh, wh, ws_before, a);
        a.upd = upd != 0;
        VjpBar bb;
        for (int k = 0; k < 3; k++) {
          bb.F[k] = B.Fb[3 * ii + k] + (w == seed_w && k == s.pax[w] ? seed : 0.0);
          bb.Ti[k] = B.Tb[3 * ii + k];
          bb.Tj[k] = 0.0;
          bb.s3[k] = upd ? wsb[k] : 0.0;
        }
        law_vjp<ROLL>(a, bb);
        for (int k = 0; k < 3; k++) {
          if (k == s.pax[w]) B.xb[3 * ii + k] += bb.d[k];  // off-axis components of d are constants
          B.vb[3 * ii + k] += bb.vr[k];
          B.wb[3 * ii + k] += bb.wi[k];
          wsb[k] = bb.sh[k] + (upd ? 0.0 : wsb[k]);
        }
        B.rb[ii] += bb.ri;
        B.mb[ii] += bb.mi;
        B.wth[kTh * ii + 0] += bb.Y;
        B.wth[kTh * ii + 1] += bb.G;
        B.wth[kTh * ii + 2] += bb.beta;
        B.wth[kTh * ii + 3] += bb.mu;
        B.wth[kTh * ii + 4] += bb.mur;
      }
      __syncthreads();
    }
    if (MESH && valid) {  // mesh walls, per atom (the planes' writes are behind the barrier)
      double Fb[3], Tb[3], xb[3] = {0., 0., 0.}, vb[3] = {0., 0., 0.}, wb[3] = {0., 0., 0.};
      double rb = 0.0, mb = 0.0, th[kTh] = {0., 0., 0., 0., 0.};
      for (int k = 0; k < 3; k++) {
        Fb[k] = B.Fb[3 * i + k];
        Tb[k] = B.Tb[3 * i + k];
      }
      amesh_vjp<ROLL>(s, B, i, x, vh, wh, upd, ntimestep, seed_w - s.nplanes, seed_axis, seed, tmst, tmsh, tmnp, Fb,
                      Tb, xb, vb, wb, rb, mb, th);
      for (int k = 0; k < 3; k++) {
        B.xb[3 * i + k] += xb[k];
        B.vb[3 * i + k] += vb[k];
        B.wb[3 * i + k] += wb[k];
      }
      B.rb[i] += rb;
      B.mb[i] += mb;
      for (int k = 0; k < kTh; k++) B.wth[kTh * i + k] += th[k];
    }
  }
}

// reverse of ka_pair_force for one evaluation at positions x (vh/wh the
// velocities it saw, sh_before/bh_before the history before it); the input
// adjoints of each entry go to the per-entry arrays, the history adjoints
// B.sb/B.bb are replaced by those of the history before the evaluation
template <bool BONDS, bool ROLL>
__global__ void __launch_bounds__(kAB) kb_pairs(ADev s, ABar B, const double *x, const float4 *xf,
                                                const double *vh, const double *wh, const double *sh_before,
                                                const double *bh_before, int upd, long long ntimestep) {
  __shared__ int q[kAB];
  __shared__ int wcnt[kAB / 32];
  ABLOCKS(base, s.np) {
    const int p0 = base + threadIdx.x;
    bool work = false;
    if (p0 < s.np) {  // entries without a law evaluation: no input adjoints
      bool band = false;
      if (xf) {  // FP32 candidate test (beyond it: not touching, not in the band)
        work = pair_candidate(s, xf, p0);
      } else {
        const VjpIn a = pair_in(s, x, p0, vh, wh, sh_before);
        const bool touch = pair_touch(a);
        band = pair_band(s, a);
        work = touch || (BONDS && band);
      }
      if (!work) {
        for (int k = 0; k < 3; k++) {
          B.pd[3 * p0 + k] = B.pv[3 * p0 + k] = B.pwi[3 * p0 + k] = B.pwj[3 * p0 + k] = 0.0;
          if (band) B.sb[3 * p0 + k] = 0.0;  // history cleared: no dependence
        }  // else: history unchanged, its adjoint passes through
        B.pri[p0] = B.prj[p0] = B.pmi[p0] = B.pmj[p0] = 0.0;
      }
    }
    const int tot = block_queue(work, p0, q, wcnt);
    if (threadIdx.x < tot) {
      const int p = q[threadIdx.x];
      VjpIn a = pair_in(s, x, p, vh, wh, sh_before);
      a.upd = upd != 0;
      const int i = s.pi[p], j = s.pj[p];
      const bool local = s.sh[p] == kNoShift;
      const bool touch = pair_touch(a), band = pair_band(s, a);
      double Fb[3], Tib[3], Tjb[3];
      for (int k = 0; k < 3; k++) {
        Fb[k] = B.Fb[3 * i + k] - (local ? B.Fb[3 * j + k] : 0.0);
        Tib[k] = B.Tb[3 * i + k];
        Tjb[k] = local ? B.Tb[3 * j + k] : 0.0;
      }
      double d[3] = {0., 0., 0.}, vr[3] = {0., 0., 0.}, wi[3] = {0., 0., 0.}, wj[3] = {0., 0., 0.};
      double ri = 0.0, rj = 0.0, mi = 0.0, mj = 0.0, th[kTh] = {0., 0., 0., 0., 0.};
      int st = kBondNone;
      if (BONDS && (touch || band)) {
        const BondArgs b = bond_in(s, a, x, i, ntimestep);
        double hin[kBondValues], houtb[kBondValues], hinb[kBondValues];
        double *bb = B.bb + (size_t)kBondValues * p;
        for (int k = 0; k < kBondValues; k++) {
          hin[k] = bh_before[(size_t)kBondValues * p + k];
          houtb[k] = bb[k];
        }
        BondArgsBar ab;
        st = bond_vjp(b, s.bp, hin, Fb, Tib, Tjb, houtb, ab, hinb);
        for (int k = 0; k < kBondValues; k++) bb[k] = hinb[k];
        for (int k = 0; k < 3; k++) {
          d[k] += ab.d[k];
          vr[k] += ab.vr[k];
          wi[k] += ab.wi[k];
          wj[k] += ab.wj[k];
        }
        ri += ab.ri;
        rj += ab.rj;
      }
      if (touch) {
        a.bonded = st == kBondActive;
        VjpBar bb;
        for (int k = 0; k < 3; k++) {
          bb.F[k] = Fb[k];
          bb.Ti[k] = Tib[k];
          bb.Tj[k] = Tjb[k];
          bb.s3[k] = upd ? B.sb[3 * p + k] : 0.0;
        }
        law_vjp<ROLL>(a, bb);
        for (int k = 0; k < 3; k++) {
          d[k] += bb.d[k];
          vr[k] += bb.vr[k];
          wi[k] += bb.wi[k];
          wj[k] += bb.wj[k];  // F_i and T_i depend on w_j for periodic images too
          B.sb[3 * p + k] = bb.sh[k] + (upd ? 0.0 : B.sb[3 * p + k]);
        }
        ri += bb.ri;
        rj += bb.rj;
        mi += bb.mi;
        mj += bb.mj;
        th[0] = bb.Y;
        th[1] = bb.G;
        th[2] = bb.beta;
        th[3] = bb.mu;
        th[4] = bb.mur;
      } else if (band) {
        for (int k = 0; k < 3; k++) B.sb[3 * p + k] = 0.0;  // history cleared: no dependence
      }
      for (int k = 0; k < 3; k++) {
        B.pd[3 * p + k] = d[k];
        B.pv[3 * p + k] = vr[k];
        B.pwi[3 * p + k] = wi[k];
        B.pwj[3 * p + k] = wj[k];
      }
      B.pri[p] = ri;
      B.prj[p] = rj;
      B.pmi[p] = mi;
      B.pmj[p] = mj;
      for (int k = 0; k < kTh; k++) B.pth[kTh * p + k] += th[k];  // summed over the segment's steps
    }
    __syncthreads();
  }
}

// per atom: pair adjoints in list order (own row, then reverse list), then
// the drift x' = x + dt vh and the first half-kick vh = v + a F, wh = w + b T
// with Fn/Tn the forces at the step's start; drift = 0 for the setup pass
__global__ void kb_gather_kick(ADev s, ABar B, const double *Fn, const double *Tn, int drift) {
  AGRID(i, s.n) {
    double xb[3], vb[3], wb[3], rb = 0.0, mb = 0.0;
    for (int k = 0; k < 3; k++) {
      xb[k] = B.xb[3 * i + k];
      vb[k] = B.vb[3 * i + k];
      wb[k] = B.wb[3 * i + k];
    }
    for (int p = s.row[i]; p < s.row[i + 1]; p++) {
      for (int k = 0; k < 3; k++) {
        xb[k] += B.pd[3 * p + k];
        vb[k] += B.pv[3 * p + k];
        wb[k] += B.pwi[3 * p + k];
      }
      rb += B.pri[p];
      mb += B.pmi[p];
    }
    for (int q = s.rev_start[i]; q < s.rev_start[i + 1]; q++) {
      const int p = s.rev[q];
      for (int k = 0; k < 3; k++) {
        xb[k] -= B.pd[3 * p + k];
        vb[k] -= B.pv[3 * p + k];
        wb[k] += B.pwj[3 * p + k];
      }
      rb += B.prj[p];
      mb += B.pmj[p];
    }
    if (!drift) {  // setup force pass: adjoints of the initial state
      for (int k = 0; k < 3; k++) {
        B.xb[3 * i + k] = xb[k];
        B.vb[3 * i + k] = vb[k];
        B.wb[3 * i + k] = wb[k];
      }
      B.rb[i] += rb;
      B.mb[i] += mb;
      continue;
    }
    const double a = s.ka[i], b = s.kb[i];
    double fv = 0.0, tw = 0.0;
    for (int k = 0; k < 3; k++) {
      vb[k] += s.dt * xb[k];
      B.xb[3 * i + k] = xb[k];
      B.vb[3 * i + k] = vb[k];
      B.wb[3 * i + k] = wb[k];
      B.Fb[3 * i + k] = a * vb[k];
      B.Tb[3 * i + k] = b * wb[k];
      fv += Fn[3 * i + k] * vb[k];
      tw += Tn[3 * i + k] * wb[k];
    }
    B.rb[i] += rb - s.kbr[i] * tw;
    B.mb[i] += mb - s.kam[i] * fv - s.kbm[i] * tw;
  }
}

// deterministic sum of cnt rows of kTh doubles: per-block partials, then one
// thread per component adds them in block order into acc
__global__ void kb_reduce_th(const double *in, int cnt, double *part) {
  __shared__ double sm[kTh][kAB];
  double acc[kTh] = {0., 0., 0., 0., 0.};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += gridDim.x * blockDim.x)
    for (int k = 0; k < kTh; k++) acc[k] += in[kTh * q + k];
  for (int k = 0; k < kTh; k++) sm[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int st = kAB / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < kTh; k++) sm[k][threadIdx.x] += sm[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < kTh; k++) part[kTh * blockIdx.x + k] = sm[k][0];
}
__global__ void kb_accum_th(const double *part, int nb, double *acc) {
  if (threadIdx.x >= kTh) return;
  double v = acc[threadIdx.x];
  for (int b = 0; b < nb; b++) v += part[kTh * b + threadIdx.x];
  acc[threadIdx.x] = v;
}

// history adjoints at a build back to the previous list's entries: direct
// copies first, then the flipped copies of old local entries (each old entry
// has at most one source of each kind, so both passes are race-free); bb_new
// and bb_old (bond values) may be null
__global__ void kb_uncarry(int np_new, const int *carry, const double *sb_new, double *sb_old, int flipped,
                           const double *bb_new, double *bb_old) {
  AGRID(p, np_new) {
    const int c = carry[p];
    if (!flipped && c >= 0) {
      for (int k = 0; k < 3; k++) sb_old[3 * c + k] += sb_new[3 * p + k];
      if (bb_new)
        for (int k = 0; k < kBondValues; k++)
          bb_old[(size_t)kBondValues * c + k] += bb_new[(size_t)kBondValues * p + k];
    }
    if (flipped && c <= -2) {
      const int e = -c - 2;
      for (int k = 0; k < 3; k++) sb_old[3 * e + k] -= sb_new[3 * p + k];
      if (bb_new)
        for (int k = 0; k < kBondValues; k++)
          bb_old[(size_t)kBondValues * e + k] +=
              ((k >= 5 && k <= 13) ? -1.0 : 1.0) * bb_new[(size_t)kBondValues * p + k];
    }
  }
}

int grid_of(long n) { return (int)std::max<long>(1, std::min<long>((n + kAB - 1) / kAB, kMaxGrid)); }

// device memory of one run: a bump arena sized by the previous run's demand
// (repeated runs of the same problem allocate nothing), spilling to
// cudaMalloc when a run needs more
struct Arena {
  char *base = nullptr;
  size_t cap = 0, used = 0, want = 0;
  std::vector<void *> spill;
  void *get(size_t bytes) {
    bytes = (std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
    want += bytes;
    if (used + bytes <= cap) {
      void *p = base + used;
      used += bytes;
      return p;
    }
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    spill.push_back(p);
    return p;
  }
  cudaError_t reset() {
    for (void *p : spill) cudaFree(p);
    spill.clear();
    if (want > cap) {
      if (base) cudaFree(base);
      base = nullptr;
      cap = 0;
      const size_t c = want + want / 4;
      cudaError_t e = cudaMalloc(&base, c);
      if (e != cudaSuccess) return e;
      cap = c;
    }
    used = 0;
    want = 0;
    return cudaSuccess;
  }
  void release() {
    for (void *p : spill) cudaFree(p);
    spill.clear();
    if (base) cudaFree(base);
    base = nullptr;
    cap = used = want = 0;
  }
};

}  // namespace

struct dem_adjoint {
  dem_adjoint_config cfg{};
  ADev s{};
  int n = 0;
  std::vector<void *> owned;  // freed with the handle
  Arena arena;                // per-run checkpoints, lists and tape
  cudaStream_t st = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  // the backward pass's replays run on st2, beside the reverse sweeps on st:
  // evq[b] = the replay into tape b is done, evq[2 + b] = the reverse sweep
  // over tape b is done
  cudaStream_t st2 = nullptr;
  cudaEvent_t evq[4] = {nullptr, nullptr, nullptr, nullptr};
  std::string err;
  double *x0 = nullptr, *v0 = nullptr, *w0 = nullptr, *r0 = nullptr;  // initial state
  double rmax0 = 0.0;
  double *xref = nullptr;  // positions at the last build
  double *wallF = nullptr;
  int *scan_tmp = nullptr, *rcnt = nullptr, *rfill = nullptr;
  Sys nosys{};  // the scan helper's gate argument (ungated here)
  int pcap = 0;
  ABar B{};
  double *part = nullptr;
  double last_fwd_ms = 0.0, last_bwd_ms = 0.0;
  int last_nseg = 0, last_maxnp = 0;
  dem_bond_settings bond_settings{};
  int tape_mode = 2;          // 0 replay, 1 record every step, 2 record when it fits
  double tape_max_bytes = 0;  // budget of mode 2 (0: half the free device memory)
  int last_recorded = 0;
  double last_grad_mur = 0.0;  // d(loss)/d(rolling coefficient) of the last gradient
};

#define ATRY(h, call)                                                \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) {                                         \
      (h)->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
      return DEM_ERR_CUDA;                                           \
    }                                                                \
  } while (0)

#define AGET(h, ptr, type, count)                                                \
  do {                                                                           \
    (ptr) = static_cast<type *>((h)->arena.get((size_t)(count) * sizeof(type))); \
    if (!(ptr)) {                                                                \
      (h)->err = "device memory exhausted";                                      \
      return DEM_ERR_CUDA;                                                       \
    }                                                                            \
  } while (0)

namespace {

template <typename T>
cudaError_t dmalloc(std::vector<void *> &owned, T **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
  if (e == cudaSuccess) {
    owned.push_back(q);
    *p = static_cast<T *>(q);
  }
  return e;
}

// per-step record of one segment: positions, half-step velocities and the
// history each force evaluation saw, and its forces; ps: entries per step of
// the pair parts
struct Tape {
  double *x = nullptr, *vh = nullptr, *wh = nullptr, *F = nullptr, *T = nullptr, *ws = nullptr;
  double *sh = nullptr, *bh = nullptr;
  float4 *xf = nullptr;
  int *mst = nullptr, *mnp = nullptr;  // mesh slot state before each evaluation
  double *msh = nullptr;
  size_t ps = 0;
};

struct Checkpoint {
  double *x, *v, *w, *F, *T, *ws;  // state before the segment's first drift
  double *sh0, *bh0;               // the list's history as carried at the build
  int *mst0, *mnp0;                // mesh slot state at the segment's first force evaluation
  double *msh0;
  AList L;
  Tape tape;                       // recorded in the forward pass (tape mode), else replayed
};

// neighbour list of the current positions; old: the previous list (with its
// current history and flags) or np = 0
int build_list(dem_adjoint *h, AList &L, const AList &old, long long step) {
  ADev &s = h->s;
  const int n = h->n;
  const cudaStream_t st = h->st;
  ATRY(h, cudaMemsetAsync(s.cell_count, 0, (s.ncell + 2) * sizeof(int), st));
  ATRY(h, cudaMemsetAsync(s.cell_fill, 0, (s.ncell + 2) * sizeof(int), st));
  ka_cell<<<grid_of(n), kAB, 0, st>>>(s);
  scan_exclusive(h->nosys, s.cell_count, s.cell_start, s.ncell + 1, h->scan_tmp, false, st);
  ka_scatter<<<grid_of(n), kAB, 0, st>>>(s);
  ka_cellsort<<<grid_of(s.ncell), kAB, 0, st>>>(s);
  ka_pairs<false><<<grid_of(n), kAB, 0, st>>>(s, nullptr, nullptr, nullptr, nullptr);
  ATRY(h, cudaMemsetAsync(s.pcount + n, 0, sizeof(int), st));
  AGET(h, L.row, int, n + 1);
  scan_exclusive(h->nosys, s.pcount, L.row, n + 1, h->scan_tmp, false, st);
  int np = 0;
  ATRY(h, cudaMemcpyAsync(&np, L.row + n, sizeof(int), cudaMemcpyDeviceToHost, st));
  ATRY(h, cudaStreamSynchronize(st));
  L.np = np;
  AGET(h, L.pi, int, np);
  AGET(h, L.pj, int, np);
  AGET(h, L.sh, uint8_t, np);
  AGET(h, L.flag, uint8_t, np);
  AGET(h, L.rev_start, int, n + 1);
  AGET(h, L.rev, int, np);
  AGET(h, L.carry, int, np);
  AGET(h, L.shear, double, 3 * (size_t)np);
  if (s.bonds) AGET(h, L.bond, double, (size_t)kBondValues * np);
  ka_pairs<true><<<grid_of(n), kAB, 0, st>>>(s, L.pi, L.pj, L.sh, L.row);
  ATRY(h, cudaMemsetAsync(h->rcnt, 0, (n + 1) * sizeof(int), st));
  ATRY(h, cudaMemsetAsync(h->rfill, 0, (n + 1) * sizeof(int), st));
  if (np > 0) ka_rev_count<<<grid_of(np), kAB, 0, st>>>(np, L.pj, h->rcnt);
  scan_exclusive(h->nosys, h->rcnt, L.rev_start, n + 1, h->scan_tmp, false, st);
  if (np > 0) {
    ka_rev_fill<<<grid_of(np), kAB, 0, st>>>(np, L.pj, L.rev_start, h->rfill, L.rev);
    ka_carry<<<grid_of(np), kAB, 0, st>>>(s, L, old);
  }
  ka_rev_sort<<<grid_of(n), kAB, 0, st>>>(n, L.rev_start, L.rev);
  if (s.nmeshes) {
    const size_t nb = (size_t)s.nmeshes * n;
    AGET(h, L.mcn, int, nb);
    AGET(h, L.mcand, int, nb * kAMC);
    AGET(h, L.mmap, int, nb * kAMC);
    ka_mesh_build<<<grid_of(n), kAB, 0, st>>>(s, step, L.mcn, L.mcand, L.mmap);
  }
  ATRY(h, cudaGetLastError());
  return DEM_OK;
}

void use_list_on(ADev &s, const AList &L, double *shear, double *bond) {
  s.bh = bond;
  s.np = L.np;
  s.pi = L.pi;
  s.pj = L.pj;
  s.sh = L.sh;
  s.flag = L.flag;
  s.row = L.row;
  s.rev_start = L.rev_start;
  s.rev = L.rev;
  s.shear = shear;
  s.mcn = L.mcn;
  s.mcand = L.mcand;
}

void use_list(dem_adjoint *h, const AList &L, double *shear, double *bond) { use_list_on(h->s, L, shear, bond); }

int ensure_pairs(dem_adjoint *h, int np) {
  if (np <= h->pcap) return DEM_OK;
  const int cap = std::max(np, 1024) + std::max(np, 1024) / 4;
  double **d3[] = {&h->s.pF, &h->s.pTi, &h->s.pTj, &h->B.pd, &h->B.pv, &h->B.pwi, &h->B.pwj, &h->B.sb};
  for (double **q : d3) ATRY(h, dmalloc(h->owned, q, 3 * (size_t)cap));
  double **d1[] = {&h->B.pri, &h->B.prj, &h->B.pmi, &h->B.pmj};
  for (double **q : d1) ATRY(h, dmalloc(h->owned, q, (size_t)cap));
  ATRY(h, dmalloc(h->owned, &h->B.pth, kTh * (size_t)cap));
  if (h->s.bonds) ATRY(h, dmalloc(h->owned, &h->B.bb, (size_t)kBondValues * cap));
  ATRY(h, dmalloc(h->owned, &h->s.active, (size_t)cap));
  h->pcap = cap;
  return DEM_OK;
}

// Yeff, Geff, betaeff of one material against itself
// (src/global_properties.cpp: Yeff, Geff, betaeff) and their derivatives
void derive(double E, double nu, double e, double &Y, double &G, double &beta, double &dYdE,
            double &dGdE, double &dbde) {
  Y = 1. / ((1. - nu * nu) / E + (1. - nu * nu) / E);
  G = 1. / (2. * (2. - nu) * (1. + nu) / E + 2. * (2. - nu) * (1. + nu) / E);
  const double lg = std::log(e);
  beta = lg / std::sqrt(lg * lg + M_PI * M_PI);
  dYdE = Y / E;
  dGdE = G / E;
  dbde = (1.0 / e) * (M_PI * M_PI) / std::pow(lg * lg + M_PI * M_PI, 1.5);
}

// one force evaluation of state s on stream st
void force_pass_on(const ADev &s, cudaStream_t st, const double *vh, const double *wh, int upd,
                   long long ntimestep, double *tape_sh, double *tape_bh, double *tape_ws, int final_kick,
                   double *wallF, double *tape_F = nullptr, double *tape_T = nullptr, int *tape_mst = nullptr,
                   double *tape_msh = nullptr, int *tape_mnp = nullptr, NextKick nk = NextKick{}) {
  const int g = grid_of(s.np), ga = grid_of(s.n);
  if (s.np > 0) {
    if (s.bonds && s.rolling) ka_pair_force<true, true><<<g, kAB, 0, st>>>(s, vh, wh, upd, ntimestep, tape_sh, tape_bh);
    else if (s.bonds) ka_pair_force<true, false><<<g, kAB, 0, st>>>(s, vh, wh, upd, ntimestep, tape_sh, tape_bh);
    else if (s.rolling) ka_pair_force<false, true><<<g, kAB, 0, st>>>(s, vh, wh, upd, ntimestep, tape_sh, tape_bh);
    else ka_pair_force<false, false><<<g, kAB, 0, st>>>(s, vh, wh, upd, ntimestep, tape_sh, tape_bh);
  }
#define A_GATHER(R, M)                                                                                        \
  ka_gather<R, M><<<ga, kAB, 0, st>>>(s, vh, wh, upd, final_kick, tape_ws, wallF, tape_F, tape_T, tape_mst, tape_msh, \
                                      tape_mnp, ntimestep, nk)
  if (s.rolling && s.nmeshes) A_GATHER(true, true);
  else if (s.rolling) A_GATHER(true, false);
  else if (s.nmeshes) A_GATHER(false, true);
  else A_GATHER(false, false);
#undef A_GATHER
}

void force_pass(dem_adjoint *h, const double *vh, const double *wh, int upd, long long ntimestep,
                double *tape_sh, double *tape_bh, double *tape_ws, int final_kick, double *wallF,
                double *tape_F = nullptr, double *tape_T = nullptr, int *tape_mst = nullptr,
                double *tape_msh = nullptr, int *tape_mnp = nullptr, NextKick nk = NextKick{}) {
  force_pass_on(h->s, h->st, vh, wh, upd, ntimestep, tape_sh, tape_bh, tape_ws, final_kick, wallF, tape_F, tape_T,
                tape_mst, tape_msh, tape_mnp, nk);
}

void pairs_vjp(dem_adjoint *h, const double *x, const float4 *xf, const double *vh, const double *wh,
               const double *sh_before, const double *bh_before, int upd, long long ntimestep) {
  const ADev &s = h->s;
  if (s.np <= 0) return;
  const int g = grid_of(s.np);
#define A_PAIRS(BD, R) \
  kb_pairs<BD, R><<<g, kAB, 0, h->st>>>(s, h->B, x, xf, vh, wh, sh_before, bh_before, upd, ntimestep)
  if (s.bonds && s.rolling) A_PAIRS(true, true);
  else if (s.bonds) A_PAIRS(true, false);
  else if (s.rolling) A_PAIRS(false, true);
  else A_PAIRS(false, false);
#undef A_PAIRS
}

void walls_vjp(dem_adjoint *h, const double *x, const double *vh, const double *wh, const double *ws_before, int upd,
               int seed_w, double seed, const double *Fn1, const double *Tn1, const int *tmst, const double *tmsh,
               const int *tmnp, long long ntimestep, int seed_axis = -1) {
  const ADev &s = h->s;
  const int g = grid_of(h->n);
#define A_WALLS(R, M) \
  kb_walls<R, M><<<g, kAB, 0, h->st>>>(s, h->B, x, vh, wh, ws_before, upd, seed_w, seed, Fn1, Tn1, tmst, tmsh, tmnp, \
                                       ntimestep, seed_axis)
  if (s.rolling && s.nmeshes) A_WALLS(true, true);
  else if (s.rolling) A_WALLS(true, false);
  else if (s.nmeshes) A_WALLS(false, true);
  else A_WALLS(false, false);
#undef A_WALLS
}

void accumulate(dem_adjoint *h, const double *in, int cnt) {
  if (cnt <= 0) return;
  const int g = std::min(grid_of(cnt), 304);
  kb_reduce_th<<<g, kAB, 0, h->st>>>(in, cnt, h->part);
  kb_accum_th<<<1, 32, 0, h->st>>>(h->part, g, h->B.th);
}

void copyd_on(cudaStream_t st, double *dst, const double *src, size_t count) {
  if (count) cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyDeviceToDevice, st);
}

void copyd(dem_adjoint *h, double *dst, const double *src, size_t count) { copyd_on(h->st, dst, src, count); }

}  // namespace

extern "C" {

int dem_adjoint_create(const dem_adjoint_config *cfg, dem_adjoint **out) {
  if (!cfg || !out) return DEM_ERR_BAD_ARG;
  *out = nullptr;
  if (!(cfg->dt > 0) || !(cfg->skin > 0) || !(cfg->density > 0) || cfg->nplanes < 0 || cfg->nplanes > 8 ||
      !(cfg->poisson > -1.0 && cfg->poisson < 0.5))
    return DEM_ERR_BAD_ARG;
  for (int d = 0; d < 3; d++)
    if (!(cfg->boxhi[d] > cfg->boxlo[d])) return DEM_ERR_BAD_ARG;
  for (int w = 0; w < cfg->nplanes; w++)
    if (cfg->plane_axis[w] < 0 || cfg->plane_axis[w] > 2) return DEM_ERR_BAD_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DEM_ERR_NO_DEVICE;
  dem_adjoint *h = new dem_adjoint();
  h->cfg = *cfg;
  bool ok = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&h->ev[0]) == cudaSuccess && cudaEventCreate(&h->ev[1]) == cudaSuccess;
  for (cudaEvent_t &e : h->evq) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    dem_adjoint_destroy(h);
    return DEM_ERR_CUDA;
  }
  ADev &s = h->s;
  for (int d = 0; d < 3; d++) {
    s.lo[d] = cfg->boxlo[d];
    s.hi[d] = cfg->boxhi[d];
    s.prd[d] = cfg->boxhi[d] - cfg->boxlo[d];
    s.per[d] = cfg->periodic[d] ? 1 : 0;
    s.g[d] = cfg->gravity[d];
  }
  s.gravity_on = cfg->gravity_on ? 1 : 0;
  s.dt = cfg->dt;
  s.skin = cfg->skin;
  s.nplanes = cfg->nplanes;
  for (int w = 0; w < cfg->nplanes; w++) {
    s.pax[w] = cfg->plane_axis[w];
    s.ppos[w] = cfg->plane_pos[w];
  }
  // FixNVESphere: dtf = dt/2 (force units 1), dtfrot = dtf / INERTIA (0.4)
  s.dtf = 0.5 * cfg->dt;
  s.dtfrot = s.dtf / 0.4;
  s.bonds = 0;
  s.cdf = 1.0;
  s.nmeshes = 0;
  s.rolling = 0;
  s.mur = 0.0;
  *out = h;
  return DEM_OK;
}

int dem_adjoint_set_mesh_motion(dem_adjoint *h, int mesh_id, const double *vel) {
  if (!h || h->n || !vel || mesh_id < 0 || mesh_id >= h->s.nmeshes) return DEM_ERR_BAD_ARG;
  AMesh &M = h->s.mesh[mesh_id];
  M.moving = 1;
  for (int k = 0; k < 3; k++) M.vel[k] = vel[k];
  return DEM_OK;
}

int dem_adjoint_set_rolling(dem_adjoint *h, double mur) {
  if (!h || h->n || !(mur >= 0)) return DEM_ERR_BAD_ARG;
  h->s.rolling = 1;
  h->s.mur = mur;
  return DEM_OK;
}

int dem_adjoint_add_mesh(dem_adjoint *h, int ntri, const double *nodes, const unsigned char *edge_active,
                         const unsigned char *corner_active) {
  if (!h || h->n || ntri < 1 || !nodes) return DEM_ERR_BAD_ARG;
  ADev &s = h->s;
  if (s.nmeshes >= kAMeshes) {
    h->err = "at most 4 meshes";
    return DEM_ERR_BAD_ARG;
  }
  MeshHost mh;
  const int rc = mesh_prepare(ntri, nodes, edge_active, corner_active, mh);
  if (rc != DEM_OK) {
    h->err = "mesh preparation failed";
    return rc;
  }
  double *tri;
  int *meta, *cs, *cl;
  ATRY(h, dmalloc(h->owned, &tri, mh.tri.size()));
  ATRY(h, dmalloc(h->owned, &meta, mh.meta.size()));
  ATRY(h, dmalloc(h->owned, &cs, mh.cn_start.size()));
  ATRY(h, dmalloc(h->owned, &cl, std::max<size_t>(1, mh.cn_list.size())));
  ATRY(h, cudaMemcpy(tri, mh.tri.data(), mh.tri.size() * sizeof(double), cudaMemcpyHostToDevice));
  ATRY(h, cudaMemcpy(meta, mh.meta.data(), mh.meta.size() * sizeof(int), cudaMemcpyHostToDevice));
  ATRY(h, cudaMemcpy(cs, mh.cn_start.data(), mh.cn_start.size() * sizeof(int), cudaMemcpyHostToDevice));
  if (!mh.cn_list.empty())
    ATRY(h, cudaMemcpy(cl, mh.cn_list.data(), mh.cn_list.size() * sizeof(int), cudaMemcpyHostToDevice));
  AMesh &M = s.mesh[s.nmeshes++];
  M.moving = 0;
  M.vel[0] = M.vel[1] = M.vel[2] = 0.0;
  M.ntri = ntri;
  M.tri = tri;
  M.meta = meta;
  M.cn_start = cs;
  M.cn_list = cl;
  return DEM_OK;
}

int dem_adjoint_set_bonds(dem_adjoint *h, const double *values, const dem_bond_settings *st) {
  if (!h || !values || !st || h->n) return DEM_ERR_BAD_ARG;
  for (int k = 0; k < kBondTables; k++)
    if (!std::isfinite(values[k])) return DEM_ERR_BAD_ARG;
  for (int k = kBondDampFn; k <= kBondDampTt; k++)
    if (values[k] < 0.0 || values[k] > 1.0) return DEM_ERR_BAD_ARG;
  if (st->stressBreak && values[kBondKfn2] <= 1e-15) {
    h->err = "stress breakage needs stiffnessPerUnitAreaK_fn2 > 0";
    return DEM_ERR_BAD_ARG;
  }
  ADev &s = h->s;
  for (int k = 0; k < kBondTables; k++) s.bp.t[k] = values[k];
  // the settings as dem_set_bond_params maps them
  int fl = 0;
  if (st->stressBreak) fl |= kBondStressBreak;
  if (st->tensionStress) fl |= kBondTension;
  if (st->compressionStress) fl |= kBondCompression;
  if (st->shearStress) fl |= kBondShear;
  if (st->normalTorqueStress) fl |= kBondNormalTorque;
  if (st->shearTorqueStress) fl |= kBondShearTorque;
  if (st->createBondAlways) fl |= kBondCreateAlways;
  if (st->dampingBond || st->dampingBondSmooth) fl |= kBondDamping;
  if (st->dampingBondSmooth) fl |= kBondDampingSmooth;
  if (st->ratioTCBond) fl |= kBondUseRatioTC;
  s.bp.flags = fl;
  s.ts_create = (long long)(int)st->tsCreate;
  s.bonds = values[kBondLambda] >= 1e-15 ? 1 : 0;
  h->bond_settings = *st;
  return DEM_OK;
}

int dem_adjoint_destroy(dem_adjoint *h) {
  if (!h) return DEM_ERR_BAD_ARG;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->st2) cudaStreamSynchronize(h->st2);
  h->arena.release();
  for (void *p : h->owned) cudaFree(p);
  for (cudaEvent_t e : h->ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : h->evq)
    if (e) cudaEventDestroy(e);
  if (h->st) cudaStreamDestroy(h->st);
  if (h->st2) cudaStreamDestroy(h->st2);
  delete h;
  return DEM_OK;
}

int dem_adjoint_set_state(dem_adjoint *h, int n, const double *x, const double *v, const double *omega,
                          const double *radius) {
  if (!h || n < 1 || !x || !v || !omega || !radius || h->n) return DEM_ERR_BAD_ARG;
  ADev &s = h->s;
  double rmax = 0.0;
  for (int i = 0; i < n; i++) {
    if (!(radius[i] > 0.0)) return DEM_ERR_BAD_ARG;
    rmax = std::max(rmax, radius[i]);
  }
  // contact distance factor of cohesion bond/nonlinear
  // (neighbor->register_contact_dist_factor, connectToProperties,
  // src/cohesion_model_bond_nonlinear.h:330-380) from the smallest radius
  if (s.bonds) {
    double minrad = radius[0];
    for (int i = 1; i < n; i++) minrad = std::min(minrad, radius[i]);
    const dem_bond_settings &bs = h->bond_settings;
    double one;
    if (!bs.stressBreak) {
      one = 1.1 * 0.5 * s.bp.t[kBondMaxDist] / minrad;
    } else {
      double stress = s.bp.t[kBondMaxSigma];
      if (bs.ratioTCBond) stress = std::fmax(stress, stress * s.bp.t[kBondRatioTC]);
      one = 0.5 * 1.1 * s.bp.t[kBondCreateDist] / minrad + 0.5 * 1.1 * stress / (s.bp.t[kBondKfn2] * minrad);
    }
    s.cdf = std::max(1.0, one);
    if (s.cdf > 10.0) {
      h->err = "bond distance above 10 particle diameters";
      return DEM_ERR_BAD_ARG;
    }
  }
  // cells at least one neighbour cutoff wide for radii up to 1 % larger
  // than the initial ones
  const double cut = 2.0 * rmax * 1.01 * s.cdf + s.skin;
  long ncell = 1;
  int nc[3];
  for (int d = 0; d < 3; d++) {
    long c = (long)std::floor(s.prd[d] / (cut * (1.0 + 1e-9)));
    c = std::max(1L, std::min(c, 1024L));
    if (s.per[d] && c < 3) return DEM_ERR_BOX;
    nc[d] = (int)c;
    ncell *= c;
  }
  if (ncell > 16000000L) return DEM_ERR_BAD_ARG;
  h->n = n;
  h->rmax0 = rmax;
  s.n = n;
  for (int d = 0; d < 3; d++) {
    s.nc[d] = nc[d];
    s.csz[d] = s.prd[d] / nc[d];
  }
  s.ncell = (int)ncell;
  double **d3[] = {&s.x, &s.v, &s.w, &s.F, &s.T, &h->x0, &h->v0, &h->w0, &h->xref,
                   &h->B.xb, &h->B.vb, &h->B.wb, &h->B.Fb, &h->B.Tb};
  for (double **q : d3) ATRY(h, dmalloc(h->owned, q, 3 * (size_t)n));
  double **d1[] = {&s.r, &s.m, &h->r0, &h->B.rb, &h->B.mb, &s.ka, &s.kb, &s.kam, &s.kbm, &s.kbr};
  for (double **q : d1) ATRY(h, dmalloc(h->owned, q, (size_t)n));
  const size_t W3 = 3 * (size_t)std::max(1, s.nplanes) * n;
  ATRY(h, dmalloc(h->owned, &s.ws, W3));
  ATRY(h, dmalloc(h->owned, &s.xf, (size_t)n));
  // mesh walls: the neighbour cutoff (Neighbor::cutneighmax, (maxrad_i +
  // maxrad_j) cdf + skin) bounds the contacts considered, and static meshes
  // take candidates within r cdf + skin/2 (FixNeighlistMesh::pre_force)
  s.cutneighmax = 2.0 * rmax * s.cdf + s.skin;
  s.mtskin = 0.5 * s.skin;
  if (s.nmeshes) {
    const size_t nb = (size_t)s.nmeshes * n;
    ATRY(h, dmalloc(h->owned, &s.mst, nb * kAMC));
    ATRY(h, dmalloc(h->owned, &s.msh, nb * kAMC * 3));
    ATRY(h, dmalloc(h->owned, &s.mnp, nb));
    ATRY(h, dmalloc(h->owned, &s.mns, nb));
    ATRY(h, dmalloc(h->owned, &h->B.msb, nb * kAMC * 3));
  }
  // the FP32 mirror's margin: coordinates and image shifts below X in size
  // round by at most 2^-24 X each, a difference by 4 such roundings; 4e-6 X
  // is more than ten times the bound on the distance error
  double X = 0.0, P = 0.0;
  for (int d = 0; d < 3; d++) {
    X = std::max(X, std::max(std::fabs(s.lo[d]), std::fabs(s.hi[d])));
    P = std::max(P, s.prd[d]);
    s.prdf[d] = (float)s.prd[d];
  }
  s.fm = (float)(4e-6 * (X + P));
  ATRY(h, dmalloc(h->owned, &h->B.wsb, W3));
  ATRY(h, dmalloc(h->owned, &h->wallF, 3 * (size_t)(s.nplanes + kAMeshes) * n));  // planes, then meshes
  ATRY(h, dmalloc(h->owned, &h->B.wth, kTh * (size_t)n));
  ATRY(h, dmalloc(h->owned, &h->B.th, kTh));
  ATRY(h, dmalloc(h->owned, &h->part, kTh * (size_t)kMaxGrid));
  ATRY(h, dmalloc(h->owned, &s.cell_of, (size_t)n));
  ATRY(h, dmalloc(h->owned, &s.cell_count, (size_t)ncell + 2));
  ATRY(h, dmalloc(h->owned, &s.cell_start, (size_t)ncell + 2));
  ATRY(h, dmalloc(h->owned, &s.cell_fill, (size_t)ncell + 2));
  ATRY(h, dmalloc(h->owned, &s.order, (size_t)n));
  ATRY(h, dmalloc(h->owned, &s.pcount, (size_t)n + 1));
  ATRY(h, dmalloc(h->owned, &h->rcnt, (size_t)n + 1));
  ATRY(h, dmalloc(h->owned, &h->rfill, (size_t)n + 1));
  ATRY(h, dmalloc(h->owned, &s.err, 4));
  const long maxlen = std::max<long>(n + 1, ncell + 2);
  ATRY(h, dmalloc(h->owned, &h->scan_tmp, (size_t)((maxlen + 4095) / 4096 + 2)));
  ATRY(h, cudaMemcpy(h->x0, x, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  ATRY(h, cudaMemcpy(h->v0, v, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  ATRY(h, cudaMemcpy(h->w0, omega, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  ATRY(h, cudaMemcpy(h->r0, radius, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  return DEM_OK;
}

static int adj_run(dem_adjoint *h, double E, double e, double mu, const double *radius, int nsteps,
                   int seg, const dem_adjoint_loss *loss, double *loss_out, double *gE, double *ge,
                   double *gmu, double *gr, bool backward) {
  if (!h || !h->n || nsteps < 1 || seg < 1 || !loss || !loss_out || !(E > 0) || !(e > 0 && e < 1) ||
      !(mu >= 0))
    return DEM_ERR_BAD_ARG;
  if (backward && (!gE || !ge || !gmu || !gr)) return DEM_ERR_BAD_ARG;
  ADev &s = h->s;
  const int n = h->n;
  const cudaStream_t st = h->st;
  std::vector<double> rr(n), mm(n);
  if (radius) {
    for (int i = 0; i < n; i++) rr[i] = radius[i];
  } else {
    ATRY(h, cudaMemcpy(rr.data(), h->r0, n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  for (int i = 0; i < n; i++) {
    if (!(rr[i] > 0) || rr[i] > 1.01 * h->rmax0) return DEM_ERR_BAD_ARG;
    mm[i] = 4.0 * M_PI / 3.0 * rr[i] * rr[i] * rr[i] * h->cfg.density;  // FixDensity: rmass = 4/3 pi r^3 rho
  }
  ATRY(h, cudaStreamSynchronize(st));
  ATRY(h, h->arena.reset());
  double Y, G, beta, dYdE, dGdE, dbde;
  derive(E, h->cfg.poisson, e, Y, G, beta, dYdE, dGdE, dbde);
  s.Y = Y;
  s.G = G;
  s.beta = beta;
  s.mu = mu;
  const size_t S3 = 3 * (size_t)n, W3 = 3 * (size_t)std::max(1, s.nplanes) * n;
  ATRY(h, cudaMemcpyAsync(s.r, rr.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  ATRY(h, cudaMemcpyAsync(s.m, mm.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  ka_consts<<<grid_of(n), kAB, 0, st>>>(s);
  copyd(h, s.x, h->x0, S3);
  copyd(h, s.v, h->v0, S3);
  copyd(h, s.w, h->w0, S3);
  ATRY(h, cudaMemsetAsync(s.ws, 0, W3 * sizeof(double), st));
  const size_t NBM = (size_t)s.nmeshes * n;  // (mesh, atom) slot-state records
  if (s.nmeshes) {  // no mesh contacts before the setup pass
    ATRY(h, cudaMemsetAsync(s.mst, 0xff, NBM * kAMC * sizeof(int), st));
    ATRY(h, cudaMemsetAsync(s.msh, 0, NBM * kAMC * 3 * sizeof(double), st));
    ATRY(h, cudaMemsetAsync(s.mnp, 0, NBM * sizeof(int), st));
    ATRY(h, cudaMemsetAsync(s.mns, 0, NBM * sizeof(int), st));
  }
  ATRY(h, cudaMemsetAsync(s.err, 0, 4 * sizeof(int), st));
  ATRY(h, cudaEventRecord(h->ev[0], st));
  // ------------------------------------------------------------ forward
  // segment k covers steps max(1, kL) .. min(N, (k+1)L - 1); its list is
  // built after the drift of step kL (k >= 1) or at setup (k = 0)
  const int nseg = nsteps / seg + 1;
  std::vector<Checkpoint> cps(nseg);
  // tape mode: 1 records every step in the forward pass (no replay), 0
  // replays each segment from its checkpoint, 2 decides by the budget
  bool record = h->tape_mode == 1;
  size_t tape_budget = 0;
  if (h->tape_mode == 2) {
    size_t fr = 0, tot = 0;
    ATRY(h, cudaMemGetInfo(&fr, &tot));
    const size_t avail = (fr + h->arena.cap) / 2;  // the arena of the previous run is reused
    tape_budget = h->tape_max_bytes > 0 ? std::min((size_t)h->tape_max_bytes, avail) : avail;
  }
  int rc;
  AList none;
  int maxnp = 1;
  for (int k = 0; k < nseg; k++) {
    Checkpoint &c = cps[k];
    const int first = std::max(1, k * seg), last = std::min(nsteps, (k + 1) * seg - 1);
    AGET(h, c.x, double, S3);
    AGET(h, c.v, double, S3);
    AGET(h, c.w, double, S3);
    AGET(h, c.F, double, S3);
    AGET(h, c.T, double, S3);
    AGET(h, c.ws, double, W3);
    if (k == 0) {
      ka_wrap<<<grid_of(n), kAB, 0, st>>>(s);
      rc = build_list(h, c.L, none, 0);
      if (rc) return rc;
      rc = ensure_pairs(h, c.L.np);
      if (rc) return rc;
      use_list(h, c.L, c.L.shear, c.L.bond);
      force_pass(h, s.v, s.w, 0, 0, nullptr, nullptr, nullptr, 0, nullptr);  // Verlet::setup
      copyd(h, h->xref, s.x, S3);
      AGET(h, c.sh0, double, 3 * (size_t)c.L.np);
      copyd(h, c.sh0, c.L.shear, 3 * (size_t)c.L.np);
      if (s.nmeshes) {
        AGET(h, c.mst0, int, NBM * kAMC);
        AGET(h, c.msh0, double, NBM * kAMC * 3);
        AGET(h, c.mnp0, int, NBM);
        ATRY(h, cudaMemcpyAsync(c.mst0, s.mst, NBM * kAMC * sizeof(int), cudaMemcpyDeviceToDevice, st));
        copyd(h, c.msh0, s.msh, NBM * kAMC * 3);
        ATRY(h, cudaMemcpyAsync(c.mnp0, s.mnp, NBM * sizeof(int), cudaMemcpyDeviceToDevice, st));
      }
      if (s.bonds) {
        AGET(h, c.bh0, double, (size_t)kBondValues * c.L.np);
        copyd(h, c.bh0, c.L.bond, (size_t)kBondValues * c.L.np);
      }
    }
    const int nst = last - first + 1;
    if (k == 0 && h->tape_mode == 2) {
      // record every step when the whole tape fits the budget (the pair
      // parts estimated from the first list, with room to grow)
      const size_t pe = (size_t)(1.5 * cps[0].L.np) + 1024;
      const size_t per = (5 * S3 + W3 + 2 * (size_t)n + (3 + (s.bonds ? kBondValues : 0)) * pe) * sizeof(double);
      record = per * (size_t)nsteps <= tape_budget;
    }
    if (record && nst > 0) {
      Tape &T = c.tape;
      AGET(h, T.x, double, S3 * nst);
      AGET(h, T.vh, double, S3 * nst);
      AGET(h, T.wh, double, S3 * nst);
      AGET(h, T.F, double, S3 * nst);
      AGET(h, T.T, double, S3 * nst);
      AGET(h, T.ws, double, W3 * nst);
      AGET(h, T.xf, float4, (size_t)n * nst);
      if (s.nmeshes) {
        AGET(h, T.mst, int, NBM * kAMC * nst);
        AGET(h, T.msh, double, NBM * kAMC * 3 * nst);
        AGET(h, T.mnp, int, NBM * nst);
      }
    }
    copyd(h, c.x, s.x, S3);
    copyd(h, c.v, s.v, S3);
    copyd(h, c.w, s.w, S3);
    copyd(h, c.F, s.F, S3);
    copyd(h, c.T, s.T, S3);
    copyd(h, c.ws, s.ws, W3);
    for (int t = first; t <= last; t++) {
      const bool build = (k > 0 && t == first);
      const int q = t - first;
      Tape &T = c.tape;
      const bool rec = T.x != nullptr;
      if (t == first)  // later steps of the segment: kicked and drifted by the previous gather
        ka_kick_drift<<<grid_of(n), kAB, 0, st>>>(s, build ? nullptr : h->xref, build ? 1 : 0,
                                                  rec ? T.x + S3 * q : nullptr, rec ? T.vh + S3 * q : nullptr,
                                                  rec ? T.wh + S3 * q : nullptr,
                                                  rec ? T.xf + (size_t)n * q : nullptr);
      if (build) {
        rc = build_list(h, c.L, cps[k - 1].L, t);
        if (rc) return rc;
        rc = ensure_pairs(h, c.L.np);
        if (rc) return rc;
        use_list(h, c.L, c.L.shear, c.L.bond);
        copyd(h, h->xref, s.x, S3);
        AGET(h, c.sh0, double, 3 * (size_t)c.L.np);
        copyd(h, c.sh0, c.L.shear, 3 * (size_t)c.L.np);
        if (s.nmeshes) {
          AGET(h, c.mst0, int, NBM * kAMC);
          AGET(h, c.msh0, double, NBM * kAMC * 3);
          AGET(h, c.mnp0, int, NBM);
          ATRY(h, cudaMemcpyAsync(c.mst0, s.mst, NBM * kAMC * sizeof(int), cudaMemcpyDeviceToDevice, st));
          copyd(h, c.msh0, s.msh, NBM * kAMC * 3);
          ATRY(h, cudaMemcpyAsync(c.mnp0, s.mnp, NBM * sizeof(int), cudaMemcpyDeviceToDevice, st));
        }
        if (s.bonds) {
          AGET(h, c.bh0, double, (size_t)kBondValues * c.L.np);
          copyd(h, c.bh0, c.L.bond, (size_t)kBondValues * c.L.np);
        }
      }
      if (rec && q == 0) {  // the pair parts, sized by this segment's list
        T.ps = std::max(1, c.L.np);
        AGET(h, T.sh, double, 3 * T.ps * nst);
        if (s.bonds) AGET(h, T.bh, double, kBondValues * T.ps * nst);
      }
      const bool mrec = rec && s.nmeshes;
      NextKick nk{};
      if (t < last) {
        nk.on = 1;
        nk.xref = h->xref;
        if (rec) {
          nk.tx = T.x + S3 * (q + 1);
          nk.tv = T.vh + S3 * (q + 1);
          nk.tw = T.wh + S3 * (q + 1);
          nk.txf = T.xf + (size_t)n * (q + 1);
        }
      }
      force_pass(h, s.v, s.w, 1, t, rec ? T.sh + 3 * T.ps * q : nullptr,
                 rec && s.bonds ? T.bh + kBondValues * T.ps * q : nullptr, rec ? T.ws + W3 * q : nullptr, 1,
                 t == nsteps ? h->wallF : nullptr, rec ? T.F + S3 * q : nullptr, rec ? T.T + S3 * q : nullptr,
                 mrec ? T.mst + NBM * kAMC * q : nullptr, mrec ? T.msh + NBM * kAMC * 3 * q : nullptr,
                 mrec ? T.mnp + NBM * q : nullptr, nk);
    }
    maxnp = std::max(maxnp, c.L.np);
  }
  ATRY(h, cudaGetLastError());
  int flag = 0, mflag = 0;
  ATRY(h, cudaMemcpyAsync(&flag, s.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  ATRY(h, cudaMemcpyAsync(&mflag, s.err + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  const size_t WF = 3 * (size_t)(s.nplanes + s.nmeshes) * n;
  std::vector<double> xf(S3), vf(S3), wf(S3), wallf(std::max<size_t>(1, WF));
  ATRY(h, cudaMemcpyAsync(xf.data(), s.x, S3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  ATRY(h, cudaMemcpyAsync(vf.data(), s.v, S3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  ATRY(h, cudaMemcpyAsync(wf.data(), s.w, S3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (WF) ATRY(h, cudaMemcpyAsync(wallf.data(), h->wallF, WF * sizeof(double), cudaMemcpyDeviceToHost, st));
  ATRY(h, cudaEventRecord(h->ev[1], st));
  ATRY(h, cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
  h->last_fwd_ms = ms;
  h->last_nseg = nseg;
  h->last_recorded = record ? 1 : 0;
  h->last_maxnp = maxnp;
  if (flag) {
    h->err = "an atom moved more than skin/2 from its position at the list build: use shorter segments or a larger skin";
    return DEM_ERR_BAD_ARG;
  }
  if (mflag) {
    h->err = "an atom has more candidate mesh triangles (or contacts) than its history slots";
    return DEM_ERR_BAD_ARG;
  }
  // loss of the final state
  double ke = 0.0, hz = 0.0, fw = 0.0;
  for (int i = 0; i < n; i++) {
    const double I = 0.4 * mm[i] * rr[i] * rr[i];
    for (int k = 0; k < 3; k++)
      ke += 0.5 * mm[i] * vf[3 * i + k] * vf[3 * i + k] + 0.5 * I * wf[3 * i + k] * wf[3 * i + k];
    hz += xf[3 * i + 2];
  }
  hz /= n;
  const int lw = loss->wall_id;
  const bool use_wall = lw >= 0 && lw < s.nplanes + s.nmeshes;
  if (lw >= s.nplanes && use_wall && (loss->wall_axis < 0 || loss->wall_axis > 2)) {
    h->err = "wall_axis must be 0, 1 or 2 for a mesh";
    return DEM_ERR_BAD_ARG;
  }
  const int wax = lw < s.nplanes ? (use_wall ? s.pax[lw] : 0) : loss->wall_axis;
  if (use_wall)
    for (int i = 0; i < n; i++) fw += wallf[((size_t)lw * n + i) * 3 + wax];
  *loss_out = loss->w_ke * ke + loss->w_height * (hz - loss->height_target) * (hz - loss->height_target) +
              (use_wall ? loss->w_wallforce * (fw - loss->wallforce_target) * (fw - loss->wallforce_target) : 0.0);
  if (!backward) return DEM_OK;
  // ----------------------------------------------------------- backward
  ATRY(h, cudaEventRecord(h->ev[0], st));
  ABar &B = h->B;
  {  // adjoints of the final state
    std::vector<double> xb(S3, 0.0), vb(S3), wb(S3), mb(n), rb(n);
    for (int i = 0; i < n; i++) {
      const double I = 0.4 * mm[i] * rr[i] * rr[i];
      double v2 = 0.0, w2 = 0.0;
      for (int k = 0; k < 3; k++) {
        vb[3 * i + k] = loss->w_ke * mm[i] * vf[3 * i + k];
        wb[3 * i + k] = loss->w_ke * I * wf[3 * i + k];
        v2 += vf[3 * i + k] * vf[3 * i + k];
        w2 += wf[3 * i + k] * wf[3 * i + k];
      }
      xb[3 * i + 2] = loss->w_height * 2.0 * (hz - loss->height_target) / n;
      mb[i] = loss->w_ke * (0.5 * v2 + 0.2 * rr[i] * rr[i] * w2);
      rb[i] = loss->w_ke * 0.4 * mm[i] * rr[i] * w2;
    }
    ATRY(h, cudaMemcpyAsync(B.xb, xb.data(), S3 * sizeof(double), cudaMemcpyHostToDevice, st));
    ATRY(h, cudaMemcpyAsync(B.vb, vb.data(), S3 * sizeof(double), cudaMemcpyHostToDevice, st));
    ATRY(h, cudaMemcpyAsync(B.wb, wb.data(), S3 * sizeof(double), cudaMemcpyHostToDevice, st));
    ATRY(h, cudaMemcpyAsync(B.mb, mb.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    ATRY(h, cudaMemcpyAsync(B.rb, rb.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    ATRY(h, cudaStreamSynchronize(st));  // the host vectors go out of scope
  }
  ATRY(h, cudaMemsetAsync(B.Fb, 0, S3 * sizeof(double), st));
  ATRY(h, cudaMemsetAsync(B.Tb, 0, S3 * sizeof(double), st));
  ATRY(h, cudaMemsetAsync(B.wsb, 0, W3 * sizeof(double), st));
  ATRY(h, cudaMemsetAsync(B.sb, 0, 3 * (size_t)h->pcap * sizeof(double), st));
  if (s.bonds) ATRY(h, cudaMemsetAsync(B.bb, 0, (size_t)kBondValues * h->pcap * sizeof(double), st));
  ATRY(h, cudaMemsetAsync(B.th, 0, kTh * sizeof(double), st));
  ATRY(h, cudaMemsetAsync(B.wth, 0, kTh * (size_t)n * sizeof(double), st));
  const double fw_seed = use_wall ? loss->w_wallforce * 2.0 * (fw - loss->wallforce_target) : 0.0;
  // Replay (tape mode 0): segment k-1 is replayed from its checkpoint on
  // the second stream, with its own state s2 and into one of two tapes,
  // while the reverse sweep of segment k reads the other tape on the
  // handle's stream.  (Segments recorded in the forward pass use their own
  // tape.)
  Tape shared[2];
  ADev s2 = s;
  double *shr2 = nullptr, *bhr2 = nullptr;
  if (!record) {
    for (Tape &tp : shared) {
      tp.ps = (size_t)maxnp;
      AGET(h, tp.x, double, S3 * seg);
      AGET(h, tp.vh, double, S3 * seg);
      AGET(h, tp.wh, double, S3 * seg);
      AGET(h, tp.F, double, S3 * seg);
      AGET(h, tp.T, double, S3 * seg);
      AGET(h, tp.ws, double, W3 * seg);
      AGET(h, tp.sh, double, 3 * (size_t)maxnp * seg);
      AGET(h, tp.xf, float4, (size_t)n * seg);
      if (s.bonds) AGET(h, tp.bh, double, kBondValues * (size_t)maxnp * seg);
      if (s.nmeshes) {
        AGET(h, tp.mst, int, NBM * kAMC * seg);
        AGET(h, tp.msh, double, NBM * kAMC * 3 * seg);
        AGET(h, tp.mnp, int, NBM * seg);
      }
    }
    // the replay's own positions, velocities, forces, wall and slot
    // histories, FP32 mirror, pair outputs and carried histories
    AGET(h, s2.x, double, S3);
    AGET(h, s2.v, double, S3);
    AGET(h, s2.w, double, S3);
    AGET(h, s2.F, double, S3);
    AGET(h, s2.T, double, S3);
    AGET(h, s2.ws, double, W3);
    AGET(h, s2.xf, float4, (size_t)n);
    AGET(h, s2.pF, double, 3 * (size_t)maxnp);
    AGET(h, s2.pTi, double, 3 * (size_t)maxnp);
    AGET(h, s2.pTj, double, 3 * (size_t)maxnp);
    AGET(h, s2.active, uint8_t, (size_t)maxnp);
    if (s.nmeshes) {
      AGET(h, s2.mst, int, NBM * kAMC);
      AGET(h, s2.msh, double, NBM * kAMC * 3);
      AGET(h, s2.mnp, int, NBM);
    }
    AGET(h, shr2, double, 3 * (size_t)maxnp);
    if (s.bonds) AGET(h, bhr2, double, kBondValues * (size_t)maxnp);
  }
  // replay of segment k into tape T on the second stream, recording the
  // positions, half-step velocities, histories and forces of every step
  auto replay = [&](int k, Tape &T) {
    Checkpoint &c = cps[k];
    const int first = std::max(1, k * seg), last = std::min(nsteps, (k + 1) * seg - 1);
    const cudaStream_t q2 = h->st2;
    copyd_on(q2, s2.x, c.x, S3);
    copyd_on(q2, s2.v, c.v, S3);
    copyd_on(q2, s2.w, c.w, S3);
    copyd_on(q2, s2.F, c.F, S3);
    copyd_on(q2, s2.T, c.T, S3);
    copyd_on(q2, s2.ws, c.ws, W3);
    copyd_on(q2, shr2, c.sh0, 3 * (size_t)c.L.np);
    if (s.bonds) copyd_on(q2, bhr2, c.bh0, (size_t)kBondValues * c.L.np);
    if (s.nmeshes) {
      cudaMemcpyAsync(s2.mst, c.mst0, NBM * kAMC * sizeof(int), cudaMemcpyDeviceToDevice, q2);
      copyd_on(q2, s2.msh, c.msh0, NBM * kAMC * 3);
      cudaMemcpyAsync(s2.mnp, c.mnp0, NBM * sizeof(int), cudaMemcpyDeviceToDevice, q2);
    }
    use_list_on(s2, c.L, shr2, bhr2);
    const size_t PS = T.ps;
    for (int t = first; t <= last; t++) {
      const int q = t - first;
      if (t == first)  // later steps: kicked and drifted by the previous gather
        ka_kick_drift<<<grid_of(n), kAB, 0, q2>>>(s2, nullptr, k > 0 ? 1 : 0, T.x + S3 * q, T.vh + S3 * q,
                                                  T.wh + S3 * q, T.xf + (size_t)n * q);
      NextKick nk{};
      if (t < last) {
        nk.on = 1;
        nk.tx = T.x + S3 * (q + 1);
        nk.tv = T.vh + S3 * (q + 1);
        nk.tw = T.wh + S3 * (q + 1);
        nk.txf = T.xf + (size_t)n * (q + 1);
      }
      force_pass_on(s2, q2, T.vh + S3 * q, T.wh + S3 * q, 1, t, T.sh + 3 * PS * q,
                    s.bonds ? T.bh + kBondValues * PS * q : nullptr, T.ws + W3 * q, 1, nullptr, T.F + S3 * q,
                    T.T + S3 * q, s.nmeshes ? T.mst + NBM * kAMC * q : nullptr,
                    s.nmeshes ? T.msh + NBM * kAMC * 3 * q : nullptr, s.nmeshes ? T.mnp + NBM * q : nullptr, nk);
    }
  };
  // the mesh slot state before the setup pass (empty) and the slot-history
  // adjoints of the previous list at a build
  int *mst_e = nullptr, *mnp_e = nullptr;
  double *msh_e = nullptr, *msb_prev = nullptr;
  if (s.nmeshes) {
    AGET(h, mst_e, int, NBM * kAMC);
    AGET(h, mnp_e, int, NBM);
    AGET(h, msh_e, double, NBM * kAMC * 3);
    AGET(h, msb_prev, double, NBM * kAMC * 3);
    ATRY(h, cudaMemsetAsync(mst_e, 0xff, NBM * kAMC * sizeof(int), st));
    ATRY(h, cudaMemsetAsync(mnp_e, 0, NBM * sizeof(int), st));
    ATRY(h, cudaMemsetAsync(msh_e, 0, NBM * kAMC * 3 * sizeof(double), st));
    ATRY(h, cudaMemsetAsync(B.msb, 0, NBM * kAMC * 3 * sizeof(double), st));
  }
  double *shr, *sb_prev, *tws0;
  AGET(h, shr, double, 3 * (size_t)maxnp);
  AGET(h, sb_prev, double, 3 * (size_t)maxnp);
  AGET(h, tws0, double, W3);
  double *bhr = nullptr, *bb_prev = nullptr;
  const size_t NB = kBondValues * (size_t)maxnp;
  if (s.bonds) {
    AGET(h, bhr, double, NB);
    AGET(h, bb_prev, double, NB);
  }
  const bool replayed = !record;
  if (replayed) {  // the last segment's replay; each earlier one is queued a segment ahead
    ATRY(h, cudaEventRecord(h->evq[2], st));  // the state above is in place before the replays start
    ATRY(h, cudaStreamWaitEvent(h->st2, h->evq[2], 0));
    replay(nseg - 1, shared[(nseg - 1) & 1]);
    ATRY(h, cudaEventRecord(h->evq[(nseg - 1) & 1], h->st2));
  }
  for (int k = nseg - 1; k >= 0; k--) {
    Checkpoint &c = cps[k];
    const int first = std::max(1, k * seg), last = std::min(nsteps, (k + 1) * seg - 1);
    if (replayed && k >= 1) {
      // segment k-1 into the tape of segment k+1, once that one's reverse sweep is done
      if (k + 1 < nseg) ATRY(h, cudaStreamWaitEvent(h->st2, h->evq[2 + ((k + 1) & 1)], 0));
      replay(k - 1, shared[(k - 1) & 1]);
      ATRY(h, cudaEventRecord(h->evq[(k - 1) & 1], h->st2));
    }
    if (replayed) ATRY(h, cudaStreamWaitEvent(st, h->evq[k & 1], 0));
    const Tape &T = replayed ? shared[k & 1] : c.tape;
    const size_t PS = T.ps;
    use_list(h, c.L, shr, bhr);
    // reverse over the segment's steps; the pair parameter adjoints of the
    // segment's list are summed per entry over its steps, then reduced
    if (s.np > 0) ATRY(h, cudaMemsetAsync(B.pth, 0, kTh * (size_t)s.np * sizeof(double), st));
    for (int t = last; t >= first; t--) {
      const int q = t - first;
      const double *xs = T.x + S3 * q, *vh = T.vh + S3 * q, *wh = T.wh + S3 * q;
      walls_vjp(h, xs, vh, wh, T.ws + W3 * q, 1, t == nsteps ? lw : -1, t == nsteps ? fw_seed : 0.0, T.F + S3 * q,
                T.T + S3 * q, s.nmeshes ? T.mst + NBM * kAMC * q : nullptr,
                s.nmeshes ? T.msh + NBM * kAMC * 3 * q : nullptr, s.nmeshes ? T.mnp + NBM * q : nullptr, t,
                loss->wall_axis);
      if (s.np > 0)
        pairs_vjp(h, xs, T.xf + (size_t)n * q, vh, wh, T.sh + 3 * PS * q,
                  s.bonds ? T.bh + kBondValues * PS * q : nullptr, 1, t);
      const double *Fn = q > 0 ? T.F + S3 * (q - 1) : c.F;
      const double *Tn = q > 0 ? T.T + S3 * (q - 1) : c.T;
      kb_gather_kick<<<grid_of(n), kAB, 0, st>>>(s, B, Fn, Tn, 1);
    }
    if (k > 0) accumulate(h, B.pth, s.np);  // segment 0: after the setup pass below
    if (k > 0) {  // history adjoints back through the carry at this build
      const AList &po = cps[k - 1].L;
      ATRY(h, cudaMemsetAsync(sb_prev, 0, 3 * (size_t)std::max(1, po.np) * sizeof(double), st));
      if (s.bonds)
        ATRY(h, cudaMemsetAsync(bb_prev, 0, (size_t)kBondValues * std::max(1, po.np) * sizeof(double), st));
      if (c.L.np > 0) {
        double *bn = s.bonds ? B.bb : nullptr, *bo = s.bonds ? bb_prev : nullptr;
        kb_uncarry<<<grid_of(c.L.np), kAB, 0, st>>>(c.L.np, c.L.carry, B.sb, sb_prev, 0, bn, bo);
        kb_uncarry<<<grid_of(c.L.np), kAB, 0, st>>>(c.L.np, c.L.carry, B.sb, sb_prev, 1, bn, bo);
      }
      copyd(h, B.sb, sb_prev, 3 * (size_t)po.np);
      if (s.bonds) copyd(h, B.bb, bb_prev, (size_t)kBondValues * po.np);
      if (s.nmeshes) {
        ATRY(h, cudaMemsetAsync(msb_prev, 0, NBM * kAMC * 3 * sizeof(double), st));
        kb_mesh_uncarry<<<grid_of((long)NBM), kAB, 0, st>>>((int)NBM, c.L.mmap, B.msb, msb_prev);
        copyd(h, B.msb, msb_prev, NBM * kAMC * 3);
      }
    }
    if (replayed) ATRY(h, cudaEventRecord(h->evq[2 + (k & 1)], st));
  }
  {  // Verlet::setup force pass: initial state, zero history, no update
    Checkpoint &c = cps[0];
    ATRY(h, cudaMemsetAsync(tws0, 0, W3 * sizeof(double), st));
    ATRY(h, cudaMemsetAsync(shr, 0, 3 * (size_t)maxnp * sizeof(double), st));
    if (s.bonds) ATRY(h, cudaMemsetAsync(bhr, 0, NB * sizeof(double), st));
    use_list(h, c.L, shr, bhr);
    walls_vjp(h, c.x, c.v, c.w, tws0, 0, -1, 0.0, nullptr, nullptr, mst_e, msh_e, mnp_e, 0);
    pairs_vjp(h, c.x, nullptr, c.v, c.w, shr, bhr, 0, 0);
    kb_gather_kick<<<grid_of(n), kAB, 0, st>>>(s, B, nullptr, nullptr, 0);
    accumulate(h, B.pth, s.np);  // segment 0's steps and the setup pass
    accumulate(h, B.wth, n);     // every step's wall contacts
  }
  ATRY(h, cudaGetLastError());
  std::vector<double> rb(n), mb(n), th(kTh);
  ATRY(h, cudaMemcpyAsync(rb.data(), B.rb, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  ATRY(h, cudaMemcpyAsync(mb.data(), B.mb, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  ATRY(h, cudaMemcpyAsync(th.data(), B.th, kTh * sizeof(double), cudaMemcpyDeviceToHost, st));
  ATRY(h, cudaEventRecord(h->ev[1], st));
  ATRY(h, cudaStreamSynchronize(st));
  cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
  h->last_bwd_ms = ms;
  for (int i = 0; i < n; i++) gr[i] = rb[i] + mb[i] * 3.0 * mm[i] / rr[i];  // dm/dr = 3 m / r
  *gE = th[0] * dYdE + th[1] * dGdE;
  *ge = th[2] * dbde;
  *gmu = th[3];
  h->last_grad_mur = th[4];
  return DEM_OK;
}

int dem_adjoint_forward(dem_adjoint *h, double E, double restitution, double friction, const double *radius,
                        int nsteps, int segment, const dem_adjoint_loss *loss, double *loss_out) {
  return adj_run(h, E, restitution, friction, radius, nsteps, segment, loss, loss_out, nullptr, nullptr,
                 nullptr, nullptr, false);
}

int dem_adjoint_gradient(dem_adjoint *h, double E, double restitution, double friction, const double *radius,
                         int nsteps, int segment, const dem_adjoint_loss *loss, double *loss_out,
                         double *grad_E, double *grad_restitution, double *grad_friction, double *grad_radius) {
  return adj_run(h, E, restitution, friction, radius, nsteps, segment, loss, loss_out, grad_E, grad_restitution,
                 grad_friction, grad_radius, true);
}

int dem_adjoint_download(dem_adjoint *h, double *x, double *v, double *omega) {
  if (!h || !h->n) return DEM_ERR_BAD_ARG;
  const size_t b = 3 * (size_t)h->n * sizeof(double);
  ATRY(h, cudaStreamSynchronize(h->st));
  if (x) ATRY(h, cudaMemcpy(x, h->s.x, b, cudaMemcpyDeviceToHost));
  if (v) ATRY(h, cudaMemcpy(v, h->s.v, b, cudaMemcpyDeviceToHost));
  if (omega) ATRY(h, cudaMemcpy(omega, h->s.w, b, cudaMemcpyDeviceToHost));
  return DEM_OK;
}

int dem_adjoint_times(dem_adjoint *h, double *forward_ms, double *backward_ms, int *segments, int *max_pairs) {
  if (!h) return DEM_ERR_BAD_ARG;
  if (forward_ms) *forward_ms = h->last_fwd_ms;
  if (backward_ms) *backward_ms = h->last_bwd_ms;
  if (segments) *segments = h->last_nseg;
  if (max_pairs) *max_pairs = h->last_maxnp;
  return DEM_OK;
}

int dem_adjoint_set_tape(dem_adjoint *h, int mode, double max_bytes) {
  if (!h || mode < 0 || mode > 2 || !(max_bytes >= 0)) return DEM_ERR_BAD_ARG;
  h->tape_mode = mode;
  h->tape_max_bytes = max_bytes;
  return DEM_OK;
}

int dem_adjoint_rolling_gradient(dem_adjoint *h, double *grad_mur) {
  if (!h || !grad_mur) return DEM_ERR_BAD_ARG;
  *grad_mur = h->last_grad_mur;
  return DEM_OK;
}

int dem_adjoint_tape_recorded(dem_adjoint *h, int *recorded) {
  if (!h || !recorded) return DEM_ERR_BAD_ARG;
  *recorded = h->last_recorded;
  return DEM_OK;
}

const char *dem_adjoint_last_error(dem_adjoint *h) { return h ? h->err.c_str() : "null handle"; }

}  // extern "C"
