// GB300 kernels of the sphere-DEM timestep.
//
// One step = k_particle (force gather of the previous step + walls + gravity +
// nve/sphere final and initial half-kicks + skin check) -> k_decide ->
// [rebuild kernels, no-ops unless ctrl->rebuild] -> k_pair.  All decisions
// live in device memory (Ctrl), so many steps are queued without a host sync.
//
// Determinism: every force is the sum of per-pair results in a fixed order
// (owner row ascending, then partner list ascending); no floating-point
// atomics anywhere.  Integer atomics are only used for counting; each
// resulting order is made canonical by a per-cell / per-atom sort.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <stdint.h>

#include "bond_law.cuh"
#include "contact_law.cuh"
#include "dem_device.cuh"
#include "dem_kernels.h"
#include "mesh_device.cuh"

namespace gb300 {

#define GRID_STRIDE(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

__device__ __forceinline__ bool gated(const Ctrl *c) { return c->halt != 0 || c->rebuild == 0; }

// Exact reference arithmetic (no contraction) for everything that decides
// membership of the pair set.
__device__ __forceinline__ double rsq_rn(double dx, double dy, double dz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ void shift_decode(int c, int &sx, int &sy, int &sz) {
  sx = c % 3 - 1;
  sy = (c / 3) % 3 - 1;
  sz = c / 9 - 1;
}

// ghost image x_j + pbc*prd exactly as CommBrick::borders/forward_comm
// (src/atom_vec_sphere.cpp:213-223): fl(x + (+-prd)) per shifted dimension.
__device__ __forceinline__ void image(const Sys &s, int code, double &xj, double &yj, double &zj) {
  if (code == kNoShift) return;
  int sx, sy, sz;
  shift_decode(code, sx, sy, sz);
  // +-prd by selection: sx * prd would convert sx to FP64 and multiply on
  // the FP64 pipe (and the compiler hoists that out of candidate loops)
  if (sx) xj = __dadd_rn(xj, sx > 0 ? s.prd[0] : -s.prd[0]);
  if (sy) yj = __dadd_rn(yj, sy > 0 ? s.prd[1] : -s.prd[1]);
  if (sz) zj = __dadd_rn(zj, sz > 0 ? s.prd[2] : -s.prd[2]);
}

// Whether the periodic image of j (shift sv) exists as a ghost atom:
// CommBrick::borders sends an atom across a periodic boundary only when it
// lies within slab_offset + its radius of that boundary (the granular
// criterion of CommBrick::decide, src/comm_brick.cpp:443,1613-1624).  With a
// contact distance factor above 1 this band is narrower than the pair cutoff
// and some periodic pairs near the cutoff do not exist in the reference.
__device__ __forceinline__ bool ghost_exists(const Sys &s, const AtomArrays &A, int j, const int sv[3]) {
  const double rad = A.r[j];
  const double pos[3] = {A.x[j], A.y[j], A.z[j]};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (sv[d] > 0 && !(pos[d] <= __dadd_rn(__dadd_rn(s.boxlo[d], s.ghost_slab), rad))) return false;
    if (sv[d] < 0 && !(pos[d] >= __dadd_rn(__dadd_rn(s.boxhi[d], -s.ghost_slab), -rad))) return false;
  }
  return true;
}

// The cells are wider than the neighbour cutoff by a relative 1e-9 at least,
// far above the rounding of this product, so atoms within the cutoff are
// never more than one cell apart; every kernel bins through this function.
// FP32 image shift -1, 0 or +1 times the period, by selection (no conversion)
__device__ __forceinline__ float fshift(int sv, float prd) { return sv == 0 ? 0.0f : (sv > 0 ? prd : -prd); }

__device__ __forceinline__ int cell_coord(const Sys &s, double x, int d) {
  int c = (int)((x - s.boxlo[d]) * s.icsz[d]);
  c = c < 0 ? 0 : c;
  c = c >= s.nc[d] ? s.nc[d] - 1 : c;
  return c;
}

// ----------------------------------------------------------------------------
// step control
// ----------------------------------------------------------------------------

// Neighbor::decide (src/neighbor.cpp:1362-1376): a fix that forces a
// rebuild at this step (FixMesh::next_reneighbor) comes before the
// ago/every/delay/check logic.  A moving mesh that travelled more than skin/2
// on a step without rebuild forces one at the next step.
// An ensemble decides per system, as each system running alone would; the
// rebuild stage runs when any system rebuilds, and the others keep their
// atom order, list and histories.  Called by every thread of a single
// block (one thread per system at a time); the result is the block's.  The
// displacement flags are read past L1 (the last block of k_particle decides
// while the flags other blocks set may sit stale in its SM's L1).
__device__ __forceinline__ int decide_rebuild(const Sys &s, Ctrl *c) {
  const int force = c->force_rebuild;
  int r_any = 0;
  for (int k = threadIdx.x; k < s.nsys; k += blockDim.x) {
    int r = 1;
    if (!force) {
      const int ago = ++s.sys_ago[k];
      r = (ago >= s.neigh_delay && ago % s.neigh_every == 0) ? (s.neigh_check ? __ldcg(&s.sys_moved[k]) : 1)
                                                             : 0;
    }
    s.sys_reb[k] = r;
    s.sys_moved[k] = 0;
    r_any |= r;
  }
  int reb = __syncthreads_or(r_any);
  if (threadIdx.x == 0) {
    if (force) {
      reb = 1;
    } else if (!s.nsys) {
      c->ago++;
      if (c->ago >= s.neigh_delay && c->ago % s.neigh_every == 0) reb = s.neigh_check ? __ldcg(&c->moved) : 1;
    }
    c->force_rebuild = reb ? 0 : c->mesh_moved;
    c->mesh_moved = 0;
    c->rebuild = reb;
    c->moved = 0;
  }
  return reb;
}

// this atom's system rebuilds at the current rebuild stage
__device__ __forceinline__ bool sys_rebuilds(const Sys &s, int type) { return s.nsys == 0 || s.sys_reb[type - 1]; }

__global__ void k_decide(Sys s) {
  Ctrl *c = s.ctrl;
  if (c->halt) return;
  if (threadIdx.x == 0) c->ntimestep++;
  decide_rebuild(s, c);
}

// k_decide for the graph-resident step loop: also drives the IF node around
// the rebuild and the WHILE node around the whole step.
__global__ void k_decide_loop(Sys s, cudaGraphConditionalHandle hreb, cudaGraphConditionalHandle hloop) {
  Ctrl *c = s.ctrl;
  if (c->halt) {
    if (threadIdx.x == 0) {
      cudaGraphSetConditional(hreb, 0);
      cudaGraphSetConditional(hloop, 0);
    }
    return;
  }
  if (threadIdx.x == 0) c->ntimestep++;
  const int reb = decide_rebuild(s, c);
  if (threadIdx.x == 0) {
    c->loop_left--;
    cudaGraphSetConditional(hreb, reb ? 1u : 0u);
    cudaGraphSetConditional(hloop, c->loop_left > 0 ? 1u : 0u);
  }
}

__global__ void k_set_loop(Sys s, int n) { s.ctrl->loop_left = n; }

__global__ void k_set_rebuild(Sys s, int v) {
  if (s.ctrl->halt) return;
  if (threadIdx.x == 0) {
    s.ctrl->rebuild = v;
    s.ctrl->moved = 0;
  }
  for (int k = threadIdx.x; k < s.nsys; k += blockDim.x) {
    s.sys_reb[k] = v;
    s.sys_moved[k] = 0;
  }
}

__global__ void k_zero_gated(Sys s, int *a, int n) {
  if (gated(s.ctrl)) return;
  GRID_STRIDE(i, n) a[i] = 0;
}

// ----------------------------------------------------------------------------
// exclusive scan (warp-shuffle prefix sums), 4096 items per block
// ----------------------------------------------------------------------------

__device__ __forceinline__ int warp_incl_scan(int x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  return x;
}

// out[k] = sum(in[0..k-1]) within the block's 4096 items; bsum[block] = total.
// gate: 0 always runs; 1 only while the system rebuilds; 2 also not in an
// ensemble rebuild that keeps the other systems in place (Ctrl::pmode)
__device__ __forceinline__ bool scan_gated(const Ctrl *c, int gate) {
  return gate && (gated(c) || (gate == 2 && c->pmode));
}

__global__ void __launch_bounds__(1024) k_scan_blocks(Sys s, const int *__restrict__ in, int *out,
                                                      int len, int *bsum, int gate) {
  if (scan_gated(s.ctrl, gate)) return;
  __shared__ int wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const long base = (long)blockIdx.x * 4096 + 4 * t;
  int v[4], tot = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v[k] = (base + k < len) ? in[base + k] : 0;
    tot += v[k];
  }
  int incl = warp_incl_scan(tot);
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) wsum[lane] = warp_incl_scan(wsum[lane]);
  __syncthreads();
  int run = incl - tot + (w ? wsum[w - 1] : 0);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (base + k < len) out[base + k] = run;
    run += v[k];
  }
  if (t == 1023 && bsum) bsum[blockIdx.x] = run;
}

__global__ void k_scan_add(Sys s, int *out, int len, const int *__restrict__ bsum, int gate) {
  if (scan_gated(s.ctrl, gate)) return;
  const int add = bsum[blockIdx.x];
  const long base = (long)blockIdx.x * 4096;
  for (int k = threadIdx.x; k < 4096; k += blockDim.x)
    if (base + k < len) out[base + k] += add;
}

// ----------------------------------------------------------------------------
// ensemble rebuilds that keep the other systems in place
// ----------------------------------------------------------------------------
//
// A rebuild of an ensemble where only some systems rebuild (Ctrl::pmode)
// runs the rebuild kernels over those systems' atoms, cells and list
// segments alone, through compact indices: atom t of the rebuilding systems
// (prefix sums rpre over rlist), cell u (ens_ncell per system), segment
// entry u (prefix sums cpre of the segments' capacities).  Every other
// system keeps its atoms, cells, list entries, histories and holds where
// they are.  The whole-list path runs instead when a rebuilding system loses
// atoms (the systems behind it would move), and its list layout (Ctrl::lmode
// 0) when a rebuilding system's entries outgrow its segment.  Both paths
// give the same atom order, entries and values for every system.

// largest q in [0, n) with pre[q] <= t (pre ascending from 0, pre[n] > t)
__device__ __forceinline__ int seg_find(const int *pre, int n, int t) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// atom of compact index t (t < nra); systems keep their ranges in pmode
__device__ __forceinline__ int ens_atom(const Sys &s, const Ctrl *c, int t) {
  const int q = seg_find(s.rpre, c->nR, t);
  return s.sys_start[s.rlist[q]] + (t - s.rpre[q]);
}

// list entry of compact segment index u (u < ncr)
__device__ __forceinline__ int ens_entry(const Sys &s, const Ctrl *c, int u) {
  const int q = seg_find(s.cpre, c->nR, u);
  return s.seg_start[s.rlist[q]] + (u - s.cpre[q]);
}

// cell of compact index u (u < nR * ens_ncell)
__device__ __forceinline__ int ens_cell(const Sys &s, int u) {
  return s.rlist[u / s.ens_ncell] * s.ens_ncell + u % s.ens_ncell;
}

__device__ __forceinline__ bool ens_partial(const Sys &s, const Ctrl *c) { return s.nsys && c->pmode; }
__device__ __forceinline__ bool ens_list_partial(const Sys &s, const Ctrl *c) { return s.nsys && c->lmode; }

// exclusive block-wide prefix sum of one int per thread (blockDim.x a
// multiple of 32); *tot = the block's total
__device__ int block_excl_scan(int v, int *tot) {
  __shared__ int ws[32];
  __shared__ int wt;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int incl = warp_incl_scan(v);
  if (lane == 31) ws[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int y = warp_incl_scan(lane < nw ? ws[lane] : 0);
    if (lane < nw) ws[lane] = y;
    if (lane == 31) wt = y;
  }
  __syncthreads();
  const int ex = incl - v + (w ? ws[w - 1] : 0);
  *tot = wt;
  __syncthreads();  // ws and wt are reused by the next call
  return ex;
}

// out[i] = base + sum(in[b..i)) for i in [b, e), and out_end[i] = out[i] +
// in[i] when out_end is set, by one block of 1024 threads in chunks of 4096;
// returns the range's total (every thread)
__device__ int block_range_scan(const int *__restrict__ in, int b, int e, int base, int *out, int *out_end) {
  __shared__ int wsum[32];
  __shared__ int carry;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) carry = base;
  __syncthreads();
  for (int c0 = b; c0 < e; c0 += 4096) {
    const int i0 = c0 + 4 * t;
    int v[4], tot = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[k] = (i0 + k < e) ? in[i0 + k] : 0;
      tot += v[k];
    }
    const int incl = warp_incl_scan(tot);
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) wsum[lane] = warp_incl_scan(wsum[lane]);
    __syncthreads();
    int run = carry + incl - tot + (w ? wsum[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (i0 + k < e) {
        out[i0 + k] = run;
        if (out_end) out_end[i0 + k] = run + v[k];
      }
      run += v[k];
    }
    __syncthreads();  // every thread has read carry and wsum
    if (t == 1023) carry = run;
    __syncthreads();
  }
  const int total = carry - base;
  __syncthreads();
  return total;
}

// Domain::pbc (src/domain.cpp:550-600) of one atom's position, in place;
// true when the atom is then outside the box in any dimension, which
// CommBrick::exchange deletes (src/comm_brick.cpp:784-808)
__device__ __forceinline__ bool pbc_wrap(const Sys &s, double xv[3]) {
  bool lost = false;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (s.periodic[d]) {
      if (xv[d] < s.boxlo[d]) xv[d] = __dadd_rn(xv[d], s.prd[d]);
      if (xv[d] >= s.boxhi[d]) {
        xv[d] = __dadd_rn(xv[d], -s.prd[d]);
        if (xv[d] < s.boxlo[d]) xv[d] = s.boxlo[d];
      }
    }
    if (xv[d] < s.boxlo[d] || xv[d] >= s.boxhi[d]) lost = true;
  }
  return lost;
}

// Compacts the rebuilding systems and picks the path: in place (pmode 1)
// when the list is in segments, some system does not rebuild and the
// whole-list path is not forced.  One block.
__global__ void k_ens_plan(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  __shared__ int cr, ca, cc;
  if (threadIdx.x == 0) cr = ca = cc = 0;
  __syncthreads();
  for (int b = 0; b < s.nsys; b += blockDim.x) {
    const int k = b + threadIdx.x;
    const int r = k < s.nsys ? s.sys_reb[k] : 0;
    const int na = r ? s.sys_start[k + 1] - s.sys_start[k] : 0;
    const int ne = r ? s.seg_start[k + 1] - s.seg_start[k] : 0;
    int tr, ta, te;
    const int xr = block_excl_scan(r, &tr);
    const int xa = block_excl_scan(na, &ta);
    const int xe = block_excl_scan(ne, &te);
    if (r) {
      s.rlist[cr + xr] = k;
      s.rpre[cr + xr] = ca + xa;
      s.cpre[cr + xr] = cc + xe;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      cr += tr;
      ca += ta;
      cc += te;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    s.rpre[cr] = ca;
    s.cpre[cr] = cc;
    c->nR = cr;
    c->nra = ca;
    c->ncr = cc;
    const int part = (c->seg_ok && !s.ens_full && cr < s.nsys) ? 1 : 0;
    c->pmode = part;
    c->lmode = part;
    c->np_new = c->np;
  }
}

// in-place path: a rebuilding system that loses an atom moves every system
// behind it, so the whole-list path takes this rebuild
__global__ void k_ens_lost(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c) || !c->pmode) return;
  const AtomArrays &A = s.atoms[0];
  GRID_STRIDE(t, c->nra) {
    const int i = ens_atom(s, c, t);
    double xv[3] = {A.x[i], A.y[i], A.z[i]};
    if (pbc_wrap(s, xv)) {
      c->pmode = 0;
      c->lmode = 0;
    }
  }
}

__global__ void k_ens_zero_cells(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  if (c->pmode) {
    const int tot = c->nR * s.ens_ncell;
    GRID_STRIDE(u, tot) {
      const int cell = ens_cell(s, u);
      s.cell_count[cell] = 0;
      s.cell_fill[cell] = 0;
    }
  } else {
    GRID_STRIDE(u, s.ncell + 2) {
      s.cell_count[u] = 0;
      s.cell_fill[u] = 0;
    }
  }
}

// the in-place path's block-per-system prefix sums
enum { kEnsScanCells = 0, kEnsScanRowsPartial = 1, kEnsScanRowsFull = 2, kEnsScanRev = 3 };

// atoms of system k after this rebuild's cell sort: [lo, hi)
__device__ __forceinline__ void ens_range(const Sys &s, int k, int &lo, int &hi) {
  lo = s.cell_start[k * s.ens_ncell];
  hi = s.cell_start[(k + 1) * s.ens_ncell];
}

__global__ void __launch_bounds__(1024) k_ens_scan(Sys s, int what) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const PairArrays &M = s.pairs[1];
  bool all = false;
  if (what == kEnsScanCells || what == kEnsScanRowsPartial) {
    if (!(what == kEnsScanCells ? c->pmode : c->lmode)) return;
  } else if (what == kEnsScanRowsFull) {
    if (c->lmode) return;
    all = true;
  } else {
    all = !c->lmode;
  }
  const int nlist = all ? s.nsys : c->nR;
  for (int q = blockIdx.x; q < nlist; q += gridDim.x) {
    const int k = all ? q : s.rlist[q];
    int lo, hi;
    if (what == kEnsScanCells) {
      // the system's cells, from its first atom (its range is unchanged)
      block_range_scan(s.cell_count, k * s.ens_ncell, (k + 1) * s.ens_ncell, s.sys_start[k], s.cell_start, nullptr);
      continue;
    }
    ens_range(s, k, lo, hi);
    if (what == kEnsScanRev) {
      block_range_scan(s.rev_count, lo, hi, s.seg_start[k], M.rev_start, M.reve);
      continue;
    }
    // owner rows: into the system's own segment, or relative (the layout
    // kernel places the segments) on the whole-list path
    const int base = what == kEnsScanRowsPartial ? s.seg_start[k] : 0;
    const int used = block_range_scan(s.pcount, lo, hi, base, M.row, M.rowe);
    if (threadIdx.x == 0) {
      s.seg_used[k] = used;
      if (what == kEnsScanRowsPartial && used > s.seg_start[k + 1] - s.seg_start[k]) c->lmode = 0;
    }
  }
}

// in place for the atoms, whole list for the entries: the systems that do
// not rebuild keep their atoms where they are (perm = identity) and count
// their current rows
__global__ void k_ens_kept(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c) || !c->pmode || c->lmode) return;
  const AtomArrays &A = s.atoms[0];
  const PairArrays &L = s.pairs[0];
  GRID_STRIDE(i, c->n) {
    if (s.sys_reb[A.type[i] - 1]) continue;
    s.pcount[i] = L.rowe[i] - L.row[i];
    s.perm[i] = i;
  }
}

// whole-list path: every system gets a segment of its entries plus slack
// (ens_slack percent and 64 more; none with ens_slack 0), so that later
// rebuilds of it alone stay in place while it grows.  One block.
__global__ void k_ens_layout(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c) || c->lmode) return;
  __shared__ int run;
  if (threadIdx.x == 0) run = 0;
  __syncthreads();
  for (int b = 0; b < s.nsys; b += blockDim.x) {
    const int k = b + threadIdx.x;
    int cap = 0;
    if (k < s.nsys) {
      const long u = s.seg_used[k];
      cap = (int)(u + (u * s.ens_slack) / 100 + (s.ens_slack ? 64 : 0));
    }
    int tot;
    const int x = block_excl_scan(cap, &tot);
    if (k < s.nsys) s.seg_start[k] = run + x;
    __syncthreads();
    if (threadIdx.x == 0) run += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    s.seg_start[s.nsys] = run;
    c->np_new = run;
  }
}

// whole-list path: relative rows into the system's segment
__global__ void k_ens_rows_base(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c) || c->lmode) return;
  const AtomArrays &A = s.atoms[0];
  const PairArrays &M = s.pairs[1];
  GRID_STRIDE(i, c->n_new) {
    const int b = s.seg_start[A.type[i] - 1];
    M.row[i] += b;
    M.rowe[i] += b;
  }
}

__global__ void k_ens_zero_rev(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  if (c->lmode) {
    GRID_STRIDE(t, c->nra) {
      const int i = ens_atom(s, c, t);
      s.rev_count[i] = 0;
      s.rev_fill[i] = 0;
    }
  } else {
    GRID_STRIDE(i, s.nmax + 1) {
      s.rev_count[i] = 0;
      s.rev_fill[i] = 0;
    }
  }
}

// unused entries at the end of each (rebuilt) segment
__global__ void k_ens_holes(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const PairArrays &M = s.pairs[1];
  const bool part = c->lmode;
  const int nlist = part ? c->nR : s.nsys;
  for (int q = blockIdx.x; q < nlist; q += gridDim.x) {
    const int k = part ? s.rlist[q] : q;
    for (int p = s.seg_start[k] + s.seg_used[k] + threadIdx.x; p < s.seg_start[k + 1]; p += blockDim.x) {
      M.i[p] = -1;
      M.j[p] = -1;
      M.sh[p] = (uint8_t)kHole;
      M.flag[p] = 0;
    }
  }
}

// ----------------------------------------------------------------------------
// rebuild: pbc wrap, cell sort, permutation
// ----------------------------------------------------------------------------

// Domain::pbc then CommBrick::exchange deletion of atoms outside the box
// (pbc_wrap), and the atoms' neighbour cells.
__device__ __forceinline__ void cell_count_atom(const Sys &s, const AtomArrays &A, int i) {
  double xv[3] = {A.x[i], A.y[i], A.z[i]};
  const bool lost = pbc_wrap(s, xv);
  A.x[i] = xv[0];
  A.y[i] = xv[1];
  A.z[i] = xv[2];
  int cell = s.ncell;
  if (!lost) {
    const int cx = cell_coord(s, xv[0], 0), cy = cell_coord(s, xv[1], 1), cz = cell_coord(s, xv[2], 2);
    cell = cx + s.nc[0] * (cy + s.nc[1] * cz) + (s.ens_ncell ? (A.type[i] - 1) * s.ens_ncell : 0);
  }
  s.pcount[i] = cell;  // reused as per-atom cell id until the pair count
  atomicAdd(&s.cell_count[cell], 1);
}

__global__ void k_cell_count(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const AtomArrays &A = s.atoms[0];
  if (ens_partial(s, c)) {
    GRID_STRIDE(t, c->nra) cell_count_atom(s, A, ens_atom(s, c, t));
    return;
  }
  const int n = c->n;
  // a system that does not rebuild keeps its atoms in order in its first
  // cell: its count is set once, not added per atom
  GRID_STRIDE(k, s.nsys)
    if (!s.sys_reb[k]) s.cell_count[k * s.ens_ncell] = s.sys_start[k + 1] - s.sys_start[k];
  GRID_STRIDE(i, n) {
    if (!sys_rebuilds(s, A.type[i])) {
      s.pcount[i] = (A.type[i] - 1) * s.ens_ncell;
      continue;
    }
    cell_count_atom(s, A, i);
  }
}

__global__ void k_cell_scatter(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const AtomArrays &A = s.atoms[0];
  if (ens_partial(s, c)) {
    GRID_STRIDE(t, c->nra) {
      const int i = ens_atom(s, c, t);
      const int cell = s.pcount[i];
      s.order[s.cell_start[cell] + atomicAdd(&s.cell_fill[cell], 1)] = i;
    }
    return;
  }
  const int n = c->n;
  GRID_STRIDE(i, n) {
    const int cell = s.pcount[i];
    int slot;
    if (!sys_rebuilds(s, A.type[i])) slot = s.cell_start[cell] + (i - s.sys_start[A.type[i] - 1]);
    else slot = s.cell_start[cell] + atomicAdd(&s.cell_fill[cell], 1);
    s.order[slot] = i;
  }
}

// canonical order inside every cell: ascending previous index
__device__ __forceinline__ void cell_sort_one(const Sys &s, int cell) {
  const int b = s.cell_start[cell], e = s.cell_start[cell + 1];
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

__global__ void k_cell_sort(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  if (ens_partial(s, c)) {
    const int tot = c->nR * s.ens_ncell;
    GRID_STRIDE(u, tot) cell_sort_one(s, ens_cell(s, u));
  } else {
    GRID_STRIDE(cell, s.ncell) {
      if (s.nsys && !s.sys_reb[cell / s.ens_ncell]) continue;  // already in order
      cell_sort_one(s, cell);
    }
  }
  // (in place, cell_start[ncell] is the atom count of the last whole build
  // and no atom is lost)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    c->n_new = s.cell_start[s.ncell];
    c->nmlist = 0;
    c->lost_step = c->n - c->n_new;
  }
}

// gather atoms into the new order (buffer 1), xhold = x, primitive-wall
// neighbour lists (PrimitiveWall::buildNeighList, src/primitive_wall.h:129-138)
__device__ __forceinline__ void permute_atom(const Sys &s, const AtomArrays &A, const AtomArrays &B, int i) {
  {
    const int o = s.order[i];
    s.perm[i] = o;
    const bool reb = sys_rebuilds(s, A.type[o]);
    const double x = A.x[o], y = A.y[o], z = A.z[o];
    B.x[i] = x; B.y[i] = y; B.z[i] = z;
    if (reb) {
      B.xh[i] = x; B.yh[i] = y; B.zh[i] = z;
    } else {  // a system that does not rebuild keeps its holds
      B.xh[i] = A.xh[o]; B.yh[i] = A.yh[o]; B.zh[i] = A.zh[o];
    }
    B.vx[i] = A.vx[o]; B.vy[i] = A.vy[o]; B.vz[i] = A.vz[o];
    B.wx[i] = A.wx[o]; B.wy[i] = A.wy[o]; B.wz[i] = A.wz[o];
    // f and torque are not moved: a rebuild comes after the step's initial
    // integration, and the step's gather writes them again before they are
    // read (they are live only between dem_step calls)
    const double r = A.r[o];
    B.r[i] = r; B.m[i] = A.m[o]; B.dtfm[i] = A.dtfm[o]; B.dtir[i] = A.dtir[o];
    B.type[i] = A.type[o]; B.tag[i] = A.tag[o]; B.lidx[i] = A.lidx[o];
    uint8_t bits = 0;
    for (int w = 0; w < s.nplanes; w++) {
      for (int d = 0; d < 3; d++)
        B.whist[(size_t)(w * 3 + d) * s.nmax + i] = A.whist[(size_t)(w * 3 + d) * s.nmax + o];
      const Plane &pl = s.planes[w];
      const double dMax = __dadd_rn(r, s.skin);
      if (pl.kind == 1) {
        // Cylinder<dim>::resolveNeighlist (src/primitive_wall_definitions.h:192-198)
        const double xo[3] = {x, y, z};
        const double dy = __dadd_rn(xo[(pl.axis + 1) % 3], -pl.c1), dz = __dadd_rn(xo[(pl.axis + 2) % 3], -pl.c2);
        const double dist = __dadd_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dz, dz))), -pl.pos);
        if (dMax < dist || -dMax < dist) bits |= (uint8_t)(1u << w);
        continue;
      }
      const double pos = pl.axis == 0 ? x : (pl.axis == 1 ? y : z);
      const double dist = pos - plane_pos(pl, A.type[o]);
      const double absdist = (dist > 0.0) ? dist : -dist;
      if (absdist <= dMax) bits |= (uint8_t)(1u << w);
    }
    B.wbits[i] = reb ? bits : A.wbits[o];
    for (int k = 0; k < s.nmeshes; k++) {  // FixContactHistoryMesh per-atom slots travel too
      const MeshDev &M = s.meshes[k];
      const int ns = M.nslot[0][o];
      M.nslot[1][i] = ns;
      M.npart[1][i] = M.npart[0][o];
      for (int q = 0; q < ns; q++) {
        M.slot_tri[1][(size_t)q * s.nmax + i] = M.slot_tri[0][(size_t)q * s.nmax + o];
        for (int d = 0; d < 3; d++)
          M.slot_hist[1][(size_t)(3 * q + d) * s.nmax + i] = M.slot_hist[0][(size_t)(3 * q + d) * s.nmax + o];
      }
    }
  }
}

__global__ void k_permute(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const AtomArrays &A = s.atoms[0];
  const AtomArrays &B = s.atoms[1];
  if (ens_partial(s, c)) {
    GRID_STRIDE(t, c->nra) permute_atom(s, A, B, ens_atom(s, c, t));
    return;
  }
  const int n = c->n_new;
  GRID_STRIDE(i, n) permute_atom(s, A, B, i);
}

__device__ __forceinline__ void copy_atom(const Sys &s, const AtomArrays &A, const AtomArrays &B, int i) {
  {
    A.x[i] = B.x[i]; A.y[i] = B.y[i]; A.z[i] = B.z[i];
    A.xh[i] = B.xh[i]; A.yh[i] = B.yh[i]; A.zh[i] = B.zh[i];
    A.vx[i] = B.vx[i]; A.vy[i] = B.vy[i]; A.vz[i] = B.vz[i];
    A.wx[i] = B.wx[i]; A.wy[i] = B.wy[i]; A.wz[i] = B.wz[i];
    A.r[i] = B.r[i]; A.m[i] = B.m[i]; A.dtfm[i] = B.dtfm[i]; A.dtir[i] = B.dtir[i];
    A.type[i] = B.type[i]; A.tag[i] = B.tag[i]; A.lidx[i] = B.lidx[i];
    const float4 xf = make_float4((float)B.x[i], (float)B.y[i], (float)B.z[i], (float)B.r[i]);
    s.xf[i] = xf;
    // xhold = x at this build (k_permute), or kept by a system that did not rebuild
    s.xhf[i] = sys_rebuilds(s, B.type[i]) ? xf : make_float4((float)B.xh[i], (float)B.yh[i], (float)B.zh[i], xf.w);
    for (int w = 0; w < s.nplanes; w++)
      for (int d = 0; d < 3; d++)
        A.whist[(size_t)(w * 3 + d) * s.nmax + i] = B.whist[(size_t)(w * 3 + d) * s.nmax + i];
    A.wbits[i] = B.wbits[i];
    for (int k = 0; k < s.nmeshes; k++) {
      const MeshDev &M = s.meshes[k];
      const int ns = M.nslot[1][i];
      M.nslot[0][i] = ns;
      M.npart[0][i] = M.npart[1][i];
      for (int q = 0; q < ns; q++) {
        M.slot_tri[0][(size_t)q * s.nmax + i] = M.slot_tri[1][(size_t)q * s.nmax + i];
        for (int d = 0; d < 3; d++)
          M.slot_hist[0][(size_t)(3 * q + d) * s.nmax + i] = M.slot_hist[1][(size_t)(3 * q + d) * s.nmax + i];
      }
    }
  }
}

__global__ void k_copy_atoms(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const AtomArrays &A = s.atoms[0];
  const AtomArrays &B = s.atoms[1];
  if (ens_partial(s, c)) {
    GRID_STRIDE(t, c->nra) copy_atom(s, A, B, ens_atom(s, c, t));
    return;
  }
  const int n = c->n_new;
  GRID_STRIDE(i, n) copy_atom(s, A, B, i);
}

// ----------------------------------------------------------------------------
// rebuild: triangle-mesh candidate lists (FixNeighlistMesh::pre_force) and
// history slot maintenance (FixContactHistoryMesh::pre_exchange/pre_force)
// ----------------------------------------------------------------------------

__device__ __forceinline__ void mslot_swap(const MeshDev &M, size_t nmax, int i, int a, int b) {
  const int t = M.slot_tri[0][a * nmax + i];
  M.slot_tri[0][a * nmax + i] = M.slot_tri[0][b * nmax + i];
  M.slot_tri[0][b * nmax + i] = t;
  for (int d = 0; d < 3; d++) {
    const double h = M.slot_hist[0][(3 * a + d) * nmax + i];
    M.slot_hist[0][(3 * a + d) * nmax + i] = M.slot_hist[0][(3 * b + d) * nmax + i];
    M.slot_hist[0][(3 * b + d) * nmax + i] = h;
  }
}

// MeshMoverLinear::initial_integrate + MultiNodeMesh::move (nodes and
// centres += dx, src/multi_node_mesh_I.h:502-520), then
// MultiNodeMesh::decideRebuild (any node > skin/2 from its position at the
// last build, src/multi_node_mesh_I.h:792-823); the decision is used by
// k_decide only on steps that do not rebuild anyway (FixMesh::pre_force).
// MathExtra::quatquat (src/math_extra.h:596-602) and
// MathExtraLiggghts::vec_quat_rotate (src/math_extra_liggghts.h:455-471) in
// the reference's operation order, exactly rounded: rotated nodes are
// bit-identical to the reference's
__device__ __forceinline__ void quatquat_rn(const double *a, const double *b, double *c) {
  c[0] = __dsub_rn(__dsub_rn(__dsub_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2])),
                   __dmul_rn(a[3], b[3]));
  c[1] = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[0], b[1]), __dmul_rn(b[0], a[1])), __dmul_rn(a[2], b[3])),
                   __dmul_rn(a[3], b[2]));
  c[2] = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[0], b[2]), __dmul_rn(b[0], a[2])), __dmul_rn(a[3], b[1])),
                   __dmul_rn(a[1], b[3]));
  c[3] = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[0], b[3]), __dmul_rn(b[0], a[3])), __dmul_rn(a[1], b[2])),
                   __dmul_rn(a[2], b[1]));
}
__device__ __forceinline__ void vec_quat_rotate_rn(double *v, const double *q) {
  const double vq[4] = {0., v[0], v[1], v[2]};
  const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
  double t[4], r[4];
  quatquat_rn(q, vq, t);
  quatquat_rn(t, qc, r);
  v[0] = r[1];
  v[1] = r[2];
  v[2] = r[3];
}

// MeshMoverRotate::initial_integrate (src/mesh_mover_rotation.cpp:105-131):
// nodes and centres (MultiNodeMesh::rotate(dQ, origin),
// src/multi_node_mesh_I.h:643-668), the rotating element vectors edgeVec,
// edgeNorm, surfaceNorm (CustomValueTracker::rotate), node velocities
// 0 + w x (node - O); then the node-travel test of decideRebuild
__global__ void k_mesh_rotate(Sys s, int k) {
  Ctrl *c = s.ctrl;
  if (c->halt) return;
  const MeshDev &M = s.meshes[k];
  const double trigger = __dmul_rn(__dmul_rn(0.25, s.skin), s.skin);
  const double *o = M.rorig, *q = M.rq, *w = M.romega;
  const bool trans = __dadd_rn(__dadd_rn(__dmul_rn(o[0], o[0]), __dmul_rn(o[1], o[1])), __dmul_rn(o[2], o[2])) > 0.;
  const double third = 1. / 3.;
  bool moved = false;
  GRID_STRIDE(t, M.ntri) {
    double *g = M.tri + (size_t)t * kTriStride;
    double cen[3] = {0., 0., 0.};
    for (int j = 0; j < 3; j++) {
      double nd[3] = {g[3 * j], g[3 * j + 1], g[3 * j + 2]};
      if (trans)
        for (int d = 0; d < 3; d++) nd[d] = __dsub_rn(nd[d], o[d]);
      vec_quat_rotate_rn(nd, q);
      if (trans)
        for (int d = 0; d < 3; d++) nd[d] = __dadd_rn(nd[d], o[d]);
      double dsq = 0.0;
      for (int d = 0; d < 3; d++) {
        g[3 * j + d] = nd[d];
        cen[d] = __dadd_rn(nd[d], cen[d]);
        const double e = __dadd_rn(nd[d], -M.node_last[(size_t)t * 9 + 3 * j + d]);
        dsq = d == 0 ? __dmul_rn(e, e) : __dadd_rn(dsq, __dmul_rn(e, e));
      }
      moved |= dsq > trigger;
      const double r[3] = {__dsub_rn(nd[0], o[0]), __dsub_rn(nd[1], o[1]), __dsub_rn(nd[2], o[2])};
      double *v = M.nodev + (size_t)t * 9 + 3 * j;
      v[0] = __dadd_rn(0.0, __dsub_rn(__dmul_rn(w[1], r[2]), __dmul_rn(w[2], r[1])));
      v[1] = __dadd_rn(0.0, __dsub_rn(__dmul_rn(w[2], r[0]), __dmul_rn(w[0], r[2])));
      v[2] = __dadd_rn(0.0, __dsub_rn(__dmul_rn(w[0], r[1]), __dmul_rn(w[1], r[0])));
    }
    for (int d = 0; d < 3; d++) g[33 + d] = __dmul_rn(third, cen[d]);
    for (int j = 0; j < 3; j++) vec_quat_rotate_rn(g + 9 + 3 * j, q);   // edgeVec
    for (int j = 0; j < 3; j++) vec_quat_rotate_rn(g + 18 + 3 * j, q);  // edgeNorm
    vec_quat_rotate_rn(g + 30, q);                                      // surfaceNorm
    M.trif[2 * (size_t)t] = make_float4((float)g[0], (float)g[1], (float)g[2], 0.f);
    M.trif[2 * (size_t)t + 1] = make_float4((float)g[30], (float)g[31], (float)g[32], 0.f);
  }
  if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(&c->mesh_moved, 1);
}

__global__ void k_mesh_move(Sys s, int k) {
  Ctrl *c = s.ctrl;
  if (c->halt) return;
  const MeshDev &M = s.meshes[k];
  const double trigger = __dmul_rn(__dmul_rn(0.25, s.skin), s.skin);
  bool moved = false;
  GRID_STRIDE(t, M.ntri) {
    double *g = M.tri + (size_t)t * kTriStride;
    for (int q = 0; q < 3; q++) {
      double dsq = 0.0;
      for (int d = 0; d < 3; d++) {
        const double x = __dadd_rn(g[3 * q + d], M.dx[d]);
        g[3 * q + d] = x;
        const double e = __dadd_rn(x, -M.node_last[(size_t)t * 9 + 3 * q + d]);
        dsq = d == 0 ? __dmul_rn(e, e) : __dadd_rn(dsq, __dmul_rn(e, e));
      }
      moved |= dsq > trigger;
    }
    for (int d = 0; d < 3; d++) g[33 + d] = __dadd_rn(g[33 + d], M.dx[d]);
    M.trif[2 * (size_t)t] = make_float4((float)g[0], (float)g[1], (float)g[2], 0.f);
  }
  if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(&c->mesh_moved, 1);
}

// sort_contacts: move filled slots forward (swap first empty <-> last filled)
__global__ void k_mesh_sort(Sys s, int k) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const MeshDev &M = s.meshes[k];
  const int n = c->n_new;
  const size_t nmax = s.nmax;
  GRID_STRIDE(i, n) {
    const int nn = M.nslot[0][i];
    int fe, lf;
    do {
      fe = lf = -1;
      for (int j = 0; j < nn; j++) {
        const int p = M.slot_tri[0][j * nmax + i];
        if (fe == -1 && p == -1) fe = j;
        if (p >= 0) lf = j;
      }
      if (fe > -1 && lf > -1 && fe < lf) mslot_swap(M, nmax, i, fe, lf);
    } while (fe > -1 && lf > -1 && fe < lf);
  }
}

__device__ __forceinline__ void tri_cell_range(const Sys &s, const MeshDev &M, int t, int lo[3], int hi[3]) {
  const double *g = M.tri + (size_t)t * kTriStride;
  for (int d = 0; d < 3; d++) {
    double a = g[d], b = g[d];
    for (int q = 1; q < 3; q++) {
      a = fmin(a, g[3 * q + d]);
      b = fmax(b, g[3 * q + d]);
    }
    lo[d] = cell_coord(s, a - M.distmax, d);
    hi[d] = cell_coord(s, b + M.distmax, d);
  }
}

__global__ void k_tri_count(Sys s, int k) {
  if (gated(s.ctrl)) return;
  const MeshDev &M = s.meshes[k];
  GRID_STRIDE(t, M.ntri) {
    if (M.moving)  // FixMesh::pre_force on a rebuild step: storeNodePosRebuild
      for (int q = 0; q < 9; q++) M.node_last[(size_t)t * 9 + q] = M.tri[(size_t)t * kTriStride + q];
    int lo[3], hi[3];
    tri_cell_range(s, M, t, lo, hi);
    for (int z = lo[2]; z <= hi[2]; z++)
      for (int y = lo[1]; y <= hi[1]; y++)
        for (int x = lo[0]; x <= hi[0]; x++) atomicAdd(&M.tc_count[x + s.nc[0] * (y + s.nc[1] * z)], 1);
  }
}

__global__ void k_tri_fill(Sys s, int k) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const MeshDev &M = s.meshes[k];
  if (M.tc_start[s.ncell] > M.tc_cap) {  // the host grows tc_list to tc_start[ncell] and resumes
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      c->status = kStatMeshReg;
      c->halt = 1;
    }
    return;
  }
  GRID_STRIDE(t, M.ntri) {
    int lo[3], hi[3];
    tri_cell_range(s, M, t, lo, hi);
    for (int z = lo[2]; z <= hi[2]; z++)
      for (int y = lo[1]; y <= hi[1]; y++)
        for (int x = lo[0]; x <= hi[0]; x++) {
          const int cell = x + s.nc[0] * (y + s.nc[1] * z);
          M.tc_list[M.tc_start[cell] + atomicAdd(&M.tc_fill[cell], 1)] = t;
        }
  }
}

// per atom: candidate triangles of its cell that pass resolveTriSphereNeighbuild,
// ascending; then cleanUpContactJumps and the re-paging of the slots
__global__ void k_mesh_cand(Sys s, int k) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const MeshDev &M = s.meshes[k];
  const AtomArrays &A = s.atoms[0];
  const int n = c->n_new;
  const size_t nmax = s.nmax;
  const int cap = M.ccap;
  bool over = false;
  GRID_STRIDE(i, n) {
    const double xv[3] = {A.x[i], A.y[i], A.z[i]};
    const int cell = cell_coord(s, xv[0], 0) + s.nc[0] * (cell_coord(s, xv[1], 1) + s.nc[1] * cell_coord(s, xv[2], 2));
    const double rS = __dmul_rn(A.r[i], s.cdf);
    int *cand = M.cand + i;  // [q*nmax]
    int nc = 0, need = 0;
    for (int q = M.tc_start[cell]; q < M.tc_start[cell + 1]; q++) {
      const int t = M.tc_list[q];
      if (!tri_sphere_neighbuild(M.tri + (size_t)t * kTriStride, rS, xv, M.tskin)) continue;
      need++;
      if (nc == cap) continue;  // counted only: the host grows the capacity
      int m = nc++;
      while (m > 0 && cand[(size_t)(m - 1) * nmax] > t) {
        cand[(size_t)m * nmax] = cand[(size_t)(m - 1) * nmax];
        m--;
      }
      cand[(size_t)m * nmax] = t;
    }
    if (need > cap) {  // leave this atom's slots untouched; the rebuild resumes here after growth
      over = true;
      atomicMax(&c->mesh_need, need);
      continue;
    }
    M.cand_n[i] = nc;
    // cleanUpContactJumps: drop partners whose triangle no longer lists the atom
    int np = M.npart[0][i];
    int ip = 0;
    while (ip < np) {
      const int t = M.slot_tri[0][ip * nmax + i];
      bool listed = false;
      for (int q = 0; q < nc; q++) listed |= (cand[(size_t)q * nmax] == t);
      if (!listed) {
        M.slot_tri[0][ip * nmax + i] = -1;
        for (int d = 0; d < 3; d++) M.slot_hist[0][(3 * ip + d) * nmax + i] = 0.0;
        mslot_swap(M, nmax, i, ip, np - 1);
        np--;
      } else {
        ip++;
      }
    }
    for (int q = np; q < nc; q++) {
      M.slot_tri[0][q * nmax + i] = -1;
      for (int d = 0; d < 3; d++) M.slot_hist[0][(3 * q + d) * nmax + i] = 0.0;
    }
    M.npart[0][i] = np;
    M.nslot[0][i] = nc;
  }
  if (over) {
    c->status = kStatMeshCand;
    c->halt = 1;
  }
}

// end of atom i's owner row and of its partner list
__device__ __forceinline__ int row_end(const Sys &s, const PairArrays &L, int i) {
  return s.nsys ? L.rowe[i] : L.row[i + 1];
}
__device__ __forceinline__ int rev_end(const Sys &s, const PairArrays &L, int i) {
  return s.nsys ? L.reve[i] : L.rev_start[i + 1];
}

// Entry of the old list for the atom pair (owner o, partner q) in old
// indices: o's own row first, then the entries where o was the partner
// (flip = true).  Only flagged entries carry history (pre_exchange keeps
// those).  Returns -1 when none.
__device__ __forceinline__ int find_old(const Sys &s, const PairArrays &L, int o, int q, bool &flip) {
  flip = false;
  for (int k = L.row[o]; k < row_end(s, L, o); k++)
    if (L.j[k] == q && L.flag[k] != 0) return k;
  for (int k = L.rev_start[o]; k < rev_end(s, L, o); k++) {
    const int e = L.rev[k];
    if (L.i[e] == q && L.flag[e] != 0) {
      flip = true;
      return e;
    }
  }
  return -1;
}

// atoms in a primitive wall's neighbour list or with candidate triangles on
// any mesh: bit 7 of wbits and the compact list the wall kernel walks (its
// order does not matter: one thread computes all of an atom's wall forces)
__global__ void __launch_bounds__(256) k_wall_list(Sys s) {
  __shared__ int wc[8], wbase;
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const AtomArrays &A = s.atoms[0];
  const int n = c->n_new;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // one reservation per block keeps each block's atoms ascending and
  // contiguous in the list (coalesced per-atom loads in the wall kernel)
  for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const int i = base + threadIdx.x;
    bool has = false;
    if (i < n) {
      has = (A.wbits[i] & 0x7fu) != 0;
      for (int k = 0; k < s.nmeshes; k++) has |= s.meshes[k].cand_n[i] > 0;
      A.wbits[i] = has ? (uint8_t)(A.wbits[i] | 0x80u) : (uint8_t)(A.wbits[i] & 0x7fu);
    }
    const unsigned m = __ballot_sync(0xffffffffu, has);
    if (lane == 0) wc[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < 8; w++) tot += wc[w];
      wbase = tot ? atomicAdd(&c->nmlist, tot) : 0;
    }
    __syncthreads();
    int off = wbase;
    for (int w = 0; w < warp; w++) off += wc[w];
    if (has) s.mlist[off + __popc(m & ((1u << lane) - 1u))] = i;
    __syncthreads();
  }
}

// ----------------------------------------------------------------------------
// rebuild: granular half list (Neighbor::granular_bin_no_newton,
// src/neigh_gran.cpp:485-644), 27-cell stencil with periodic images.  The
// count pass keeps each atom's first kStash entries (partner and image code
// in one int); the fill pass copies them into the atom's row, and searches
// again only for atoms with more.
// ----------------------------------------------------------------------------

// One run of candidates [jb, je) of the cell-sorted order, all with image
// code `code` (shift sv): FP32 prefilter of rsq <= (radsum*cdf + skin)^2;
// candidates clearly outside (or clearly inside) by more than the bound of
// the FP32 rounding are decided without FP64; the rest, and every entry the
// fill pass writes, use the exact FP64 test.
template <bool FILL>
__device__ __forceinline__ void pairs_scan(const Sys &s, const AtomArrays &A, const PairArrays &M, int i,
                                           const float4 &pi, double xi, double yi, double zi, double radi,
                                           float cdff, float skinf, float hi_f, float lo_f, int jb, int je,
                                           int code, const int sv[3], int &cnt, int &out, int out_end) {
  // image shifts by selection: an int-to-float conversion would issue on the FP64 pipe
  const float sxf = fshift(sv[0], s.prdf[0]), syf = fshift(sv[1], s.prdf[1]), szf = fshift(sv[2], s.prdf[2]);
  for (int j = jb; j < je; j++) {
    if (code == kNoShift && j <= i) continue;
    const float4 pj = s.xf[j];
    const float fx = pi.x - (pj.x + sxf), fy = pi.y - (pj.y + syf), fz = pi.z - (pj.z + szf);
    const float rsqf = fx * fx + fy * fy + fz * fz;
    const float csf = (pi.w + pj.w) * cdff + skinf;
    const float cs2f = csf * csf;
    if (rsqf > cs2f * hi_f) continue;
    if (code != kNoShift && !ghost_exists(s, A, j, sv)) continue;
    const bool clear_in = rsqf < cs2f * lo_f;
    if (!FILL && clear_in) {
      if (cnt < kStash) s.stash[(size_t)cnt * s.nmax + i] = j | (code << 24);
      cnt++;
      continue;
    }
    double xj = A.x[j], yj = A.y[j], zj = A.z[j];
    image(s, code, xj, yj, zj);
    const double delx = __dadd_rn(xi, -xj);
    const double dely = __dadd_rn(yi, -yj);
    const double delz = __dadd_rn(zi, -zj);
    const double rsq = rsq_rn(delx, dely, delz);
    const double radj = A.r[j];
    const double radsum = __dmul_rn(__dadd_rn(radi, radj), s.cdf);
    const double cs = __dadd_rn(radsum, s.skin);
    if (!(rsq <= __dmul_rn(cs, cs))) continue;
    if (!FILL) {
      if (cnt < kStash) s.stash[(size_t)cnt * s.nmax + i] = j | (code << 24);
      cnt++;
      continue;
    }
    if (out >= out_end) continue;  // count and fill passes agree; guard only
    const int p = out++;
    M.i[p] = i;
    M.j[p] = j;
    M.sh[p] = (uint8_t)code;
    if (s.nsys) M.rev[p] = -1;  // a fresh entry (source of copied ones: see pairs_atom)
  }
}

template <bool FILL>
__device__ __forceinline__ void pairs_atom(const Sys &s, const AtomArrays &A, const PairArrays &L,
                                           const PairArrays &M, int i) {
  {
    if (!sys_rebuilds(s, A.type[i])) {
      // a system that does not rebuild keeps its entries, in their order,
      // with partners renumbered by its block's shift (pairs never cross
      // systems); k_pair_init copies their history from the source entry
      const int sy = A.type[i] - 1;
      const int o = s.perm[i];
      const int eb = L.row[o], ee = row_end(s, L, o);
      if (!FILL) {
        s.pcount[i] = ee - eb;
        return;
      }
      const int shift = s.cell_start[sy * s.ens_ncell] - s.sys_start[sy];
      int out = M.row[i];
      for (int e = eb; e < ee; e++, out++) {
        M.i[out] = i;
        M.j[out] = L.j[e] + shift;
        M.sh[out] = L.sh[e];
        M.rev[out] = e;
      }
      return;
    }
    if (FILL) {  // the count pass kept the atom's entries unless it had more than kStash
      const int beg = M.row[i], ne = row_end(s, M, i) - beg;
      if (ne <= kStash) {
        for (int e = 0; e < ne; e++) {
          const int v = s.stash[(size_t)e * s.nmax + i];
          M.i[beg + e] = i;
          M.j[beg + e] = v & 0xffffff;
          M.sh[beg + e] = (uint8_t)(v >> 24);
          if (s.nsys) M.rev[beg + e] = -1;  // a fresh entry (source of copied ones: see above)
        }
        return;
      }
    }
    const double xi = A.x[i], yi = A.y[i], zi = A.z[i];
    const double radi = A.r[i];
    const int ci[3] = {cell_coord(s, xi, 0), cell_coord(s, yi, 1), cell_coord(s, zi, 2)};
    const float4 pi = s.xf[i];
    const int cell_base = s.ens_ncell ? (A.type[i] - 1) * s.ens_ncell : 0;
    const float cdff = s.cdff, skinf = s.skinf;
    const float hi_f = 1.0f + s.pf_margin, lo_f = 1.0f - s.pf_margin;
    int cnt = 0;
    int out = FILL ? M.row[i] : 0;
    const int out_end = FILL ? row_end(s, M, i) : 0;
    // per dimension: the neighbour coordinate, image shift and validity of
    // the offsets -1, 0, +1
    int nb[3][3], sv3[3][3];
    bool ok3[3][3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const int o = k - 1;
        int cc = ci[d] + o, sv = 0;
        bool ok = !(s.nc[d] == 1 && o != 0);
        if (cc < 0) {
          ok = ok && s.periodic[d];
          cc += s.nc[d];
          sv = -1;
        } else if (cc >= s.nc[d]) {
          ok = ok && s.periodic[d];
          cc -= s.nc[d];
          sv = 1;
        }
        nb[d][k] = cc;
        sv3[d][k] = sv;
        ok3[d][k] = ok;
      }
    }
    // the 27 cells in the stencil's order (z, then y, then x offsets): along
    // x the unwrapped cells of a row are consecutive, so their atoms are one
    // contiguous run of the cell-sorted order, scanned in one loop (the same
    // candidates in the same order as cell by cell); a cell that wraps
    // around a periodic x boundary is scanned alone, with its image shift
    const bool lwrap = ok3[0][0] && sv3[0][0] != 0, rwrap = ok3[0][2] && sv3[0][2] != 0;
    const int x0 = (ok3[0][0] && !lwrap) ? nb[0][0] : nb[0][1];
    const int x1 = (ok3[0][2] && !rwrap) ? nb[0][2] : nb[0][1];
#pragma unroll
    for (int kz = 0; kz < 3; kz++) {
#pragma unroll
      for (int ky = 0; ky < 3; ky++) {
        if (!ok3[2][kz] || !ok3[1][ky]) continue;
        const int rowb = s.nc[0] * (nb[1][ky] + s.nc[1] * nb[2][kz]) + cell_base;
        const int syz = 3 * (sv3[1][ky] + 1) + 9 * (sv3[2][kz] + 1);
        if (lwrap) {
          const int sv[3] = {-1, sv3[1][ky], sv3[2][kz]};
          pairs_scan<FILL>(s, A, M, i, pi, xi, yi, zi, radi, cdff, skinf, hi_f, lo_f, s.cell_start[rowb + nb[0][0]],
                           s.cell_start[rowb + nb[0][0] + 1], syz, sv, cnt, out, out_end);
        }
        {
          const int sv[3] = {0, sv3[1][ky], sv3[2][kz]};
          pairs_scan<FILL>(s, A, M, i, pi, xi, yi, zi, radi, cdff, skinf, hi_f, lo_f, s.cell_start[rowb + x0],
                           s.cell_start[rowb + x1 + 1], 1 + syz, sv, cnt, out, out_end);
        }
        if (rwrap) {
          const int sv[3] = {1, sv3[1][ky], sv3[2][kz]};
          pairs_scan<FILL>(s, A, M, i, pi, xi, yi, zi, radi, cdff, skinf, hi_f, lo_f, s.cell_start[rowb + nb[0][2]],
                           s.cell_start[rowb + nb[0][2] + 1], 2 + syz, sv, cnt, out, out_end);
        }
      }
    }
    if (!FILL) s.pcount[i] = cnt;
  }
}

template <bool FILL>
__global__ void k_pairs(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const AtomArrays &A = s.atoms[0];
  const PairArrays &L = s.pairs[0];  // old list (old atom order)
  const PairArrays &M = s.pairs[1];  // new list
  // count: in place for the rebuilding systems' atoms (pmode); fill: also
  // in place for their segments (lmode)
  if (FILL ? ens_list_partial(s, c) : ens_partial(s, c)) {
    GRID_STRIDE(t, c->nra) pairs_atom<FILL>(s, A, L, M, ens_atom(s, c, t));
    return;
  }
  const int n = c->n_new;
  const int total = FILL ? n : s.nmax + 1;
  GRID_STRIDE(i, total) {
    if (!FILL && i >= n) {
      s.pcount[i] = 0;
      continue;
    }
    pairs_atom<FILL>(s, A, L, M, i);
  }
}

// Per new list entry (one thread each, dense): exact distance, history
// carry-over, per-pair contact constants, reverse-list count.  The carry-over
// is the reference's (pre_exchange partner lists + the lookup of
// src/neigh_gran.cpp:590-620): the new entry's reference owner R (lower lidx
// of an owned pair, else i) takes its partner-list entry for the other atom:
// its own old entry, or the partner copy of an old owned pair, in which the
// values registered with newtonflag 1 change sign.  The shear is then
// expressed in the list's own orientation; history is carried only when the
// pair is within radsum*cdf at the build.
__device__ __forceinline__ void pair_init_entry(const Sys &s, const AtomArrays &A, const PairArrays &L,
                                                const PairArrays &M, int p) {
  {
    const int code = M.sh[p];
    if (code == kHole) return;  // an unused entry of an ensemble segment
    const int i = M.i[p], j = M.j[p];
    const int src = s.nsys ? M.rev[p] : -1;
    if (src >= 0) {  // kept entry of a system that does not rebuild: as it was
      M.flag[p] = L.flag[src];
      for (int d = 0; d < s.dnum; d++) M.hist[(size_t)d * s.pcap + p] = L.hist[(size_t)d * s.pcap + src];
      M.reff[p] = L.reff[src];
      M.c0[p] = L.c0[src];
      M.c1[p] = L.c1[src];
      if (code == kNoShift) atomicAdd(&s.rev_count[j], 1);
      return;
    }
    double xj = A.x[j], yj = A.y[j], zj = A.z[j];
    image(s, code, xj, yj, zj);
    const double rsq = rsq_rn(__dadd_rn(A.x[i], -xj), __dadd_rn(A.y[i], -yj), __dadd_rn(A.z[i], -zj));
    const double radi = A.r[i], radj = A.r[j];
    const double radsum = __dmul_rn(__dadd_rn(radi, radj), s.cdf);
    int e = -1;
    double ssign = 1.0;
    bool quirk = false;
    if (rsq < __dmul_rn(radsum, radsum)) {
      const bool rj = s.bond && code == kNoShift && A.lidx[i] > A.lidx[j];
      bool fl;
      e = rj ? find_old(s, L, s.perm[j], s.perm[i], fl) : find_old(s, L, s.perm[i], s.perm[j], fl);
      ssign = (fl ? -1.0 : 1.0) * (rj ? -1.0 : 1.0);
      quirk = s.bond && e >= 0 && !rj && code != kNoShift && L.sh[e] == kNoShift && A.lidx[i] > A.lidx[j];
    }
    M.flag[p] = e >= 0 ? 1 : 0;
    for (int d = 0; d < kDnumShear; d++)
      M.hist[(size_t)d * s.pcap + p] = e >= 0 ? ssign * L.hist[(size_t)d * s.pcap + e] : 0.0;
    for (int d = kDnumShear; d < s.dnum; d++) {
      double hv = e >= 0 ? L.hist[(size_t)d * s.pcap + e] : 0.0;
      if (quirk && d >= kDnumShear + 5 && d <= kDnumShear + 13) hv = -hv;
      M.hist[(size_t)d * s.pcap + p] = hv;
    }
    const double mi = A.m[i], mj = A.m[j];
    const double meff = mi * mj / (mi + mj);
    const double reff = radi * radj / (radi + radj);
    const TypePair tp = load_typepair(s.params, s.ntypes, A.type[i], A.type[j]);
    double c0, c1;
    if (s.normal == kHertz) contact_consts<kHertz>(tp, meff, reff, s.charVel, s.tdamp, c0, c1);
    else contact_consts<kHooke>(tp, meff, reff, s.charVel, s.tdamp, c0, c1);
    M.reff[p] = reff;
    M.c0[p] = c0;
    M.c1[p] = c1;
    if (code == kNoShift) atomicAdd(&s.rev_count[j], 1);
  }
}

__global__ void k_pair_init(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const AtomArrays &A = s.atoms[0];
  const PairArrays &L = s.pairs[0];  // old list (old atom order)
  const PairArrays &M = s.pairs[1];  // new list
  if (ens_list_partial(s, c)) {
    GRID_STRIDE(u, c->ncr) pair_init_entry(s, A, L, M, ens_entry(s, c, u));
    return;
  }
  const int np = c->np_new;
  GRID_STRIDE(p, np) pair_init_entry(s, A, L, M, p);
}

// after the pair-count scan: capacity check; halts on overflow
__global__ void k_pairs_total(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  // ensembles: the segments' extent (k_ens_plan or k_ens_layout)
  const int np = s.nsys ? c->np_new : s.pairs[1].row[s.nmax];
  c->np_new = np;
  if (np > s.pcap) {
    c->status = kStatPairOverflow;
    c->halt = 1;
    c->halt_step = 1;
  }
}

__device__ __forceinline__ void rev_fill_entry(const Sys &s, const PairArrays &M, int p) {
  if (M.sh[p] != kNoShift) return;  // image entries and unused ones
  const int j = M.j[p];
  M.rev[M.rev_start[j] + atomicAdd(&s.rev_fill[j], 1)] = p;
}

__global__ void k_rev_fill(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const PairArrays &M = s.pairs[1];
  if (ens_list_partial(s, c)) {
    GRID_STRIDE(u, c->ncr) rev_fill_entry(s, M, ens_entry(s, c, u));
    return;
  }
  const int np = c->np_new;
  GRID_STRIDE(p, np) rev_fill_entry(s, M, p);
}

__device__ __forceinline__ void rev_sort_atom(const Sys &s, const PairArrays &M, int i) {
  const int b = M.rev_start[i], e = rev_end(s, M, i);
  for (int k = b + 1; k < e; k++) {
    const int v = M.rev[k];
    int m = k - 1;
    while (m >= b && M.rev[m] > v) {
      M.rev[m + 1] = M.rev[m];
      m--;
    }
    M.rev[m + 1] = v;
  }
}

__global__ void k_rev_sort(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const PairArrays &M = s.pairs[1];
  if (ens_list_partial(s, c)) {
    GRID_STRIDE(t, c->nra) rev_sort_atom(s, M, ens_atom(s, c, t));
    return;
  }
  const int n = c->n_new;
  GRID_STRIDE(i, n) rev_sort_atom(s, M, i);
}

__device__ __forceinline__ void copy_entry(const Sys &s, const PairArrays &L, const PairArrays &M, int p) {
  L.i[p] = M.i[p];
  L.j[p] = M.j[p];
  L.sh[p] = M.sh[p];
  L.flag[p] = M.flag[p];
  for (int d = 0; d < s.dnum; d++) L.hist[(size_t)d * s.pcap + p] = M.hist[(size_t)d * s.pcap + p];
  L.reff[p] = M.reff[p];
  L.c0[p] = M.c0[p];
  L.c1[p] = M.c1[p];
  L.rev[p] = M.rev[p];
}

__device__ __forceinline__ void copy_rows(const Sys &s, const PairArrays &L, const PairArrays &M, int i) {
  L.row[i] = M.row[i];
  L.rev_start[i] = M.rev_start[i];
  if (s.nsys) {
    L.rowe[i] = M.rowe[i];
    L.reve[i] = M.reve[i];
  }
}

__global__ void k_copy_pairs(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  const PairArrays &L = s.pairs[0];
  const PairArrays &M = s.pairs[1];
  if (ens_list_partial(s, c)) {  // the rebuilt segments (with their unused entries) and rows
    GRID_STRIDE(u, c->ncr) copy_entry(s, L, M, ens_entry(s, c, u));
    GRID_STRIDE(t, c->nra) copy_rows(s, L, M, ens_atom(s, c, t));
    return;
  }
  const int np = c->np_new;
  const int nrow = s.nmax + 1;
  const int tot = np > nrow ? np : nrow;
  GRID_STRIDE(p, tot) {
    if (p < np) copy_entry(s, L, M, p);
    if (p < nrow) copy_rows(s, L, M, p);
  }
}

__global__ void k_finish_rebuild(Sys s) {
  Ctrl *c = s.ctrl;
  if (gated(c)) return;
  int live = 0;
  for (int k = threadIdx.x; k < s.nsys; k += blockDim.x) {
    if (s.sys_reb[k]) {
      s.sys_nreb[k]++;
      s.sys_ago[k] = 0;
    }
    s.sys_start[k] = s.cell_start[k * s.ens_ncell];
    live += s.seg_used[k];
  }
  int tot = 0;
  if (s.nsys) block_excl_scan(live, &tot);
  __syncthreads();  // every thread has read the gate before it changes
  if (threadIdx.x == 0) {
    if (s.nsys) {
      s.sys_start[s.nsys] = s.cell_start[s.ncell];
      c->seg_ok = 1;
      c->np_live = tot;
      if (c->pmode) {
        if (c->lmode) c->ens_inplace++;
        else c->ens_relayout++;
      }
    }
    c->lost += c->lost_step;
    c->n = c->n_new;
    c->np = c->np_new;
    if (!s.nsys) c->np_live = c->np_new;
    c->nrebuilds++;
    c->ago = 0;
  }
}

// ----------------------------------------------------------------------------
// pair forces: one thread per half-list entry, results to the pair buffer
// ----------------------------------------------------------------------------

// The pair kernels test list entries per lane (phase 1) and queue the ones
// that need the FP64 laws in a per-warp shared-memory queue (warp ballots),
// so phase 2 runs on full warps: entries that need nothing cost no FP64
// issue slots.  Results go to the entry's own slot, so the processing order
// never changes a value.  kPairTile is k_pair_pf's block size.
constexpr int kPairTile = 256;

// The general kernel carries the bond law.  Blocks of 128 threads capped at
// 128 registers (a few spilled) let four blocks share an SM (measured on the
// 200k bonded fibre bed with one queue per tile: 0.55 ms with one 256-thread
// block per SM, 0.41 ms with three 128-thread blocks, 0.35 ms with four;
// 64-thread tiles 0.40 ms; with per-warp queues 0.27 ms).
constexpr int kBandTile = 128;

// the entry's result record: three whole 32-byte sectors in one go
__device__ __forceinline__ void store_result(const Sys &s, int q, const ContactOut &o) {
  double2 *r = reinterpret_cast<double2 *>(s.res + (size_t)kResStride * q);
  r[0] = make_double2(o.F[0], o.F[1]);
  r[1] = make_double2(o.F[2], o.Ti[0]);
  r[2] = make_double2(o.Ti[1], o.Ti[2]);
  r[3] = make_double2(o.Tj[0], o.Tj[1]);
  r[4] = make_double2(o.Tj[2], 0.0);
  r[5] = make_double2(0.0, 0.0);
}

// Phase 2 of k_pair for one queued entry q (delx, dely, delz, rsq_q from
// its exact test): the bond law, the contact law, the result record
template <int NORMAL, bool ROLL, bool BOND>
__device__ __forceinline__ void band_entry(const Sys &s, int q, double delx, double dely, double delz,
                                           double rsq_q, int shearupdate, long long ntimestep) {
  const AtomArrays &A = s.atoms[0];
  const PairArrays &L = s.pairs[0];
  const size_t P = s.pcap;
  const int i = L.i[q], j = L.j[q];
  ContactIn ci;
  ci.d[0] = delx;
  ci.d[1] = dely;
  ci.d[2] = delz;
  ci.radi = A.r[i];
  ci.radj = A.r[j];
  ci.radsum = __dadd_rn(ci.radi, ci.radj);
  ci.vr[0] = A.vx[i] - A.vx[j];
  ci.vr[1] = A.vy[i] - A.vy[j];
  ci.vr[2] = A.vz[i] - A.vz[j];
  ci.wi[0] = A.wx[i]; ci.wi[1] = A.wy[i]; ci.wi[2] = A.wz[i];
  ci.wj[0] = A.wx[j]; ci.wj[1] = A.wy[j]; ci.wj[2] = A.wz[j];
  const bool touch = !BOND || rsq_q < __dmul_rn(ci.radsum, ci.radsum);
  ContactOut bo;
  bool bonded = false;
  if (BOND) {
    // evaluated in the reference's orientation: owner = lower lidx
    // (periodic entries are directed and always owned by i)
    const bool rev = L.sh[q] == kNoShift && A.lidx[i] > A.lidx[j];
    const int a = rev ? j : i, b = rev ? i : j;
    const double sg = rev ? -1.0 : 1.0;
    BondIn bi;
    bi.d[0] = sg * ci.d[0]; bi.d[1] = sg * ci.d[1]; bi.d[2] = sg * ci.d[2];
    bi.rsq = rsq_q;
    bi.radi = A.r[a];
    bi.radj = A.r[b];
    bi.vi[0] = A.vx[a]; bi.vi[1] = A.vy[a]; bi.vi[2] = A.vz[a];
    bi.vj[0] = A.vx[b]; bi.vj[1] = A.vy[b]; bi.vj[2] = A.vz[b];
    bi.wi[0] = A.wx[a]; bi.wi[1] = A.wy[a]; bi.wi[2] = A.wz[a];
    bi.wj[0] = A.wx[b]; bi.wj[1] = A.wy[b]; bi.wj[2] = A.wz[b];
    bi.xi[0] = A.x[a]; bi.xi[1] = A.y[a]; bi.xi[2] = A.z[a];
    bi.tp = A.type[a] * (s.ntypes + 1) + A.type[b];
    ContactOut bc;
    bonded = bond_nonlinear(s, bi, L.hist + 3 * P + q, P, L.flag + q, shearupdate != 0, ntimestep, bc);
    if (bonded) {  // back to the list's orientation (i owns the entry)
      for (int k = 0; k < 3; k++) {
        bo.F[k] = sg * bc.F[k];
        bo.Ti[k] = rev ? bc.Tj[k] : bc.Ti[k];
        bo.Tj[k] = rev ? bc.Ti[k] : bc.Tj[k];
      }
    }
  }
  ContactOut o;
  if (touch) {
    // r from 1/r: within an ulp of sqrt(rsq), which moves the overlap
    // radsum - r by ~1e-13 of itself
    ci.rinv = rsqrt(rsq_q);
    ci.r = rsq_q * ci.rinv;
    ci.reff = L.reff[q];
    ci.c0 = L.c0[q];
    ci.c1 = L.c1[q];
    ci.en[0] = ci.d[0] * ci.rinv;
    ci.en[1] = ci.d[1] * ci.rinv;
    ci.en[2] = ci.d[2] * ci.rinv;
    ci.deltan_wall = 0.0;
    const TypePair tp = load_typepair(s.params, s.ntypes, A.type[i], A.type[j]);
    double sh3[3] = {L.hist[q], L.hist[P + q], L.hist[2 * P + q]};
    contact_law<NORMAL, false>(ci, tp, s.dt, s.tdamp, s.limitf, ROLL, shearupdate != 0, sh3, o,
                               (BOND && bonded) ? &bo : nullptr);
    if (shearupdate) {
      L.hist[q] = sh3[0];
      L.hist[P + q] = sh3[1];
      L.hist[2 * P + q] = sh3[2];
    }
    L.flag[q] |= (kContactNormal | kContactTangential);
  } else {
    for (int k = 0; k < 3; k++) {
      o.F[k] = bo.F[k];
      o.Ti[k] = bo.Ti[k];
      o.Tj[k] = bo.Tj[k];
    }
  }
  if (touch || bonded) {
    store_result(s, q, o);
    s.active[q] = 1;
  }
}

// Phase 1 runs per lane on 32 consecutive entries of a warp at a time; the
// entries that need phase 2 wait in the warp's shared-memory queue (with
// their exact test's delta and rsq) until 32 have gathered, so the bond and
// contact laws run on full warps.  The warps' remainders merge into one
// block batch at the end.  Each entry's result goes to its own slot and
// depends on no other entry, so the order changes no value.
template <int NORMAL, bool ROLL, bool BOND>
__global__ void __launch_bounds__(kBandTile, 4) k_pair(Sys s, int shearupdate) {
  __shared__ int q_p[kBandTile / 32][64];
  __shared__ double q_d[kBandTile / 32][4][64];
  __shared__ int rest_p[kBandTile];
  __shared__ double rest_d[4][kBandTile];
  __shared__ int nrest;
  Ctrl *c = s.ctrl;
  if (c->halt) return;
  const AtomArrays &A = s.atoms[0];
  const PairArrays &L = s.pairs[0];
  const int np = c->np;
  const size_t P = s.pcap;
  const double cdm = s.cdf * s.cdf;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  int *qp = q_p[warp];
  double(*qd)[64] = q_d[warp];
  // cohesion bond/nonlinear: a bond can be created in this pass
  const long long ntimestep = BOND ? c->ntimestep : 0;
  const bool may_create = BOND && shearupdate &&
                          ((s.bond_flags & kBondCreateAlways) || ntimestep == s.bond_ts_create);
  int qn = 0;  // the same in every lane
  const long stride = (long)gridDim.x * kBandTile;
  for (long base = (long)blockIdx.x * kBandTile + warp * 32; base < np; base += stride) {
    const int p = (int)base + lane;
    bool queue = false;
    double delx = 0., dely = 0., delz = 0., rsq = 0.;
    const int code = p < np ? L.sh[p] : kHole;
    if (code == kHole && p < np) s.active[p] = 0;  // an unused entry of an ensemble segment
    if (code != kHole) {
      const int i = L.i[p], j = L.j[p];
      double xj = A.x[j], yj = A.y[j], zj = A.z[j];
      image(s, code, xj, yj, zj);
      delx = __dadd_rn(A.x[i], -xj);
      dely = __dadd_rn(A.y[i], -yj);
      delz = __dadd_rn(A.z[i], -zj);
      rsq = rsq_rn(delx, dely, delz);
      const double radsum = __dadd_rn(A.r[i], A.r[j]);
      queue = rsq < __dmul_rn(radsum, radsum);
      if (!queue) {
        s.active[p] = 0;
        if (rsq < __dmul_rn(__dmul_rn(cdm, radsum), radsum)) {
          // TangentialModel<TANGENTIAL_HISTORY>::surfacesClose
          L.flag[p] &= ~kContactTangential;
          L.hist[p] = 0.0;
          L.hist[P + p] = 0.0;
          L.hist[2 * P + p] = 0.0;
          // CohesionModel::surfacesClose: bonded pairs (and pairs that may
          // bond in this pass) are evaluated in phase 2
          if (BOND && (may_create || L.hist[3 * P + p] >= 1.e-15)) {
            const int tp = A.type[i] * (s.ntypes + 1) + A.type[j];
            queue = __ldg(s.bondp + tp) >= 1.e-15;
          }
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, queue);
    if (queue) {
      const int slot = qn + __popc(m & below);
      qp[slot] = p;
      qd[0][slot] = delx;
      qd[1][slot] = dely;
      qd[2][slot] = delz;
      qd[3][slot] = rsq;
    }
    qn += __popc(m);
    __syncwarp();
    if (qn >= 32) {
      band_entry<NORMAL, ROLL, BOND>(s, qp[lane], qd[0][lane], qd[1][lane], qd[2][lane], qd[3][lane], shearupdate,
                                     ntimestep);
      const int rem = qn - 32;
      __syncwarp();
      int vp = 0;
      double v0 = 0., v1 = 0., v2 = 0., v3 = 0.;
      if (lane < rem) {
        vp = qp[32 + lane];
        v0 = qd[0][32 + lane];
        v1 = qd[1][32 + lane];
        v2 = qd[2][32 + lane];
        v3 = qd[3][32 + lane];
      }
      __syncwarp();
      if (lane < rem) {
        qp[lane] = vp;
        qd[0][lane] = v0;
        qd[1][lane] = v1;
        qd[2][lane] = v2;
        qd[3][lane] = v3;
      }
      qn = rem;
      __syncwarp();
    }
  }
  // the warps' remainders (at most 31 each) into one block batch
  if (threadIdx.x == 0) nrest = 0;
  __syncthreads();
  int at = 0;
  if (lane == 0 && qn) at = atomicAdd(&nrest, qn);
  at = __shfl_sync(0xffffffffu, at, 0);
  if (lane < qn) {
    rest_p[at + lane] = qp[lane];
    for (int k = 0; k < 4; k++) rest_d[k][at + lane] = qd[k][lane];
  }
  __syncthreads();
  if (threadIdx.x < nrest)
    band_entry<NORMAL, ROLL, BOND>(s, rest_p[threadIdx.x], rest_d[0][threadIdx.x], rest_d[1][threadIdx.x],
                                   rest_d[2][threadIdx.x], rest_d[3][threadIdx.x], shearupdate, ntimestep);
}

// Pair forces without cohesion and with contact distance factor 1 (an entry
// that is not touching needs no work).  A warp tests 32 consecutive entries
// at a time in FP32 (x, y, z, r refreshed by every drift): entries apart by
// more than the bound of the FP32 rounding (pf_margin_touch) only clear
// their active flag.  The rest are queued in the warp's shared-memory queue;
// whenever 32 have gathered, the warp runs the exact test and the FP64
// contact law on all its lanes (the FP64 pipe issues per warp, so idle lanes
// would waste it).  No block-wide barrier inside the loop: the warps of a
// block reach their FP64 phases at different times (a block-wide queue
// of 256 held all eight warps at three barriers per tile; the pair kernel
// took 0.143 ms on the 1M-atom hopper that way, 0.136 ms this way).
template <int NORMAL, bool ROLL>
__device__ __forceinline__ void pair_entry(const Sys &s, int q, int shearupdate) {
  const AtomArrays &A = s.atoms[0];
  const PairArrays &L = s.pairs[0];
  const size_t P = s.pcap;
  const int i = L.i[q], j = L.j[q];
  double xj = A.x[j], yj = A.y[j], zj = A.z[j];
  image(s, L.sh[q], xj, yj, zj);
  ContactIn ci;
  ci.d[0] = __dadd_rn(A.x[i], -xj);
  ci.d[1] = __dadd_rn(A.y[i], -yj);
  ci.d[2] = __dadd_rn(A.z[i], -zj);
  const double rsq = rsq_rn(ci.d[0], ci.d[1], ci.d[2]);
  ci.radi = A.r[i];
  ci.radj = A.r[j];
  ci.radsum = __dadd_rn(ci.radi, ci.radj);
  if (!(rsq < __dmul_rn(ci.radsum, ci.radsum))) {
    s.active[q] = 0;
    return;
  }
  ci.vr[0] = A.vx[i] - A.vx[j];
  ci.vr[1] = A.vy[i] - A.vy[j];
  ci.vr[2] = A.vz[i] - A.vz[j];
  ci.wi[0] = A.wx[i]; ci.wi[1] = A.wy[i]; ci.wi[2] = A.wz[i];
  ci.wj[0] = A.wx[j]; ci.wj[1] = A.wy[j]; ci.wj[2] = A.wz[j];
  // r from 1/r: within an ulp of sqrt(rsq), which moves the overlap
  // radsum - r by ~1e-13 of itself
  ci.rinv = rsqrt(rsq);
  ci.r = rsq * ci.rinv;
  ci.reff = L.reff[q];
  ci.c0 = L.c0[q];
  ci.c1 = L.c1[q];
  ci.en[0] = ci.d[0] * ci.rinv;
  ci.en[1] = ci.d[1] * ci.rinv;
  ci.en[2] = ci.d[2] * ci.rinv;
  ci.deltan_wall = 0.0;
  const TypePair tp = load_typepair(s.params, s.ntypes, A.type[i], A.type[j]);
  double sh3[3] = {L.hist[q], L.hist[P + q], L.hist[2 * P + q]};
  ContactOut o;
  contact_law<NORMAL, false>(ci, tp, s.dt, s.tdamp, s.limitf, ROLL, shearupdate != 0, sh3, o);
  if (shearupdate) {
    L.hist[q] = sh3[0];
    L.hist[P + q] = sh3[1];
    L.hist[2 * P + q] = sh3[2];
  }
  L.flag[q] |= (kContactNormal | kContactTangential);
  store_result(s, q, o);
  s.active[q] = 1;
}

template <int NORMAL, bool ROLL, int MINB>
__global__ void __launch_bounds__(kPairTile, MINB) k_pair_pf(Sys s, int shearupdate) {
  __shared__ int qbuf[kPairTile / 32][64];
  Ctrl *c = s.ctrl;
  if (c->halt) return;
  const PairArrays &L = s.pairs[0];
  const int np = c->np;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  int *q = qbuf[warp];
  const float hi_f = 1.0f + s.pf_margin_touch;
  const float px = s.prdf[0], py = s.prdf[1], pz = s.prdf[2];
  int qn = 0;  // the same in every lane
  const long stride = (long)gridDim.x * kPairTile;
  for (long base = (long)blockIdx.x * kPairTile + warp * 32; base < np; base += stride) {
    const int p = (int)base + lane;
    bool maybe = false;
    const int code = p < np ? L.sh[p] : kHole;
    if (code != kHole) {
      const float4 a = s.xf[L.i[p]], b = s.xf[L.j[p]];
      float sx = 0.f, sy = 0.f, sz = 0.f;
      if (code != kNoShift) {
        sx = fshift(code % 3 - 1, px);
        sy = fshift((code / 3) % 3 - 1, py);
        sz = fshift(code / 9 - 1, pz);
      }
      const float fx = a.x - (b.x + sx), fy = a.y - (b.y + sy), fz = a.z - (b.z + sz);
      const float rs = a.w + b.w;
      maybe = !(fx * fx + fy * fy + fz * fz > rs * rs * hi_f);
    }
    if (!maybe && p < np) s.active[p] = 0;
    const unsigned m = __ballot_sync(0xffffffffu, maybe);
    if (maybe) q[qn + __popc(m & below)] = p;
    qn += __popc(m);
    __syncwarp();
    if (qn >= 32) {
      pair_entry<NORMAL, ROLL>(s, q[lane], shearupdate);
      const int rem = qn - 32;
      __syncwarp();
      const int v = lane < rem ? q[32 + lane] : 0;
      __syncwarp();
      if (lane < rem) q[lane] = v;
      qn = rem;
      __syncwarp();
    }
  }
  // the warps' remainders (at most 31 each) into one block queue, so that a
  // block ends with one partial batch instead of one per warp
  __shared__ int rest[kPairTile];
  __shared__ int nrest;
  if (threadIdx.x == 0) nrest = 0;
  __syncthreads();
  int at = 0;
  if (lane == 0 && qn) at = atomicAdd(&nrest, qn);
  at = __shfl_sync(0xffffffffu, at, 0);
  if (lane < qn) rest[at + lane] = q[lane];
  __syncthreads();
  if (threadIdx.x < nrest) pair_entry<NORMAL, ROLL>(s, rest[threadIdx.x], shearupdate);
}

// ----------------------------------------------------------------------------
// per-atom kernel: force gather + gravity + primitive walls + nve/sphere
// ----------------------------------------------------------------------------

// Walls::Granular::compute_force (src/fix_wall_gran_base.h:159-372) for one
// wall contact: overlap -deltan, delta = closest wall point - centre, wall
// velocity vwall; h points at the history (stride hs between components)
template <int NORMAL>
__device__ __forceinline__ void wall_force(const Sys &s, const AtomArrays &A, int i, double deltan,
                                           const double delta[3], const double vwall[3],
                                           int wall_type, bool rolling, double *h, size_t hs,
                                           int shearupdate, const double v[3], const double om[3],
                                           double &fx, double &fy, double &fz, double &tx,
                                           double &ty, double &tz) {
  const double radi = A.r[i];
  if (deltan <= 0) {
    ContactIn ci;
    ci.radi = radi;
    ci.radj = 0.0;
    ci.deltan_wall = -deltan;
    ci.d[0] = -delta[0];
    ci.d[1] = -delta[1];
    ci.d[2] = -delta[2];
    ci.r = radi - ci.deltan_wall;
    ci.rinv = 1.0 / ci.r;
    ci.en[0] = ci.d[0] * ci.rinv;
    ci.en[1] = ci.d[1] * ci.rinv;
    ci.en[2] = ci.d[2] * ci.rinv;
    ci.radsum = radi;
    ci.reff = radi;
    ci.vr[0] = v[0] - vwall[0];
    ci.vr[1] = v[1] - vwall[1];
    ci.vr[2] = v[2] - vwall[2];
    ci.wi[0] = om[0]; ci.wi[1] = om[1]; ci.wi[2] = om[2];
    ci.wj[0] = ci.wj[1] = ci.wj[2] = 0.0;
    const TypePair tp = load_typepair(s.params, s.ntypes, A.type[i], wall_type);
    contact_consts<NORMAL>(tp, A.m[i], radi, s.charVel, s.tdamp, ci.c0, ci.c1);
    double sh3[3] = {h[0], h[hs], h[2 * hs]};
    ContactOut o;
    contact_law<NORMAL, true>(ci, tp, s.dt, s.tdamp, s.limitf, rolling, shearupdate != 0, sh3, o);
    if (shearupdate) {
      h[0] = sh3[0];
      h[hs] = sh3[1];
      h[2 * hs] = sh3[2];
    }
    fx += o.F[0]; fy += o.F[1]; fz += o.F[2];
    tx += o.Ti[0]; ty += o.Ti[1]; tz += o.Ti[2];
  } else {
    h[0] = 0.0; h[hs] = 0.0; h[2 * hs] = 0.0;  // surfacesClose
  }
}

template <int NORMAL>
__device__ __forceinline__ void plane_contact(const Sys &s, const AtomArrays &A, int i, int w,
                                              int shearupdate, double v[3], double om[3],
                                              double xv[3], double &fx, double &fy, double &fz,
                                              double &tx, double &ty, double &tz) {
  const Plane &pl = s.planes[w];
  const int ax = pl.axis, ay = (ax + 1) % 3, az = (ax + 2) % 3;
  const double radi = A.r[i];
  const double ppos = plane_pos(pl, A.type[i]);
  double delta[3];
  double deltan;
  if (pl.kind == 1) {
    // Cylinder<dim>::resolveContact, src/primitive_wall_definitions.h:170-190,
    // in the reference's operations and order
    const double dy = __dadd_rn(xv[ay], -pl.c1), dz = __dadd_rn(xv[az], -pl.c2);
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dz, dz)));
    if (dist < 1e-13 && dist > -1e-13) {  // compDouble(dist, 0.0)
      delta[0] = delta[1] = delta[2] = 0.;
      deltan = 0.0;
    } else if (dist > ppos) {
      deltan = __dadd_rn(__dadd_rn(dist, -ppos), -radi);
      const double fact = __ddiv_rn(__dadd_rn(dist, -ppos), dist);
      delta[ax] = 0.;
      delta[ay] = __dmul_rn(-dy, fact);
      delta[az] = __dmul_rn(-dz, fact);
    } else {
      deltan = __dadd_rn(__dadd_rn(ppos, -dist), -radi);
      const double fact = __ddiv_rn(__dadd_rn(ppos, -dist), dist);
      delta[ax] = 0.;
      delta[ay] = __dmul_rn(dy, fact);
      delta[az] = __dmul_rn(dz, fact);
    }
  } else if (xv[ax] > ppos) {  // Plane<dim>::resolveContact, src/primitive_wall_definitions.h:123-140
    delta[ax] = ppos - xv[ax];
    deltan = xv[ax] - ppos - radi;
  } else {
    delta[ax] = ppos - xv[ax];
    deltan = ppos - xv[ax] - radi;
  }
  if (pl.kind == 0) {
    delta[ay] = 0.;
    delta[az] = 0.;
  }
  if (deltan > s.cutneighmax) return;
  double *h = A.whist + (size_t)(w * 3) * s.nmax + i;
  const size_t hs = s.nmax;
  const double cdm1 = s.cdf - 1.0;
  if (deltan <= 0 || deltan < cdm1 * radi) {
    const double vwall[3] = {0., 0., 0.};
    wall_force<NORMAL>(s, A, i, deltan, delta, vwall, pl.wall_type ? pl.wall_type : A.type[i],
                       pl.rolling != 0, h, hs, shearupdate, v, om, fx, fy, fz, tx, ty, tz);
  } else {
    h[0] = 0.0; h[hs] = 0.0; h[2 * hs] = 0.0;
  }
}

// barycentric node velocity at the contact point (src/fix_wall_gran.cpp:929-934):
// the linear mover's node velocities are all vel, the rotating mover's nodev
__device__ __forceinline__ void mesh_vwall(const MeshDev &M, int t, const double bary[3], double vwall[3]) {
  if (M.rotating) {
    const double *vn = M.nodev + (size_t)t * 9;
    for (int d = 0; d < 3; d++) vwall[d] = (bary[0] * vn[d] + bary[1] * vn[3 + d] + bary[2] * vn[6 + d]);
  } else {
    for (int d = 0; d < 3; d++) vwall[d] = (bary[0] * M.vel[d] + bary[1] * M.vel[d] + bary[2] * M.vel[d]);
  }
}

// SurfaceMesh::areCoplanarNodeNeighs from the precomputed lists
__device__ __forceinline__ bool mesh_coplanar(const MeshDev &M, int a, int b) {
  for (int q = M.cn_start[a]; q < M.cn_start[a + 1]; q++)
    if (M.cn_list[q] == b) return true;
  return false;
}

// triangle id of a slot entry (-1: empty), without the kept mark
__device__ __forceinline__ int slot_tri_of(int v) { return v < 0 ? -1 : (v & ~kSlotKept); }

// The closest-feature contacts of atom i with mesh k, one candidate at a
// time in ascending triangle order (FixWallGran::post_force_mesh with
// FixContactHistoryMesh::handleContact, coplanarContactAlready,
// checkCoplanarContactHistory and cleanUpContacts).  A slot touched in this
// evaluation carries kSlotKept in slot_tri until the clean-up, so the number
// of candidates has no fixed bound.
template <int NORMAL>
__device__ void mesh_contacts(const Sys &s, const AtomArrays &A, int i, int k, int shearupdate,
                              double v[3], double om[3], double xv[3], double &fx, double &fy,
                              double &fz, double &tx, double &ty, double &tz, bool &bad, double msum[3]) {
  const MeshDev &M = s.meshes[k];
  const int nc = M.cand_n[i];
  if (nc == 0) return;
  const size_t nmax = s.nmax;
  int *st = M.slot_tri[0];
  double *sh = M.slot_hist[0];
  int np = M.npart[0][i];
  const double radi = A.r[i];
  const double cdm1 = s.cdf - 1.0;
  // a triangle is at least as far as its plane: candidates whose plane is
  // clearly beyond the contact range (relative margin 1e-9, far above the
  // rounding of either side) skip the closest-feature resolution; the
  // resolution would return deltan > 0 and skip them as well
  const double reach = __dmul_rn(__dadd_rn(radi, fmax(0.0, __dmul_rn(cdm1, radi))), 1.0 + 1e-9);
  // FP32 test first: the plane distance in FP32 is within 5*2^-24*S of the
  // FP64 one (S: sum of the magnitudes of the atom's and node 0's
  // coordinates), so a candidate farther than reach plus 2^-21*S is beyond
  // reach in FP64 too; the rest take the FP64 path below
  const float4 xa = s.xf[i];
  const float reach_f = (float)reach * (1.0f + 0x1p-20f);
  for (int q = 0; q < nc; q++) {
    const int t = M.cand[(size_t)q * nmax + i];
    {
      const float4 n0 = M.trif[2 * (size_t)t], sn = M.trif[2 * (size_t)t + 1];
      const float dnf = sn.x * (xa.x - n0.x) + sn.y * (xa.y - n0.y) + sn.z * (xa.z - n0.z);
      const float mag = fabsf(xa.x) + fabsf(xa.y) + fabsf(xa.z) + fabsf(n0.x) + fabsf(n0.y) + fabsf(n0.z);
      if (fabsf(dnf) > reach_f + mag * 0x1p-21f) continue;
    }
    const double *g = M.tri + (size_t)t * kTriStride;
    {
      const double *sn = tri_sn(g), *n0 = tri_node(g, 0);
      const double dn = sn[0] * (xv[0] - n0[0]) + sn[1] * (xv[1] - n0[1]) + sn[2] * (xv[2] - n0[2]);
      if (fabs(dn) > reach) continue;
    }
    double delta[3], bary[3];
    int bs;
    const double deltan = resolve_tri_sphere(g, M.meta[t], radi, xv, delta, bary, bs);
    if (deltan > s.cutneighmax) continue;
    if (!(deltan <= 0 || deltan < cdm1 * radi)) continue;
    int slot = -1;
    for (int u = 0; u < nc; u++)
      if (slot_tri_of(st[u * nmax + i]) == t) { slot = u; break; }
    if (slot >= 0) {
      st[slot * nmax + i] |= kSlotKept;
    } else {
      const bool face = bs == 7;
      if (face) {  // coplanarContactAlready
        bool already = false;
        for (int u = 0; u < nc; u++) {
          const int sv = st[u * nmax + i];
          const int p = slot_tri_of(sv);
          if (p >= 0 && p != t && (sv & kSlotKept) && mesh_coplanar(M, p, t)) already = true;
        }
        if (already) continue;
      }
      if (np >= nc) { bad = true; continue; }
      for (int u = 0; u < nc; u++)
        if (st[u * nmax + i] == -1) { slot = u; break; }
      st[slot * nmax + i] = t | kSlotKept;
      for (int d = 0; d < 3; d++) sh[(3 * slot + d) * nmax + i] = 0.0;
      np++;
      if (face)  // checkCoplanarContactHistory
        for (int u = 0; u < nc; u++) {
          const int p = slot_tri_of(st[u * nmax + i]);
          if (p >= 0 && p != t && mesh_coplanar(M, p, t))
            for (int d = 0; d < 3; d++) sh[(3 * slot + d) * nmax + i] = sh[(3 * u + d) * nmax + i];
        }
    }
    double vwall[3] = {0., 0., 0.};
    if (M.moving && M.vel_on) mesh_vwall(M, t, bary, vwall);
    double cfx = 0., cfy = 0., cfz = 0., ctx = 0., cty = 0., ctz = 0.;
    wall_force<NORMAL>(s, A, i, deltan, delta, vwall, M.wall_type, M.rolling != 0,
                         sh + (size_t)(3 * slot) * nmax + i, nmax, shearupdate, v, om, cfx, cfy, cfz, ctx, cty, ctz);
    fx += cfx; fy += cfy; fz += cfz;
    tx += ctx; ty += cty; tz += ctz;
    msum[0] += cfx; msum[1] += cfy; msum[2] += cfz;
  }
  for (int u = 0; u < nc; u++) {  // cleanUpContacts
    const int sv = st[u * nmax + i];
    if (sv >= 0 && (sv & kSlotKept)) {
      st[u * nmax + i] = sv & ~kSlotKept;
    } else {
      if (sv > -1) np--;
      st[u * nmax + i] = -1;
      for (int d = 0; d < 3; d++) sh[(3 * u + d) * nmax + i] = 0.0;
    }
  }
  M.npart[0][i] = np;
}

// FixWallGran::post_force_primitive / post_force_mesh for the atoms near a
// wall (the compact list of k_wall_list): wall forces and torques of the
// current state, planes then meshes in order, into fm/tm.  Independent of
// the pair kernel of the same step (it reads positions and velocities and
// writes only the wall histories, mesh slots and fm/tm), so the two run side
// by side; the per-atom kernel adds fm/tm.
//
// A block takes a tile of kWallTile listed atoms (one thread each) and, per
// mesh, runs the FP64-heavy parts densely over the tile's work instead of
// per atom (the FP64 pipe issues per warp instruction, and atoms differ in
// their number of candidates and contacts):
//   A  per atom, FP32: the candidates whose plane is within reach (see
//      mesh_contacts), queued in ascending order;
//   B  per queued candidate: exact plane test and closest feature
//      (TriMesh::resolveTriSphereContactBary), kept when touching;
//   C  per atom, integer work in candidate order: FixContactHistoryMesh's
//      slot semantics (handleContact, coplanarContactAlready); an atom whose
//      new face contact would copy a coplanar neighbour's history
//      (checkCoplanarContactHistory) takes the sequential path instead,
//      since that copy depends on the order of the contact updates;
//   D  per contact: the contact law with the slot's history;
//   E  per atom: contact forces summed in candidate order, slot clean-up.
// A tile whose queue would exceed its capacity (cap entries, a launch
// parameter) runs the sequential path for all its atoms.  Both paths give
// the same result.  The queue lives in dynamic shared memory, kWallQ bytes
// per entry: a smaller cap leaves room for more blocks beside the pair
// kernel that runs concurrently.
constexpr int kWallTile = 64;
constexpr int kWallCapDefault = 6;  // queue entries per tile atom (LIGGGHTS_GB300_WALL_CAP)
constexpr int kWallRes = 7;  // doubles per queued candidate: deltan, delta[3], vwall[3]; then F[3], T[3]
constexpr int kWallQ = kWallRes * 8 + 4 + 2;  // result doubles, state int, atom and candidate bytes

__device__ __forceinline__ int wall_tile_scan(int v, int &total, int *wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  int base = 0;
  total = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
    if (w < warp) base += wsum[w];
    total += wsum[w];
  }
  __syncthreads();
  return base + inc - v;
}

template <int NORMAL>
__global__ void __launch_bounds__(kWallTile) k_wall_force(Sys s, int shearupdate, int cap) {
  extern __shared__ double wres[];             // [cap * kWallRes], then qst, qa, qq
  int *qst = reinterpret_cast<int *>(wres + (size_t)cap * kWallRes);  // bit 0 touching, bit 1 face,
                                                                       // bits 8+: contact slot + 1
  unsigned char *qa = reinterpret_cast<unsigned char *>(qst + cap);
  unsigned char *qq = qa + cap;
  __shared__ int wsum[kWallTile / 32];
  Ctrl *c = s.ctrl;
  if (c->halt) return;
  const AtomArrays &A = s.atoms[0];
  const int nl = c->nmlist;
  const size_t nmax = s.nmax;
  const double cdm1 = s.cdf - 1.0;
  bool meshbad = false;
  for (int base = blockIdx.x * kWallTile; base < nl; base += gridDim.x * kWallTile) {
    const int a = threadIdx.x;
    const bool valid = base + a < nl;
    const int i = valid ? s.mlist[base + a] : 0;
    double v[3] = {0., 0., 0.}, om[3] = {0., 0., 0.}, xv[3] = {0., 0., 0.};
    double fx = 0., fy = 0., fz = 0., tx = 0., ty = 0., tz = 0.;
    if (valid) {
      v[0] = A.vx[i]; v[1] = A.vy[i]; v[2] = A.vz[i];
      om[0] = A.wx[i]; om[1] = A.wy[i]; om[2] = A.wz[i];
      xv[0] = A.x[i]; xv[1] = A.y[i]; xv[2] = A.z[i];
      const uint8_t bits = A.wbits[i];
      for (int w = 0; w < s.nplanes; w++) {
        double pfx = 0., pfy = 0., pfz = 0., ptx = 0., pty = 0., ptz = 0.;
        if (bits & (1u << w)) plane_contact<NORMAL>(s, A, i, w, shearupdate, v, om, xv, pfx, pfy, pfz, ptx, pty, ptz);
        fx += pfx; fy += pfy; fz += pfz;
        tx += ptx; ty += pty; tz += ptz;
        s.wforce[(size_t)(3 * w) * nmax + i] = pfx;
        s.wforce[(size_t)(3 * w + 1) * nmax + i] = pfy;
        s.wforce[(size_t)(3 * w + 2) * nmax + i] = pfz;
      }
    }
    for (int k = 0; k < s.nmeshes; k++) {
      const MeshDev &M = s.meshes[k];
      int *st = M.slot_tri[0];
      double *sh = M.slot_hist[0];
      // ---- A: FP32 candidate pass
      const int nc = valid ? M.cand_n[i] : 0;
      const double radi = valid ? A.r[i] : 0.0;
      const double reach = __dmul_rn(__dadd_rn(radi, fmax(0.0, __dmul_rn(cdm1, radi))), 1.0 + 1e-9);
      unsigned todo = 0u;
      const bool big = nc > kMeshFastCand;  // beyond the 32-bit masks: sequential path
      if (nc > 0 && !big) {
        const float4 xa = s.xf[i];
        const float reach_f = (float)reach * (1.0f + 0x1p-20f);
        for (int q = 0; q < nc; q++) {
          const int t = M.cand[(size_t)q * nmax + i];
          const float4 n0 = M.trif[2 * (size_t)t], sn = M.trif[2 * (size_t)t + 1];
          const float dn = sn.x * (xa.x - n0.x) + sn.y * (xa.y - n0.y) + sn.z * (xa.z - n0.z);
          const float mag = fabsf(xa.x) + fabsf(xa.y) + fabsf(xa.z) + fabsf(n0.x) + fabsf(n0.y) + fabsf(n0.z);
          if (!(fabsf(dn) > reach_f + mag * 0x1p-21f)) todo |= 1u << q;
        }
      }
      const int cnt = __popc(todo);
      int total;
      const int off = wall_tile_scan(cnt, total, wsum);
      double msum[3] = {0., 0., 0.};
      double *const wf = s.wforce + (size_t)(3 * (s.nplanes + k)) * nmax;
      if (total > cap) {  // sequential path for this tile
        if (nc > 0) mesh_contacts<NORMAL>(s, A, i, k, shearupdate, v, om, xv, fx, fy, fz, tx, ty, tz, meshbad, msum);
        if (valid)
          for (int d = 0; d < 3; d++) wf[(size_t)d * nmax + i] = msum[d];
        __syncthreads();
        continue;
      }
      {
        unsigned m = todo;
        for (int e = off; m; e++) {
          qa[e] = (unsigned char)a;
          qq[e] = (unsigned char)(__ffs(m) - 1);
          m &= m - 1u;
        }
      }
      __syncthreads();
      // ---- B: exact plane test and closest feature per queued candidate
      for (int e = threadIdx.x; e < total; e += kWallTile) {
        const int ie = s.mlist[base + qa[e]];
        const int t = M.cand[(size_t)qq[e] * nmax + ie];
        const double *g = M.tri + (size_t)t * kTriStride;
        const double xe[3] = {A.x[ie], A.y[ie], A.z[ie]};
        const double re = A.r[ie];
        const double reach_e = __dmul_rn(__dadd_rn(re, fmax(0.0, __dmul_rn(cdm1, re))), 1.0 + 1e-9);
        int state = 0;
        const double *snv = tri_sn(g), *n0 = tri_node(g, 0);
        const double dn = snv[0] * (xe[0] - n0[0]) + snv[1] * (xe[1] - n0[1]) + snv[2] * (xe[2] - n0[2]);
        if (!(fabs(dn) > reach_e)) {
          double delta[3], bary[3];
          int bs;
          const double deltan = resolve_tri_sphere(g, M.meta[t], re, xe, delta, bary, bs);
          if (!(deltan > s.cutneighmax) && (deltan <= 0 || deltan < cdm1 * re)) {
            state = 1 | (bs == 7 ? 2 : 0);
            double *r = wres + (size_t)e * kWallRes;
            r[0] = deltan;
            r[1] = delta[0]; r[2] = delta[1]; r[3] = delta[2];
            double vwall[3] = {0., 0., 0.};
            if (M.moving && M.vel_on) mesh_vwall(M, t, bary, vwall);
            r[4] = vwall[0]; r[5] = vwall[1]; r[6] = vwall[2];
          }
        }
        qst[e] = state;
      }
      __syncthreads();
      // ---- C: slot semantics per atom, in candidate order
      bool fallback = big;
      unsigned keep = 0u;
      int np = 0;
      if (nc > 0 && !big) {
        np = M.npart[0][i];
        int stl[kMeshFastCand];
        for (int u = 0; u < nc; u++) stl[u] = st[u * nmax + i];
        unsigned fresh = 0u;
        for (int e = off; e < off + cnt && !fallback; e++) {
          if (!(qst[e] & 1)) continue;
          const int t = M.cand[(size_t)qq[e] * nmax + i];
          int slot = -1;
          for (int u = 0; u < nc; u++)
            if (stl[u] == t) { slot = u; break; }
          if (slot >= 0) {
            keep |= 1u << slot;
          } else {
            const bool face = (qst[e] & 2) != 0;
            if (face) {  // coplanarContactAlready
              bool already = false;
              for (int u = 0; u < nc; u++)
                if (stl[u] >= 0 && stl[u] != t && ((keep >> u) & 1u) && mesh_coplanar(M, stl[u], t)) already = true;
              if (already) continue;
            }
            if (np >= nc) { meshbad = true; continue; }
            for (int u = 0; u < nc; u++)
              if (stl[u] == -1) { slot = u; break; }
            if (face)  // checkCoplanarContactHistory would copy: order-dependent
              for (int u = 0; u < nc; u++)
                if (stl[u] >= 0 && stl[u] != t && mesh_coplanar(M, stl[u], t)) fallback = true;
            if (fallback) break;
            stl[slot] = t;
            keep |= 1u << slot;
            fresh |= 1u << slot;
            np++;
          }
          qst[e] |= (slot + 1) << 8;
        }
        if (fallback) {
          for (int e = off; e < off + cnt; e++) qst[e] &= 0xff;
        } else {
          for (int u = 0; u < nc; u++)
            if ((fresh >> u) & 1u) {
              st[u * nmax + i] = stl[u];
              for (int d = 0; d < 3; d++) sh[(3 * u + d) * nmax + i] = 0.0;
            }
        }
      }
      __syncthreads();
      // ---- D: contact law per contact
      for (int e = threadIdx.x; e < total; e += kWallTile) {
        const int slot = (qst[e] >> 8) - 1;
        if (slot < 0) continue;
        const int ie = s.mlist[base + qa[e]];
        double *r = wres + (size_t)e * kWallRes;
        const double delta[3] = {r[1], r[2], r[3]};
        const double vwall[3] = {r[4], r[5], r[6]};
        double ve[3] = {A.vx[ie], A.vy[ie], A.vz[ie]};
        double oe[3] = {A.wx[ie], A.wy[ie], A.wz[ie]};
        double cfx = 0., cfy = 0., cfz = 0., ctx = 0., cty = 0., ctz = 0.;
        wall_force<NORMAL>(s, A, ie, r[0], delta, vwall, M.wall_type, M.rolling != 0,
                           sh + (size_t)(3 * slot) * nmax + ie, nmax, shearupdate, ve, oe, cfx, cfy, cfz, ctx,
                           cty, ctz);
        r[0] = cfx; r[1] = cfy; r[2] = cfz;
        r[3] = ctx; r[4] = cty; r[5] = ctz;
      }
      __syncthreads();
      // ---- E: sums in candidate order, clean-up (or the sequential path)
      if (nc > 0) {
        if (fallback) {
          mesh_contacts<NORMAL>(s, A, i, k, shearupdate, v, om, xv, fx, fy, fz, tx, ty, tz, meshbad, msum);
        } else {
          for (int e = off; e < off + cnt; e++) {
            if ((qst[e] >> 8) == 0) continue;
            const double *r = wres + (size_t)e * kWallRes;
            fx += r[0]; fy += r[1]; fz += r[2];
            tx += r[3]; ty += r[4]; tz += r[5];
            msum[0] += r[0]; msum[1] += r[1]; msum[2] += r[2];
          }
          for (int u = 0; u < nc; u++)  // cleanUpContacts
            if (!((keep >> u) & 1u)) {
              if (st[u * nmax + i] > -1) np--;
              st[u * nmax + i] = -1;
              for (int d = 0; d < 3; d++) sh[(3 * u + d) * nmax + i] = 0.0;
            }
          M.npart[0][i] = np;
        }
      }
      if (valid)
        for (int d = 0; d < 3; d++) wf[(size_t)d * nmax + i] = msum[d];
      __syncthreads();
    }
    if (valid) {
      A.fmx[i] = fx; A.fmy[i] = fy; A.fmz[i] = fz;
      A.tmx[i] = tx; A.tmy[i] = ty; A.tmz[i] = tz;
    }
  }
  if (__any_sync(0xffffffffu, meshbad) && (threadIdx.x & 31) == 0) atomicExch(&c->status, kStatMeshSlots);
}

// Force gather of one atom: its own row (ascending), then its reverse list
// (ascending), the reference's per-atom order.  The FP64 pipe issues per warp
// instruction, so additions inside a loop over all list entries cost one
// issue per entry of the warp's longest row, active or not.  Here a first,
// integer-only pass collects the active entries of up to 32 entries per list
// as bit masks (gather_masks); one loop over the set bits then does the FP64
// additions (gather_sum).  A reverse contribution adds the negated force
// (sign bit flipped on the integer pipe: a + (-b) is exactly a - b) and Tj
// instead of Ti.  k_particle hands the loops of a block's atoms to its
// threads sorted by contact count, so that a warp's lanes run loops of equal
// length (see there).
__device__ __forceinline__ bool gather_masks(const Sys &s, const PairArrays &L, int i, int &pb, int &rb,
                                             unsigned &om, unsigned &rm) {
  pb = L.row[i];
  rb = L.rev_start[i];
  const int pe = row_end(s, L, i), re = rev_end(s, L, i);
  if (pe - pb > 32 || re - rb > 32) return false;
  om = 0u;
  rm = 0u;
  for (int k = 0; k < pe - pb; k++) om |= (s.active[pb + k] ? 1u : 0u) << k;
  for (int k = 0; k < re - rb; k++) rm |= (s.active[L.rev[rb + k]] ? 1u : 0u) << k;
  return true;
}

__device__ __forceinline__ void gather_sum(const Sys &s, const PairArrays &L, int pb, int rb, unsigned om,
                                           unsigned rm, double &fx, double &fy, double &fz, double &tx, double &ty,
                                           double &tz) {
  const int cnt = __popc(om) + __popc(rm);
  for (int t = 0; t < cnt; t++) {
    int p;
    unsigned long long sg;
    int to;  // offset of the torque in the record: Ti (own row) or Tj (partner)
    if (om) {
      p = pb + __ffs(om) - 1;
      om &= om - 1u;
      sg = 0ull;
      to = 3;
    } else {
      p = L.rev[rb + __ffs(rm) - 1];
      rm &= rm - 1u;
      sg = 0x8000000000000000ull;
      to = 6;
    }
    const double *r = s.res + (size_t)kResStride * p;
    fx += __longlong_as_double(__double_as_longlong(r[0]) ^ sg);
    fy += __longlong_as_double(__double_as_longlong(r[1]) ^ sg);
    fz += __longlong_as_double(__double_as_longlong(r[2]) ^ sg);
    tx += r[to];
    ty += r[to + 1];
    tz += r[to + 2];
  }
}

// lists longer than 32 entries: one pass over every entry
__device__ __forceinline__ void gather_long(const Sys &s, const PairArrays &L, int i, double &fx, double &fy,
                                            double &fz, double &tx, double &ty, double &tz) {
  const int pb = L.row[i], pe = row_end(s, L, i);
  const int rb = L.rev_start[i], re = rev_end(s, L, i);
  for (int p = pb; p < pe; p++) {
    if (!s.active[p]) continue;
    const double *r = s.res + (size_t)kResStride * p;
    fx += r[0]; fy += r[1]; fz += r[2];
    tx += r[3]; ty += r[4]; tz += r[5];
  }
  for (int k = rb; k < re; k++) {
    const int p = L.rev[k];
    if (!s.active[p]) continue;
    const double *r = s.res + (size_t)kResStride * p;
    fx -= r[0]; fy -= r[1]; fz -= r[2];
    tx += r[6]; ty += r[7]; tz += r[8];
  }
}

// the block-level sort of k_particle's gather: loops of up to kGatherKeys-1
// contacts by count, longer ones together in the last key
constexpr int kGatherKeys = 32;
constexpr int kParticleMaxThreads = 256;

// Per atom: force gather, gravity, wall totals, nve/sphere, FP32 copy,
// displacement check.  The gather runs in three block-wide phases, because a
// warp's contact loops issue their FP64 additions once per contact of its
// busiest atom: (1) every thread forms its atom's start sums (gravity) and
// contact masks; (2) the atoms with contacts are sorted by their contact
// count in shared memory; (3) thread t runs the loop of the t-th atom in that
// order, so that a warp's lanes run loops of equal length, and the sums go
// back to the owner.  Each atom's sum keeps its order and its one thread, so
// the result does not depend on the sort or the launch shape.
// Graph steps without moving meshes: the last block of k_particle to finish
// takes the step's rebuild decision and sets the loop's conditionals, as
// k_decide_loop does after it otherwise (one node and one dependency fewer
// per step).
struct LoopCond {
  int on;
  cudaGraphConditionalHandle hreb, hloop;
};

template <int NORMAL, bool GATHER, bool FINAL, bool INITIAL>
__global__ void __launch_bounds__(kParticleMaxThreads, 4) k_particle(Sys s, int shearupdate, LoopCond lp) {
  __shared__ double gsum[GATHER ? 6 : 1][GATHER ? kParticleMaxThreads : 1];
  __shared__ int gpb[GATHER ? kParticleMaxThreads : 1], grb[GATHER ? kParticleMaxThreads : 1];
  __shared__ unsigned gom[GATHER ? kParticleMaxThreads : 1], grm[GATHER ? kParticleMaxThreads : 1];
  __shared__ short gsorted[GATHER ? kParticleMaxThreads : 1];
  __shared__ int gcount[kGatherKeys], gfill[kGatherKeys], gstart[kGatherKeys], gnq;
  __shared__ int last_block;
  Ctrl *c = s.ctrl;
  if (c->halt) {
    if (lp.on && blockIdx.x == 0 && threadIdx.x == 0) {
      cudaGraphSetConditional(lp.hreb, 0);
      cudaGraphSetConditional(lp.hloop, 0);
    }
    return;
  }
  const AtomArrays &A = s.atoms[0];
  const PairArrays &L = s.pairs[0];
  const int n = c->n;
  const double dtv = s.dt;
  const double trigger = 0.25 * s.skin * s.skin;
  const int tid = threadIdx.x;
  bool moved = false, bad = false;
  if (GATHER) {
    if (tid < kGatherKeys) {
      gcount[tid] = 0;
      gfill[tid] = 0;
    }
    __syncthreads();
  }
  for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const int i = base + tid;
    const bool valid = i < n;
    double fx = 0.0, fy = 0.0, fz = 0.0, tx = 0.0, ty = 0.0, tz = 0.0;
    double v[3] = {0.0, 0.0, 0.0}, om[3] = {0.0, 0.0, 0.0}, xv[3] = {0.0, 0.0, 0.0};
    if (valid) {
      v[0] = A.vx[i]; v[1] = A.vy[i]; v[2] = A.vz[i];
      om[0] = A.wx[i]; om[1] = A.wy[i]; om[2] = A.wz[i];
      xv[0] = A.x[i]; xv[1] = A.y[i]; xv[2] = A.z[i];
    }
    if (GATHER) {
      // FixGravity::post_force (src/fix_gravity.cpp:329-337) adds m*g after
      // the pair forces; starting the sum from it instead changes only the
      // rounding order and saves three FP64 additions
      if (valid && s.gravity_on) {
        const double massone = A.m[i];
        fx = __dmul_rn(massone, s.g[0]);
        fy = __dmul_rn(massone, s.g[1]);
        fz = __dmul_rn(massone, s.g[2]);
      }
      // (1) masks and counts; lists longer than 32 entries are summed here
      // by the owner (gcount and gfill are zero: cleared after the last use)
      int key = 0;
      if (valid) {
        int pb, rb;
        unsigned mo, mr;
        if (gather_masks(s, L, i, pb, rb, mo, mr)) {
          const int cnt = __popc(mo) + __popc(mr);
          if (cnt) {
            key = cnt < kGatherKeys ? cnt : kGatherKeys - 1;
            gpb[tid] = pb;
            grb[tid] = rb;
            gom[tid] = mo;
            grm[tid] = mr;
            gsum[0][tid] = fx; gsum[1][tid] = fy; gsum[2][tid] = fz;
            gsum[3][tid] = tx; gsum[4][tid] = ty; gsum[5][tid] = tz;
          }
        } else {
          gather_long(s, L, i, fx, fy, fz, tx, ty, tz);
        }
      }
      // (2) counting sort of the block's atoms with contacts by their count
      if (key) atomicAdd(&gcount[key], 1);
      __syncthreads();
      if (tid < 32) {
        const int v0 = tid < kGatherKeys ? gcount[tid] : 0;
        const int inc = warp_incl_scan(v0);
        if (tid < kGatherKeys) gstart[tid] = inc - v0;
        if (tid == 31) gnq = inc;
      }
      __syncthreads();
      if (key) gsorted[gstart[key] + atomicAdd(&gfill[key], 1)] = (short)tid;
      __syncthreads();
      if (tid < kGatherKeys) {  // read by no one until the next block of atoms counts
        gcount[tid] = 0;
        gfill[tid] = 0;
      }
      // (3) the loops, one atom per thread in sorted order
      if (tid < gnq) {
        const int a = gsorted[tid];
        double sx = gsum[0][a], sy = gsum[1][a], sz = gsum[2][a];
        double qx = gsum[3][a], qy = gsum[4][a], qz = gsum[5][a];
        gather_sum(s, L, gpb[a], grb[a], gom[a], grm[a], sx, sy, sz, qx, qy, qz);
        gsum[0][a] = sx; gsum[1][a] = sy; gsum[2][a] = sz;
        gsum[3][a] = qx; gsum[4][a] = qy; gsum[5][a] = qz;
      }
      __syncthreads();
      if (key) {
        fx = gsum[0][tid]; fy = gsum[1][tid]; fz = gsum[2][tid];
        tx = gsum[3][tid]; ty = gsum[4][tid]; tz = gsum[5][tid];
      }
    }
    if (!valid) continue;
    if (GATHER) {
      if (A.wbits[i] & 0x80u) {  // walls, computed by k_wall_force for this step
        fx += A.fmx[i]; fy += A.fmy[i]; fz += A.fmz[i];
        tx += A.tmx[i]; ty += A.tmy[i]; tz += A.tmz[i];
      }
      // the sums are kept for the download and the next call's first
      // step; inside a run (FINAL && INITIAL) nothing reads them
      if (!(FINAL && INITIAL)) {
        A.fx[i] = fx; A.fy[i] = fy; A.fz[i] = fz;
        A.tx[i] = tx; A.ty[i] = ty; A.tz[i] = tz;
      }
    } else {
      fx = A.fx[i]; fy = A.fy[i]; fz = A.fz[i];
      tx = A.tx[i]; ty = A.ty[i]; tz = A.tz[i];
    }
    if (FINAL || INITIAL) {
      // FixNVESphere half-kicks and drift as fused multiply-adds: one FP64
      // instruction each (the FP64 pipe bounds this kernel on GB300); the
      // single rounding moves positions by at most an ulp from the reference.
      // The final half-kick of step n and the initial one of step n+1 use
      // the same force: fused into one FMA with 2*dtfm (2*dtir), exact
      // scalings, one rounding instead of two.
      const double dtfm = A.dtfm[i], dtir = A.dtir[i];
      if (FINAL && INITIAL) {
        v[0] = fma(2.0 * dtfm, fx, v[0]);
        v[1] = fma(2.0 * dtfm, fy, v[1]);
        v[2] = fma(2.0 * dtfm, fz, v[2]);
        om[0] = fma(2.0 * dtir, tx, om[0]);
        om[1] = fma(2.0 * dtir, ty, om[1]);
        om[2] = fma(2.0 * dtir, tz, om[2]);
      } else if (FINAL || INITIAL) {
        v[0] = fma(dtfm, fx, v[0]);
        v[1] = fma(dtfm, fy, v[1]);
        v[2] = fma(dtfm, fz, v[2]);
        om[0] = fma(dtir, tx, om[0]);
        om[1] = fma(dtir, ty, om[1]);
        om[2] = fma(dtir, tz, om[2]);
      }
      if (INITIAL) {
        xv[0] = fma(dtv, v[0], xv[0]);
        xv[1] = fma(dtv, v[1], xv[1]);
        xv[2] = fma(dtv, v[2], xv[2]);
        A.x[i] = xv[0]; A.y[i] = xv[1]; A.z[i] = xv[2];
        // the FP32 radius of the copy does not change: no conversion
        const float4 nf = make_float4((float)xv[0], (float)xv[1], (float)xv[2], s.xf[i].w);
        s.xf[i] = nf;
        // Neighbor::check_distance (src/neighbor.cpp:1426-1466) with an FP32
        // prefilter: only displacements within the rounding band of skin/2
        // take the exact FP64 test, so the decision is the reference's
        const float4 hf = s.xhf[i];
        const float ex = nf.x - hf.x, ey = nf.y - hf.y, ez = nf.z - hf.z;
        const float rf2 = ex * ex + ey * ey + ez * ez;
        bool mv = false;
        if (rf2 > s.skin_hi2) {
          mv = true;
        } else if (rf2 > s.skin_lo2) {
          const double dx = __dadd_rn(xv[0], -A.xh[i]);
          const double dy = __dadd_rn(xv[1], -A.yh[i]);
          const double dz = __dadd_rn(xv[2], -A.zh[i]);
          if (rsq_rn(dx, dy, dz) > trigger) mv = true;
        }
        if (mv && s.nsys) s.sys_moved[A.type[i] - 1] = 1;  // this atom's system (ensembles)
        moved |= mv;
        // a non-finite coordinate converts to a non-finite float (so does one
        // beyond the FP32 range, which no granular box reaches)
        if (!(isfinite(nf.x) && isfinite(nf.y) && isfinite(nf.z))) bad = true;
      }
      A.vx[i] = v[0]; A.vy[i] = v[1]; A.vz[i] = v[2];
      A.wx[i] = om[0]; A.wy[i] = om[1]; A.wz[i] = om[2];
    }
  }
  (void)shearupdate;
  if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(&c->moved, 1);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) {
    atomicExch(&c->status, kStatNan);
  }
  if (lp.on) {  // the last block to finish decides (k_decide_loop's work)
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      last_block = atomicAdd(&c->pdone, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (last_block) {
      __threadfence();
      if (threadIdx.x == 0) {
        c->pdone = 0;
        c->ntimestep++;
      }
      const int reb = decide_rebuild(s, c);
      if (threadIdx.x == 0) {
        c->loop_left--;
        cudaGraphSetConditional(lp.hreb, reb ? 1u : 0u);
        cudaGraphSetConditional(lp.hloop, c->loop_left > 0 ? 1u : 0u);
      }
    }
  }
}

// ----------------------------------------------------------------------------
// insertion (dem_insert_atoms): new atoms are staged into the unused slots
// [first, first + k) of atom buffer 0 between steps and join the system at
// the next step after its initial integration, with a forced rebuild, as
// FixInsert::pre_exchange adds them in the reference (src/fix_insert.cpp,
// pre_exchange with next_reneighbor = the insertion step)
// ----------------------------------------------------------------------------

__global__ void k_insert_stage(Sys s, InsertStage in, int first, int k, int lidx0) {
  const AtomArrays &A = s.atoms[0];
  const size_t nmax = s.nmax;
  GRID_STRIDE(q, k) {
    const int i = first + q;
    A.x[i] = in.x[3 * q]; A.y[i] = in.x[3 * q + 1]; A.z[i] = in.x[3 * q + 2];
    A.vx[i] = in.v[3 * q]; A.vy[i] = in.v[3 * q + 1]; A.vz[i] = in.v[3 * q + 2];
    A.wx[i] = in.w[3 * q]; A.wy[i] = in.w[3 * q + 1]; A.wz[i] = in.w[3 * q + 2];
    A.fx[i] = A.fy[i] = A.fz[i] = 0.0;
    A.tx[i] = A.ty[i] = A.tz[i] = 0.0;
    A.xh[i] = A.x[i]; A.yh[i] = A.y[i]; A.zh[i] = A.z[i];
    A.r[i] = in.r[q]; A.m[i] = in.m[q];
    A.dtfm[i] = in.dtfm[q]; A.dtir[i] = in.dtir[q];
    A.type[i] = in.type[q]; A.tag[i] = in.tag[q]; A.lidx[i] = lidx0 + q;
    for (int w = 0; w < s.nplanes; w++)
      for (int d = 0; d < 3; d++) A.whist[(size_t)(w * 3 + d) * nmax + i] = 0.0;
    A.wbits[i] = 0;
    A.fmx[i] = A.fmy[i] = A.fmz[i] = A.tmx[i] = A.tmy[i] = A.tmz[i] = 0.0;
    const float4 f = make_float4((float)A.x[i], (float)A.y[i], (float)A.z[i], (float)A.r[i]);
    s.xf[i] = f;
    s.xhf[i] = f;
    for (int m = 0; m < s.nmeshes; m++) {
      const MeshDev &M = s.meshes[m];
      M.cand_n[i] = 0;
      M.nslot[0][i] = 0;
      M.npart[0][i] = 0;
      for (int u = 0; u < M.ccap; u++) {
        M.slot_tri[0][(size_t)u * nmax + i] = -1;
        for (int d = 0; d < 3; d++) M.slot_hist[0][(size_t)(3 * u + d) * nmax + i] = 0.0;
      }
    }
  }
}

// the new atoms get empty rows in the current (old) list, so that the
// rebuild's history carry-over finds nothing for them
__global__ void k_insert_commit(Sys s, int k) {
  __shared__ int n_old;
  Ctrl *c = s.ctrl;
  if (c->halt) return;
  if (threadIdx.x == 0) n_old = c->n;
  __syncthreads();
  const PairArrays &L = s.pairs[0];
  const int r = L.row[n_old], rv = L.rev_start[n_old];
  for (int q = threadIdx.x; q < k; q += blockDim.x) {
    L.row[n_old + 1 + q] = r;
    L.rev_start[n_old + 1 + q] = rv;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    c->n = n_old + k;
    c->force_rebuild = 1;
  }
}

// ----------------------------------------------------------------------------
// atom transfer: caller AoS <-> device SoA (dem_upload_atoms, dem_download_atoms)
// ----------------------------------------------------------------------------

__global__ void k_upload_atoms(Sys s, AtomsIn in, int n, double dtf, double dtfrotate, UploadCheck *chk) {
  const AtomArrays &A = s.atoms[0];
  const size_t nmax = s.nmax;
  unsigned long long rmin = ~0ull, rmax = 0ull;
  int bad_type = 0, bad_value = 0, nonfinite = 0;
  GRID_STRIDE(i, n) {
    const double x0 = in.x[3 * i], x1 = in.x[3 * i + 1], x2 = in.x[3 * i + 2];
    const double v0 = in.v[3 * i], v1 = in.v[3 * i + 1], v2 = in.v[3 * i + 2];
    const double w0 = in.w[3 * i], w1 = in.w[3 * i + 1], w2 = in.w[3 * i + 2];
    const double r = in.r[i], m = in.m[i];
    const int t = in.type[i];
    bad_type += (t < 1 || t > s.ntypes) ? 1 : 0;
    const bool okv = r > 0.0 && m > 0.0 && isfinite(r) && isfinite(m);
    bad_value += okv ? 0 : 1;
    const bool fin = isfinite(x0) && isfinite(x1) && isfinite(x2) && isfinite(v0) && isfinite(v1) &&
                     isfinite(v2) && isfinite(w0) && isfinite(w1) && isfinite(w2);
    nonfinite += fin ? 0 : 1;
    A.x[i] = x0; A.y[i] = x1; A.z[i] = x2;
    A.vx[i] = v0; A.vy[i] = v1; A.vz[i] = v2;
    A.wx[i] = w0; A.wy[i] = w1; A.wz[i] = w2;
    A.r[i] = r; A.m[i] = m;
    A.type[i] = t; A.tag[i] = in.tag[i]; A.lidx[i] = i;
    // FixNVESphere per-atom factors, as its init/initial_integrate form them
    // (src/fix_nve_sphere.cpp:150-178): dtf/(m*(1+CAdd/rho)) with no added
    // mass, dtfrotate/(r*r*m)
    A.dtfm[i] = dtf / (m * (1. + 0.0));
    A.dtir[i] = dtfrotate / (r * r * m);
    A.fx[i] = A.fy[i] = A.fz[i] = 0.0;
    A.tx[i] = A.ty[i] = A.tz[i] = 0.0;
    A.xh[i] = A.yh[i] = A.zh[i] = 0.0;
    for (int k = 0; k < 3 * s.nplanes; k++) A.whist[(size_t)k * nmax + i] = 0.0;
    A.wbits[i] = 0;
    A.fmx[i] = A.fmy[i] = A.fmz[i] = A.tmx[i] = A.tmy[i] = A.tmz[i] = 0.0;
    if (okv) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(r);
      rmin = b < rmin ? b : rmin;
      rmax = b > rmax ? b : rmax;
    }
  }
  // positive doubles order as their bit patterns
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_down_sync(0xffffffffu, rmin, o);
    const unsigned long long b = __shfl_down_sync(0xffffffffu, rmax, o);
    rmin = a < rmin ? a : rmin;
    rmax = b > rmax ? b : rmax;
    bad_type += __shfl_down_sync(0xffffffffu, bad_type, o);
    bad_value += __shfl_down_sync(0xffffffffu, bad_value, o);
    nonfinite += __shfl_down_sync(0xffffffffu, nonfinite, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (rmin != ~0ull) atomicMin(&chk->rmin, rmin);
    if (rmax) atomicMax(&chk->rmax, rmax);
    if (bad_type) atomicAdd(&chk->bad_type, bad_type);
    if (bad_value) atomicAdd(&chk->bad_value, bad_value);
    if (nonfinite) atomicAdd(&chk->nonfinite, nonfinite);
  }
}

// One block writes a tile of kDownTile atoms. Each 3-vector goes through
// shared memory so that a warp's stores cover 256 contiguous bytes of the
// caller's array: strided stores (one component per instruction) left two
// thirds of every line they touched for later instructions, which over the
// host link took 2.9 ms for 1M atoms against 0.8 ms this way.
constexpr int kDownTile = 256;

__global__ void __launch_bounds__(kDownTile) k_download_atoms(Sys s, AtomsOut out, int n) {
  const AtomArrays &A = s.atoms[0];
  __shared__ double tile[3 * kDownTile];
  double *dst[5] = {out.x, out.v, out.w, out.f, out.t};
  const double *src[5][3] = {{A.x, A.y, A.z}, {A.vx, A.vy, A.vz}, {A.wx, A.wy, A.wz},
                             {A.fx, A.fy, A.fz}, {A.tx, A.ty, A.tz}};
  for (int b = blockIdx.x; (long)b * kDownTile < n; b += gridDim.x) {
    const int a0 = b * kDownTile, cnt = min(kDownTile, n - a0);
    const int t = threadIdx.x, i = a0 + t;
    for (int k = 0; k < 5; k++) {
      if (!dst[k]) continue;  // the same for the whole block
      if (t < cnt) {
        tile[3 * t] = src[k][0][i];
        tile[3 * t + 1] = src[k][1][i];
        tile[3 * t + 2] = src[k][2][i];
      }
      __syncthreads();
      double *base = dst[k] + 3 * (size_t)a0;
      for (int q = t; q < 3 * cnt; q += kDownTile) base[q] = tile[q];
      __syncthreads();
    }
    if (t < cnt) {
      if (out.r) out.r[i] = A.r[i];
      if (out.m) out.m[i] = A.m[i];
      if (out.tag) out.tag[i] = A.tag[i];
      if (out.type) out.type[i] = A.type[i];
    }
  }
}

int launch_upload_atoms(const Sys &s, const AtomsIn &in, int n, double dtf, double dtfrotate, UploadCheck *chk,
                        cudaStream_t st) {
  if (n <= 0) return 0;
  k_upload_atoms<<<std::min((n + 255) / 256, 152 * 16), 256, 0, st>>>(s, in, n, dtf, dtfrotate, chk);
  return 1;
}

int launch_download_atoms(const Sys &s, const AtomsOut &out, int n, cudaStream_t st) {
  if (n <= 0) return 0;
  k_download_atoms<<<std::min((n + kDownTile - 1) / kDownTile, 152 * 8), kDownTile, 0, st>>>(s, out, n);
  return 1;
}

int launch_insert_stage(const Sys &s, const InsertStage &in, int first, int k, int lidx0, cudaStream_t st) {
  k_insert_stage<<<(k + 127) / 128, 128, 0, st>>>(s, in, first, k, lidx0);
  return 1;
}

int launch_insert_commit(const Sys &s, int k, cudaStream_t st) {
  k_insert_commit<<<1, 256, 0, st>>>(s, k);
  return 1;
}

// ----------------------------------------------------------------------------
// diagnostics (dem_get_diagnostics): deterministic per-block partial sums,
// added in block order by the host
// ----------------------------------------------------------------------------

constexpr int kDiagBlock = 256;

__device__ __forceinline__ double block_sum(double v, double *sm) {
  sm[threadIdx.x] = v;
  __syncthreads();
  for (int st = kDiagBlock / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sm[threadIdx.x] += sm[threadIdx.x + st];
    __syncthreads();
  }
  const double r = sm[0];
  __syncthreads();
  return r;
}

// ComputeKE (sum m v^2), ComputeERotateSphere (sum w^2 r^2 m) and the solid
// volume (sum r^3) of the atoms whose centre lies in [lo, hi)
__global__ void __launch_bounds__(kDiagBlock) k_diag_atoms(Sys s, double3 lo, double3 hi, double *part) {
  __shared__ double sm[kDiagBlock];
  const AtomArrays &A = s.atoms[0];
  const int n = s.ctrl->n;
  double ke = 0.0, er = 0.0, vol = 0.0;
  GRID_STRIDE(i, n) {
    const double m = A.m[i], r = A.r[i];
    ke += m * (A.vx[i] * A.vx[i] + A.vy[i] * A.vy[i] + A.vz[i] * A.vz[i]);
    er += (A.wx[i] * A.wx[i] + A.wy[i] * A.wy[i] + A.wz[i] * A.wz[i]) * r * r * m;
    const double x = A.x[i], y = A.y[i], z = A.z[i];
    if (x >= lo.x && x < hi.x && y >= lo.y && y < hi.y && z >= lo.z && z < hi.z) vol += r * r * r;
  }
  ke = block_sum(ke, sm);
  er = block_sum(er, sm);
  vol = block_sum(vol, sm);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = ke;
    part[3 * blockIdx.x + 1] = er;
    part[3 * blockIdx.x + 2] = vol;
  }
}

// per-wall force sums over the listed wall atoms: part[(blk*nw + w)*3 + d]
__global__ void __launch_bounds__(kDiagBlock) k_diag_walls(Sys s, int nw, double *part) {
  __shared__ double sm[kDiagBlock];
  const int nl = s.ctrl->nmlist;
  for (int w = 0; w < nw; w++)
    for (int d = 0; d < 3; d++) {
      const double *wf = s.wforce + (size_t)(3 * w + d) * s.nmax;
      double acc = 0.0;
      GRID_STRIDE(q, nl) acc += wf[s.mlist[q]];
      acc = block_sum(acc, sm);
      if (threadIdx.x == 0) part[((size_t)blockIdx.x * nw + w) * 3 + d] = acc;
    }
}

// list entries with a contact force in the last force evaluation
__global__ void k_diag_contacts(Sys s, unsigned long long *cnt) {
  const int np = s.ctrl->np;
  unsigned long long c = 0;
  GRID_STRIDE(p, np) c += s.active[p] ? 1ull : 0ull;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(cnt, c);
}

int launch_diagnostics(const Sys &s, const LaunchCfg &lc, const double lo[3], const double hi[3], double *part_atoms,
                       double *part_walls, unsigned long long *contacts, int nblocks, cudaStream_t st) {
  const int nw = s.nplanes + s.nmeshes;
  k_diag_atoms<<<nblocks, kDiagBlock, 0, st>>>(s, make_double3(lo[0], lo[1], lo[2]),
                                               make_double3(hi[0], hi[1], hi[2]), part_atoms);
  if (nw > 0) k_diag_walls<<<nblocks, kDiagBlock, 0, st>>>(s, nw, part_walls);
  cudaMemsetAsync(contacts, 0, sizeof(unsigned long long), st);
  const int gc = (int)std::max<long>(1, std::min<long>(((long)s.pcap + 255) / 256, lc.max_grid));
  k_diag_contacts<<<gc, 256, 0, st>>>(s, contacts);
  return nw > 0 ? 3 : 2;
}

// ----------------------------------------------------------------------------
// launchers
// ----------------------------------------------------------------------------

static inline int grid_for(long n, int block, int cap) {
  long g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

int scan_exclusive(const Sys &s, const int *in, int *out, int len, int *tmp, int gate,
                   cudaStream_t st) {
  const int nb = (len + 4095) / 4096;
  k_scan_blocks<<<nb, 1024, 0, st>>>(s, in, out, len, tmp, gate);
  if (nb > 1) {
    // nb <= 4096: one block scans the block totals in place
    k_scan_blocks<<<1, 1024, 0, st>>>(s, tmp, tmp, nb, nullptr, gate);
    k_scan_add<<<nb, 256, 0, st>>>(s, out, len, tmp, gate);
    return 3;
  }
  return 1;
}

// one block: one thread per ensemble system (up to 256 at a time)
static inline int sys_threads(const Sys &s) { return s.nsys > 32 ? 256 : 32; }

// Ensemble rebuild: in place for the rebuilding systems where that is
// possible (see k_ens_plan), else the whole list; the kernels of both paths
// are launched and each runs the path that Ctrl selects.  Stage 1 resumes
// after a pair-capacity overflow (whole-list path only).
static int launch_rebuild_ens(const Sys &s, const LaunchCfg &lc, cudaStream_t st, int stage) {
  int nl = 0;
  const int B = 256;
  const int gN = grid_for(s.nmax + 1, B, lc.max_grid);
  const int gC = grid_for(s.ncell + 2, B, lc.max_grid);
  const int gP = grid_for(s.pcap, B, lc.max_grid);
  const int gS = std::max(1, std::min(s.nsys, 2 * lc.sms));  // a block per system
  const int T = sys_threads(s);
  if (stage <= 0) {
    k_ens_plan<<<1, T, 0, st>>>(s);
    k_ens_lost<<<gN, B, 0, st>>>(s);
    k_ens_zero_cells<<<gC, B, 0, st>>>(s);
    k_cell_count<<<gN, B, 0, st>>>(s);
    nl += 4 + scan_exclusive(s, s.cell_count, s.cell_start, s.ncell + 2, s.scan_tmp, 2, st);
    k_ens_scan<<<gS, 1024, 0, st>>>(s, kEnsScanCells);
    k_cell_scatter<<<gN, B, 0, st>>>(s);
    k_cell_sort<<<gC, B, 0, st>>>(s);
    k_permute<<<gN, B, 0, st>>>(s);
    k_copy_atoms<<<gN, B, 0, st>>>(s);
    k_pairs<false><<<gN, B, 0, st>>>(s);
    k_ens_scan<<<gS, 1024, 0, st>>>(s, kEnsScanRowsPartial);
    k_ens_kept<<<gN, B, 0, st>>>(s);
    k_ens_scan<<<gS, 1024, 0, st>>>(s, kEnsScanRowsFull);
    k_ens_layout<<<1, T, 0, st>>>(s);
    k_ens_rows_base<<<gN, B, 0, st>>>(s);
    k_pairs_total<<<1, 1, 0, st>>>(s);
    nl += 13;
  }
  if (stage <= 1) {
    k_ens_zero_rev<<<gN, B, 0, st>>>(s);
    k_ens_holes<<<gS, B, 0, st>>>(s);
    k_pairs<true><<<gN, B, 0, st>>>(s);
    k_pair_init<<<gP, B, 0, st>>>(s);
    k_ens_scan<<<gS, 1024, 0, st>>>(s, kEnsScanRev);
    k_rev_fill<<<gP, B, 0, st>>>(s);
    k_rev_sort<<<gN, B, 0, st>>>(s);
    k_copy_pairs<<<grid_for((long)s.pcap > s.nmax + 1 ? s.pcap : s.nmax + 1, B, lc.max_grid), B, 0, st>>>(s);
    nl += 8;
  }
  if (s.nplanes > 0) {
    k_wall_list<<<gN, B, 0, st>>>(s);
    nl++;
  }
  k_finish_rebuild<<<1, T, 0, st>>>(s);
  return nl + 1;
}

int launch_rebuild(const Sys &s, const LaunchCfg &lc, cudaStream_t st, int stage) {
  if (s.nsys) return launch_rebuild_ens(s, lc, st, stage);
  int nl = 0;
  const int B = 256;
  const int gN = grid_for(s.nmax + 1, B, lc.max_grid);
  const int gC = grid_for(s.ncell + 2, B, lc.max_grid);
  const int gP = grid_for(s.pcap, B, lc.max_grid);
  // stage 0: the whole rebuild; stage 1: from the pair fill (after the host
  // grew the pair list); stage 2: from the mesh stages (after it grew mesh
  // slots or registrations).  Every resumed stage is idempotent.
  if (stage <= 0) {
    k_zero_gated<<<gC, B, 0, st>>>(s, s.cell_count, s.ncell + 2);
    k_zero_gated<<<gC, B, 0, st>>>(s, s.cell_fill, s.ncell + 2);
    k_cell_count<<<gN, B, 0, st>>>(s);
    nl += 3 + scan_exclusive(s, s.cell_count, s.cell_start, s.ncell + 2, s.scan_tmp, true, st);
    k_cell_scatter<<<gN, B, 0, st>>>(s);
    k_cell_sort<<<gC, B, 0, st>>>(s);
    k_permute<<<gN, B, 0, st>>>(s);
    k_copy_atoms<<<gN, B, 0, st>>>(s);
    k_pairs<false><<<gN, B, 0, st>>>(s);
    nl += 5 + scan_exclusive(s, s.pcount, s.pairs[1].row, s.nmax + 1, s.scan_tmp, true, st);
    k_pairs_total<<<1, 1, 0, st>>>(s);
    nl += 1;
  }
  if (stage <= 1) {
    k_zero_gated<<<gN, B, 0, st>>>(s, s.rev_count, s.nmax + 1);
    k_zero_gated<<<gN, B, 0, st>>>(s, s.rev_fill, s.nmax + 1);
    k_pairs<true><<<gN, B, 0, st>>>(s);
    k_pair_init<<<gP, B, 0, st>>>(s);
    nl += 4 + scan_exclusive(s, s.rev_count, s.pairs[1].rev_start, s.nmax + 1, s.scan_tmp, true, st);
    k_rev_fill<<<gP, B, 0, st>>>(s);
    k_rev_sort<<<gN, B, 0, st>>>(s);
    k_copy_pairs<<<grid_for((long)s.pcap > s.nmax + 1 ? s.pcap : s.nmax + 1, B, lc.max_grid), B, 0, st>>>(s);
  }
  for (int k = 0; k < s.nmeshes; k++) {
    const MeshDev &M = s.meshes[k];
    const int gT = grid_for(M.ntri, B, lc.max_grid);
    k_mesh_sort<<<gN, B, 0, st>>>(s, k);
    k_zero_gated<<<gC, B, 0, st>>>(s, M.tc_count, s.ncell + 2);
    k_zero_gated<<<gC, B, 0, st>>>(s, M.tc_fill, s.ncell + 2);
    k_tri_count<<<gT, B, 0, st>>>(s, k);
    nl += 6 + scan_exclusive(s, M.tc_count, M.tc_start, s.ncell + 2, s.scan_tmp, true, st);
    k_tri_fill<<<gT, B, 0, st>>>(s, k);
    k_mesh_cand<<<gN, B, 0, st>>>(s, k);
  }
  if (s.nmeshes > 0 || s.nplanes > 0) {
    k_wall_list<<<gN, B, 0, st>>>(s);
    nl++;
  }
  k_finish_rebuild<<<1, sys_threads(s), 0, st>>>(s);
  return nl + 4;
}

// Builds the executable graph of `steps 2..n` of dem_step:
//   WHILE(loop) { k_particle(gather+final+initial) -> k_decide_loop ->
//                 IF(rebuild) { rebuild kernels } -> k_pair }
// (without moving meshes, the last block of k_particle decides instead of
// k_decide_loop)
// The host sets ctrl->loop_left with launch_set_loop() before each launch.
static int launch_particle_lp(const Sys &s, const LaunchCfg &lc, int mode, int shearupdate, const LoopCond &lp,
                              cudaStream_t st);

cudaError_t build_step_graph(const Sys &s, const LaunchCfg &lc, cudaStream_t st, cudaStream_t st2,
                             cudaGraphExec_t *exec, int *kernels_per_step, int *kernels_per_rebuild) {
  cudaGraph_t g = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  // every failure leaves through here: end a capture still open on either
  // stream (its graph belongs to g), destroy the events and the graph
  auto fail = [&](cudaError_t err) -> cudaError_t {
    const cudaStream_t qs[2] = {st, st2};
    for (cudaStream_t q : qs) {
      cudaStreamCaptureStatus cs0 = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(q, &cs0) == cudaSuccess && cs0 != cudaStreamCaptureStatusNone) {
        cudaGraph_t part = nullptr;
        cudaStreamEndCapture(q, &part);
      }
    }
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (g) cudaGraphDestroy(g);
    return err;
  };
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return fail(e);
  cudaGraphConditionalHandle hloop, hreb;
  if ((e = cudaGraphConditionalHandleCreate(&hloop, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return fail(e);
  if ((e = cudaGraphConditionalHandleCreate(&hreb, g, 0, cudaGraphCondAssignDefault)) != cudaSuccess) return fail(e);
  cudaGraphNodeParams wp = {};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = hloop;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  cudaGraphNode_t wnode;
  if ((e = cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp)) != cudaSuccess) return fail(e);
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  if ((e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return fail(e);
  bool moving = false;
  for (int m = 0; m < s.nmeshes; m++) moving |= s.meshes[m].moving != 0;
  int k = 0;
  if (moving) {  // the mesh moves between the particle kernel and the decision
    k += launch_particle(s, lc, kModeGatherFinalInitial, 1, st);
    k += launch_mesh_move(s, lc, st);
    k_decide_loop<<<1, sys_threads(s), 0, st>>>(s, hreb, hloop);
    k++;
  } else {
    k += launch_particle_lp(s, lc, kModeGatherFinalInitial, 1, LoopCond{1, hreb, hloop}, st);
  }
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  cudaGraph_t cg;
  if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &nd)) != cudaSuccess) return fail(e);
  cudaGraphNodeParams ip = {};
  ip.type = cudaGraphNodeTypeConditional;
  ip.conditional.handle = hreb;
  ip.conditional.type = cudaGraphCondTypeIf;
  ip.conditional.size = 1;
  cudaGraphNode_t inode;
  if ((e = cudaGraphAddNode(&inode, cg, deps, nullptr, nd, &ip)) != cudaSuccess) return fail(e);
  cudaGraph_t rbody = ip.conditional.phGraph_out[0];
  if ((e = cudaStreamUpdateCaptureDependencies(st, &inode, nullptr, 1, cudaStreamSetCaptureDependencies)) != cudaSuccess)
    return fail(e);
  // the pair kernel and the wall kernel of the step run side by side
  const bool walls = s.nmeshes > 0 || s.nplanes > 0;
  if (walls) {
    if ((e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
    if ((e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
    if ((e = cudaEventRecord(fork, st)) != cudaSuccess) return fail(e);
    if ((e = cudaStreamWaitEvent(st2, fork, 0)) != cudaSuccess) return fail(e);
    k += launch_wall_force(s, lc, 1, st2);
    if ((e = cudaEventRecord(join, st2)) != cudaSuccess) return fail(e);
  }
  k += launch_pair(s, lc, 1, st);
  if (walls && (e = cudaStreamWaitEvent(st, join, 0)) != cudaSuccess) return fail(e);
  cudaGraph_t out = nullptr;
  if ((e = cudaStreamEndCapture(st, &out)) != cudaSuccess) return fail(e);
  if (fork) cudaEventDestroy(fork);
  if (join) cudaEventDestroy(join);
  fork = join = nullptr;
  if ((e = cudaStreamBeginCaptureToGraph(st2, rbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return fail(e);
  const int kr = launch_rebuild(s, lc, st2, 0);
  if ((e = cudaStreamEndCapture(st2, &out)) != cudaSuccess) return fail(e);
  e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  g = nullptr;
  *kernels_per_step = k;
  *kernels_per_rebuild = kr;
  return e;
}

// The wall kernel walks a short list (atoms near walls) with long per-atom
// dependency chains; it is launched with the device's highest priority so
// that its blocks start before those of the pair kernel beside it.
int launch_wall_force(const Sys &s, const LaunchCfg &lc, int shearupdate, cudaStream_t st) {
  if (s.nmeshes == 0 && s.nplanes == 0) return 0;
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  // queue entries per tile: LIGGGHTS_GB300_WALL_CAP per atom (1..16)
  static int cap_per_atom = 0;
  if (!cap_per_atom) {
    const char *e = getenv("LIGGGHTS_GB300_WALL_CAP");
    cap_per_atom = e ? std::max(1, std::min(16, atoi(e))) : kWallCapDefault;
    const int bytes = cap_per_atom * kWallTile * kWallQ;
    cudaFuncSetAttribute(k_wall_force<kHertz>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_wall_force<kHooke>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  }
  const int cap = cap_per_atom * kWallTile;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid_for(s.nmax, kWallTile, 2 * lc.max_grid));
  cfg.blockDim = dim3(kWallTile);
  cfg.dynamicSmemBytes = (size_t)cap * kWallQ;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = hi;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (s.normal == kHertz) cudaLaunchKernelEx(&cfg, k_wall_force<kHertz>, s, shearupdate, cap);
  else cudaLaunchKernelEx(&cfg, k_wall_force<kHooke>, s, shearupdate, cap);
  return 1;
}

int launch_mesh_move(const Sys &s, const LaunchCfg &lc, cudaStream_t st) {
  int nl = 0;
  for (int k = 0; k < s.nmeshes; k++) {
    if (!s.meshes[k].moving) continue;
    if (s.meshes[k].rotating)
      k_mesh_rotate<<<grid_for(s.meshes[k].ntri, 256, lc.max_grid), 256, 0, st>>>(s, k);
    else
      k_mesh_move<<<grid_for(s.meshes[k].ntri, 256, lc.max_grid), 256, 0, st>>>(s, k);
    nl++;
  }
  return nl;
}

int launch_set_loop(const Sys &s, int n, cudaStream_t st) {
  k_set_loop<<<1, 1, 0, st>>>(s, n);
  return 1;
}

int launch_decide(const Sys &s, cudaStream_t st) {
  k_decide<<<1, sys_threads(s), 0, st>>>(s);
  return 1;
}
int launch_set_rebuild(const Sys &s, int v, cudaStream_t st) {
  k_set_rebuild<<<1, sys_threads(s), 0, st>>>(s, v);
  return 1;
}

int launch_pair(const Sys &s, const LaunchCfg &lc, int shearupdate, cudaStream_t st) {
  const int B = 256;
  const int g = grid_for(s.pcap, B, lc.max_grid);
  const int Bb = kBandTile;
  const int gb = grid_for(s.pcap, Bb, 2 * lc.max_grid);
  if (s.bond) {
    if (s.normal == kHertz) {
      if (s.rolling) k_pair<kHertz, true, true><<<gb, Bb, 0, st>>>(s, shearupdate);
      else k_pair<kHertz, false, true><<<gb, Bb, 0, st>>>(s, shearupdate);
    } else {
      if (s.rolling) k_pair<kHooke, true, true><<<gb, Bb, 0, st>>>(s, shearupdate);
      else k_pair<kHooke, false, true><<<gb, Bb, 0, st>>>(s, shearupdate);
    }
    return 1;
  }
  if (s.cdf == 1.0) {
    // blocks per SM the kernel is compiled for (registers: 80 at 3, 64 at
    // 4 with some spilling): 3 with mesh walls, whose wall kernel runs
    // beside this one (the 1M hopper's graph step 2 % faster than at 4),
    // else 4 (the 256-system ensemble 12 % faster than at 3; the dense bed
    // 1.6 % slower); LIGGGHTS_GB300_PAIR_MINB 3 or 4 sets it.  The grid:
    // LIGGGHTS_GB300_PAIR_GRID (0: up to 8 blocks per SM, the default, which
    // leaves room for the wall kernel beside it; 1: one resident wave, the
    // tiles taken grid-stride: the pair kernel alone runs faster, the step
    // slower).  Results do not depend on either.
    static int env_minb = -1, wave = 0;
    if (env_minb < 0) {
      const char *e = getenv("LIGGGHTS_GB300_PAIR_MINB");
      env_minb = (e && (atoi(e) == 3 || atoi(e) == 4)) ? atoi(e) : 0;
      const char *w = getenv("LIGGGHTS_GB300_PAIR_GRID");
      wave = (w && atoi(w) == 1) ? 1 : 0;
    }
    const int minb = env_minb ? env_minb : (s.nmeshes > 0 ? 3 : 4);
    const int gp = wave ? std::min(g, lc.sms * minb) : g;
    if (minb == 4) {
      if (s.normal == kHertz) {
        if (s.rolling) k_pair_pf<kHertz, true, 4><<<gp, B, 0, st>>>(s, shearupdate);
        else k_pair_pf<kHertz, false, 4><<<gp, B, 0, st>>>(s, shearupdate);
      } else {
        if (s.rolling) k_pair_pf<kHooke, true, 4><<<gp, B, 0, st>>>(s, shearupdate);
        else k_pair_pf<kHooke, false, 4><<<gp, B, 0, st>>>(s, shearupdate);
      }
    } else {
      if (s.normal == kHertz) {
        if (s.rolling) k_pair_pf<kHertz, true, 3><<<gp, B, 0, st>>>(s, shearupdate);
        else k_pair_pf<kHertz, false, 3><<<gp, B, 0, st>>>(s, shearupdate);
      } else {
        if (s.rolling) k_pair_pf<kHooke, true, 3><<<gp, B, 0, st>>>(s, shearupdate);
        else k_pair_pf<kHooke, false, 3><<<gp, B, 0, st>>>(s, shearupdate);
      }
    }
    return 1;
  }
  if (s.normal == kHertz) {
    if (s.rolling) k_pair<kHertz, true, false><<<gb, Bb, 0, st>>>(s, shearupdate);
    else k_pair<kHertz, false, false><<<gb, Bb, 0, st>>>(s, shearupdate);
  } else {
    if (s.rolling) k_pair<kHooke, true, false><<<gb, Bb, 0, st>>>(s, shearupdate);
    else k_pair<kHooke, false, false><<<gb, Bb, 0, st>>>(s, shearupdate);
  }
  return 1;
}

template <int NORMAL>
static void launch_particle_n(const Sys &s, int g, int B, int mode, int shearupdate, const LoopCond &lp,
                              cudaStream_t st) {
  switch (mode) {
    case kModeInitial: k_particle<NORMAL, false, false, true><<<g, B, 0, st>>>(s, shearupdate, lp); break;
    case kModeGather: k_particle<NORMAL, true, false, false><<<g, B, 0, st>>>(s, shearupdate, lp); break;
    case kModeGatherFinal: k_particle<NORMAL, true, true, false><<<g, B, 0, st>>>(s, shearupdate, lp); break;
    case kModeGatherFinalInitial:
      k_particle<NORMAL, true, true, true><<<g, B, 0, st>>>(s, shearupdate, lp);
      break;
  }
}

static int launch_particle_lp(const Sys &s, const LaunchCfg &lc, int mode, int shearupdate, const LoopCond &lp,
                              cudaStream_t st) {
  // one particle per thread; smaller blocks give the same number of threads
  // in more, smaller blocks (each particle's sums do not depend on it)
  const int B = lc.particle_threads;
  const int g = grid_for(s.nmax, B, lc.max_grid * (256 / B));
  if (s.normal == kHertz) launch_particle_n<kHertz>(s, g, B, mode, shearupdate, lp, st);
  else launch_particle_n<kHooke>(s, g, B, mode, shearupdate, lp, st);
  return 1;
}

int launch_particle(const Sys &s, const LaunchCfg &lc, int mode, int shearupdate, cudaStream_t st) {
  return launch_particle_lp(s, lc, mode, shearupdate, LoopCond{0, 0, 0}, st);
}

}  // namespace gb300
