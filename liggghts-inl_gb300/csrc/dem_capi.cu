// Host runtime of one resident granular system and the C ABI of
// include/liggghts_gb300.h.  The host owns device buffers and one stream per
// handle, queues whole timesteps without synchronising (rebuild decisions are
// taken on the device), and checks the device control block every
// kCheckEvery steps and at the end of each call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/liggghts_gb300.h"
#include "contact_law.cuh"
#include "dem_device.cuh"
#include "dem_kernels.h"
#include "dem_mesh_host.h"

using namespace gb300;

namespace {
constexpr int kCheckEvery = 256;
// the two-level exclusive scan covers 4096 * 4096 items
constexpr long kMaxScan = 4096L * 4096L - 2;
static_assert(kMaxScan < (1L << 24), "the neighbour stash packs atom indices in 24 bits");
constexpr long kMaxCells = 16000000L;
}  // namespace

struct dem_handle {
  dem_config cfg{};
  Sys s{};
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int device = 0;
  std::string err;
  bool have_params = false, have_atoms = false, setup_done = false;
  std::vector<void *> allocs_atoms, allocs_pairs, allocs_misc, allocs_cells;
  std::vector<void *> allocs_mslots[kMaxMeshes], allocs_tclist[kMaxMeshes];  // grown on overflow
  // atom transfers: kernels read and write the caller's arrays directly
  // when the device reaches pageable host memory through the host's page
  // tables (cudaDevAttrPageableMemoryAccessUsesHostPageTables, Grace
  // C2C systems); else through this device staging buffer
  bool host_direct = false;
  void *stage = nullptr;
  size_t stage_bytes = 0;
  UploadCheck *chk = nullptr;       // device: k_upload_atoms results
  UploadCheck *chk_host = nullptr;  // pinned host copy
  double *diag_buf = nullptr;  // dem_get_diagnostics partial sums
  LaunchCfg lc{152 * 8};
  float last_ms = 0.f;
  Ctrl host_ctrl{};
  // per-kernel timing (dem_profile)
  bool profile = false;
  std::vector<cudaEvent_t> evpool;
  int evused = 0;
  std::vector<int> evkind;  // 0 particle, 1 neigh, 2 pair, 3 wall: kind of interval ending at event k
  dem_kernel_times kt{};
  // graph-resident step loop
  bool use_graph = true;
  cudaStream_t st2 = nullptr;
  cudaGraphExec_t gexec = nullptr;
  long long graph_gen = -1, sys_gen = 0;  // rebuilt when device pointers change
  int graph_kps = 0, graph_kpr = 0;
  std::vector<MeshHost> mesh_host;
  std::vector<double> bond_tables;  // host copy for the cutoff derivation
  double cell_scale = 1.0;          // neighbour cell edge / cutneighmax (dem_set_tuning)
  int ens_nsys = 0;                 // batched ensemble: number of systems (dem_set_ensemble)
  // insertion (dem_set_capacity / dem_insert_atoms)
  int cap_n = 0;                    // atom capacity (0: the uploaded count)
  double cap_rmin = 0.0, cap_rmax = 0.0;  // radius range inserted atoms may take
  double eff_rmin = 0.0, eff_rmax = 0.0;  // radii the neighbour cutoff was sized for
  int pending_insert = 0;           // staged atoms that join at the next step
  int next_lidx = 0;                // caller-order index of the next inserted atom
  dem_bond_settings bond_settings{};
};

static int ensure_graph(dem_handle *h) {
  if (h->gexec && h->graph_gen == h->sys_gen) return DEM_OK;
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  cudaError_t e = build_step_graph(h->s, h->lc, h->st, h->st2, &h->gexec, &h->graph_kps, &h->graph_kpr);
  if (e != cudaSuccess) {
    h->err = std::string("build_step_graph: ") + cudaGetErrorString(e);
    return DEM_ERR_CUDA;
  }
  h->graph_gen = h->sys_gen;
  return DEM_OK;
}

// Records an event closing an interval of the given kind (profiling only).
static void mark(dem_handle *h, int kind) {
  if (!h->profile) return;
  if (h->evused >= (int)h->evpool.size()) return;
  cudaEventRecord(h->evpool[h->evused], h->st);
  h->evkind[h->evused] = kind;
  h->evused++;
}

static void mark_start(dem_handle *h) { mark(h, -1); }

// Folds the recorded intervals into the totals (the stream must be idle).
static void harvest(dem_handle *h) {
  if (!h->profile || h->evused == 0) return;
  for (int k = 1; k < h->evused; k++) {
    if (h->evkind[k] < 0) continue;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->evpool[k - 1], h->evpool[k]);
    if (h->evkind[k] == 0) { h->kt.particle_ms += ms; h->kt.particle_launches++; }
    if (h->evkind[k] == 1) { h->kt.neigh_ms += ms; h->kt.neigh_stages++; }
    if (h->evkind[k] == 2) { h->kt.pair_ms += ms; h->kt.pair_launches++; }
    if (h->evkind[k] == 3) { h->kt.wall_ms += ms; h->kt.wall_launches++; }
  }
  h->evused = 0;
}

#define CUDA_TRY(h, call)                                                                  \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      (h)->err = std::string(#call) + ": " + cudaGetErrorString(e_);                       \
      return DEM_ERR_CUDA;                                                                 \
    }                                                                                      \
  } while (0)

static int fail(dem_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

template <typename T>
static cudaError_t dalloc(std::vector<void *> &list, T **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
  if (e == cudaSuccess) {
    list.push_back(q);
    *p = static_cast<T *>(q);
  }
  return e;
}

// One device allocation carved into 256-byte aligned arrays: a carving
// function runs once to size the block (base unset), then again to hand out
// the pointers.  Replaces one cudaMalloc per array.
struct Arena {
  char *base = nullptr;
  size_t off = 0;
  template <typename T>
  void take(T **p, size_t n) {
    off = (off + 255) & ~(size_t)255;
    if (base) *p = reinterpret_cast<T *>(base + off);
    off += std::max<size_t>(n, 1) * sizeof(T);
  }
  cudaError_t commit(std::vector<void *> &list) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(off, 256));
    if (e == cudaSuccess) {
      list.push_back(q);
      base = static_cast<char *>(q);
    }
    off = 0;
    return e;
  }
};

static void free_list(std::vector<void *> &l) {
  for (void *p : l) cudaFree(p);
  l.clear();
}

// Per-atom candidate lists and history slots of mesh k (the pages of
// FixContactHistoryMesh) at `cap` per atom.  With keep, the live slots
// (buffer 0) move to the new arrays and the added rows start empty; the
// candidate lists are rebuilt by the resumed k_mesh_cand.
static int alloc_mesh_slots(dem_handle *h, int k, int cap, bool keep) {
  Sys &s = h->s;
  MeshDev &M = s.meshes[k];
  const size_t nmax = s.nmax;
  MeshDev N = M;
  std::vector<void *> nl;
  auto carve = [&](Arena &ar) {
    ar.take(&N.cand_n, nmax);
    ar.take(&N.cand, (size_t)cap * nmax);
    for (int b = 0; b < 2; b++) {
      ar.take(&N.nslot[b], nmax);
      ar.take(&N.npart[b], nmax);
      ar.take(&N.slot_tri[b], (size_t)cap * nmax);
      ar.take(&N.slot_hist[b], (size_t)3 * cap * nmax);
    }
  };
  Arena ar;
  carve(ar);
  CUDA_TRY(h, ar.commit(nl));
  carve(ar);
  const size_t old = keep ? (size_t)std::min(M.ccap, cap) : 0;
  if (keep) {
    CUDA_TRY(h, cudaMemcpyAsync(N.cand_n, M.cand_n, nmax * sizeof(int), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.nslot[0], M.nslot[0], nmax * sizeof(int), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.npart[0], M.npart[0], nmax * sizeof(int), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.slot_tri[0], M.slot_tri[0], old * nmax * sizeof(int), cudaMemcpyDeviceToDevice,
                                h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.slot_hist[0], M.slot_hist[0], 3 * old * nmax * sizeof(double),
                                cudaMemcpyDeviceToDevice, h->st));
  } else {
    CUDA_TRY(h, cudaMemsetAsync(N.cand_n, 0, nmax * sizeof(int), h->st));
    CUDA_TRY(h, cudaMemsetAsync(N.nslot[0], 0, nmax * sizeof(int), h->st));
    CUDA_TRY(h, cudaMemsetAsync(N.npart[0], 0, nmax * sizeof(int), h->st));
  }
  CUDA_TRY(h, cudaMemsetAsync(N.slot_tri[0] + old * nmax, 0xff, ((size_t)cap - old) * nmax * sizeof(int), h->st));
  CUDA_TRY(h, cudaMemsetAsync(N.slot_hist[0] + 3 * old * nmax, 0, 3 * ((size_t)cap - old) * nmax * sizeof(double),
                              h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));  // the old arrays are read until here
  free_list(h->allocs_mslots[k]);
  h->allocs_mslots[k] = nl;
  M.cand_n = N.cand_n;
  M.cand = N.cand;
  for (int b = 0; b < 2; b++) {
    M.nslot[b] = N.nslot[b];
    M.npart[b] = N.npart[b];
    M.slot_tri[b] = N.slot_tri[b];
    M.slot_hist[b] = N.slot_hist[b];
  }
  M.ccap = cap;
  h->sys_gen++;
  return DEM_OK;
}

// Triangle-to-cell registrations of mesh k (FixNeighlistMesh's per-bin
// triangle lists) at M.tc_cap entries.
static int alloc_tc_list(dem_handle *h, int k) {
  MeshDev &M = h->s.meshes[k];
  std::vector<void *> nl;
  int *p = nullptr;
  CUDA_TRY(h, dalloc(nl, &p, (size_t)M.tc_cap));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  free_list(h->allocs_tclist[k]);
  h->allocs_tclist[k] = nl;
  M.tc_list = p;
  h->sys_gen++;
  return DEM_OK;
}

static int alloc_atoms(dem_handle *h, int nmax) {
  Sys &s = h->s;
  free_list(h->allocs_atoms);
  h->sys_gen++;
  s.nmax = nmax;
  auto carve = [&](Arena &ar) {
    for (int b = 0; b < 2; b++) {
      AtomArrays &A = s.atoms[b];
      double **d[] = {&A.x, &A.y, &A.z, &A.vx, &A.vy, &A.vz, &A.wx, &A.wy, &A.wz, &A.fx, &A.fy,
                      &A.fz, &A.tx, &A.ty, &A.tz, &A.r, &A.m, &A.dtfm, &A.dtir, &A.xh, &A.yh, &A.zh};
      for (double **pp : d) ar.take(pp, nmax);
      ar.take(&A.type, nmax);
      ar.take(&A.tag, nmax);
      ar.take(&A.lidx, nmax);
      ar.take(&A.whist, (size_t)3 * std::max(1, s.nplanes) * nmax);  // walls are added before atoms
      ar.take(&A.wbits, nmax);
      double **fm[] = {&A.fmx, &A.fmy, &A.fmz, &A.tmx, &A.tmy, &A.tmz};
      for (double **pp : fm) ar.take(pp, nmax);
    }
    for (int b = 0; b < 2; b++) {
      ar.take(&s.pairs[b].row, nmax + 1);
      ar.take(&s.pairs[b].rev_start, nmax + 1);
      if (s.nsys) {  // ensembles: row ends (segmented list)
        ar.take(&s.pairs[b].rowe, nmax + 1);
        ar.take(&s.pairs[b].reve, nmax + 1);
      } else {
        s.pairs[b].rowe = s.pairs[b].reve = nullptr;
      }
    }
    ar.take(&s.perm, nmax);
    ar.take(&s.xf, nmax);
    ar.take(&s.xhf, nmax);
    ar.take(&s.mlist, nmax);
    ar.take(&s.stash, (size_t)kStash * nmax);
    ar.take(&s.wforce, (size_t)3 * std::max(1, s.nplanes + s.nmeshes) * nmax);
    ar.take(&s.order, nmax);
    ar.take(&s.pcount, nmax + 1);
    ar.take(&s.rev_count, nmax + 1);
    ar.take(&s.rev_fill, nmax + 1);
  };
  Arena ar;
  carve(ar);
  CUDA_TRY(h, ar.commit(h->allocs_atoms));
  carve(ar);
  for (int b = 0; b < 2; b++) {
    PairArrays &P = s.pairs[b];
    CUDA_TRY(h, cudaMemsetAsync(P.row, 0, (nmax + 1) * sizeof(int), h->st));
    CUDA_TRY(h, cudaMemsetAsync(P.rev_start, 0, (nmax + 1) * sizeof(int), h->st));
    if (P.rowe) {
      CUDA_TRY(h, cudaMemsetAsync(P.rowe, 0, (nmax + 1) * sizeof(int), h->st));
      CUDA_TRY(h, cudaMemsetAsync(P.reve, 0, (nmax + 1) * sizeof(int), h->st));
    }
  }
  CUDA_TRY(h, cudaMemsetAsync(s.wforce, 0, (size_t)3 * std::max(1, s.nplanes + s.nmeshes) * nmax * sizeof(double), h->st));
  for (int k = 0; k < s.nmeshes; k++) {
    int rc = alloc_mesh_slots(h, k, s.meshes[k].ccap, false);
    if (rc) return rc;
  }
  return DEM_OK;
}

// The arrays sized by the neighbour cells and the mesh cell registrations
// (known once the radius range is): cell counts and starts, the scan's
// block sums, the triangle-to-cell lists.
static int alloc_cells(dem_handle *h) {
  Sys &s = h->s;
  free_list(h->allocs_cells);
  auto carve = [&](Arena &ar) {
    ar.take(&s.cell_count, (size_t)s.ncell + 2);
    ar.take(&s.cell_start, (size_t)s.ncell + 2);
    ar.take(&s.cell_fill, (size_t)s.ncell + 2);
    long maxlen = std::max<long>(s.nmax + 1, s.ncell + 2);
    ar.take(&s.scan_tmp, (maxlen + 4095) / 4096 + 1);
    for (int k = 0; k < s.nmeshes; k++) {
      MeshDev &M = s.meshes[k];
      ar.take(&M.tc_count, (size_t)s.ncell + 2);
      ar.take(&M.tc_start, (size_t)s.ncell + 2);
      ar.take(&M.tc_fill, (size_t)s.ncell + 2);
    }
  };
  Arena ar;
  carve(ar);
  CUDA_TRY(h, ar.commit(h->allocs_cells));
  carve(ar);
  for (int k = 0; k < s.nmeshes; k++) {
    int rc = alloc_tc_list(h, k);
    if (rc) return rc;
  }
  h->sys_gen++;
  return DEM_OK;
}

// Device staging for atom transfers where the device cannot reach the
// caller's pageable memory (grown on demand, kept by the handle).
static int ensure_stage(dem_handle *h, size_t bytes) {
  if (h->stage_bytes >= bytes) return DEM_OK;
  if (h->stage) cudaFree(h->stage);
  h->stage = nullptr;
  h->stage_bytes = 0;
  CUDA_TRY(h, cudaMalloc(&h->stage, bytes));
  h->stage_bytes = bytes;
  return DEM_OK;
}

// (Re)allocates every pcap-sized array; keeps the current list (pairs[0]).
static int alloc_pairs(dem_handle *h, int pcap, int keep_np) {
  Sys &s = h->s;
  std::vector<void *> nl;
  PairArrays np_[2];
  double *rres = nullptr;
  uint8_t *act = nullptr;
  auto carve = [&](Arena &ar) {
    for (int b = 0; b < 2; b++) {
      PairArrays &P = np_[b];
      P = s.pairs[b];
      ar.take(&P.i, pcap);
      ar.take(&P.j, pcap);
      ar.take(&P.sh, pcap);
      ar.take(&P.flag, pcap);
      ar.take(&P.hist, (size_t)s.dnum * pcap);
      ar.take(&P.reff, pcap);
      ar.take(&P.c0, pcap);
      ar.take(&P.c1, pcap);
      ar.take(&P.rev, pcap);
    }
    ar.take(&rres, (size_t)kResStride * pcap);
    ar.take(&act, pcap);
  };
  Arena ar;
  carve(ar);
  CUDA_TRY(h, ar.commit(nl));
  carve(ar);
  if (keep_np > 0 && s.pcap > 0) {
    const PairArrays &O = s.pairs[0];
    PairArrays &N = np_[0];
    const size_t k = keep_np;
    CUDA_TRY(h, cudaMemcpyAsync(N.i, O.i, k * sizeof(int), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.j, O.j, k * sizeof(int), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.sh, O.sh, k, cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.flag, O.flag, k * sizeof(int), cudaMemcpyDeviceToDevice, h->st));
    for (int d = 0; d < s.dnum; d++)
      CUDA_TRY(h, cudaMemcpyAsync(N.hist + (size_t)d * pcap, O.hist + (size_t)d * s.pcap,
                             k * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.reff, O.reff, k * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.c0, O.c0, k * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.c1, O.c1, k * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(N.rev, O.rev, k * sizeof(int), cudaMemcpyDeviceToDevice, h->st));
  }
  free_list(h->allocs_pairs);
  h->allocs_pairs = nl;
  s.pairs[0] = np_[0];
  s.pairs[1] = np_[1];
  s.res = rres;
  s.active = act;
  s.pcap = pcap;
  h->sys_gen++;
  return DEM_OK;
}

static int read_ctrl(dem_handle *h) {
  CUDA_TRY(h, cudaMemcpyAsync(&h->host_ctrl, h->s.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  harvest(h);
  return DEM_OK;
}

// If the device halted on a pair-capacity overflow: grow, clear the halt and
// finish the interrupted rebuild.  Returns DEM_OK when nothing is pending.
static int recover(dem_handle *h, bool *resumed) {
  *resumed = false;
  int rc = read_ctrl(h);
  if (rc) return rc;
  Ctrl &c = h->host_ctrl;
  if (c.status == kStatNan) return fail(h, DEM_ERR_NAN, "non-finite particle position");
  if (c.status == kStatMeshSlots)
    return fail(h, DEM_ERR_CAPACITY, "a mesh contact found no free history slot (inconsistent slots)");
  if (!c.halt) return DEM_OK;
  if (c.status == kStatMeshCand || c.status == kStatMeshReg) {
    // FixContactHistoryMesh pages and FixNeighlistMesh bin lists grow without
    // a bound in the reference: grow the arrays that overflowed, then finish
    // the interrupted rebuild from its mesh stages
    Sys &s = h->s;
    if (c.status == kStatMeshCand) {
      const int need = c.mesh_need;
      for (int k = 0; k < s.nmeshes; k++)
        if (s.meshes[k].ccap < need) {
          rc = alloc_mesh_slots(h, k, std::max(need, 2 * s.meshes[k].ccap), true);
          if (rc) return fail(h, DEM_ERR_CAPACITY, "cannot grow the mesh history slots: " + h->err);
        }
      c.mesh_need = 0;
    } else {
      for (int k = 0; k < s.nmeshes; k++) {
        MeshDev &M = s.meshes[k];
        int tot = 0;
        CUDA_TRY(h, cudaMemcpyAsync(&tot, M.tc_start + s.ncell, sizeof(int), cudaMemcpyDeviceToHost, h->st));
        CUDA_TRY(h, cudaStreamSynchronize(h->st));
        if (tot > M.tc_cap) {
          M.tc_cap = (int)std::min<long>(2147000000L, (long)tot * 5 / 4 + 4096);
          rc = alloc_tc_list(h, k);
          if (rc) return fail(h, DEM_ERR_CAPACITY, "cannot grow the mesh cell registrations: " + h->err);
        }
      }
    }
    c.halt = 0;
    c.status = kStatOk;
    CUDA_TRY(h, cudaMemcpyAsync(h->s.ctrl, &c, sizeof(Ctrl), cudaMemcpyHostToDevice, h->st));
    h->kt.kernel_launches += launch_rebuild(h->s, h->lc, h->st, 2);
    *resumed = true;
    return DEM_OK;
  }
  if (c.status != kStatPairOverflow) return fail(h, DEM_ERR_CUDA, "device halted");
  const int want = (int)std::min<long>(2147000000L, std::max<long>((long)c.np_new * 5 / 4 + 1024, 2L * h->s.pcap));
  rc = alloc_pairs(h, want, c.np);
  if (rc) return fail(h, DEM_ERR_NEIGH_OVERFLOW, "cannot grow neighbour list: " + h->err);
  c.halt = 0;
  c.status = kStatOk;
  CUDA_TRY(h, cudaMemcpyAsync(h->s.ctrl, &c, sizeof(Ctrl), cudaMemcpyHostToDevice, h->st));
  h->kt.kernel_launches += launch_rebuild(h->s, h->lc, h->st, 1);
  *resumed = true;
  return DEM_OK;
}

extern "C" {

const char *dem_version(void) { return "liggghts-inl-gb300 0.1 (sm_103a)"; }

int dem_create(const dem_config *cfg, dem_handle **out) {
  if (!cfg || !out) return DEM_ERR_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DEM_ERR_NO_DEVICE;
  if (cfg->cohesion_model != DEM_COHESION_OFF && cfg->cohesion_model != DEM_COHESION_BOND_NONLINEAR)
    return DEM_ERR_UNSUPPORTED;
  if (cfg->normal_model != DEM_NORMAL_HERTZ && cfg->normal_model != DEM_NORMAL_HOOKE)
    return DEM_ERR_UNSUPPORTED;
  if (cfg->dt <= 0 || cfg->skin < 0 || cfg->neigh_every < 1 || cfg->contact_distance_factor < 1.0)
    return DEM_ERR_BAD_ARG;
  dem_handle *h = new dem_handle();
  h->cfg = *cfg;
  cudaGetDevice(&h->device);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, h->device) == cudaSuccess) {
    h->lc.max_grid = prop.multiProcessorCount * 8;
    h->lc.sms = prop.multiProcessorCount;
  }
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess) {
    delete h;
    return DEM_ERR_CUDA;
  }
  // LIGGGHTS_GB300_NO_GRAPH=1 queues every kernel from the host instead of
  // running the step loop as one graph (same results; for debugging)
  const char *ng = getenv("LIGGGHTS_GB300_NO_GRAPH");
  h->use_graph = !(ng && ng[0] == '1');
  Sys &s = h->s;
  if (cudaMalloc(&s.ctrl, sizeof(Ctrl)) != cudaSuccess) {
    delete h;
    return DEM_ERR_CUDA;
  }
  h->allocs_misc.push_back(s.ctrl);
  cudaMemset(s.ctrl, 0, sizeof(Ctrl));
  if (cudaMalloc(&h->chk, sizeof(UploadCheck)) != cudaSuccess ||
      cudaMallocHost(&h->chk_host, sizeof(UploadCheck)) != cudaSuccess) {
    delete h;
    return DEM_ERR_CUDA;
  }
  h->allocs_misc.push_back(h->chk);
  cudaDeviceSynchronize();
  {  // direct access to the caller's pageable arrays: hardware coherence
     // through the host page tables only (not software page migration);
     // LIGGGHTS_GB300_STAGED_COPIES=1 forces the staged copies
    int pma = 0, hpt = 0;
    cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, h->device);
    cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, h->device);
    const char *sc = getenv("LIGGGHTS_GB300_STAGED_COPIES");
    h->host_direct = pma == 1 && hpt == 1 && !(sc && sc[0] == '1');
  }
  for (int d = 0; d < 3; d++) {
    s.boxlo[d] = cfg->boxlo[d];
    s.boxhi[d] = cfg->boxhi[d];
    s.prd[d] = cfg->boxhi[d] - cfg->boxlo[d];
    s.periodic[d] = cfg->periodic[d] ? 1 : 0;
    s.g[d] = cfg->gravity[d];
  }
  s.dt = cfg->dt;
  s.skin = cfg->skin;
  s.cdf = cfg->contact_distance_factor;
  s.neigh_every = cfg->neigh_every;
  s.neigh_delay = cfg->neigh_delay;
  s.neigh_check = cfg->neigh_check;
  s.normal = cfg->normal_model;
  s.rolling = cfg->rolling_model;
  s.tdamp = cfg->tangential_damping;
  s.limitf = cfg->limit_force;
  s.gravity_on = cfg->gravity_on;
  s.bond = cfg->cohesion_model == DEM_COHESION_BOND_NONLINEAR ? 1 : 0;
  s.dnum = s.bond ? kDnumBond : kDnumShear;
  *out = h;
  return DEM_OK;
}

// Device history index of the reference's history value r (bond values
// first, then shear; device: shear first).
static inline int dev_hist_index(const Sys &s, int r) {
  if (!s.bond) return r;
  return r < kBondValues ? kDnumShear + r : r - kBondValues;
}

int dem_destroy(dem_handle *h) {
  if (!h) return DEM_ERR_BAD_ARG;
  if (h->st) cudaStreamSynchronize(h->st);
  free_list(h->allocs_pairs);
  free_list(h->allocs_atoms);
  free_list(h->allocs_misc);
  free_list(h->allocs_cells);
  for (int k = 0; k < kMaxMeshes; k++) {
    free_list(h->allocs_mslots[k]);
    free_list(h->allocs_tclist[k]);
  }
  if (h->stage) cudaFree(h->stage);
  if (h->chk_host) cudaFreeHost(h->chk_host);
  if (h->diag_buf) cudaFree(h->diag_buf);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  for (auto &e : h->evpool) cudaEventDestroy(e);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->st) cudaStreamDestroy(h->st);
  if (h->st2) cudaStreamDestroy(h->st2);
  delete h;
  return DEM_OK;
}

int dem_derive_hertz_tables(int nt, const double *Y, const double *v, const double *e,
                            double *Yeff, double *Geff, double *betaeff, double *restlog) {
  if (nt < 1 || !Y || !v || !e) return DEM_ERR_BAD_ARG;
  const int m = nt + 1;
  for (int k = 0; k < m * m; k++) {
    if (Yeff) Yeff[k] = 0.0;
    if (Geff) Geff[k] = 0.0;
    if (betaeff) betaeff[k] = 0.0;
    if (restlog) restlog[k] = 0.0;
  }
  for (int i = 1; i <= nt; i++)
    for (int j = 1; j <= nt; j++) {
      const double Yi = Y[i - 1], Yj = Y[j - 1], vi = v[i - 1], vj = v[j - 1];
      // src/global_properties.cpp:449, :480, :518, :556
      if (Yeff) Yeff[i * m + j] = 1. / ((1. - pow(vi, 2.)) / Yi + (1. - pow(vj, 2.)) / Yj);
      if (Geff) Geff[i * m + j] = 1. / (2. * (2. - vi) * (1. + vi) / Yi + 2. * (2. - vj) * (1. + vj) / Yj);
      const double lg = log(e[(i - 1) * nt + (j - 1)]);
      if (restlog) restlog[i * m + j] = lg;
      if (betaeff) betaeff[i * m + j] = lg / sqrt(pow(lg, 2.) + pow(M_PI, 2.));
    }
  return DEM_OK;
}

int dem_set_pair_params(dem_handle *h, int ntypes, const double *Yeff, const double *Geff,
                        const double *betaeff, const double *coeffFrict,
                        const double *coeffRollFrict, const double *coeffRestLog, double charVel) {
  if (!h || ntypes < 1 || !Yeff || !Geff || !coeffFrict) return DEM_ERR_BAD_ARG;
  if (h->cfg.normal_model == DEM_NORMAL_HERTZ && !betaeff) return fail(h, DEM_ERR_BAD_ARG, "betaeff required");
  if (h->cfg.normal_model == DEM_NORMAL_HOOKE && !coeffRestLog) return fail(h, DEM_ERR_BAD_ARG, "coeffRestLog required");
  const int m = (ntypes + 1) * (ntypes + 1);
  std::vector<double> tab(kTypeTables * (size_t)m, 0.0);
  const double *src[6] = {Yeff, Geff, betaeff, coeffFrict, coeffRollFrict, coeffRestLog};
  for (int k = 0; k < 6; k++)
    if (src[k]) std::memcpy(&tab[(size_t)k * m], src[k], m * sizeof(double));
  derive_type_tables(m, tab.data());
  if (h->s.params) {
    cudaFree(h->s.params);
    h->allocs_misc.erase(std::remove(h->allocs_misc.begin(), h->allocs_misc.end(), (void *)h->s.params),
                         h->allocs_misc.end());
  }
  CUDA_TRY(h, dalloc(h->allocs_misc, &h->s.params, tab.size()));
  CUDA_TRY(h, cudaMemcpyAsync(h->s.params, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  h->s.ntypes = ntypes;
  h->s.charVel = charVel;
  h->have_params = true;
  h->sys_gen++;
  return DEM_OK;
}

int dem_set_bond_params(dem_handle *h, const double *tables, const dem_bond_settings *st) {
  if (!h || !tables || !st) return DEM_ERR_BAD_ARG;
  if (!h->s.bond) return fail(h, DEM_ERR_BAD_ARG, "cohesion_model is not DEM_COHESION_BOND_NONLINEAR");
  if (!h->have_params) return fail(h, DEM_ERR_BAD_ARG, "set pair parameters first");
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "set bond parameters before uploading atoms");
  const size_t m = (size_t)(h->s.ntypes + 1) * (h->s.ntypes + 1);
  for (size_t q = 0; q < (size_t)kBondTables * m; q++)
    if (!std::isfinite(tables[q])) return fail(h, DEM_ERR_BAD_ARG, "non-finite bond parameter");
  // sanity range of the damping tables, createPerTypePairProperty(..., 0.0, 1.0)
  for (int t = kBondDampFn; t <= kBondDampTt; t++)
    for (size_t q = 0; q < m; q++)
      if (tables[t * m + q] < 0.0 || tables[t * m + q] > 1.0)
        return fail(h, DEM_ERR_BAD_ARG, "bond damping coefficients must lie in [0, 1]");
  if (h->s.bondp) {
    cudaFree(h->s.bondp);
    h->allocs_misc.erase(std::remove(h->allocs_misc.begin(), h->allocs_misc.end(), (void *)h->s.bondp),
                         h->allocs_misc.end());
  }
  CUDA_TRY(h, dalloc(h->allocs_misc, &h->s.bondp, (size_t)(kBondTables + kBondDerived) * m));
  {
    std::vector<double> all(tables, tables + (size_t)kBondTables * m);
    all.resize((size_t)(kBondTables + kBondDerived) * m);
    auto T = [&](int t, size_t q) { return tables[(size_t)t * m + q]; };
    for (size_t q = 0; q < m; q++) {
      all[(size_t)kBondRatioTn * m + q] = (T(kBondKutn, q) - T(kBondKtn, q)) / (T(kBondKutn, q) + T(kBondKctn, q));
      all[(size_t)kBondRatioTt * m + q] = (T(kBondKutt, q) - T(kBondKtt, q)) / (T(kBondKutt, q) + T(kBondKctt, q));
      all[(size_t)kBondRatioFn1 * m + q] =
          (T(kBondKufn1, q) - T(kBondKfn1, q)) / (T(kBondKufn1, q) + T(kBondKcfn1, q));
      all[(size_t)kBondRatioFn2 * m + q] =
          (T(kBondKufn2, q) - T(kBondKfn2, q)) / (T(kBondKufn2, q) + T(kBondKcfn2, q));
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->s.bondp, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  }
  h->bond_tables.assign(tables, tables + (size_t)kBondTables * m);
  h->bond_settings = *st;
  int fl = 0;
  if (st->stressBreak) fl |= kBondStressBreak;
  if (st->tensionStress) fl |= kBondTension;
  if (st->compressionStress) fl |= kBondCompression;
  if (st->shearStress) fl |= kBondShear;
  if (st->normalTorqueStress) fl |= kBondNormalTorque;
  if (st->shearTorqueStress) fl |= kBondShearTorque;
  if (st->createBondAlways) fl |= kBondCreateAlways;
  // dampingBondSmooth implies dampingBond (connectToProperties, :285)
  if (st->dampingBond || st->dampingBondSmooth) fl |= kBondDamping;
  if (st->dampingBondSmooth) fl |= kBondDampingSmooth;
  if (st->ratioTCBond) fl |= kBondUseRatioTC;
  h->s.bond_flags = fl;
  h->s.bond_ts_create = (long long)(int)st->tsCreate;
  h->sys_gen++;
  return DEM_OK;
}

// neighbor->register_contact_dist_factor of cohesion bond/nonlinear
// (connectToProperties, src/cohesion_model_bond_nonlinear.h:330-380): the
// cutoff grows with the largest breakage distance relative to the smallest
// radius.  Returns 0 or a DEM_ERR_*.
static int bond_contact_distance_factor(dem_handle *h, double minrad, double *cdf) {
  const int nt = h->s.ntypes;
  const size_t m = (size_t)(nt + 1) * (nt + 1);
  auto T = [&](int t, int i, int j) { return h->bond_tables[t * m + (size_t)i * (nt + 1) + j]; };
  const dem_bond_settings &st = h->bond_settings;
  double cdf_all = 1.;
  for (int i = 1; i < nt + 1; i++)
    for (int j = 1; j < nt + 1; j++) {
      double one;
      if (!st.stressBreak) {
        one = 1.1 * 0.5 * T(kBondMaxDist, i, j) / minrad;
      } else {
        double stress = T(kBondMaxSigma, i, j);
        if (st.ratioTCBond) stress = std::fmax(stress, stress * T(kBondRatioTC, i, j));
        if (T(kBondKfn2, i, j) <= 1e-15) return fail(h, DEM_ERR_BAD_ARG, "stress breakage needs K_fn2 > 0");
        one = 0.5 * 1.1 * T(kBondCreateDist, i, j) / minrad + 0.5 * 1.1 * stress / (T(kBondKfn2, i, j) * minrad);
      }
      cdf_all = one > cdf_all ? one : cdf_all;
    }
  if (cdf_all > 10.) return fail(h, DEM_ERR_BAD_ARG, "bond distance above 10 particle diameters");
  *cdf = cdf_all;
  return DEM_OK;
}

int dem_add_plane(dem_handle *h, int axis, double pos, int wall_type, int rolling_model, int *wall_id) {
  if (!h || axis < 0 || axis > 2 || wall_type < 1) return DEM_ERR_BAD_ARG;
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "add walls before uploading atoms");
  if (h->s.nplanes >= kMaxPlanes) return fail(h, DEM_ERR_BAD_ARG, "too many primitive walls");
  Plane &p = h->s.planes[h->s.nplanes];
  p = Plane{};
  p.axis = axis;
  p.pos = pos;
  p.pos_t = nullptr;
  p.wall_type = wall_type;
  p.rolling = rolling_model == DEM_ROLLING_CDT ? 1 : 0;
  if (wall_id) *wall_id = h->s.nplanes;
  h->s.nplanes++;
  h->sys_gen++;
  return DEM_OK;
}

int dem_add_cylinder(dem_handle *h, int axis, double radius, double center1, double center2, int wall_type,
                     int rolling_model, int *wall_id) {
  if (!h || axis < 0 || axis > 2 || wall_type < 1 || !(radius > 0.0) || !std::isfinite(radius) ||
      !std::isfinite(center1) || !std::isfinite(center2))
    return DEM_ERR_BAD_ARG;
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "add walls before uploading atoms");
  if (h->s.nplanes >= kMaxPlanes) return fail(h, DEM_ERR_BAD_ARG, "too many primitive walls");
  Plane &p = h->s.planes[h->s.nplanes];
  p = Plane{};
  p.axis = axis;
  p.pos = radius;
  p.kind = 1;
  p.c1 = center1;
  p.c2 = center2;
  p.pos_t = nullptr;
  p.wall_type = wall_type;
  p.rolling = rolling_model == DEM_ROLLING_CDT ? 1 : 0;
  if (wall_id) *wall_id = h->s.nplanes;
  h->s.nplanes++;
  h->sys_gen++;
  return DEM_OK;
}

int dem_add_plane_per_type(dem_handle *h, int axis, const double *pos_by_type, int rolling_model,
                           int *wall_id) {
  if (!h || axis < 0 || axis > 2 || !pos_by_type) return DEM_ERR_BAD_ARG;
  if (!h->have_params) return fail(h, DEM_ERR_BAD_ARG, "set pair parameters first");
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "add walls before uploading atoms");
  if (h->s.nplanes >= kMaxPlanes) return fail(h, DEM_ERR_BAD_ARG, "too many primitive walls");
  double *dpos = nullptr;
  CUDA_TRY(h, dalloc(h->allocs_misc, &dpos, (size_t)h->s.ntypes + 1));
  CUDA_TRY(h, cudaMemcpyAsync(dpos, pos_by_type, ((size_t)h->s.ntypes + 1) * sizeof(double), cudaMemcpyHostToDevice, h->st));
  Plane &p = h->s.planes[h->s.nplanes];
  p = Plane{};
  p.axis = axis;
  p.pos = pos_by_type[1];
  p.pos_t = dpos;
  p.wall_type = 0;
  p.rolling = rolling_model == DEM_ROLLING_CDT ? 1 : 0;
  if (wall_id) *wall_id = h->s.nplanes;
  h->s.nplanes++;
  h->sys_gen++;
  return DEM_OK;
}

int dem_set_ensemble(dem_handle *h, int nsys) {
  if (!h || nsys < 1) return DEM_ERR_BAD_ARG;
  if (!h->have_params || h->s.ntypes != nsys)
    return fail(h, DEM_ERR_BAD_ARG, "an ensemble of nsys systems needs ntypes == nsys (system k = type k+1)");
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "declare the ensemble before uploading atoms");
  if (h->s.nmeshes > 0) return fail(h, DEM_ERR_UNSUPPORTED, "mesh walls are not supported in ensembles");
  h->ens_nsys = nsys;
  // per-system neighbour decisions: moved, rebuild, ago, build count [nsys]
  // and the systems' first atoms [nsys+1]; list segments: start [nsys+1],
  // used [nsys]; the in-place rebuild's compaction: rlist [nsys], rpre and
  // cpre [nsys+1]
  const size_t nbuf = (size_t)10 * nsys + 4;
  int *buf = nullptr;
  CUDA_TRY(h, dalloc(h->allocs_misc, &buf, nbuf));
  CUDA_TRY(h, cudaMemsetAsync(buf, 0, nbuf * sizeof(int), h->st));
  Sys &s = h->s;
  s.nsys = nsys;
  s.sys_moved = buf;
  s.sys_reb = buf + nsys;
  s.sys_ago = buf + 2 * nsys;
  s.sys_nreb = buf + 3 * nsys;
  s.sys_start = buf + 4 * nsys;            // [nsys+1]
  s.seg_start = buf + 5 * nsys + 1;        // [nsys+1]
  s.seg_used = buf + 6 * nsys + 2;         // [nsys]
  s.rlist = buf + 7 * nsys + 2;            // [nsys]
  s.rpre = buf + 8 * nsys + 2;             // [nsys+1]
  s.cpre = buf + 9 * nsys + 3;             // [nsys+1]
  // LIGGGHTS_GB300_ENS_FULL=1 takes the whole-list path at every rebuild;
  // LIGGGHTS_GB300_ENS_SLACK sets the segments' unused share in percent
  // (default 12; 0 makes every growth re-lay the list): both for tests
  const char *ef = getenv("LIGGGHTS_GB300_ENS_FULL");
  s.ens_full = (ef && atoi(ef) != 0) ? 1 : 0;
  const char *es = getenv("LIGGGHTS_GB300_ENS_SLACK");
  s.ens_slack = es ? std::max(0, std::min(400, atoi(es))) : 12;
  h->sys_gen++;
  return DEM_OK;
}

int dem_ensemble_rebuilds(dem_handle *h, int *counts) {
  if (!h || !counts || h->ens_nsys < 1) return DEM_ERR_BAD_ARG;
  CUDA_TRY(h, cudaMemcpyAsync(counts, h->s.sys_nreb, (size_t)h->ens_nsys * sizeof(int), cudaMemcpyDeviceToHost,
                              h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  return DEM_OK;
}

int dem_set_tuning(dem_handle *h, int blocks_per_sm, double cell_scale) {
  if (!h || blocks_per_sm < 1 || blocks_per_sm > 64 || !(cell_scale >= 1.0) || cell_scale > 4.0)
    return DEM_ERR_BAD_ARG;
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "set the tuning before uploading atoms");
  cudaDeviceProp prop;
  int sms = 152;
  if (cudaGetDeviceProperties(&prop, h->device) == cudaSuccess) sms = prop.multiProcessorCount;
  h->lc.max_grid = sms * blocks_per_sm;
  h->cell_scale = cell_scale;
  h->sys_gen++;
  return DEM_OK;
}

int dem_set_particle_threads(dem_handle *h, int threads) {
  if (!h || (threads != 64 && threads != 128 && threads != 256)) return DEM_ERR_BAD_ARG;
  h->lc.particle_threads = threads;
  h->sys_gen++;  // the step graph is rebuilt with the new launch shape
  return DEM_OK;
}

int dem_add_mesh(dem_handle *h, int ntri, const double *nodes, int wall_type, int rolling_model,
                 const unsigned char *edge_active, const unsigned char *corner_active, int *mesh_id) {
  if (!h || ntri < 1 || !nodes || wall_type < 1) return DEM_ERR_BAD_ARG;
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "add meshes before uploading atoms");
  if (h->s.nmeshes >= kMaxMeshes) return fail(h, DEM_ERR_BAD_ARG, "too many mesh walls");
  MeshHost mh;
  int rc = mesh_prepare(ntri, nodes, edge_active, corner_active, mh);
  if (rc) return fail(h, rc, "degenerate mesh element");
  MeshDev &M = h->s.meshes[h->s.nmeshes];
  M = MeshDev{};
  M.ntri = ntri;
  M.wall_type = wall_type;
  M.rolling = rolling_model == DEM_ROLLING_CDT ? 1 : 0;
  // initial candidate triangles per atom; grown on demand.
  // LIGGGHTS_GB300_MESH_CAND sets a smaller start (tests of the growth path)
  M.ccap = kMeshCandInit;
  if (const char *e = getenv("LIGGGHTS_GB300_MESH_CAND")) M.ccap = std::max(1, atoi(e));
  auto &L = h->allocs_misc;
  CUDA_TRY(h, dalloc(L, &M.tri, mh.tri.size()));
  CUDA_TRY(h, cudaMemcpyAsync(M.tri, mh.tri.data(), mh.tri.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, dalloc(L, &M.meta, mh.meta.size()));
  CUDA_TRY(h, cudaMemcpyAsync(M.meta, mh.meta.data(), mh.meta.size() * sizeof(int), cudaMemcpyHostToDevice, h->st));
  {
    std::vector<float4> tf(2 * (size_t)ntri);
    for (int t = 0; t < ntri; t++) {
      const double *g = &mh.tri[(size_t)t * kTriStride];
      tf[2 * (size_t)t] = make_float4((float)g[0], (float)g[1], (float)g[2], 0.f);
      tf[2 * (size_t)t + 1] = make_float4((float)g[30], (float)g[31], (float)g[32], 0.f);
    }
    CUDA_TRY(h, dalloc(L, &M.trif, tf.size()));
    CUDA_TRY(h, cudaMemcpyAsync(M.trif, tf.data(), tf.size() * sizeof(float4), cudaMemcpyHostToDevice, h->st));
  }
  CUDA_TRY(h, dalloc(L, &M.cn_start, mh.cn_start.size()));
  CUDA_TRY(h, cudaMemcpyAsync(M.cn_start, mh.cn_start.data(), mh.cn_start.size() * sizeof(int), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, dalloc(L, &M.cn_list, std::max<size_t>(1, mh.cn_list.size())));
  if (!mh.cn_list.empty())
    CUDA_TRY(h, cudaMemcpyAsync(M.cn_list, mh.cn_list.data(), mh.cn_list.size() * sizeof(int), cudaMemcpyHostToDevice, h->st));
  // bounding boxes for the cell-registration estimate of each upload
  mh.bbox.resize(6 * (size_t)ntri);
  for (int t = 0; t < ntri; t++) {
    const double *g = &mh.tri[(size_t)t * kTriStride];
    for (int d = 0; d < 3; d++) {
      mh.bbox[6 * (size_t)t + d] = std::min(g[d], std::min(g[3 + d], g[6 + d]));
      mh.bbox[6 * (size_t)t + 3 + d] = std::max(g[d], std::max(g[3 + d], g[6 + d]));
    }
  }
  if (mesh_id) *mesh_id = h->s.nmeshes;
  h->mesh_host.push_back(std::move(mh));
  h->s.nmeshes++;
  h->sys_gen++;
  return DEM_OK;
}

int dem_set_mesh_motion(dem_handle *h, int mesh_id, const double *vel) {
  if (!h || !vel || mesh_id < 0 || mesh_id >= h->s.nmeshes) return DEM_ERR_BAD_ARG;
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "set mesh motion before uploading atoms");
  MeshDev &M = h->s.meshes[mesh_id];
  for (int d = 0; d < 3; d++) {
    if (!std::isfinite(vel[d])) return fail(h, DEM_ERR_BAD_ARG, "non-finite mesh velocity");
    M.vel[d] = vel[d];
    M.dx[d] = h->s.dt * vel[d];  // vectorScalarMult3D(vel_, dt, dx)
  }
  if (!M.node_last) {
    CUDA_TRY(h, dalloc(h->allocs_misc, &M.node_last, (size_t)9 * M.ntri));
    std::vector<double> nl((size_t)9 * M.ntri);
    const MeshHost &mh = h->mesh_host[mesh_id];
    for (int t = 0; t < M.ntri; t++)
      for (int q = 0; q < 9; q++) nl[(size_t)t * 9 + q] = mh.tri[(size_t)t * kTriStride + q];
    CUDA_TRY(h, cudaMemcpyAsync(M.node_last, nl.data(), nl.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  }
  M.moving = 1;
  M.vel_on = 0;
  h->sys_gen++;
  return DEM_OK;
}

int dem_set_mesh_rotation(dem_handle *h, int mesh_id, const double *origin, const double *axis, double period) {
  if (!h || !origin || !axis || mesh_id < 0 || mesh_id >= h->s.nmeshes) return DEM_ERR_BAD_ARG;
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "set mesh motion before uploading atoms");
  if (!(period != 0.0) || !std::isfinite(period)) return fail(h, DEM_ERR_BAD_ARG, "bad rotation period");
  MeshDev &M = h->s.meshes[mesh_id];
  if (M.moving) return fail(h, DEM_ERR_BAD_ARG, "one mover per mesh");
  // MeshMoverRotate: axis_ normalised by vectorNormalize3D, omega_ = 2 pi / T
  double ax[3] = {axis[0], axis[1], axis[2]};
  const double norm = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
  if (!(norm > 0.0)) return fail(h, DEM_ERR_BAD_ARG, "zero rotation axis");
  const double invnorm = 1. / norm;
  for (int d = 0; d < 3; d++) ax[d] *= invnorm;
  const double omega = 2. * M_PI / period;
  const double dangle = omega * h->s.dt;  // incrementalPhi = omega_ * dt
  // MultiNodeMesh::rotate(dAngle, axis, p): axisNorm = axis / |axis|, dQ
  double an[3] = {ax[0], ax[1], ax[2]};
  const double mag = std::sqrt(an[0] * an[0] + an[1] * an[1] + an[2] * an[2]);
  const double sinv = 1. / mag;
  for (int d = 0; d < 3; d++) an[d] = sinv * an[d];
  M.rq[0] = std::cos(dangle * 0.5);
  for (int d = 0; d < 3; d++) M.rq[d + 1] = an[d] * std::sin(dangle * 0.5);
  for (int d = 0; d < 3; d++) {
    M.rorig[d] = origin[d];
    M.romega[d] = ax[d] * omega;  // vectorScalarMult3D(axis_, omega_, omegaVec)
    M.vel[d] = 0.0;
    M.dx[d] = 0.0;
  }
  CUDA_TRY(h, dalloc(h->allocs_misc, &M.nodev, (size_t)9 * M.ntri));
  CUDA_TRY(h, cudaMemsetAsync(M.nodev, 0, (size_t)9 * M.ntri * sizeof(double), h->st));
  if (!M.node_last) {
    CUDA_TRY(h, dalloc(h->allocs_misc, &M.node_last, (size_t)9 * M.ntri));
    std::vector<double> nl((size_t)9 * M.ntri);
    const MeshHost &mh = h->mesh_host[mesh_id];
    for (int t = 0; t < M.ntri; t++)
      for (int q = 0; q < 9; q++) nl[(size_t)t * 9 + q] = mh.tri[(size_t)t * kTriStride + q];
    CUDA_TRY(h, cudaMemcpyAsync(M.node_last, nl.data(), nl.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  }
  M.rotating = 1;
  M.moving = 1;
  M.vel_on = 0;
  h->sys_gen++;
  return DEM_OK;
}

int dem_download_mesh_nodes(dem_handle *h, int mesh_id, double *nodes) {
  if (!h || !nodes || mesh_id < 0 || mesh_id >= h->s.nmeshes) return DEM_ERR_BAD_ARG;
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  const MeshDev &M = h->s.meshes[mesh_id];
  std::vector<double> g((size_t)kTriStride * M.ntri);
  CUDA_TRY(h, cudaMemcpyAsync(g.data(), M.tri, g.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  for (int t = 0; t < M.ntri; t++)
    for (int q = 0; q < 9; q++) nodes[(size_t)t * 9 + q] = g[(size_t)t * kTriStride + q];
  return DEM_OK;
}

static void set_mesh_velocity_on(dem_handle *h, int on) {
  for (int k = 0; k < h->s.nmeshes; k++) {
    MeshDev &M = h->s.meshes[k];
    if (M.moving && M.vel_on != on) {
      M.vel_on = on;
      h->sys_gen++;  // kernels of an existing graph hold the old value
    }
  }
}

int dem_mesh_ncontacts(dem_handle *h, int mesh_id, int *nc) {
  if (!h || !h->have_atoms || !nc || mesh_id < 0 || mesh_id >= h->s.nmeshes) return DEM_ERR_BAD_ARG;
  int rc = read_ctrl(h);
  if (rc) return rc;
  const int n = h->host_ctrl.n;
  std::vector<int> np(n);
  CUDA_TRY(h, cudaMemcpyAsync(np.data(), h->s.meshes[mesh_id].npart[0], n * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  long t = 0;
  for (int v : np) t += v;
  *nc = (int)t;
  return DEM_OK;
}

int dem_download_mesh_contacts(dem_handle *h, int mesh_id, int *tag, int *tri, int *slot, double *hist) {
  if (!h || !h->have_atoms || mesh_id < 0 || mesh_id >= h->s.nmeshes) return DEM_ERR_BAD_ARG;
  int rc = read_ctrl(h);
  if (rc) return rc;
  const int n = h->host_ctrl.n;
  const size_t nmax = h->s.nmax;
  const MeshDev &M = h->s.meshes[mesh_id];
  std::vector<int> ns(n), st((size_t)M.ccap * nmax), tags(n);
  std::vector<double> sh((size_t)3 * M.ccap * nmax);
  CUDA_TRY(h, cudaMemcpyAsync(ns.data(), M.nslot[0], n * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(st.data(), M.slot_tri[0], st.size() * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(sh.data(), M.slot_hist[0], sh.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(tags.data(), h->s.atoms[0].tag, n * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  int c = 0;
  for (int i = 0; i < n; i++)
    for (int q = 0; q < ns[i]; q++) {
      const int t = st[(size_t)q * nmax + i];
      if (t < 0) continue;
      if (tag) tag[c] = tags[i];
      if (tri) tri[c] = t;
      if (slot) slot[c] = q;
      if (hist)
        for (int d = 0; d < 3; d++) hist[3 * (size_t)c + d] = sh[(size_t)(3 * q + d) * nmax + i];
      c++;
    }
  return DEM_OK;
}

int dem_upload_atoms(dem_handle *h, int n, const int *tag, const int *type, const double *x,
                     const double *v, const double *omega, const double *radius,
                     const double *rmass) {
  if (!h || n < 1 || !tag || !type || !x || !v || !omega || !radius || !rmass) return DEM_ERR_BAD_ARG;
  if (!h->have_params) return fail(h, DEM_ERR_BAD_ARG, "set pair parameters first");
  Sys &s = h->s;
  if ((long)n > kMaxScan) return fail(h, DEM_ERR_BAD_ARG, "too many atoms for one handle");
  for (int w = 0; w < s.nplanes; w++)
    if (s.planes[w].wall_type > s.ntypes) return fail(h, DEM_ERR_BAD_ARG, "wall type out of range");
  for (int k = 0; k < s.nmeshes; k++)
    if (s.meshes[k].wall_type > s.ntypes) return fail(h, DEM_ERR_BAD_ARG, "mesh wall type out of range");
  if (h->cap_n > 0 && h->cap_n < n) return fail(h, DEM_ERR_CAPACITY, "more atoms than the capacity set");
  h->have_atoms = false;
  h->setup_done = false;
  int rc = alloc_atoms(h, std::max(n, h->cap_n));
  if (rc) return rc;

  // the caller's arrays into the SoA state, with the checks and the radius
  // range, in one pass on the device
  AtomsIn in{tag, type, x, v, omega, radius, rmass};
  if (!h->host_direct) {
    const size_t nd = (size_t)n * sizeof(double), ni = (size_t)n * sizeof(int);
    rc = ensure_stage(h, 11 * nd + 2 * ni);
    if (rc) return rc;
    char *p = static_cast<char *>(h->stage);
    double *dx = reinterpret_cast<double *>(p), *dv = dx + 3 * (size_t)n, *dw = dv + 3 * (size_t)n;
    double *dr = dw + 3 * (size_t)n, *dm = dr + n;
    int *dtag = reinterpret_cast<int *>(dm + n), *dtype = dtag + n;
    CUDA_TRY(h, cudaMemcpyAsync(dx, x, 3 * nd, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(dv, v, 3 * nd, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(dw, omega, 3 * nd, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(dr, radius, nd, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(dm, rmass, nd, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(dtag, tag, ni, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(dtype, type, ni, cudaMemcpyHostToDevice, h->st));
    in = AtomsIn{dtag, dtype, dx, dv, dw, dr, dm};
  }
  UploadCheck *ck = h->chk_host;
  *ck = UploadCheck{~0ull, 0ull, 0, 0, 0, 0};
  CUDA_TRY(h, cudaMemcpyAsync(h->chk, ck, sizeof(UploadCheck), cudaMemcpyHostToDevice, h->st));
  // FixNVESphere's dtf and dtfrotate (src/fix_nve_sphere.cpp:150-178)
  const double dtf = 0.5 * s.dt * 1.0;
  const double dtfrotate = dtf / 0.4;
  h->kt.kernel_launches += launch_upload_atoms(s, in, n, dtf, dtfrotate, h->chk, h->st);
  CUDA_TRY(h, cudaGetLastError());
  CUDA_TRY(h, cudaMemcpyAsync(ck, h->chk, sizeof(UploadCheck), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  if (ck->bad_type) return fail(h, DEM_ERR_BAD_ARG, "atom type out of range");
  if (ck->bad_value) return fail(h, DEM_ERR_BAD_ARG, "radius and rmass must be finite and > 0");
  if (ck->nonfinite) return fail(h, DEM_ERR_NAN, "non-finite position, velocity or angular velocity");
  double maxrad, minrad;
  {
    long long a = (long long)ck->rmax, b = (long long)ck->rmin;
    std::memcpy(&maxrad, &a, sizeof a);
    std::memcpy(&minrad, &b, sizeof b);
  }
  // cutneighmax = (maxrad_i + maxrad_j)*cdf + skin, src/pair_gran.cpp:591-602,
  // src/neighbor.cpp:316-337
  // radii that later insertions may bring (PairGran::init_one takes the
  // insertion templates' radii into maxrad/minrad the same way)
  if (h->cap_rmax > 0.0) maxrad = std::max(maxrad, h->cap_rmax);
  if (h->cap_rmin > 0.0) minrad = std::min(minrad, h->cap_rmin);
  h->eff_rmin = minrad;
  h->eff_rmax = maxrad;
  s.cdf = h->cfg.contact_distance_factor;
  if (s.bond) {
    if (!s.bondp) return fail(h, DEM_ERR_BAD_ARG, "cohesion bond/nonlinear needs dem_set_bond_params");
    double cdf_bond = 1.0;
    int rcb = bond_contact_distance_factor(h, minrad, &cdf_bond);
    if (rcb) return rcb;
    s.cdf = std::max(s.cdf, cdf_bond);
  }
  const double cutoff = (maxrad + maxrad) * s.cdf;
  s.cutneighmax = std::sqrt(cutoff * cutoff) + s.skin;
  s.ghost_slab = s.cutneighmax / 2. + s.skin / 2.;
  {  // FP32 neighbour prefilter margin: bound of the FP32 error of rsq
     // relative to the smallest cutoff^2, times 4, at least 1e-4
    double cmax = 0.0, pmax = 0.0;
    for (int d = 0; d < 3; d++) {
      cmax = std::max(cmax, std::max(std::fabs(s.boxlo[d]), std::fabs(s.boxhi[d])));
      pmax = std::max(pmax, s.prd[d]);
    }
    const double e = 3.0 * std::ldexp(cmax + pmax, -24);  // per component of delta
    const double cmin = 2.0 * minrad * s.cdf + s.skin;
    const double rel = 2.0 * std::sqrt(3.0) * e / cmin + 3.0 * e * e / (cmin * cmin) + 1e-6;
    s.pf_margin = (float)std::min(0.5, std::max(1e-4, 4.0 * rel));
    const double tmin = 2.0 * minrad;
    const double relt = 2.0 * std::sqrt(3.0) * e / tmin + 3.0 * e * e / (tmin * tmin) + 1e-6;
    s.pf_margin_touch = (float)std::min(0.5, std::max(1e-4, 4.0 * relt));
    // displacement prefilter: |(float)x - (float)xhold| is within
    // sqrt(3)*2^-23*C + 4*2^-24*|d| of |x - xhold| (C bounds coordinates);
    // four times that is the band the exact test decides
    const double hs = 0.5 * s.skin;
    const double band = 4.0 * (std::sqrt(3.0) * std::ldexp(cmax + pmax, -23) + 4.0 * std::ldexp(hs, -24));
    s.skin_lo2 = hs > band ? (float)((hs - band) * (hs - band) * (1.0 - 1e-6)) : -1.0f;
    s.skin_hi2 = (float)((hs + band) * (hs + band) * (1.0 + 1e-6));
  }
  long ncell = 1;
  for (int d = 0; d < 3; d++) {
    long nc = (long)std::floor(s.prd[d] / (s.cutneighmax * h->cell_scale * (1.0 + 1e-9)));
    if (nc < 1) nc = 1;
    if (s.periodic[d] && nc < 3)
      return fail(h, DEM_ERR_BOX, "periodic box dimension shorter than 3 neighbour cutoffs");
    s.nc[d] = (int)std::min<long>(nc, 4096);
    ncell *= s.nc[d];
  }
  const long nsys = std::max(1, h->ens_nsys);
  while (ncell * nsys > kMaxCells) {  // very sparse boxes: coarser cells stay conservative
    int d = (s.nc[0] >= s.nc[1] && s.nc[0] >= s.nc[2]) ? 0 : (s.nc[1] >= s.nc[2] ? 1 : 2);
    if (s.periodic[d] && s.nc[d] <= 3) break;
    s.nc[d] = std::max(s.periodic[d] ? 3 : 1, s.nc[d] / 2);
    ncell = (long)s.nc[0] * s.nc[1] * s.nc[2];
  }
  for (int d = 0; d < 3; d++) {
    s.csz[d] = s.prd[d] / s.nc[d];
    s.icsz[d] = 1.0 / s.csz[d];
    s.prdf[d] = (float)s.prd[d];
  }
  s.cdff = (float)s.cdf;
  s.skinf = (float)s.skin;
  s.ens_ncell = h->ens_nsys > 0 ? (int)ncell : 0;
  s.ncell = (int)(ncell * nsys);
  // FixNeighlistMesh::pre_force distmax/skin (static meshes), src/fix_neighlist_mesh.cpp:249-264
  for (int k = 0; k < s.nmeshes; k++) {
    MeshDev &M = s.meshes[k];
    const double rmax = 0.5 * (s.cutneighmax - s.skin);
    const double small_delta = s.skin / (70. * M_PI);
    M.distmax = M.moving ? s.cutneighmax + small_delta : s.cutneighmax - rmax + small_delta;
    M.tskin = M.moving ? s.skin : 0.5 * s.skin;
    // capacity of the triangle-to-cell registrations, from the initial mesh
    const MeshHost &mh = h->mesh_host[k];
    long tot = 0;
    for (int t = 0; t < mh.ntri; t++) {
      long cells = 1;
      for (int d = 0; d < 3; d++) {
        const double a = mh.bbox[6 * (size_t)t + d], b = mh.bbox[6 * (size_t)t + 3 + d];
        auto cc = [&](double x) {  // an estimate: the rebuild grows the list if it is short
          long c = (long)((x - s.boxlo[d]) * s.icsz[d]);
          return std::min<long>(std::max<long>(c, 0), s.nc[d] - 1);
        };
        cells *= cc(b + M.distmax) - cc(a - M.distmax) + 1 + (M.moving ? 2 : 0);
      }
      tot += cells;
    }
    M.tc_cap = (int)std::min<long>(2147000000L, 2 * tot + 4096);
    // LIGGGHTS_GB300_MESH_REG sets a smaller start (tests of the growth path)
    if (const char *e = getenv("LIGGGHTS_GB300_MESH_REG")) M.tc_cap = std::max(1, atoi(e));
  }
  rc = alloc_cells(h);
  if (rc) return rc;
  h->pending_insert = 0;
  h->next_lidx = n;
  // Initial pair capacity: 16 entries per atom.  LIGGGHTS_GB300_PAIRS_PER_ATOM
  // overrides it; a deliberately small value exercises the overflow path
  // (device halt, host growth, resumed rebuild) in tests.
  long ppa = 16;
  if (const char *e = getenv("LIGGGHTS_GB300_PAIRS_PER_ATOM")) ppa = std::max(0L, atol(e));
  rc = alloc_pairs(h, (int)std::max<long>(ppa * n, ppa >= 16 ? 4096 : 1), 0);
  if (rc) return rc;
  Ctrl c{};
  c.n = n;
  h->host_ctrl = c;
  CUDA_TRY(h, cudaMemcpyAsync(s.ctrl, &h->host_ctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  h->have_atoms = true;
  return DEM_OK;
}

int dem_set_capacity(dem_handle *h, int natoms_max, double rmin, double rmax) {
  if (!h || natoms_max < 0 || rmin < 0.0 || rmax < 0.0 || (rmin > 0.0 && rmax > 0.0 && rmin > rmax))
    return DEM_ERR_BAD_ARG;
  if (h->have_atoms) return fail(h, DEM_ERR_BAD_ARG, "set the capacity before uploading atoms");
  if ((long)natoms_max > kMaxScan) return fail(h, DEM_ERR_BAD_ARG, "capacity too large for one handle");
  h->cap_n = natoms_max;
  h->cap_rmin = rmin;
  h->cap_rmax = rmax;
  return DEM_OK;
}

int dem_insert_atoms(dem_handle *h, int k, const int *tag, const int *type, const double *x, const double *v,
                     const double *omega, const double *radius, const double *rmass) {
  if (!h || k < 0 || (k > 0 && (!tag || !type || !x || !v || !omega || !radius || !rmass))) return DEM_ERR_BAD_ARG;
  if (!h->have_atoms || !h->setup_done) return fail(h, DEM_ERR_BAD_ARG, "insert after dem_setup");
  if (h->ens_nsys > 0) return fail(h, DEM_ERR_UNSUPPORTED, "insertion into an ensemble");
  if (k == 0) return DEM_OK;
  Sys &s = h->s;
  for (int q = 0; q < k; q++) {
    if (type[q] < 1 || type[q] > s.ntypes) return fail(h, DEM_ERR_BAD_ARG, "atom type out of range");
    if (!(rmass[q] > 0.0)) return fail(h, DEM_ERR_BAD_ARG, "rmass must be > 0");
    if (!(radius[q] >= h->eff_rmin && radius[q] <= h->eff_rmax))
      return fail(h, DEM_ERR_BAD_ARG, "inserted radius outside the range the neighbour cutoff was sized for "
                                      "(dem_set_capacity)");
    for (int d = 0; d < 3; d++)
      if (!std::isfinite(x[3 * q + d]) || !std::isfinite(v[3 * q + d]) || !std::isfinite(omega[3 * q + d]))
        return fail(h, DEM_ERR_BAD_ARG, "non-finite inserted state");
  }
  int rc = read_ctrl(h);
  if (rc) return rc;
  const int first = h->host_ctrl.n + h->pending_insert;
  if ((long)first + k > (long)s.nmax) return fail(h, DEM_ERR_CAPACITY, "atom capacity exceeded (dem_set_capacity)");
  // FixNVESphere per-atom constants as at upload
  const double dtf = 0.5 * s.dt * 1.0;
  const double dtfrotate = dtf / 0.4;
  std::vector<double> dtfm(k), dtir(k);
  for (int q = 0; q < k; q++) {
    dtfm[q] = dtf / (rmass[q] * (1. + 0.0));
    dtir[q] = dtfrotate / (radius[q] * radius[q] * rmass[q]);
  }
  double *buf = nullptr;
  int *ibuf = nullptr;
  const size_t nd = (size_t)k * (9 + 4);
  CUDA_TRY(h, cudaMalloc(&buf, nd * sizeof(double)));
  CUDA_TRY(h, cudaMalloc(&ibuf, (size_t)2 * k * sizeof(int)));
  const double *src[] = {x, v, omega};
  for (int a = 0; a < 3; a++)
    CUDA_TRY(h, cudaMemcpyAsync(buf + (size_t)3 * k * a, src[a], (size_t)3 * k * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(buf + (size_t)9 * k, radius, (size_t)k * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(buf + (size_t)10 * k, rmass, (size_t)k * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(buf + (size_t)11 * k, dtfm.data(), (size_t)k * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(buf + (size_t)12 * k, dtir.data(), (size_t)k * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(ibuf, type, (size_t)k * sizeof(int), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(ibuf + k, tag, (size_t)k * sizeof(int), cudaMemcpyHostToDevice, h->st));
  InsertStage in;
  in.x = buf;
  in.v = buf + (size_t)3 * k;
  in.w = buf + (size_t)6 * k;
  in.r = buf + (size_t)9 * k;
  in.m = buf + (size_t)10 * k;
  in.dtfm = buf + (size_t)11 * k;
  in.dtir = buf + (size_t)12 * k;
  in.type = ibuf;
  in.tag = ibuf + k;
  h->kt.kernel_launches += launch_insert_stage(s, in, first, k, h->next_lidx, h->st);
  CUDA_TRY(h, cudaGetLastError());
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  cudaFree(buf);
  cudaFree(ibuf);
  h->next_lidx += k;
  h->pending_insert += k;
  return DEM_OK;
}

int dem_upload_contact_history(dem_handle *h, int ne, const int *towner, const int *tpartner,
                               const double *hist) {
  if (!h || !h->have_atoms || ne < 0 || (ne > 0 && (!towner || !tpartner || !hist)))
    return DEM_ERR_BAD_ARG;
  if (h->setup_done) return fail(h, DEM_ERR_BAD_ARG, "contact history must precede dem_setup");
  const int n = h->host_ctrl.n;
  std::vector<int> tags(n);
  CUDA_TRY(h, cudaMemcpyAsync(tags.data(), h->s.atoms[0].tag, n * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  // tag -> local index, as the reference's atom map array (Atom::map_set)
  int maxtag = 0;
  for (int i = 0; i < n; i++) maxtag = std::max(maxtag, tags[i]);
  std::vector<int> t2i((size_t)maxtag + 1, -1);
  for (int i = 0; i < n; i++)
    if (tags[i] >= 0) t2i[tags[i]] = i;
  auto find = [&](int t) -> int { return (t >= 0 && t <= maxtag) ? t2i[t] : -1; };
  std::vector<int> oi(ne), oj(ne), row(n + 1, 0);
  for (int k = 0; k < ne; k++) {
    oi[k] = find(towner[k]);
    oj[k] = find(tpartner[k]);
    if (oi[k] < 0 || oj[k] < 0) return fail(h, DEM_ERR_BAD_ARG, "contact history names an unknown tag");
    row[oi[k] + 1]++;
  }
  for (int i = 0; i < n; i++) row[i + 1] += row[i];
  if (ne > h->s.pcap) {
    int rc = alloc_pairs(h, ne + 1024, 0);
    if (rc) return rc;
  }
  const size_t P = h->s.pcap;
  const int dnum = h->s.dnum;
  std::vector<int> pi(ne), pj(ne), fl(ne, 1), fill(row.begin(), row.end() - 1);
  std::vector<double> hh((size_t)dnum * ne);  // [d*ne + p]: one block per history value
  for (int k = 0; k < ne; k++) {
    const int p = fill[oi[k]]++;
    pi[p] = oi[k];
    pj[p] = oj[k];
    for (int r = 0; r < dnum; r++) hh[(size_t)dev_hist_index(h->s, r) * ne + p] = hist[(size_t)k * dnum + r];
  }
  const PairArrays &L = h->s.pairs[0];
  if (ne) {
    // each entry is its owner's own partner-list copy: marked as a directed
    // (image) entry so that the first build takes it as it is
    std::vector<uint8_t> dsh(ne, 0);
    CUDA_TRY(h, cudaMemcpyAsync(L.i, pi.data(), ne * sizeof(int), cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(L.j, pj.data(), ne * sizeof(int), cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(L.sh, dsh.data(), ne, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(L.flag, fl.data(), ne * sizeof(int), cudaMemcpyHostToDevice, h->st));
    for (int d = 0; d < dnum; d++)
      CUDA_TRY(h, cudaMemcpyAsync(L.hist + (size_t)d * P, hh.data() + (size_t)d * ne, (size_t)ne * sizeof(double),
                                  cudaMemcpyHostToDevice, h->st));
  }
  CUDA_TRY(h, cudaMemcpyAsync(L.row, row.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaMemsetAsync(L.rev_start, 0, (h->s.nmax + 1) * sizeof(int), h->st));
  if (L.rowe) {  // ensembles: the rows' ends (no segments before the first build)
    CUDA_TRY(h, cudaMemcpyAsync(L.rowe, row.data() + 1, n * sizeof(int), cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemsetAsync(L.reve, 0, (h->s.nmax + 1) * sizeof(int), h->st));
  }
  CUDA_TRY(h, cudaStreamSynchronize(h->st));  // the host vectors go out of scope
  return DEM_OK;
}

int dem_upload_wall_history(dem_handle *h, int wall_id, const double *hist) {
  if (!h || !h->have_atoms || !hist || wall_id < 0 || wall_id >= h->s.nplanes) return DEM_ERR_BAD_ARG;
  if (h->setup_done) return fail(h, DEM_ERR_BAD_ARG, "wall history must precede dem_setup");
  const int n = h->host_ctrl.n;
  std::vector<double> hb(n);
  for (int d = 0; d < 3; d++) {
    for (int i = 0; i < n; i++) hb[i] = hist[3 * (size_t)i + d];
    CUDA_TRY(h, cudaMemcpyAsync(h->s.atoms[0].whist + (size_t)(wall_id * 3 + d) * h->s.nmax, hb.data(),
                           n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  }
  return DEM_OK;
}

int dem_setup(dem_handle *h) {
  if (!h || !h->have_atoms) return DEM_ERR_BAD_ARG;
  cudaGetLastError();
  set_mesh_velocity_on(h, 0);  // FixMoveMesh::setup: node velocities 0
  h->kt.kernel_launches += launch_set_rebuild(h->s, 1, h->st);
  h->kt.kernel_launches += launch_rebuild(h->s, h->lc, h->st, 0);
  bool resumed = true;
  while (resumed) {
    int rc = recover(h, &resumed);
    if (rc) return rc;
  }
  h->kt.kernel_launches += launch_pair(h->s, h->lc, 0, h->st);
  h->kt.kernel_launches += launch_wall_force(h->s, h->lc, 0, h->st);
  h->kt.kernel_launches += launch_particle(h->s, h->lc, kModeGather, 0, h->st);
  CUDA_TRY(h, cudaGetLastError());
  bool dummy;
  int rc = recover(h, &dummy);
  if (rc) return rc;
  h->setup_done = true;
  return DEM_OK;
}

int dem_step(dem_handle *h, int nsteps) {
  if (!h || nsteps < 0) return DEM_ERR_BAD_ARG;
  if (!h->setup_done) return fail(h, DEM_ERR_BAD_ARG, "dem_setup must precede dem_step");
  if (nsteps == 0) return DEM_OK;
  set_mesh_velocity_on(h, 1);
  int rc = read_ctrl(h);
  if (rc) return rc;
  const long long ts0 = h->host_ctrl.ntimestep;
  CUDA_TRY(h, cudaEventRecord(h->ev0, h->st));
  long long done = 0;  // steps whose rebuild+pair stage has been queued
  bool first = true;
  const bool graph = h->use_graph && !h->profile;
  while (done < nsteps) {
    const long long chunk = graph ? nsteps - done : std::min<long long>(kCheckEvery, nsteps - done);
    long long k0 = 0;
    mark_start(h);
    if (first) {  // step 1 starts from stored forces: initial_integrate only
      h->kt.kernel_launches += launch_particle(h->s, h->lc, kModeInitial, 1, h->st);
      h->kt.kernel_launches += launch_mesh_move(h->s, h->lc, h->st);
      if (h->pending_insert > 0) {  // staged atoms join now and force a rebuild
        h->kt.kernel_launches += launch_insert_commit(h->s, h->pending_insert, h->st);
        h->pending_insert = 0;
      }
      mark(h, 0);
      h->kt.kernel_launches += launch_decide(h->s, h->st);
      h->kt.kernel_launches += launch_rebuild(h->s, h->lc, h->st, 0);
      mark(h, 1);
      h->kt.kernel_launches += launch_pair(h->s, h->lc, 1, h->st);
      mark(h, 2);
      h->kt.kernel_launches += launch_wall_force(h->s, h->lc, 1, h->st);
      mark(h, 3);
      first = false;
      k0 = 1;
    }
    if (graph && chunk > k0) {
      rc = ensure_graph(h);
      if (rc) return rc;
      rc = read_ctrl(h);
      if (rc) return rc;
      const long long rb0 = h->host_ctrl.nrebuilds;
      h->kt.kernel_launches += launch_set_loop(h->s, (int)(chunk - k0), h->st);
      CUDA_TRY(h, cudaGraphLaunch(h->gexec, h->st));
      rc = read_ctrl(h);
      if (rc) return rc;
      const long long iters = std::min<long long>(chunk - k0, h->host_ctrl.ntimestep - (ts0 + done + k0));
      h->kt.kernel_launches += iters * h->graph_kps + (h->host_ctrl.nrebuilds - rb0) * h->graph_kpr;
    } else {
      for (long long k = k0; k < chunk; k++) {
        h->kt.kernel_launches += launch_particle(h->s, h->lc, kModeGatherFinalInitial, 1, h->st);
        h->kt.kernel_launches += launch_mesh_move(h->s, h->lc, h->st);
        mark(h, 0);
        h->kt.kernel_launches += launch_decide(h->s, h->st);
        h->kt.kernel_launches += launch_rebuild(h->s, h->lc, h->st, 0);
        mark(h, 1);
        h->kt.kernel_launches += launch_pair(h->s, h->lc, 1, h->st);
        mark(h, 2);
        h->kt.kernel_launches += launch_wall_force(h->s, h->lc, 1, h->st);
        mark(h, 3);
      }
    }
    CUDA_TRY(h, cudaGetLastError());
    bool resumed = false;
    rc = recover(h, &resumed);
    if (rc) return rc;
    if (resumed) {
      // the halted step's rebuild is now finished; compute its forces and
      // continue after it (later queued kernels were no-ops)
      h->kt.kernel_launches += launch_pair(h->s, h->lc, 1, h->st);
      h->kt.kernel_launches += launch_wall_force(h->s, h->lc, 1, h->st);
      bool again = true;
      while (again) {
        rc = recover(h, &again);
        if (rc) return rc;
        if (again) {
          h->kt.kernel_launches += launch_pair(h->s, h->lc, 1, h->st);
          h->kt.kernel_launches += launch_wall_force(h->s, h->lc, 1, h->st);
        }
      }
      rc = read_ctrl(h);
      if (rc) return rc;
      done = h->host_ctrl.ntimestep - ts0;
    } else {
      done += chunk;
    }
  }
  mark_start(h);
  h->kt.kernel_launches += launch_particle(h->s, h->lc, kModeGatherFinal, 1, h->st);
  mark(h, 0);
  CUDA_TRY(h, cudaEventRecord(h->ev1, h->st));
  CUDA_TRY(h, cudaGetLastError());
  bool dummy;
  rc = recover(h, &dummy);
  if (rc) return rc;
  cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1);
  return DEM_OK;
}

int dem_get_diagnostics(dem_handle *h, const double *region_lo, const double *region_hi, dem_diagnostics *out) {
  if (!h || !out || !h->have_atoms || !h->setup_done) return DEM_ERR_BAD_ARG;
  const Sys &s = h->s;
  const int nw = s.nplanes + s.nmeshes;
  if (nw > DEM_DIAG_MAX_WALLS) return fail(h, DEM_ERR_BAD_ARG, "more walls than DEM_DIAG_MAX_WALLS");
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = region_lo ? region_lo[d] : s.boxlo[d];
    hi[d] = region_hi ? region_hi[d] : s.boxhi[d];
    if (!(hi[d] > lo[d])) return fail(h, DEM_ERR_BAD_ARG, "empty diagnostics region");
  }
  const int nb = 2 * 152;
  if (!h->diag_buf) {
    CUDA_TRY(h, cudaMalloc(&h->diag_buf, (size_t)(nb * 3 + nb * 3 * DEM_DIAG_MAX_WALLS + 1) * sizeof(double)));
  }
  double *pa = h->diag_buf, *pw = pa + nb * 3;
  unsigned long long *cnt = reinterpret_cast<unsigned long long *>(pw + nb * 3 * DEM_DIAG_MAX_WALLS);
  int rc = read_ctrl(h);
  if (rc) return rc;
  h->kt.kernel_launches += launch_diagnostics(s, h->lc, lo, hi, pa, pw, cnt, nb, h->st);
  CUDA_TRY(h, cudaGetLastError());
  std::vector<double> host((size_t)nb * 3 + (size_t)nb * 3 * DEM_DIAG_MAX_WALLS + 1);
  CUDA_TRY(h, cudaMemcpyAsync(host.data(), h->diag_buf, host.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  double ke = 0.0, er = 0.0, vol = 0.0;
  for (int b = 0; b < nb; b++) {
    ke += host[3 * b];
    er += host[3 * b + 1];
    vol += host[3 * b + 2];
  }
  std::memset(out, 0, sizeof(*out));
  out->ke_translational = 0.5 * ke;          // ComputeKE: scalar *= 0.5 * mvv2e
  out->ke_rotational = 0.5 * 0.4 * er;       // ComputeERotateSphere: scalar *= 0.5 * INERTIA * mvv2e
  out->solid_volume = 4.0 * M_PI / 3.0 * vol;
  out->packing_fraction = out->solid_volume / ((hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]));
  out->nwalls = nw;
  for (int w = 0; w < nw; w++)
    for (int d = 0; d < 3; d++) {
      double acc = 0.0;
      for (int b = 0; b < nb; b++) acc += host[(size_t)nb * 3 + ((size_t)b * nw + w) * 3 + d];
      out->wall_force[w][d] = acc;
    }
  unsigned long long nc = 0;
  std::memcpy(&nc, &host[host.size() - 1], sizeof(nc));
  out->ncontacts = (long long)nc;
  return DEM_OK;
}

int dem_natoms(dem_handle *h, int *n) {
  if (!h || !n) return DEM_ERR_BAD_ARG;
  int rc = read_ctrl(h);
  if (rc) return rc;
  *n = h->host_ctrl.n;
  return DEM_OK;
}

int dem_download_atoms(dem_handle *h, int *tag, int *type, double *x, double *v, double *omega,
                       double *f, double *torque, double *radius, double *rmass) {
  if (!h || !h->have_atoms) return DEM_ERR_BAD_ARG;
  int rc = read_ctrl(h);
  if (rc) return rc;
  const int n = h->host_ctrl.n;
  if (n <= 0) return DEM_OK;
  AtomsOut out{tag, type, x, v, omega, f, torque, radius, rmass};
  if (h->host_direct) {  // the kernel writes the caller's arrays
    h->kt.kernel_launches += launch_download_atoms(h->s, out, n, h->st);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    return DEM_OK;
  }
  const size_t nd = (size_t)n * sizeof(double), ni = (size_t)n * sizeof(int);
  rc = ensure_stage(h, 17 * nd + 2 * ni);
  if (rc) return rc;
  double *p = static_cast<double *>(h->stage);
  AtomsOut dv{};
  double *vec[5] = {x, v, omega, f, torque};
  double **dvec[5] = {&dv.x, &dv.v, &dv.w, &dv.f, &dv.t};
  for (int k = 0; k < 5; k++)
    if (vec[k]) *dvec[k] = p + (size_t)3 * n * k;
  if (radius) dv.r = p + (size_t)15 * n;
  if (rmass) dv.m = p + (size_t)16 * n;
  int *ip = reinterpret_cast<int *>(p + (size_t)17 * n);
  if (tag) dv.tag = ip;
  if (type) dv.type = ip + n;
  h->kt.kernel_launches += launch_download_atoms(h->s, dv, n, h->st);
  CUDA_TRY(h, cudaGetLastError());
  for (int k = 0; k < 5; k++)
    if (vec[k]) CUDA_TRY(h, cudaMemcpyAsync(vec[k], *dvec[k], 3 * nd, cudaMemcpyDeviceToHost, h->st));
  if (radius) CUDA_TRY(h, cudaMemcpyAsync(radius, dv.r, nd, cudaMemcpyDeviceToHost, h->st));
  if (rmass) CUDA_TRY(h, cudaMemcpyAsync(rmass, dv.m, nd, cudaMemcpyDeviceToHost, h->st));
  if (tag) CUDA_TRY(h, cudaMemcpyAsync(tag, dv.tag, ni, cudaMemcpyDeviceToHost, h->st));
  if (type) CUDA_TRY(h, cudaMemcpyAsync(type, dv.type, ni, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  return DEM_OK;
}

int dem_npairs(dem_handle *h, int *npairs, int *dnum) {
  if (!h) return DEM_ERR_BAD_ARG;
  int rc = read_ctrl(h);
  if (rc) return rc;
  // ensembles: the entries in use (the segments' unused entries are not part
  // of the list)
  if (npairs) *npairs = h->s.nsys ? h->host_ctrl.np_live : h->host_ctrl.np;
  if (dnum) *dnum = h->s.dnum;
  return DEM_OK;
}

int dem_download_contacts(dem_handle *h, int *tag_i, int *tag_j, int *shift, int *flag, double *hist) {
  if (!h || !h->have_atoms) return DEM_ERR_BAD_ARG;
  int rc = read_ctrl(h);
  if (rc) return rc;
  const int n = h->host_ctrl.n, np = h->host_ctrl.np;
  const PairArrays &L = h->s.pairs[0];
  std::vector<int> pi(np), pj(np), tags(n), fl(np), li(n);
  std::vector<uint8_t> sh(np);
  if (np) {
    CUDA_TRY(h, cudaMemcpyAsync(pi.data(), L.i, np * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(pj.data(), L.j, np * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(sh.data(), L.sh, np, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(fl.data(), L.flag, np * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  }
  CUDA_TRY(h, cudaMemcpyAsync(tags.data(), h->s.atoms[0].tag, n * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaMemcpyAsync(li.data(), h->s.atoms[0].lidx, n * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  // pairs of two owned atoms are returned as the reference holds them: owned
  // by the atom that comes first in the caller's local order (shear negated
  // when the list holds the other orientation; bond values are kept in that
  // orientation already)
  std::vector<char> swap(np, 0);
  for (int p = 0; p < np; p++) {
    if (sh[p] == kNoShift && li[pi[p]] > li[pj[p]]) {
      swap[p] = 1;
      std::swap(pi[p], pj[p]);
    }
  }
  // output slot of each entry: ensembles skip their segments' unused entries
  std::vector<int> slot(np);
  int nout = 0;
  for (int p = 0; p < np; p++) slot[p] = sh[p] == kHole ? -1 : nout++;
  for (int p = 0; p < np; p++) {
    const int o = slot[p];
    if (o < 0) continue;
    if (tag_i) tag_i[o] = tags[pi[p]];
    if (tag_j) tag_j[o] = tags[pj[p]];
    if (shift) {
      const int c = sh[p];
      shift[3 * o] = c % 3 - 1;
      shift[3 * o + 1] = (c / 3) % 3 - 1;
      shift[3 * o + 2] = c / 9 - 1;
    }
    if (flag) flag[o] = fl[p];
  }
  if (hist && np) {
    std::vector<double> hb(np);
    const int dnum = h->s.dnum;
    for (int r = 0; r < dnum; r++) {
      const int d = dev_hist_index(h->s, r);
      CUDA_TRY(h, cudaMemcpyAsync(hb.data(), L.hist + (size_t)d * h->s.pcap, np * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->st));
      CUDA_TRY(h, cudaStreamSynchronize(h->st));
      for (int p = 0; p < np; p++)
        if (slot[p] >= 0) hist[(size_t)slot[p] * dnum + r] = (swap[p] && d < kDnumShear) ? -hb[p] : hb[p];
    }
  }
  return DEM_OK;
}

int dem_download_wall_history(dem_handle *h, int wall_id, double *hist) {
  if (!h || !h->have_atoms || !hist || wall_id < 0 || wall_id >= h->s.nplanes) return DEM_ERR_BAD_ARG;
  int rc = read_ctrl(h);
  if (rc) return rc;
  const int n = h->host_ctrl.n;
  std::vector<double> hb(n);
  for (int d = 0; d < 3; d++) {
    CUDA_TRY(h, cudaMemcpyAsync(hb.data(), h->s.atoms[0].whist + (size_t)(wall_id * 3 + d) * h->s.nmax,
                                n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    for (int i = 0; i < n; i++) hist[3 * (size_t)i + d] = hb[i];
  }
  return DEM_OK;
}

int dem_get_stats(dem_handle *h, dem_stats *out) {
  if (!h || !out) return DEM_ERR_BAD_ARG;
  int rc = read_ctrl(h);
  if (rc) return rc;
  const Ctrl &c = h->host_ctrl;
  out->ntimestep = c.ntimestep;
  out->nrebuilds = c.nrebuilds;
  out->npairs = h->s.nsys ? c.np_live : c.np;
  out->nlost = c.lost;
  out->natoms = c.n;
  out->device = h->device;
  out->pair_capacity = h->s.pcap;
  out->last_step_ms = h->last_ms;
  out->host_direct = h->host_direct ? 1 : 0;
  out->ens_inplace_builds = c.ens_inplace;
  out->ens_relayout_builds = c.ens_relayout;
  out->mesh_slot_capacity = 0;
  for (int k = 0; k < h->s.nmeshes; k++) out->mesh_slot_capacity = std::max(out->mesh_slot_capacity, h->s.meshes[k].ccap);
  return DEM_OK;
}

int dem_profile(dem_handle *h, int enable) {
  if (!h) return DEM_ERR_BAD_ARG;
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  harvest(h);
  h->kt = dem_kernel_times{};
  h->profile = enable != 0;
  if (h->profile && h->evpool.empty()) {
    const int nev = 4 * kCheckEvery + 8;
    h->evpool.resize(nev);
    h->evkind.resize(nev);
    for (auto &e : h->evpool) CUDA_TRY(h, cudaEventCreate(&e));
  }
  h->evused = 0;
  return DEM_OK;
}

int dem_get_kernel_times(dem_handle *h, dem_kernel_times *out) {
  if (!h || !out) return DEM_ERR_BAD_ARG;
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  harvest(h);
  *out = h->kt;
  return DEM_OK;
}

const char *dem_last_error(dem_handle *h) { return h ? h->err.c_str() : "null handle"; }

}  // extern "C"
