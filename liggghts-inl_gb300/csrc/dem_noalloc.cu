// dem_contact_forces_noalloc: one evaluation of the sphere contact forces for
// a caller-supplied neighbour list, with no device allocation at all.
//
// Who needs it: callers that cannot call cudaMalloc while they run — a host
// code whose GPU memory is owned by another allocator (a fixed arena, a
// framework's pool that must see every byte), or real-time / embedded loops
// that must not allocate after start-up.  They pass device pointers to their
// own input and output buffers; the scratch the evaluation needs (per-pair
// results for the deterministic reduction, row and partner indices, the
// material table) lives in one file-scope static device array of fixed size
// that every GPU which loads this library keeps until the process exits.
//
// Limits: at most kNaMaxAtoms atoms, kNaMaxPairs list entries, kNaMaxTypes
// atom types; larger inputs are rejected with DEM_ERR_BAD_ARG.  Every call
// shares the one scratch array: calls that overlap on the GPU (two streams,
// two host threads) race and must be serialised by the caller.  Each call
// clears what it accumulates before use, so results never depend on the
// previous call.
//
// When the array is taken: CUDA loads a module's device code and its static
// arrays lazily by default (CUDA_MODULE_LOADING=LAZY), i.e. on the first
// call on each device, which therefore takes the ~11 MB then.  A caller that
// must not see that happen mid-run makes one call at start-up (any valid
// input, npairs = 0 is enough) or runs with CUDA_MODULE_LOADING=EAGER; later
// calls take no device memory.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/liggghts_gb300.h"
#include "contact_law.cuh"

namespace {

using namespace gb300;

constexpr int kNaMaxAtoms = 32768;
constexpr int kNaMaxPairs = 131072;
constexpr int kNaMaxTypes = 15;
constexpr int kNaParams = kTypeTables * (kNaMaxTypes + 1) * (kNaMaxTypes + 1);

// byte offsets of the sub-arrays inside the scratch array (256-byte aligned)
constexpr size_t al(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffRes = 0;                                              // double[9][kNaMaxPairs]
constexpr size_t kOffParams = kOffRes + al(sizeof(double) * 9 * kNaMaxPairs);  // double[kNaParams]
constexpr size_t kOffRow = kOffParams + al(sizeof(double) * kNaParams);    // int[kNaMaxAtoms+1]
constexpr size_t kOffRevStart = kOffRow + al(sizeof(int) * (kNaMaxAtoms + 1));
constexpr size_t kOffRevFill = kOffRevStart + al(sizeof(int) * (kNaMaxAtoms + 1));
constexpr size_t kOffRev = kOffRevFill + al(sizeof(int) * (kNaMaxAtoms + 1));  // int[kNaMaxPairs]
constexpr size_t kOffActive = kOffRev + al(sizeof(int) * kNaMaxPairs);      // uint8[kNaMaxPairs]
constexpr size_t kOffFlag = kOffActive + al(kNaMaxPairs);                   // int error flag
constexpr size_t kScratchBytes = kOffFlag + 256;                            // ~10.8 MB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct NaArgs {
  int n, np, ntypes, normal, rolling, tdamp, limitf;
  double prd[3], charVel;
  const double *x, *v, *omega, *radius, *rmass;
  const int *type, *pi, *pj, *shift;
  const double *hist;
  double *f, *torque;
  unsigned char *base;  // device address of g_noalloc_scratch
};

__device__ __forceinline__ double *na_res(const NaArgs &a, int k) {
  return reinterpret_cast<double *>(a.base + kOffRes) + (size_t)k * kNaMaxPairs;
}
__device__ __forceinline__ int *na_int(const NaArgs &a, size_t off) {
  return reinterpret_cast<int *>(a.base + off);
}

__global__ void na_clear(NaArgs a) {
  int *row = na_int(a, kOffRow), *rs = na_int(a, kOffRevStart), *rf = na_int(a, kOffRevFill);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= a.n; i += gridDim.x * blockDim.x) {
    row[i] = 0;
    rs[i] = 0;
    rf[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *na_int(a, kOffFlag) = 0;
}

// per-pair contact (history read, not updated: the setup force pass)
template <int NORMAL>
__global__ void na_pairs(NaArgs a) {
  int *row = na_int(a, kOffRow), *rs = na_int(a, kOffRevStart);
  unsigned char *active = a.base + kOffActive;
  const double *params = reinterpret_cast<const double *>(a.base + kOffParams);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.np; p += gridDim.x * blockDim.x) {
    const int i = a.pi[p], j = a.pj[p];
    const int sx = a.shift[3 * p], sy = a.shift[3 * p + 1], sz = a.shift[3 * p + 2];
    if (i < 0 || i >= a.n || j < 0 || j >= a.n || (p > 0 && a.pi[p - 1] > i) || (i == j && !sx && !sy && !sz)) {
      atomicExch(na_int(a, kOffFlag), 1);  // out of range, not sorted by owner, or an atom with itself
      active[p] = 0;
      continue;
    }
    double xj = a.x[3 * j], yj = a.x[3 * j + 1], zj = a.x[3 * j + 2];
    if (sx) xj = __dadd_rn(xj, sx > 0 ? a.prd[0] : -a.prd[0]);  // +-prd by selection, as the
    if (sy) yj = __dadd_rn(yj, sy > 0 ? a.prd[1] : -a.prd[1]);  // resident path's image()
    if (sz) zj = __dadd_rn(zj, sz > 0 ? a.prd[2] : -a.prd[2]);
    const double delx = __dadd_rn(a.x[3 * i], -xj);
    const double dely = __dadd_rn(a.x[3 * i + 1], -yj);
    const double delz = __dadd_rn(a.x[3 * i + 2], -zj);
    const double rsq = __dadd_rn(__dadd_rn(__dmul_rn(delx, delx), __dmul_rn(dely, dely)), __dmul_rn(delz, delz));
    atomicAdd(&row[i], 1);
    if (!sx && !sy && !sz) atomicAdd(&rs[j], 1);
    const double radi = a.radius[i], radj = a.radius[j];
    const double radsum = __dadd_rn(radi, radj);
    if (!(rsq < __dmul_rn(radsum, radsum))) {
      active[p] = 0;
      continue;
    }
    const int it = a.type[i], jt = a.type[j];
    if (it < 1 || it > a.ntypes || jt < 1 || jt > a.ntypes) {
      atomicExch(na_int(a, kOffFlag), 1);
      active[p] = 0;
      continue;
    }
    const TypePair tp = load_typepair(params, a.ntypes, it, jt);
    const double mi = a.rmass[i], mj = a.rmass[j];
    ContactIn ci;
    ci.radi = radi;
    ci.radj = radj;
    ci.radsum = radsum;
    ci.r = sqrt(rsq);
    ci.rinv = rsqrt(rsq);
    ci.reff = radi * radj / (radi + radj);
    contact_consts<NORMAL>(tp, mi * mj / (mi + mj), ci.reff, a.charVel, a.tdamp, ci.c0, ci.c1);
    ci.d[0] = delx;
    ci.d[1] = dely;
    ci.d[2] = delz;
    ci.en[0] = delx * ci.rinv;
    ci.en[1] = dely * ci.rinv;
    ci.en[2] = delz * ci.rinv;
    for (int d = 0; d < 3; d++) {
      ci.vr[d] = a.v[3 * i + d] - a.v[3 * j + d];
      ci.wi[d] = a.omega[3 * i + d];
      ci.wj[d] = a.omega[3 * j + d];
    }
    ci.deltan_wall = 0.0;
    double sh3[3] = {a.hist[3 * p], a.hist[3 * p + 1], a.hist[3 * p + 2]};
    ContactOut o;
    contact_law<NORMAL, false>(ci, tp, 0.0, a.tdamp, a.limitf, a.rolling != 0, false, sh3, o);
    for (int d = 0; d < 3; d++) {
      na_res(a, d)[p] = o.F[d];
      na_res(a, 3 + d)[p] = o.Ti[d];
      na_res(a, 6 + d)[p] = o.Tj[d];
    }
    active[p] = 1;
  }
}

// single-block exclusive scan of len <= kNaMaxAtoms+1 ints, in place
__global__ void __launch_bounds__(1024) na_scan(int *v, int len) {
  __shared__ int part[1024];
  const int t = threadIdx.x;
  const int per = (len + 1023) / 1024;
  const int b = t * per, e = min(len, b + per);
  int s = 0;
  for (int k = b; k < e; k++) s += v[k];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // Hillis-Steele on the partial sums
    const int y = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += y;
    __syncthreads();
  }
  int run = part[t] - s;
  for (int k = b; k < e; k++) {
    const int c = v[k];
    v[k] = run;
    run += c;
  }
}

__global__ void na_rev_fill(NaArgs a) {
  const int *rs = na_int(a, kOffRevStart);
  int *rf = na_int(a, kOffRevFill), *rev = na_int(a, kOffRev);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.np; p += gridDim.x * blockDim.x) {
    const int j = a.pj[p];
    if (j < 0 || j >= a.n) continue;
    if (a.shift[3 * p] || a.shift[3 * p + 1] || a.shift[3 * p + 2]) continue;
    rev[rs[j] + atomicAdd(&rf[j], 1)] = p;
  }
}

// per atom: canonical partner order, then the force sum in the order of the
// resident path (own entries ascending, then partner entries ascending)
__global__ void na_gather(NaArgs a) {
  const int *row = na_int(a, kOffRow), *rs = na_int(a, kOffRevStart);
  int *rev = na_int(a, kOffRev);
  const unsigned char *active = a.base + kOffActive;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    const int b = rs[i], e = rs[i + 1];
    for (int k = b + 1; k < e; k++) {
      const int v = rev[k];
      int m = k - 1;
      while (m >= b && rev[m] > v) {
        rev[m + 1] = rev[m];
        m--;
      }
      rev[m + 1] = v;
    }
    double F[3] = {0., 0., 0.}, T[3] = {0., 0., 0.};
    for (int p = row[i]; p < row[i + 1]; p++) {
      if (!active[p]) continue;
      for (int d = 0; d < 3; d++) {
        F[d] += na_res(a, d)[p];
        T[d] += na_res(a, 3 + d)[p];
      }
    }
    for (int k = b; k < e; k++) {
      const int p = rev[k];
      if (!active[p]) continue;
      for (int d = 0; d < 3; d++) {
        F[d] -= na_res(a, d)[p];
        T[d] += na_res(a, 6 + d)[p];
      }
    }
    for (int d = 0; d < 3; d++) {
      a.f[3 * i + d] = F[d];
      a.torque[3 * i + d] = T[d];
    }
  }
}

// Device address of the scratch array on the current device.  The name
// g_noalloc_scratch in host code is only a stand-in for the symbol, not an
// address; the lookup is repeated on every call (cheap once the module is
// loaded), so a device reset or a new context never leaves a stale address.
int scratch_address(unsigned char **out) {
  void *ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return DEM_ERR_CUDA;
  *out = static_cast<unsigned char *>(ptr);
  return DEM_OK;
}

}  // namespace

extern "C" int dem_contact_forces_noalloc(int n, const double *x, const double *v,
                                          const double *omega, const double *radius,
                                          const double *rmass, const int *type, int npairs,
                                          const int *pair_i, const int *pair_j,
                                          const int *shift, const double *hist,
                                          const dem_config *cfg, int ntypes, const double *Yeff,
                                          const double *Geff, const double *betaeff,
                                          const double *coeffFrict, const double *coeffRollFrict,
                                          const double *coeffRestLog, double charVel,
                                          double *f, double *torque, void *stream) {
  if (n < 1 || n > kNaMaxAtoms || npairs < 0 || npairs > kNaMaxPairs || ntypes < 1 ||
      ntypes > kNaMaxTypes || !cfg || !x || !v || !omega || !radius || !rmass || !type || !f ||
      !torque || !Yeff || !Geff || !coeffFrict || (npairs > 0 && (!pair_i || !pair_j || !shift || !hist)))
    return DEM_ERR_BAD_ARG;
  if (cfg->normal_model == DEM_NORMAL_HERTZ && !betaeff) return DEM_ERR_BAD_ARG;
  if (cfg->normal_model == DEM_NORMAL_HOOKE && !coeffRestLog) return DEM_ERR_BAD_ARG;
  if (cfg->normal_model != DEM_NORMAL_HERTZ && cfg->normal_model != DEM_NORMAL_HOOKE) return DEM_ERR_UNSUPPORTED;
  if (cfg->cohesion_model != DEM_COHESION_OFF) return DEM_ERR_UNSUPPORTED;  // 3 history values per pair
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEM_ERR_NO_DEVICE;
  // an error left by earlier, unrelated work is not this call's
  (void)cudaGetLastError();
  unsigned char *base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // material table into the scratch (host -> device copy, no allocation)
  double tab[kNaParams];
  const int m = (ntypes + 1) * (ntypes + 1);
  const double *src[6] = {Yeff, Geff, betaeff, coeffFrict, coeffRollFrict, coeffRestLog};
  for (int k = 0; k < 6; k++)
    for (int q = 0; q < m; q++) tab[k * m + q] = src[k] ? src[k][q] : 0.0;
  derive_type_tables(m, tab);
  if (cudaMemcpyAsync(base + kOffParams, tab, sizeof(double) * kTypeTables * m, cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return DEM_ERR_CUDA;
  NaArgs a;
  a.n = n;
  a.np = npairs;
  a.ntypes = ntypes;
  a.normal = cfg->normal_model;
  a.rolling = cfg->rolling_model == DEM_ROLLING_CDT;
  a.tdamp = cfg->tangential_damping;
  a.limitf = cfg->limit_force;
  for (int d = 0; d < 3; d++) a.prd[d] = cfg->boxhi[d] - cfg->boxlo[d];
  a.charVel = charVel;
  a.x = x; a.v = v; a.omega = omega; a.radius = radius; a.rmass = rmass; a.type = type;
  a.pi = pair_i; a.pj = pair_j; a.shift = shift; a.hist = hist;
  a.f = f; a.torque = torque;
  a.base = base;
  const int B = 256;
  const int gp = std::max(1, std::min(1216, (npairs + B - 1) / B));
  const int gn = std::max(1, std::min(1216, (n + 1 + B - 1) / B));
  na_clear<<<gn, B, 0, st>>>(a);
  if (a.normal == DEM_NORMAL_HERTZ) na_pairs<kHertz><<<gp, B, 0, st>>>(a);
  else na_pairs<kHooke><<<gp, B, 0, st>>>(a);
  na_scan<<<1, 1024, 0, st>>>(reinterpret_cast<int *>(base + kOffRow), n + 1);
  na_scan<<<1, 1024, 0, st>>>(reinterpret_cast<int *>(base + kOffRevStart), n + 1);
  na_rev_fill<<<gp, B, 0, st>>>(a);
  na_gather<<<gn, B, 0, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return DEM_ERR_CUDA;  // launches of this call
  int flag = 0;
  if (cudaMemcpyAsync(&flag, base + kOffFlag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return DEM_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return DEM_ERR_CUDA;
  return flag ? DEM_ERR_BAD_ARG : DEM_OK;
}
