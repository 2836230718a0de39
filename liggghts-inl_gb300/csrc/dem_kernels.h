// Host-side launchers of the sphere-DEM kernels (dem_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "dem_device.cuh"

namespace gb300 {

struct LaunchCfg {
  int max_grid;              // grid-stride kernels never launch more blocks of 256 than this
  int particle_threads = 256;  // threads per block of the per-particle kernel (64, 128, 256)
  int sms = 152;               // multiprocessors of the device
};

enum {
  kModeInitial = 0,             // nve/sphere initial_integrate only (first step of a call)
  kModeGather = 1,              // sum forces only (setup)
  kModeGatherFinal = 2,         // sum forces + final_integrate (last step of a call)
  kModeGatherFinalInitial = 3,  // sum forces + final(n) + initial(n+1) (steady state)
};

struct InsertStage {  // new atoms, device arrays: x, v, w [3k], the rest [k]
  const double *x, *v, *w, *r, *m, *dtfm, *dtir;
  const int *type, *tag;
};
int launch_insert_stage(const Sys &s, const InsertStage &in, int first, int k, int lidx0, cudaStream_t st);
// Atom transfer between the caller's per-atom AoS arrays (atom->x[i][d] as
// x[3*i+d]) and the device's SoA arrays.  The pointers are either the
// caller's host arrays (read and written by the kernels themselves where the
// device reaches pageable host memory through the host's page tables) or
// device staging copies of them.
struct AtomsIn {
  const int *tag, *type;
  const double *x, *v, *w, *r, *m;
};
struct AtomsOut {  // null members are skipped
  int *tag, *type;
  double *x, *v, *w, *f, *t, *r, *m;
};
struct UploadCheck {         // filled by k_upload_atoms (zero-initialise rmax, counts; rmin = ~0)
  unsigned long long rmin;   // bit pattern of the smallest positive radius
  unsigned long long rmax;   // bit pattern of the largest radius
  int bad_type;              // atoms with a type outside 1..ntypes
  int bad_value;             // atoms with radius or rmass not finite and > 0
  int nonfinite;             // atoms with a non-finite position, velocity or angular velocity
  int pad;
};
// SoA state of the first n atoms (buffer 0) from `in`, the nve/sphere
// per-atom constants dtf/m and dtfrotate/(r^2 m), caller-order indices, and
// cleared forces, holds, wall histories and mesh slots; `chk` collects the
// checks and the radius range.
int launch_upload_atoms(const Sys &s, const AtomsIn &in, int n, double dtf, double dtfrotate, UploadCheck *chk,
                        cudaStream_t st);
int launch_download_atoms(const Sys &s, const AtomsOut &out, int n, cudaStream_t st);
int launch_insert_commit(const Sys &s, int k, cudaStream_t st);
int launch_diagnostics(const Sys &s, const LaunchCfg &lc, const double lo[3], const double hi[3], double *part_atoms,
                       double *part_walls, unsigned long long *contacts, int nblocks, cudaStream_t st);
// exclusive prefix sum of len ints (len <= 4096*4096 - 1); tmp holds
// (len+4095)/4096 + 1 ints; gate 0: always; 1: only while the system
// rebuilds; 2: not in an ensemble rebuild that keeps other systems in place
int scan_exclusive(const Sys &s, const int *in, int *out, int len, int *tmp, int gate,
                   cudaStream_t st);
int launch_decide(const Sys &s, cudaStream_t st);
int launch_set_rebuild(const Sys &s, int v, cudaStream_t st);
// stage 0: full rebuild; stage 1: resume after a pair-capacity overflow;
// stage 2: resume after a mesh slot or registration overflow
int launch_rebuild(const Sys &s, const LaunchCfg &lc, cudaStream_t st, int stage);
int launch_pair(const Sys &s, const LaunchCfg &lc, int shearupdate, cudaStream_t st);
int launch_particle(const Sys &s, const LaunchCfg &lc, int mode, int shearupdate, cudaStream_t st);
int launch_set_loop(const Sys &s, int n, cudaStream_t st);
// wall (plane and mesh) forces of the current state, before the particle
// kernel that gathers the step's forces; none without walls
int launch_wall_force(const Sys &s, const LaunchCfg &lc, int shearupdate, cudaStream_t st);
// fix move/mesh: moves the moving meshes by one step (after the drift)
int launch_mesh_move(const Sys &s, const LaunchCfg &lc, cudaStream_t st);
// Executable graph of the steady-state step loop (WHILE node over steps, IF
// node around the rebuild); see dem_kernels.cu.
cudaError_t build_step_graph(const Sys &s, const LaunchCfg &lc, cudaStream_t st, cudaStream_t st2,
                             cudaGraphExec_t *exec, int *kernels_per_step, int *kernels_per_rebuild);

}  // namespace gb300
