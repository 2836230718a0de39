/* run_style verlet/gb300: the Verlet timestep loop of the reference
   (Verlet::setup / Verlet::run, src/verlet.cpp:134-389) resident on the
   GPU through the GB300 library's C ABI (include/liggghts_gb300.h).

   Selected by the suffix mechanism: Update::create_integrate tries
   "verlet/gb300" before "verlet" (src/update.cpp:342-377), so input scripts
   stay unchanged when LIGGGHTS runs with "-sf gb300".

   setup(): uploads the host state (atoms, material tables, walls, meshes,
   mesh motion, gravity, neighbour settings, contact history when the host
   holds any) unless the device still holds the state the previous run left
   and nobody changed the host copy since; runs the device's setup force
   pass (dem_setup: rebuild + forces without history update); then runs the
   reference's own Verlet::setup for the host bookkeeping, during which
   pair gran/gb300 writes the device forces into atom->f.
   run(n): advances the device in one dem_step call per stretch between
   output steps, then downloads x, v, omega, f, torque (and deletes host
   atoms the device lost through a non-periodic boundary), refreshes moving
   meshes and calls Output::write, so thermo, dump and restart output see
   the device state at their steps.

   Insertion fixes (insert/pack, insert/stream, ...: FixInsert) run on the
   host at their insertion steps; the run stops one step before, lets the
   fix insert, and hands the new atoms to the device (dem_insert_atoms),
   which adds them at the insertion step after its initial integration.
   "run_style verlet/gb300 capacity N" reserves device room for N atoms.

   Scope (checked in init): one MPI rank, orthogonal box, atom map, pair
   gran/gb300, exactly one nve/sphere/gb300, any number of
   wall/gran/gb300, gravity/gb300, move/mesh/gb300 (linear, rotate),
   insertion fixes, mesh/surface and data-only fixes.  A fix that would run on the host every step is
   rejected by name: it would silently not run between output steps. */

#ifdef INTEGRATE_CLASS

IntegrateStyle(verlet/gb300,VerletGB300)

#else

#ifndef LMP_VERLET_GB300_H
#define LMP_VERLET_GB300_H

#include "verlet.h"
#include "liggghts_gb300.h"

#include <stdint.h>
#include <vector>

namespace LAMMPS_NS {

class VerletGB300 : public Verlet {
 public:
  VerletGB300(class LAMMPS *, int, char **);
  virtual ~VerletGB300();
  virtual void init();
  virtual void setup();
  virtual void setup_minimal(int);
  virtual void run(int);
  virtual void cleanup();

  /* adds the forces and torques of the last download to atom->f/torque of
     the local atoms (pair gran/gb300's compute_force) */
  void add_device_forces();
  dem_handle *handle() const { return h_; }

 private:
  dem_handle *h_;
  class PairGranGB300 *pair_;
  std::vector<class FixWallGranGB300 *> walls_;
  std::vector<class FixMoveMeshGB300 *> movers_;
  std::vector<class FixInsert *> inserts_;
  long capacity_;
  class FixGravityGB300 *gravity_;
  class FixNVESphereGB300 *nve_;
  bigint natoms_;
  uint64_t stamp_;

  // last download, in device order
  std::vector<int> tag_, type_, row_of_tag_;
  std::vector<double> x_, v_, w_, f_, t_, r_, m_;

  void check(int rc, const char *what);
  void collect_styles();
  void create_device();
  void download();
  void sync_meshes(int nsteps);
  void insert_due(bigint step);
  uint64_t host_stamp() const;
};

}

#endif
#endif
