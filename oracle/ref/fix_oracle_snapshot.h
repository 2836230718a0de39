/* Test infrastructure only: a LIGGGHTS fix that is compiled together with the
 * unmodified reference sources (never shipped, never part of the GPU product).
 *
 * fix ID group oracle/snapshot PREFIX STEP [STEP ...]
 *
 * At the listed time steps it writes one little-endian binary file
 * PREFIX.STEP.bin holding the per-atom state (local and ghost), the granular
 * half neighbour list with its contact flags and history doubles, and every
 * per-atom wall history (fix property/atom "history_<wall-fix-id>").  Step 0
 * is written from setup(), i.e. after Verlet::setup() computed the setup
 * forces (src/verlet.cpp setup(), src/pair_gran.cpp:633-635).  Other steps are
 * written from end_of_step(), i.e. after FixNVESphere::final_integrate
 * (src/fix_nve_sphere.cpp:205-244).
 */
#ifdef FIX_CLASS

FixStyle(oracle/snapshot,FixOracleSnapshot)

#else

#ifndef LMP_FIX_ORACLE_SNAPSHOT_H
#define LMP_FIX_ORACLE_SNAPSHOT_H

#include "fix.h"
#include <vector>
#include <string>

namespace LAMMPS_NS {

class FixOracleSnapshot : public Fix {
 public:
  FixOracleSnapshot(class LAMMPS *, int, char **);
  int setmask();
  void setup(int);
  void end_of_step();

 private:
  std::string prefix_;
  std::vector<long> steps_;
  void write_snapshot();
};

}

#endif
#endif
