/* fix nve/sphere/gb300: FixNVESphere (src/fix_nve_sphere.cpp) integrated on
   the GPU inside the device-resident timestep of run_style verlet/gb300
   (the C ABI's dem_step runs both half-kicks and the drift).  Selected by
   the suffix mechanism (src/modify.cpp:833-848).  The fix must act on all
   atoms (group all) without the reference's added-mass (CAddRhoFluid) or
   disc options; under verlet/gb300 its host hooks do nothing, without it
   the fix stops with an error. */

#ifdef FIX_CLASS

FixStyle(nve/sphere/gb300,FixNVESphereGB300)

#else

#ifndef LMP_FIX_NVE_SPHERE_GB300_H
#define LMP_FIX_NVE_SPHERE_GB300_H

#include "fix_nve_sphere.h"

namespace LAMMPS_NS {

class FixNVESphereGB300 : public FixNVESphere {
 public:
  FixNVESphereGB300(class LAMMPS *, int, char **);
  virtual ~FixNVESphereGB300() {}
  virtual void init();
  virtual void initial_integrate(int);
  virtual void final_integrate();
};

}

#endif
#endif
