/* fix gravity/gb300: FixGravity (src/fix_gravity.cpp) applied on the GPU
   inside the device-resident timestep of run_style verlet/gb300 (f += m g
   in the per-atom kernel).  Selected by the suffix mechanism
   (src/modify.cpp:833-848).  Constant gravity on group all; the
   acceleration handed to the device is FixGravity::get_gravity
   (magnitude times direction).  Under verlet/gb300 post_force() adds
   nothing on the host; without it the fix stops with an error. */

#ifdef FIX_CLASS

FixStyle(gravity/gb300,FixGravityGB300)

#else

#ifndef LMP_FIX_GRAVITY_GB300_H
#define LMP_FIX_GRAVITY_GB300_H

#include "fix_gravity.h"

namespace LAMMPS_NS {

class FixGravityGB300 : public FixGravity {
 public:
  FixGravityGB300(class LAMMPS *, int, char **);
  virtual ~FixGravityGB300() {}
  virtual void post_force(int);
  /* the acceleration vector for dem_config.gravity; errors on variable
     gravity or a group other than all */
  void acceleration(double *acc);
};

}

#endif
#endif
