/* fix move/mesh/gb300: see fix_move_mesh_gb300.h. */

#include "fix_move_mesh_gb300.h"

#include <stdlib.h>
#include <string.h>

#include "error.h"

using namespace LAMMPS_NS;

/* arguments as FixMoveMesh parses them (src/fix_move_mesh.cpp:70-100):
   fix ID group move/mesh mesh MESH_ID linear VX VY VZ
   fix ID group move/mesh mesh MESH_ID rotate origin OX OY OZ axis AX AY AZ period T */
FixMoveMeshGB300::FixMoveMeshGB300(LAMMPS *lmp, int narg, char **arg)
    : FixMoveMesh(lmp, narg, arg), rotating_(false), period_(0.0) {
  for (int d = 0; d < 3; d++) vel_[d] = origin_[d] = axis_[d] = 0.0;
  if (narg >= 9 && strcmp(arg[3], "mesh") == 0 && strcmp(arg[5], "linear") == 0) {
    for (int d = 0; d < 3; d++) vel_[d] = atof(arg[6 + d]);
  } else if (narg >= 16 && strcmp(arg[3], "mesh") == 0 && strcmp(arg[5], "rotate") == 0 &&
             strcmp(arg[6], "origin") == 0 && strcmp(arg[10], "axis") == 0 && strcmp(arg[14], "period") == 0) {
    rotating_ = true;
    for (int d = 0; d < 3; d++) {
      origin_[d] = atof(arg[7 + d]);
      axis_[d] = atof(arg[11 + d]);
    }
    period_ = atof(arg[15]);
  } else {
    error->all(FLERR, "fix move/mesh/gb300 supports 'linear vx vy vz' and "
                      "'rotate origin ox oy oz axis ax ay az period T'");
  }
  mesh_id_ = arg[4];
}
