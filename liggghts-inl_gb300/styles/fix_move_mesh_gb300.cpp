/* fix move/mesh/gb300: see fix_move_mesh_gb300.h. */

#include "fix_move_mesh_gb300.h"

#include <stdlib.h>
#include <string.h>

#include "error.h"

using namespace LAMMPS_NS;

/* arguments as FixMoveMesh parses them (src/fix_move_mesh.cpp:70-100):
   fix ID group move/mesh mesh MESH_ID linear VX VY VZ */
FixMoveMeshGB300::FixMoveMeshGB300(LAMMPS *lmp, int narg, char **arg) : FixMoveMesh(lmp, narg, arg) {
  if (narg < 9 || strcmp(arg[3], "mesh") != 0 || strcmp(arg[5], "linear") != 0)
    error->all(FLERR, "fix move/mesh/gb300 supports 'mesh ID linear vx vy vz' only");
  mesh_id_ = arg[4];
  for (int d = 0; d < 3; d++) vel_[d] = atof(arg[6 + d]);
}
