/* fix move/mesh/gb300: FixMoveMesh with MeshMoverLinear
   (src/fix_move_mesh.cpp, src/mesh_mover_linear.cpp) carried out on the GPU
   inside the device-resident timestep of run_style verlet/gb300 (nodes move
   by dt*vel after the particles' drift; the wall velocity seen by contacts
   is vel).  Selected by the suffix mechanism (src/modify.cpp:833-848).
   Supported: "move/mesh mesh ID linear VX VY VZ" and "move/mesh mesh ID
   rotate origin OX OY OZ axis AX AY AZ period T" (MeshMoverRotate,
   src/mesh_mover_rotation.cpp); the host mesh is brought up to date from
   the device at output steps. */

#ifdef FIX_CLASS

FixStyle(move/mesh/gb300,FixMoveMeshGB300)

#else

#ifndef LMP_FIX_MOVE_MESH_GB300_H
#define LMP_FIX_MOVE_MESH_GB300_H

#include "fix_move_mesh.h"

#include <string>

namespace LAMMPS_NS {

class FixMoveMeshGB300 : public FixMoveMesh {
 public:
  FixMoveMeshGB300(class LAMMPS *, int, char **);
  virtual ~FixMoveMeshGB300() {}
  const std::string &mesh_id() const { return mesh_id_; }
  bool rotating() const { return rotating_; }
  const double *velocity() const { return vel_; }
  const double *origin() const { return origin_; }
  const double *axis() const { return axis_; }
  double period() const { return period_; }

 private:
  std::string mesh_id_;
  bool rotating_;
  double vel_[3], origin_[3], axis_[3], period_;
};

}

#endif
#endif
