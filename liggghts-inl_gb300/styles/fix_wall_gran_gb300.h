/* fix wall/gran/gb300: the granular wall fix of the reference (FixWallGran,
   src/fix_wall_gran.h) whose contacts are computed on the GPU inside the
   device-resident timestep of run_style verlet/gb300.

   Selected by the suffix mechanism: Modify::add_fix tries "wall/gran/gb300"
   before "wall/gran" (src/modify.cpp:833-848) and passes the same
   arguments, which the reference's constructor parses as always.  This
   class records what the device needs from them: primitive planes
   ("primitive type T xplane|yplane|zplane POS") or the mesh list
   ("mesh n_meshes N meshes ID ..."), and the wall's contact model, which
   must be hertz/hooke with tangential history and rolling_friction off|cdt.

   Under verlet/gb300 post_force() adds nothing on the host (the device's
   per-atom totals already contain the wall forces); without it the fix
   stops with an error. */

#ifdef FIX_CLASS

FixStyle(wall/gran/gb300,FixWallGranGB300)

#else

#ifndef LMP_FIX_WALL_GRAN_GB300_H
#define LMP_FIX_WALL_GRAN_GB300_H

#include "fix_wall_gran.h"
#include "liggghts_gb300.h"

#include <string>
#include <vector>

namespace LAMMPS_NS {

class FixWallGranGB300 : public FixWallGran {
 public:
  FixWallGranGB300(class LAMMPS *, int, char **);
  virtual ~FixWallGranGB300() {}

  virtual void post_force(int vflag);

  /* adds this fix's walls to the device handle; wall ids are recorded */
  void upload(dem_handle *h, int ntypes);
  /* primitive-wall history of local atom i (3 doubles), as restart data */
  bool primitive_history(int i, double *h3) const;
  bool is_primitive() const { return primitive_; }
  int device_wall_id() const { return device_wall_id_; }
  const std::vector<int> &device_mesh_ids() const { return device_mesh_ids_; }
  const std::vector<std::string> &mesh_ids() const { return mesh_ids_; }

 private:
  bool primitive_;
  bool cylinder_;   // primitive {x,y,z}cylinder R C1 C2 (else a plane)
  int axis_;
  double pos_;      // plane position, or cylinder radius
  double c1_, c2_;  // cylinder centre along (axis+1)%3, (axis+2)%3
  int wall_type_;
  int rolling_;
  std::vector<std::string> mesh_ids_;
  int device_wall_id_;
  std::vector<int> device_mesh_ids_;
};

}

#endif
#endif
