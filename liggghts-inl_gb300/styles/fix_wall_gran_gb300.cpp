/* fix wall/gran/gb300: see fix_wall_gran_gb300.h. */

#include "fix_wall_gran_gb300.h"

#include <stdlib.h>
#include <string.h>

#include "atom.h"
#include "error.h"
#include "fix_mesh_surface.h"
#include "fix_property_atom.h"
#include "modify.h"
#include "tri_mesh.h"
#include "update.h"
#include "verlet_gb300.h"

using namespace LAMMPS_NS;

/* the reference's constructor parses and validates the arguments
   (src/fix_wall_gran.cpp:149-300); the keywords the device needs are read
   again here from the same argument list */
FixWallGranGB300::FixWallGranGB300(LAMMPS *lmp, int narg, char **arg)
    : FixWallGran(lmp, narg, arg), primitive_(false), cylinder_(false), axis_(-1), pos_(0.0), c1_(0.0), c2_(0.0),
      wall_type_(0),
      rolling_(DEM_ROLLING_OFF), device_wall_id_(-1) {
  for (int k = 3; k < narg; k++) {
    if (strcmp(arg[k], "primitive") == 0 && k + 4 < narg && strcmp(arg[k + 1], "type") == 0) {
      // primitive type T {x,y,z}plane P | {x,y,z}cylinder R C1 C2
      // (PRIMITIVE_WALL_DEFINITIONS::wallString/numArgs, src/primitive_wall_definitions.h:74-94)
      primitive_ = true;
      wall_type_ = atoi(arg[k + 2]);
      const char *ws = arg[k + 3];
      const char *names[] = {"xplane", "yplane", "zplane", "xcylinder", "ycylinder", "zcylinder"};
      int kind = -1;
      for (int q = 0; q < 6; q++)
        if (strcmp(ws, names[q]) == 0) kind = q;
      if (kind < 0) error->all(FLERR, "fix wall/gran/gb300: primitive walls must be planes or cylinders");
      axis_ = kind % 3;
      cylinder_ = kind >= 3;
      if (cylinder_ && k + 6 >= narg) error->all(FLERR, "fix wall/gran/gb300: a cylinder takes R C1 C2");
      pos_ = atof(arg[k + 4]);
      if (cylinder_) {
        c1_ = atof(arg[k + 5]);
        c2_ = atof(arg[k + 6]);
        k += 2;
      }
      k += 4;
    } else if (strcmp(arg[k], "meshes") == 0) {
      for (int q = k + 1; q < narg && modify->find_fix(arg[q]) >= 0; q++) mesh_ids_.push_back(arg[q]);
    }
  }
  if (!primitive_ && mesh_ids_.empty())
    error->all(FLERR, "fix wall/gran/gb300: expected a primitive plane or a mesh list");
}

void FixWallGranGB300::post_force(int) {
  if (!dynamic_cast<VerletGB300 *>(update->integrate))
    error->all(FLERR, "fix wall/gran/gb300 needs run_style verlet/gb300 (no host fallback)");
}

void FixWallGranGB300::upload(dem_handle *h, int) {
  if (contact_match("normal", "hertz") == contact_match("normal", "hooke") ||
      !contact_match("tangential", "history") || !contact_match("cohesion", "off"))
    error->all(FLERR, "fix wall/gran/gb300: wall model must be hertz or hooke, tangential history, no cohesion");
  if (contact_match("rolling_friction", "cdt")) rolling_ = DEM_ROLLING_CDT;
  else if (contact_match("rolling_friction", "off")) rolling_ = DEM_ROLLING_OFF;
  else error->all(FLERR, "fix wall/gran/gb300: rolling_friction must be off or cdt");

  if (primitive_) {
    const int rc = cylinder_ ? dem_add_cylinder(h, axis_, pos_, c1_, c2_, wall_type_, rolling_, &device_wall_id_)
                             : dem_add_plane(h, axis_, pos_, wall_type_, rolling_, &device_wall_id_);
    if (rc != DEM_OK) error->all(FLERR, dem_last_error(h));
    return;
  }
  device_mesh_ids_.clear();
  for (size_t m = 0; m < mesh_ids_.size(); m++) {
    FixMeshSurface *fm = dynamic_cast<FixMeshSurface *>(modify->fix[modify->find_fix(mesh_ids_[m].c_str())]);
    if (!fm) error->all(FLERR, "fix wall/gran/gb300: mesh fix not found");
    TriMesh *mesh = fm->triMesh();
    const int ntri = mesh->sizeLocal();
    std::vector<double> nodes(9 * (size_t)ntri);
    for (int t = 0; t < ntri; t++)
      for (int q = 0; q < 3; q++) mesh->node(t, q, &nodes[9 * (size_t)t + 3 * q]);
    int id = -1;
    // edge/corner activity: NULL lets the library derive it as
    // SurfaceMesh::buildNeighbours does
    if (dem_add_mesh(h, ntri, &nodes[0], fm->min_type(), rolling_, NULL, NULL, &id) != DEM_OK)
      error->all(FLERR, dem_last_error(h));
    device_mesh_ids_.push_back(id);
  }
}

bool FixWallGranGB300::primitive_history(int i, double *h3) const {
  if (!primitive_ || !fix_history_primitive_ || !fix_history_primitive_->array_atom) return false;
  for (int k = 0; k < 3; k++) h3[k] = fix_history_primitive_->array_atom[i][k];
  return true;
}
