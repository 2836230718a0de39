/* fix nve/sphere/gb300: see fix_nve_sphere_gb300.h. */

#include "fix_nve_sphere_gb300.h"

#include "domain.h"
#include "error.h"
#include "group.h"
#include "update.h"
#include "verlet_gb300.h"

using namespace LAMMPS_NS;

FixNVESphereGB300::FixNVESphereGB300(LAMMPS *lmp, int narg, char **arg) : FixNVESphere(lmp, narg, arg) {}

void FixNVESphereGB300::init() {
  FixNVESphere::init();
  if (igroup != group->find("all"))
    error->all(FLERR, "fix nve/sphere/gb300 integrates group all only");
  if (extra != 0 || useAM_ || domain->dimension != 3)
    error->all(FLERR, "fix nve/sphere/gb300: update dipole, added mass and 2d discs are not supported");
}

void FixNVESphereGB300::initial_integrate(int) {
  if (!dynamic_cast<VerletGB300 *>(update->integrate))
    error->all(FLERR, "fix nve/sphere/gb300 needs run_style verlet/gb300 (no host fallback)");
}

void FixNVESphereGB300::final_integrate() {
  if (!dynamic_cast<VerletGB300 *>(update->integrate))
    error->all(FLERR, "fix nve/sphere/gb300 needs run_style verlet/gb300 (no host fallback)");
}
