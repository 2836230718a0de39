/* fix gravity/gb300: see fix_gravity_gb300.h. */

#include "fix_gravity_gb300.h"

#include "error.h"
#include "group.h"
#include "update.h"
#include "verlet_gb300.h"

using namespace LAMMPS_NS;

FixGravityGB300::FixGravityGB300(LAMMPS *lmp, int narg, char **arg) : FixGravity(lmp, narg, arg) {}

void FixGravityGB300::post_force(int) {
  if (!dynamic_cast<VerletGB300 *>(update->integrate))
    error->all(FLERR, "fix gravity/gb300 needs run_style verlet/gb300 (no host fallback)");
}

void FixGravityGB300::acceleration(double *acc) {
  if (varflag != 0)  // CONSTANT in src/fix_gravity.cpp:75
    error->all(FLERR, "fix gravity/gb300: gravity given by variables is not supported");
  if (igroup != group->find("all")) error->all(FLERR, "fix gravity/gb300 acts on group all only");
  get_gravity(acc);
}
