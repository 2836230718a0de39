/* pair_style gran/gb300: the granular pair style of the reference
   (PairGranProxy, src/pair_gran_proxy.h) whose contact forces are computed
   on the GPU by the GB300 library (include/liggghts_gb300.h) inside the
   device-resident timestep of run_style verlet/gb300.

   Selected by the suffix mechanism (command-line "-sf gb300" or the input
   command "suffix gb300"): Force::new_pair tries "gran/gb300" before "gran"
   (src/force.cpp:226-246), so input scripts stay unchanged.  The class
   derives from PairGranProxy, so the reference's own keyword parsing, model
   factory, property registry, contact-history fix, FixWallGran and every
   dynamic_cast / pair_match("gran") keep working.

   Supported models (anything else is rejected at the pair_style command):
     model hertz | hooke, tangential history, surface default,
     rolling_friction off | cdt, cohesion off | bond/nonlinear,
     options tangential_damping, limitForce and the bond/nonlinear on/off
     settings.

   Under run_style verlet/gb300 compute_force() does not compute anything on
   the host: it writes the forces and torques the device computed for the
   current state into atom->f / atom->torque (so thermo and dump output at
   setup and output steps see them).  Without verlet/gb300 it stops with an
   error: there is no host fallback. */

#ifdef PAIR_CLASS

PairStyle(gran/gb300,PairGranGB300)

#else

#ifndef LMP_PAIR_GRAN_GB300_H
#define LMP_PAIR_GRAN_GB300_H

#include "pair_gran_proxy.h"
#include "liggghts_gb300.h"

#include <string>
#include <vector>

namespace LAMMPS_NS {

class PairGranGB300 : public PairGranProxy {
 public:
  PairGranGB300(class LAMMPS *);
  virtual ~PairGranGB300() {}

  virtual void settings(int nargs, char **args);
  virtual void compute_force(int eflag, int vflag);

  /* model switches of this pair style in the C ABI's terms (after settings) */
  void fill_config(dem_config &cfg) const;
  /* material tables (and bond/nonlinear tables) from force->registry into h;
     call after init (the models have connected their properties) */
  void upload_params(dem_handle *h);
  int cohesion_model() const { return cohesion_; }

 private:
  int normal_, rolling_, cohesion_;
  int tdamp_, limitf_;
  dem_bond_settings bond_;
  std::vector<std::string> args_;

  int on_off(const char *keyword, int dflt) const;
  void matrix(const char *name, int ntypes, std::vector<double> &out, bool required);
};

}

#endif
#endif
