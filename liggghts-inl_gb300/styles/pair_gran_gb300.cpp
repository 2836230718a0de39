/* pair_style gran/gb300: see pair_gran_gb300.h. */

#include "pair_gran_gb300.h"

#include <string.h>

#include "atom.h"
#include "error.h"
#include "force.h"
#include "property_registry.h"
#include "update.h"
#include "verlet_gb300.h"

using namespace LAMMPS_NS;

PairGranGB300::PairGranGB300(LAMMPS *lmp)
    : PairGranProxy(lmp), normal_(DEM_NORMAL_HERTZ), rolling_(DEM_ROLLING_OFF),
      cohesion_(DEM_COHESION_OFF), tdamp_(1), limitf_(0) {
  memset(&bond_, 0, sizeof(bond_));
}

/* the reference parses the model keywords (PairGranProxy::settings ->
   PairStyles::Factory, src/pair_gran_proxy.cpp:63-79); the GB300 style then
   checks that the selected model is one the device implements */
void PairGranGB300::settings(int nargs, char **args) {
  PairGranProxy::settings(nargs, args);
  args_.assign(args, args + nargs);

  // Force::create_pair names a suffixed style "gran/gb300", but the
  // reference finds the granular pair by its exact name "gran"
  // (FixContactHistory::init, src/fix_contact_history.cpp:218;
  // FixCheckTimestepGran::init, src/fix_check_timestep_gran.cpp:153).  The
  // style therefore reports the base name, as the class it stands in for.
  if (force->pair == this && force->pair_style && strcmp(force->pair_style, "gran/gb300") == 0) {
    delete[] force->pair_style;
    force->pair_style = new char[5];
    strcpy(force->pair_style, "gran");
  }

  if (contact_match("normal", "hertz")) normal_ = DEM_NORMAL_HERTZ;
  else if (contact_match("normal", "hooke")) normal_ = DEM_NORMAL_HOOKE;
  else error->all(FLERR, "pair gran/gb300: normal model must be hertz or hooke");

  if (!contact_match("tangential", "history"))
    error->all(FLERR, "pair gran/gb300: tangential model must be history");
  if (!contact_match("surface", "default"))
    error->all(FLERR, "pair gran/gb300: surface model must be default");

  if (contact_match("rolling_friction", "off")) rolling_ = DEM_ROLLING_OFF;
  else if (contact_match("rolling_friction", "cdt")) rolling_ = DEM_ROLLING_CDT;
  else error->all(FLERR, "pair gran/gb300: rolling_friction must be off or cdt");

  if (contact_match("cohesion", "off")) cohesion_ = DEM_COHESION_OFF;
  else if (contact_match("cohesion", "bond/nonlinear")) cohesion_ = DEM_COHESION_BOND_NONLINEAR;
  else error->all(FLERR, "pair gran/gb300: cohesion must be off or bond/nonlinear");

  // model options as the models register them (Settings::registerOnOff):
  // tangential_damping defaults to on for hertz (normal_model_hertz.h:90)
  // and for hooke (normal_model_hooke.h:98); limitForce to off
  tdamp_ = on_off("tangential_damping", 1);
  limitf_ = on_off("limitForce", 0);
  if (normal_ == DEM_NORMAL_HOOKE &&
      (on_off("viscous", 0) || on_off("ktToKnUser", 0) || on_off("heating_normal_hooke", 0)))
    error->all(FLERR, "pair gran/gb300: hooke options viscous/ktToKnUser/heating are not supported");

  // bond/nonlinear on/off settings (cohesion_model_bond_nonlinear.h:238-247)
  bond_.stressBreak = on_off("stressBreak", 0);
  bond_.tensionStress = on_off("tensionStress", 1);
  bond_.compressionStress = on_off("compressionStress", 1);
  bond_.shearStress = on_off("shearStress", 1);
  bond_.normalTorqueStress = on_off("normalTorqueStress", 1);
  bond_.shearTorqueStress = on_off("shearTorqueStress", 1);
  bond_.createBondAlways = on_off("createBondAlways", 0);
  bond_.dampingBond = on_off("dampingBond", 1);
  bond_.dampingBondSmooth = on_off("dampingBondSmooth", 0);
  bond_.ratioTCBond = on_off("ratioTensionCompressionBond", 0);
}

/* value of an on/off (yes/no) keyword on the pair_style line, else dflt */
int PairGranGB300::on_off(const char *keyword, int dflt) const {
  for (size_t k = 0; k + 1 < args_.size(); k++) {
    if (args_[k] != keyword) continue;
    const std::string &v = args_[k + 1];
    if (v == "on" || v == "yes") return 1;
    if (v == "off" || v == "no") return 0;
  }
  return dflt;
}

void PairGranGB300::fill_config(dem_config &cfg) const {
  cfg.normal_model = normal_;
  cfg.rolling_model = rolling_;
  cfg.cohesion_model = cohesion_;
  cfg.tangential_damping = tdamp_;
  cfg.limit_force = limitf_;
}

/* one (ntypes+1)^2 matrix property of the registry, row-major */
void PairGranGB300::matrix(const char *name, int ntypes, std::vector<double> &out, bool required) {
  const size_t n1 = (size_t)ntypes + 1;
  out.assign(n1 * n1, 0.0);
  if (!required) return;
  MatrixProperty *mp = force->registry.getMatrixProperty(name, "pair gran/gb300");
  if (!mp || !mp->data) error->all(FLERR, "pair gran/gb300: a material property is missing");
  for (int i = 1; i <= ntypes && i < mp->rows; i++)
    for (int j = 1; j <= ntypes && j < mp->cols; j++) out[i * n1 + j] = mp->data[i][j];
}

void PairGranGB300::upload_params(dem_handle *h) {
  const int nt = atom->ntypes;
  std::vector<double> Y, G, B, MU, MUR, RL;
  matrix("Yeff", nt, Y, true);
  matrix("Geff", nt, G, true);
  matrix("betaeff", nt, B, normal_ == DEM_NORMAL_HERTZ);
  matrix("coeffFrict", nt, MU, true);
  matrix("coeffRollFrict", nt, MUR, rolling_ == DEM_ROLLING_CDT);
  matrix("coeffRestLog", nt, RL, normal_ == DEM_NORMAL_HOOKE);
  double charVel = 0.0;
  if (normal_ == DEM_NORMAL_HOOKE) {
    ScalarProperty *sp = force->registry.getScalarProperty("charVel", "pair gran/gb300");
    if (sp) charVel = sp->data;
  }
  int rc = dem_set_pair_params(h, nt, &Y[0], &G[0], &B[0], &MU[0],
                               rolling_ == DEM_ROLLING_CDT ? &MUR[0] : NULL, &RL[0], charVel);
  if (rc != DEM_OK) error->all(FLERR, dem_last_error(h));
  if (cohesion_ != DEM_COHESION_BOND_NONLINEAR) return;

  // the 23 tables in the C ABI's order; a property the model did not
  // register for its settings stays zero (connectToProperties,
  // cohesion_model_bond_nonlinear.h:255-381)
  struct T { const char *name; bool present; };
  const bool damp = bond_.dampingBond != 0, sb = bond_.stressBreak != 0;
  const T tabs[DEM_BOND_NTABLES] = {
      {"radiusMultiplierBondnonlinear", true},
      {"stiffnessK_fn1", true}, {"stiffnessKu_fn1", true}, {"stiffnessKc_fn1", true},
      {"stiffnessK_fn2", true}, {"stiffnessKu_fn2", true}, {"stiffnessKc_fn2", true},
      {"stiffnessK_ft", true},
      {"stiffnessK_tn", true}, {"stiffnessKu_tn", true}, {"stiffnessKc_tn", true},
      {"stiffnessK_tt", true}, {"stiffnessKu_tt", true}, {"stiffnessKc_tt", true},
      {"dampingNormalForceBondnonlinear", damp}, {"dampingTangentialForceBondnonlinear", damp},
      {"dampingNormalTorqueBondnonlinear", damp}, {"dampingTangentialTorqueBondnonlinear", damp},
      {"maxDistanceBondnonlinear", !sb},
      {"maxSigmaBondnonlinear", sb}, {"maxTauBondnonlinear", sb},
      {"ratioTensionCompressionBondnonlinear", sb && bond_.ratioTCBond != 0},
      {"createDistanceBondnonlinear", true}};
  const size_t n2 = (size_t)(nt + 1) * (nt + 1);
  std::vector<double> all(DEM_BOND_NTABLES * n2, 0.0), one;
  for (int k = 0; k < DEM_BOND_NTABLES; k++) {
    matrix(tabs[k].name, nt, one, tabs[k].present);
    memcpy(&all[k * n2], &one[0], n2 * sizeof(double));
  }
  dem_bond_settings st = bond_;
  st.tsCreate = 0.0;
  if (!bond_.createBondAlways) {
    ScalarProperty *sp = force->registry.getScalarProperty("tsCreateBondnonlinear", "pair gran/gb300");
    if (sp) st.tsCreate = sp->data;
  }
  rc = dem_set_bond_params(h, &all[0], &st);
  if (rc != DEM_OK) error->all(FLERR, dem_last_error(h));
}

/* the device computed the forces of the current state; copy them in */
void PairGranGB300::compute_force(int, int) {
  VerletGB300 *v = dynamic_cast<VerletGB300 *>(update->integrate);
  if (!v) error->all(FLERR, "pair gran/gb300 needs run_style verlet/gb300 (no host fallback)");
  v->add_device_forces();
}
