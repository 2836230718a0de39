#!/bin/sh
# Test infrastructure only.  Writes the style registry headers that a LIGGGHTS
# build needs (style_*.h, version_liggghts.h, style_contact_model.h) into an
# output folder, from the unmodified reference sources.  The reference's own
# Make.sh ("sh Make.sh style", src/Make.sh:77-106) produces the same kind of
# files: for every style class, one #include per header that declares it.
# This script is our own recipe; it does not run the reference's build system.
#
# usage: gen_styles.sh REF_SRC_DIR OUT_DIR [EXTRA_STYLE_DIR]
# With EXTRA_STYLE_DIR, the style headers found there (the GB300 suffix
# styles) are registered after the reference's own.
set -e
REF="$1"
OUT="$2"
EXTRA="$3"
mkdir -p "$OUT"

style () {   # $1 = search string, $2 = header prefix, $3 = style file suffix
  tmp="$OUT/style_$3.h.tmp"
  : > "$tmp"
  for f in $(cd "$REF" && grep -sl "$1" $2*.h 2>/dev/null); do
    echo "#include \"$f\"" >> "$tmp"
  done
  if [ -n "$EXTRA" ]; then
    for f in $(cd "$EXTRA" && grep -sl "$1" $2*.h 2>/dev/null); do
      echo "#include \"$f\"" >> "$tmp"
    done
  fi
  mv "$tmp" "$OUT/style_$3.h"
}

style ANGLE_CLASS             angle_              angle
style ATOM_CLASS              atom_vec_           atom
style BODY_CLASS              body_               body
style BOND_CLASS              bond_               bond
style COMMAND_CLASS           ""                  command
style COMPUTE_CLASS           compute_            compute
style DIHEDRAL_CLASS          dihedral_           dihedral
style DUMP_CLASS              dump_               dump
style FIX_CLASS               fix_                fix
style IMPROPER_CLASS          improper_           improper
style INTEGRATE_CLASS         ""                  integrate
style KSPACE_CLASS            ""                  kspace
style MINIMIZE_CLASS          min_                minimize
style PAIR_CLASS              pair_               pair
style SURFACE_MODEL           surface_model_      surface_model
style NORMAL_MODEL            normal_model_       normal_model
style TANGENTIAL_MODEL        tangential_model_   tangential_model
style COHESION_MODEL          cohesion_model_     cohesion_model
style ROLLING_MODEL           rolling_model_      rolling_model
style READER_CLASS            reader_             reader
style REGION_CLASS            region_             region
style CFD_DATACOUPLING_CLASS  cfd_datacoupling_   cfd_datacoupling
style CFD_REGIONMODEL_CLASS   cfd_regionmodel_    cfd_regionmodel
style LB_CLASS                ""                  lb
style SPH_KERNEL_CLASS        sph_kernel_         sph_kernel
style MESHMODULE_CLASS        mesh_module_        mesh_module
style MESHMOVER_CLASS         mesh_mover_         mesh_mover

# the snapshot fix used by the parity harness
echo '#include "fix_oracle_snapshot.h"' >> "$OUT/style_fix.h"

echo "#define LIGGGHTS_VERSION \"LIGGGHTS-INL $(cat "$REF/version_liggghts.txt"), oracle build\"" \
  > "$OUT/version_liggghts.h"

# compile-time specialised contact models (the reference's whitelist mechanism,
# src/contact_models.h:87-102); these are the combinations on the GPU path
: > "$OUT/style_contact_model.h"
for n in HERTZ HOOKE; do
  for c in COHESION_OFF COHESION_BOND_NONLINEAR; do
    for r in ROLLING_OFF ROLLING_CDT; do
      echo "GRAN_MODEL($n, TANGENTIAL_HISTORY, $c, $r, SURFACE_DEFAULT)" >> "$OUT/style_contact_model.h"
    done
  done
done
