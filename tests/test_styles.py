"""LIGGGHTS suffix styles (liggghts-inl_gb300/styles): the drop-in boundary
on the reference's side.

  * every style registers under the reference's name + "/gb300", which is
    the name Force::new_pair, Modify::add_fix and Update::create_integrate try
    first when LIGGGHTS runs with "-sf gb300";
  * every style compiles (g++ -fsyntax-only) against the reference's own
    headers and this library's C ABI header.  The reference generates its
    contact-model style headers at build time (src/Make.sh); the test writes
    them the same way (one #include per header that declares a model) into a
    temporary folder.  Skipped where the reference sources are absent.
"""
import glob
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STYLES = os.path.join(ROOT, "liggghts-inl_gb300", "styles")
# the unmodified reference sources as oracle/ref/Makefile stages them
REF_SRC = os.environ.get("LIGGGHTS_REFERENCE_SRC", os.path.join(ROOT, "oracle", "_ref", "src"))

EXPECTED = {
    "pair_gran_gb300.h": ("PairStyle", "gran/gb300", "PairGranGB300", "PairGranProxy"),
    "fix_wall_gran_gb300.h": ("FixStyle", "wall/gran/gb300", "FixWallGranGB300", "FixWallGran"),
    "fix_nve_sphere_gb300.h": ("FixStyle", "nve/sphere/gb300", "FixNVESphereGB300", "FixNVESphere"),
    "fix_gravity_gb300.h": ("FixStyle", "gravity/gb300", "FixGravityGB300", "FixGravity"),
    "fix_move_mesh_gb300.h": ("FixStyle", "move/mesh/gb300", "FixMoveMeshGB300", "FixMoveMesh"),
    "verlet_gb300.h": ("IntegrateStyle", "verlet/gb300", "VerletGB300", "Verlet"),
}


def test_style_registrations():
    for hdr, (macro, name, cls, base) in EXPECTED.items():
        txt = open(os.path.join(STYLES, hdr)).read()
        assert "%s(%s,%s)" % (macro, name, cls) in txt, hdr
        assert re.search(r"class %s : public %s\b" % (cls, base), txt), hdr
        assert os.path.exists(os.path.join(STYLES, hdr.replace(".h", ".cpp"))), hdr


def _model_headers(dst):
    for kind in ("surface", "normal", "tangential", "cohesion", "rolling"):
        macro = kind.upper() + "_MODEL("
        inc = []
        for h in sorted(glob.glob(os.path.join(REF_SRC, "*.h"))):
            with open(h, errors="replace") as f:
                if any(line.startswith(macro) for line in f):
                    inc.append('#include "%s"\n' % os.path.basename(h))
        with open(os.path.join(dst, "style_%s_model.h" % kind), "w") as f:
            f.writelines(inc)


@pytest.mark.skipif(not os.path.isdir(REF_SRC) or shutil.which("g++") is None,
                    reason="reference sources or g++ not available")
@pytest.mark.parametrize("src", sorted(os.path.basename(p) for p in glob.glob(os.path.join(STYLES, "*.cpp"))))
def test_style_compiles_against_reference_headers(src, tmp_path):
    _model_headers(str(tmp_path))
    cmd = ["g++", "-std=c++11", "-fsyntax-only", "-Wall", "-I" + str(tmp_path), "-I" + REF_SRC,
           "-I" + os.path.join(REF_SRC, "STUBS"), "-I" + os.path.join(ROOT, "include"), "-I" + STYLES,
           os.path.join(STYLES, src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    own = [ln for ln in r.stderr.splitlines() if STYLES in ln and "warning" in ln]
    assert not own, "\n".join(own)
