// Host build of the adjoint's per-pair laws (liggghts-inl_gb300/csrc/
// adjoint_law.cuh, adjoint_bond.cuh) and a finite-difference check of their
// vector-Jacobian products: for random inputs, random output weights w and a
// random input direction u, the product's <grad, u> against the central
// difference of <w, outputs> along u.  Built and called by
// tests/test_adjoint_vjp.py.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "adjoint_bond.cuh"

using namespace gb300;

namespace {

struct Rng {
  uint64_t s;
  double uni() {  // [0, 1)
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  }
  double sym() { return 2.0 * uni() - 1.0; }
};

// ------------------------------------------------------------ contact law
struct LawX {  // the differentiable inputs
  double d[3], vr[3], wi[3], wj[3], sh[3], ri, rj, mi, mj, Y, G, beta, mu, mur;
};

double law_value(const VjpIn &base, const LawX &x, const double w[12], int *slide) {
  VjpIn a = base;
  for (int k = 0; k < 3; k++) {
    a.d[k] = x.d[k];
    a.vr[k] = x.vr[k];
    a.wi[k] = x.wi[k];
    a.wj[k] = x.wj[k];
    a.sh[k] = x.sh[k];
  }
  a.ri = x.ri; a.rj = x.rj; a.mi = x.mi; a.mj = x.mj;
  a.Y = x.Y; a.G = x.G; a.beta = x.beta; a.mu = x.mu; a.mur = x.mur;
  LawState S;
  double F[3], Ti[3], Tj[3], s3[3];
  law_forward(a, S, F, Ti, Tj, s3);
  *slide = (S.slide ? 1 : 0) | (S.Fn > 0 ? 2 : 0);  // |Fn| caps the friction
  double v = 0.0;
  for (int k = 0; k < 3; k++) v += w[k] * F[k] + w[3 + k] * Ti[k] + w[6 + k] * Tj[k] + w[9 + k] * s3[k];
  return v;
}

}  // namespace

extern "C" {

// ncases random contacts of the given kind (0 pair, 1 wall, 2 bonded pair),
// with (upd = 1) or without history update, with or without CDT rolling; returns the largest relative
// error of the directional derivative, and in counts[0..1] how many cases
// stuck / slid, counts[2] the cases skipped because stick/slip switched
// within the finite-difference step
double check_law(uint64_t seed, int ncases, int kind, int upd, int rolling, int *counts) {
  Rng R{seed * 2654435761ULL + 17};
  double worst = 0.0;
  counts[0] = counts[1] = counts[2] = 0;
  for (int c = 0; c < ncases; c++) {
    VjpIn a;
    memset(&a, 0, sizeof a);
    a.upd = upd != 0;
    a.wall = kind == 1;
    a.bonded = kind == 2;
    a.rolling = rolling != 0;
    a.dt = 1e-6;
    LawX x;
    x.ri = 1e-3 * (0.8 + 0.4 * R.uni());
    x.rj = kind == 1 ? 0.0 : 1e-3 * (0.8 + 0.4 * R.uni());
    x.mi = 4.0 / 3.0 * M_PI * x.ri * x.ri * x.ri * 2500.0;
    x.mj = kind == 1 ? 0.0 : 4.0 / 3.0 * M_PI * x.rj * x.rj * x.rj * 2500.0;
    const double dist = (x.ri + x.rj) * (1.0 - 0.02 * (0.05 + R.uni()));
    double dir[3] = {R.sym(), R.sym(), R.sym()};
    if (kind == 1) dir[0] = dir[1] = 0.0, dir[2] = R.uni() < 0.5 ? -1.0 : 1.0;
    const double dn = sqrt(dot3(dir, dir));
    for (int k = 0; k < 3; k++) {
      x.d[k] = dist * dir[k] / dn;
      x.vr[k] = 0.1 * R.sym();
      x.wi[k] = 100.0 * R.sym();
      x.wj[k] = kind == 1 ? 0.0 : 100.0 * R.sym();
      x.sh[k] = 2e-6 * R.sym();  // sliding for some cases, sticking for others
    }
    x.Y = 1e7 * (0.5 + R.uni());
    x.G = 4e6 * (0.5 + R.uni());
    x.beta = -0.5 * R.uni() - 0.05;
    x.mu = 0.2 + 0.5 * R.uni();
    x.mur = 0.1 + 0.4 * R.uni();
    double w[12];
    for (int k = 0; k < 12; k++) w[k] = R.sym();
    // the VJP
    for (int k = 0; k < 3; k++) a.d[k] = x.d[k], a.vr[k] = x.vr[k], a.wi[k] = x.wi[k], a.wj[k] = x.wj[k],
                                a.sh[k] = x.sh[k];
    a.ri = x.ri; a.rj = x.rj; a.mi = x.mi; a.mj = x.mj; a.Y = x.Y; a.G = x.G; a.beta = x.beta; a.mu = x.mu;
    a.mur = x.mur;
    LawState S;
    double F[3], Ti[3], Tj[3], s3[3];
    law_forward(a, S, F, Ti, Tj, s3);
    counts[S.slide ? 1 : 0]++;
    VjpBar b;
    for (int k = 0; k < 3; k++) b.F[k] = w[k], b.Ti[k] = w[3 + k], b.Tj[k] = w[6 + k], b.s3[k] = w[9 + k];
    law_vjp(a, b);
    // direction: each input scaled by its magnitude (walls: d along the normal only)
    LawX u;
    for (int k = 0; k < 3; k++) {
      u.d[k] = (kind == 1 && dir[k] == 0.0) ? 0.0 : 1e-3 * R.sym();
      u.vr[k] = 0.1 * R.sym();
      u.wi[k] = 100.0 * R.sym();
      u.wj[k] = kind == 1 ? 0.0 : 100.0 * R.sym();
      u.sh[k] = 2e-6 * R.sym();
    }
    u.ri = 1e-3 * R.sym(); u.rj = kind == 1 ? 0.0 : 1e-3 * R.sym();
    u.mi = x.mi * R.sym(); u.mj = kind == 1 ? 0.0 : x.mj * R.sym();
    u.Y = x.Y * R.sym(); u.G = x.G * R.sym(); u.beta = 0.3 * R.sym(); u.mu = 0.3 * R.sym();
    u.mur = rolling ? 0.2 * R.sym() : 0.0;
    double g = 0.0;
    for (int k = 0; k < 3; k++)
      g += b.d[k] * u.d[k] + b.vr[k] * u.vr[k] + b.wi[k] * u.wi[k] + b.wj[k] * u.wj[k] + b.sh[k] * u.sh[k];
    g += b.ri * u.ri + b.rj * u.rj + b.mi * u.mi + b.mj * u.mj + b.Y * u.Y + b.G * u.G + b.beta * u.beta +
         b.mu * u.mu + b.mur * u.mur;
    double gabs = fabs(b.ri * u.ri) + fabs(b.rj * u.rj) + fabs(b.mi * u.mi) + fabs(b.mj * u.mj) + fabs(b.Y * u.Y) +
                  fabs(b.G * u.G) + fabs(b.beta * u.beta) + fabs(b.mu * u.mu) + fabs(b.mur * u.mur);
    for (int k = 0; k < 3; k++)
      gabs += fabs(b.d[k] * u.d[k]) + fabs(b.vr[k] * u.vr[k]) + fabs(b.wi[k] * u.wi[k]) + fabs(b.wj[k] * u.wj[k]) +
              fabs(b.sh[k] * u.sh[k]);
    // fourth-order central difference along u
    const double h = 2e-6;
    double fv[4];
    bool same = true;
    for (int q = 0; q < 4; q++) {
      const double sc = (q == 0 ? 2.0 : q == 1 ? 1.0 : q == 2 ? -1.0 : -2.0) * h;
      LawX xs = x;
      double *px = &xs.d[0];
      const double *pu = &u.d[0];
      for (size_t k = 0; k < sizeof(LawX) / sizeof(double); k++) px[k] += sc * pu[k];
      int sl;
      fv[q] = law_value(a, xs, w, &sl);
      same = same && sl == ((S.slide ? 1 : 0) | (S.Fn > 0 ? 2 : 0));
    }
    if (!same) {  // stick/slip switched within the stencil
      counts[2]++;
      continue;
    }
    const double fd = (8.0 * (fv[1] - fv[2]) - (fv[0] - fv[3])) / (12.0 * h);
    const double err = fabs(g - fd) / fmax(fabs(fd), 1e-3 * gabs);
    if (err > worst) worst = err;
  }
  return worst;
}

// ------------------------------------------------------------------ bond
namespace {

struct BondX {
  double d[3], vr[3], wi[3], wj[3], ri, rj;
  double h[kBondValues];
};

// the branch decisions of one evaluation, packed
uint64_t bond_sig(const BondTape &T) {
  uint64_t s = (uint64_t)T.status | (uint64_t)T.created << 2 | (uint64_t)T.evaluated << 3;
  if (!T.evaluated) return s;
  s |= (uint64_t)T.ncomp << 4 | (uint64_t)T.dmax_new << 5 | (uint64_t)T.dmin_new << 6 | (uint64_t)T.nbr << 7;
  int b = 10;
  for (int q = 0; q < 3; q++) {
    s |= (uint64_t)T.brn[q] << b | (uint64_t)T.brt[q] << (b + 2);
    s |= (uint64_t)(T.ncomp && T.nclamp[q]) << (b + 4) | (uint64_t)T.tclamp[q] << (b + 5);
    s |= (uint64_t)(T.nm[q] > 0) << (b + 6) | (uint64_t)(T.tm[q] > 0) << (b + 7);
    // the damping laws take absolute values
    s |= (uint64_t)(T.nforce[q] > 0) << (b + 8) | (uint64_t)(T.ftp[q] > 0) << (b + 9);
    s |= (uint64_t)(T.tn[q] > 0) << (b + 10) | (uint64_t)(T.tt[q] > 0) << (b + 11);
    b += 12;
  }
  return s;
}

double bond_value(const BondArgs &base, const BondPar &P, const BondX &x, const double w[9 + kBondValues],
                  uint64_t *sig) {
  BondArgs a = base;
  for (int k = 0; k < 3; k++) a.d[k] = x.d[k], a.vr[k] = x.vr[k], a.wi[k] = x.wi[k], a.wj[k] = x.wj[k];
  a.ri = x.ri;
  a.rj = x.rj;
  BondTape T;
  double hout[kBondValues], F[3], Ti[3], Tj[3];
  bond_fwd(a, P, x.h, hout, F, Ti, Tj, T);
  *sig = bond_sig(T);
  double v = 0.0;
  for (int k = 0; k < 3; k++) v += w[k] * F[k] + w[3 + k] * Ti[k] + w[6 + k] * Tj[k];
  for (int k = 0; k < kBondValues; k++) v += w[9 + k] * hout[k];
  return v;
}

}  // namespace

// ncases random bonds with the model's on/off settings `flags` (kBond* bits;
// create: a fresh pair that bonds in this evaluation, else an existing
// bond).  Returns the largest relative error of the directional derivative;
// branches[0..5] count the normal-law branches taken, branches[6..9] the
// twisting/bending hysteresis branches, branches[10] the stress breakages,
// branches[11] the cases skipped because a branch switched within the
// finite-difference step.
double check_bond(uint64_t seed, int ncases, int flags, int create, int upd, int *branches) {
  Rng R{seed * 0x9E3779B97F4A7C15ULL + 3};
  for (int k = 0; k < 12; k++) branches[k] = 0;
  double worst = 0.0;
  BondPar P;
  for (int k = 0; k < kBondTables; k++) P.t[k] = 0.0;
  P.flags = flags;
  P.t[kBondLambda] = 1.0;
  // magnitudes chosen so that every term contributes forces of ~0.01-0.1 N
  P.t[kBondKfn1] = 1e2; P.t[kBondKufn1] = 4e2; P.t[kBondKcfn1] = 2e2;
  P.t[kBondKfn2] = 1e10; P.t[kBondKufn2] = 4e10; P.t[kBondKcfn2] = 2e10;
  P.t[kBondKft] = 6e7;
  P.t[kBondKtn] = 3e10; P.t[kBondKutn] = 9e10; P.t[kBondKctn] = 5e10;
  P.t[kBondKtt] = 2e10; P.t[kBondKutt] = 6e10; P.t[kBondKctt] = 4e10;
  P.t[kBondDampFn] = 0.3; P.t[kBondDampFt] = 0.2; P.t[kBondDampTn] = 0.25; P.t[kBondDampTt] = 0.15;
  P.t[kBondMaxDist] = 1e9;
  // with stress breakage on, about half of the bonds break
  P.t[kBondMaxSigma] = 6e4; P.t[kBondMaxTau] = 1e30; P.t[kBondRatioTC] = 1.0;
  P.t[kBondCreateDist] = 2.5e-3;
  for (int c = 0; c < ncases; c++) {
    BondArgs a;
    memset(&a, 0, sizeof a);
    a.upd = upd != 0;
    a.may_create = create != 0;
    a.dt = 1e-6;
    BondX x;
    x.ri = 1e-3 * (0.8 + 0.4 * R.uni());
    x.rj = 1e-3 * (0.8 + 0.4 * R.uni());
    const double dist = (x.ri + x.rj) * (1.0 + 0.01 * R.sym());
    double dir[3] = {R.sym(), R.sym(), R.sym()};
    const double dn = sqrt(dot3(dir, dir));
    for (int k = 0; k < 3; k++) {
      x.d[k] = dist * dir[k] / dn;
      x.vr[k] = 0.05 * R.sym();
      x.wi[k] = 50.0 * R.sym();
      x.wj[k] = 50.0 * R.sym();
      a.xi[k] = 0.01 * R.sym();
    }
    // history: an existing bond with displacement extremes and hysteresis
    // extremes around the current angles, so that every branch is taken
    for (int k = 0; k < kBondValues; k++) x.h[k] = 0.0;
    if (!create) {
      const double disp = (R.uni() < 0.5 ? -1.0 : 1.0) * (1e-7 + 2e-6 * R.uni());
      x.h[0] = 1.0;
      x.h[1] = dist + disp;
      for (int k = 0; k < 3; k++) x.h[2 + k] = 0.01 * R.sym();
      for (int k = 0; k < 3; k++) x.h[5 + k] = 0.02 * R.sym();
      for (int k = 0; k < 6; k++) x.h[8 + k] = 2e-3 * R.sym();
      const double u1 = R.uni(), u2 = R.uni();
      x.h[14] = u1 < 0.5 ? 4e-6 * R.uni() : 1e-7 * R.uni();
      x.h[27] = u2 < 0.5 ? -4e-6 * R.uni() : -1e-7 * R.uni();
      for (int k = 0; k < 6; k++) {
        x.h[15 + k] = 4e-3 * R.uni();
        x.h[21 + k] = -4e-3 * R.uni();
      }
    } else {  // leftovers of an earlier bond survive creation in 14..27
      for (int k = 14; k < kBondValues; k++) x.h[k] = (k == 27 || k >= 21) ? -3e-3 * R.uni() : 3e-3 * R.uni();
      x.h[14] = 3e-6 * R.uni();
      x.h[27] = -3e-6 * R.uni();
    }
    double w[9 + kBondValues];
    for (int k = 0; k < 9 + kBondValues; k++) w[k] = R.sym();
    w[9 + 0] = 0.0;  // bondFlag: piecewise constant
    w[9 + 2] = w[9 + 3] = w[9 + 4] = 0.0;  // contactPos: not propagated
    for (int k = 0; k < 3; k++) a.d[k] = x.d[k], a.vr[k] = x.vr[k], a.wi[k] = x.wi[k], a.wj[k] = x.wj[k];
    a.ri = x.ri;
    a.rj = x.rj;
    BondTape T;
    double hout[kBondValues], F[3], Ti[3], Tj[3];
    const int st = bond_fwd(a, P, x.h, hout, F, Ti, Tj, T);
    if (st == kBondBroken) branches[10]++;
    if (T.evaluated && T.ncomp) branches[T.nbr]++;
    if (T.evaluated && (flags & kBondNormalTorque))
      for (int q = 0; q < 3; q++) branches[6 + T.brn[q]]++;
    if (T.evaluated && (flags & kBondShearTorque))
      for (int q = 0; q < 3; q++) branches[6 + T.brt[q]]++;
    BondArgsBar ab;
    double hinb[kBondValues];
    bond_vjp(a, P, x.h, w, w + 3, w + 6, w + 9, ab, hinb);
    // direction scaled per input
    BondX u;
    for (int k = 0; k < 3; k++) {
      u.d[k] = 1e-3 * R.sym();
      u.vr[k] = 0.05 * R.sym();
      u.wi[k] = 50.0 * R.sym();
      u.wj[k] = 50.0 * R.sym();
    }
    u.ri = 1e-3 * R.sym();
    u.rj = 1e-3 * R.sym();
    const double hs[kBondValues] = {0, 1e-3, 0, 0, 0, 0.02, 0.02, 0.02, 2e-3, 2e-3, 2e-3, 2e-3, 2e-3, 2e-3,
                                    4e-6, 4e-3, 4e-3, 4e-3, 4e-3, 4e-3, 4e-3, 4e-3, 4e-3, 4e-3, 4e-3, 4e-3,
                                    4e-3, 4e-6};
    for (int k = 0; k < kBondValues; k++) u.h[k] = hs[k] * R.sym();
    double g = 0.0;
    for (int k = 0; k < 3; k++)
      g += ab.d[k] * u.d[k] + ab.vr[k] * u.vr[k] + ab.wi[k] * u.wi[k] + ab.wj[k] * u.wj[k];
    g += ab.ri * u.ri + ab.rj * u.rj;
    for (int k = 0; k < kBondValues; k++) g += hinb[k] * u.h[k];
    double gabs = 0.0;
    for (int k = 0; k < 3; k++)
      gabs += fabs(ab.d[k] * u.d[k]) + fabs(ab.vr[k] * u.vr[k]) + fabs(ab.wi[k] * u.wi[k]) + fabs(ab.wj[k] * u.wj[k]);
    gabs += fabs(ab.ri * u.ri) + fabs(ab.rj * u.rj);
    for (int k = 0; k < kBondValues; k++) gabs += fabs(hinb[k] * u.h[k]);
    // fourth-order central difference along u
    const double h = 2e-6;
    double fv[4];
    bool same = true;
    for (int q = 0; q < 4; q++) {
      const double sc = (q == 0 ? 2.0 : q == 1 ? 1.0 : q == 2 ? -1.0 : -2.0) * h;
      BondX xs = x;
      double *px = &xs.d[0];
      const double *pu = &u.d[0];
      for (size_t k = 0; k < sizeof(BondX) / sizeof(double); k++) px[k] += sc * pu[k];
      uint64_t sg;
      fv[q] = bond_value(a, P, xs, w, &sg);
      same = same && sg == bond_sig(T);
    }
    if (!same) {  // a branch switched within the stencil: no derivative there
      branches[11]++;
      continue;
    }
    const double fd = (8.0 * (fv[1] - fv[2]) - (fv[0] - fv[3])) / (12.0 * h);
    const double err = fabs(g - fd) / fmax(fabs(fd), 1e-3 * gabs);
    if (err > worst) worst = err;
  }
  return worst;
}

}  // extern "C"
