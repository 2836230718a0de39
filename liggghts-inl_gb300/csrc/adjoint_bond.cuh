// cohesion bond/nonlinear for one pair in the form the discrete adjoint
// needs: a forward evaluation that also records its branch decisions, and
// its vector-Jacobian product.
//
// Forward: CohesionModel<COHESION_BOND_NONLINEAR>::surfacesClose with
// createBondnonlinear / breakBondnonlinear
// (src/cohesion_model_bond_nonlinear.h:394-992), the same equations and
// operation order as bond_law.cuh, on the pair's 28 history values in the
// reference's order (bondFlag, initial_dist, contactPos[3], ft[3],
// thetan[3], thetat[3], deltan_max, thetan_max[3], thetat_max[3],
// thetan_min[3], thetat_min[3], deltan_min).  The pair is oriented as the
// list owns it (d = x_i - x_j).
//
// Reverse: every history value that enters a force or a later value is a
// differentiable input (initial_dist, ft, thetan, thetat and the extremes of
// the hysteresis laws); the branch decisions (bond created or broken, the
// piecewise normal law and hysteresis branches, the signs of the sign
// damping, the clamps of the smooth damping) are constants of the
// evaluation, so the product is exact for this piecewise-smooth map away
// from its switch points.  contactPos is stored but read by no force, so its
// adjoint is identically zero and is not propagated.  The projections onto
// en re-normalise en (vectorProject3D); the product treats en as the unit
// vector it is up to rounding.
//
// Host-compilable (with __device__/__forceinline__ defined empty) so that
// the product can be checked against finite differences on the CPU.
#pragma once
#include "adjoint_law.cuh"
#include "dem_device.cuh"

namespace gb300 {

struct BondPar {
  double t[kBondTables];  // one type pair, DEM_BOND_* order
  int flags;              // kBond* bits
};

struct BondArgs {
  double d[3], vr[3], wi[3], wj[3], xi[3];
  double ri, rj, dt;
  bool upd;         // update_history (false in the setup force pass)
  bool may_create;  // createBondAlways or ntimestep == tsCreateBondnonlinear
};

struct BondArgsBar {
  double d[3], vr[3], wi[3], wj[3];
  double ri, rj;
};

// bond_fwd results
enum { kBondNone = 0, kBondActive = 1, kBondBroken = 2 };

// intermediates of one forward evaluation
struct BondTape {
  int status;
  bool created, evaluated;  // evaluated: went past the distance-breakage test
  double r, rinv, en[3], rmin, rb, A, J, I, rsi, cri, crj, fi, fj;
  double vn[3], vtr[3], wr[3], wrel[3], wn[3], wt[3], minvel;
  double r0, disp, dmax, dmin;
  bool dmax_new, dmin_new, ncomp;  // ncomp: normal force active
  int nbr;                         // branch of the piecewise normal law
  double f, nforce[3], nm[3];      // nm: damping factor per component
  bool nclamp[3];                  // smooth damping clamped (or its sign form)
  double nden[3];
  bool nden_minvel[3];
  double ft0[3], ftp[3], sc, tm[3], tden[3];
  bool tclamp[3], tden_minvel[3];
  double thn1[3], tht1[3];
  double hmaxn[3], hminn[3], hmaxt[3], hmint[3];  // extremes after the sign reset
  int brn[3], brt[3];
  double tn[3], tt[3];
  double tfd[3], tor[3];
};

__device__ __forceinline__ double ab_sgn(double v) { return (double)((0.0 < v) - (v < 0.0)); }

// vectorProject3D (src/vector_liggghts.h:437-442)
__device__ __forceinline__ void ab_project(const double v[3], const double on[3], double out[3]) {
  const double norm = sqrt(on[0] * on[0] + on[1] * on[1] + on[2] * on[2]);
  const double inv = (norm == 0.) ? 0. : 1. / norm;
  const double n0 = on[0] * inv, n1 = on[1] * inv, n2 = on[2] * inv;
  const double dt = v[0] * n0 + v[1] * n1 + v[2] * n2;
  out[0] = dt * n0;
  out[1] = dt * n1;
  out[2] = dt * n2;
}

// one component of the hysteretic twisting/bending law (:677-761, :792-866);
// hmax/hmin in: stored extremes, out: new extremes; h1max/h1min: the extremes
// after the sign reset (used by the law); br: the branch taken
__device__ __forceinline__ double ab_hyst(double th, double &hmax, double &hmin, double k, double ku,
                                          double kc, double JI, double &h1max, double &h1min, int &br) {
  if (th > 0.0) hmin = 0.0;
  else if (th < 0.0) hmax = 0.0;
  h1max = hmax;
  h1min = hmin;
  const double ratio = (ku - k) / (ku + kc);
  const double c1 = ratio * hmax, c2 = ratio * hmin;
  double t;
  if ((th >= hmax) || (th <= hmin)) { t = -k * JI * th; br = 0; }
  else if (th > c1) { t = -ku * JI * th + (ku - k) * JI * hmax; br = 1; }
  else if (th >= c2) { t = kc * JI * th; br = 2; }
  else { t = -ku * JI * th + (ku - k) * JI * hmin; br = 3; }
  if (th > hmax) hmax = th;
  if (th < hmin) hmin = th;
  return t;
}

// forward; hout receives the history after the evaluation (a copy of hin
// where nothing changes).  F/Ti/Tj: the bond's force on i and torques on i
// and j, zero unless the result is kBondActive.
__device__ int bond_fwd(const BondArgs &a, const BondPar &P, const double hin[kBondValues],
                        double hout[kBondValues], double F[3], double Ti[3], double Tj[3], BondTape &T) {
  for (int k = 0; k < kBondValues; k++) hout[k] = hin[k];
  for (int k = 0; k < 3; k++) F[k] = Ti[k] = Tj[k] = 0.0;
  T.status = kBondNone;
  T.created = T.evaluated = false;
  const double lambda = P.t[kBondLambda];
  if (lambda < 1.e-15) return kBondNone;
  const int fl = P.flags;
  const double rsq = dot3(a.d, a.d);
  const double r = sqrt(rsq);
  T.r = r;
  if (a.upd) {
    if (hin[0] < 1.e-15) {
      if (!(a.may_create && r < P.t[kBondCreateDist])) return kBondNone;
      T.created = true;
      hout[0] = 1.0;
      hout[1] = r;
      for (int k = 0; k < 3; k++) hout[2 + k] = a.xi[k] - a.d[k];
      for (int k = 5; k < 14; k++) hout[k] = 0.0;
    }
  } else if (hin[0] < 1.e-15) {
    return kBondNone;
  }
  if (!(fl & kBondStressBreak) && r > P.t[kBondMaxDist] && a.upd) {
    hout[0] = 0.0;
    hout[1] = 0.0;
    T.status = kBondBroken;
    return kBondBroken;
  }
  T.evaluated = true;
  for (int k = 0; k < 3; k++) {
    T.ft0[k] = hout[5 + k];
    T.thn1[k] = hout[8 + k];
    T.tht1[k] = hout[11 + k];
  }
  T.rinv = 1. / r;
  for (int k = 0; k < 3; k++) T.en[k] = T.rinv * a.d[k];
  const double *en = T.en;
  T.rmin = a.ri < a.rj ? a.ri : a.rj;
  T.rb = lambda * T.rmin;
  T.A = 3.14159265358979323846 * T.rb * T.rb;
  T.J = 0.5 * T.A * T.rb * T.rb;
  T.I = 0.5 * T.J;
  const double dt = a.dt;
  T.rsi = 1. / (a.ri + a.rj);
  T.cri = r * a.ri * T.rsi;
  T.crj = r * a.rj * T.rsi;
  ab_project(a.vr, en, T.vn);
  T.fi = a.ri * T.rsi;
  T.fj = a.rj * T.rsi;
  for (int k = 0; k < 3; k++) T.wr[k] = T.fi * a.wi[k] + T.fj * a.wj[k];
  T.vtr[0] = (a.vr[0] - T.vn[0]) + (a.d[1] * T.wr[2] - a.d[2] * T.wr[1]);
  T.vtr[1] = (a.vr[1] - T.vn[1]) + (a.d[2] * T.wr[0] - a.d[0] * T.wr[2]);
  T.vtr[2] = (a.vr[2] - T.vn[2]) + (a.d[0] * T.wr[1] - a.d[1] * T.wr[0]);
  for (int k = 0; k < 3; k++) T.wrel[k] = a.wi[k] - a.wj[k];
  ab_project(T.wrel, en, T.wn);
  for (int k = 0; k < 3; k++) T.wt[k] = T.wrel[k] - T.wn[k];
  T.minvel = 1e-5 * T.rmin / dt;
  const bool damping = (fl & kBondDamping) != 0, smooth = (fl & kBondDampingSmooth) != 0;

  // normal force (:582-636)
  double nfd[3] = {0., 0., 0.};
  T.r0 = hout[1];
  const double disp = T.r0 - r;
  T.disp = disp;
  T.dmax_new = disp > hout[14];
  if (T.dmax_new) { hout[14] = disp; T.dmax = disp; }
  else T.dmax = hout[14];
  T.dmin_new = disp < hout[27];
  if (T.dmin_new) { hout[27] = disp; T.dmin = disp; }
  else T.dmin = hout[27];
  if (disp < 0.0) hout[14] = 0.0;
  if (disp > 0.0) hout[27] = 0.0;
  T.ncomp = ((fl & kBondTension) && disp < -1.e-15) || ((fl & kBondCompression) && disp > 1.e-15);
  T.f = 0.0;
  T.nbr = 0;
  for (int k = 0; k < 3; k++) {
    T.nforce[k] = T.nm[k] = T.tm[k] = 0.0;
    T.nden[k] = T.tden[k] = 1.0;
    T.nclamp[k] = T.tclamp[k] = true;
    T.nden_minvel[k] = T.tden_minvel[k] = true;
    T.brn[k] = T.brt[k] = 0;
    T.hmaxn[k] = T.hminn[k] = T.hmaxt[k] = T.hmint[k] = 0.0;
  }
  if (T.ncomp) {
    const double k1 = P.t[kBondKfn1], ku1 = P.t[kBondKufn1], kc1 = P.t[kBondKcfn1];
    const double k2 = P.t[kBondKfn2], ku2 = P.t[kBondKufn2], kc2 = P.t[kBondKcfn2];
    const double q1 = (ku1 - k1) / (ku1 + kc1);
    const double dc1 = q1 * q1 * T.dmax;
    const double dc2 = (ku2 - k2) / (ku2 + kc2) * T.dmin;
    const double A = T.A, dmax = T.dmax, dmin = T.dmin;
    double f;
    if (disp < dmin) { f = k2 * A * disp; T.nbr = 0; }
    else if (disp < dc2) { f = ku2 * A * disp + (k2 - ku2) * A * dmin; T.nbr = 1; }
    else if (disp < 0.0) { f = -kc2 * A * disp; T.nbr = 2; }
    else if (disp < dc1) { f = -kc1 * sqrt(fabs(disp)); T.nbr = 3; }
    else if (disp < dmax) { f = ku1 * sqrt(fabs(disp)) + (k1 - ku1) * sqrt(fabs(dmax)); T.nbr = 4; }
    else { f = k1 * sqrt(fabs(disp)); T.nbr = 5; }
    T.f = f;
    for (int k = 0; k < 3; k++) T.nforce[k] = f * en[k];
    if (damping) {
      const double dfn = P.t[kBondDampFn];
      for (int k = 0; k < 3; k++) {
        double m;
        if (smooth) {
          const double e = 0.01 * T.nforce[k] * dt;
          T.nden_minvel[k] = !(e > T.minvel);
          T.nden[k] = T.nden_minvel[k] ? T.minvel : e;
          const double q = T.vn[k] / T.nden[k];
          T.nclamp[k] = !(q > -1.0 && q < 1.0);
          m = fmin(1.0, fmax(-1.0, T.vn[k] / fmax(T.minvel, e)));
        } else {
          T.nclamp[k] = true;
          m = ab_sgn(T.vn[k]);
        }
        T.nm[k] = m;
        nfd[k] = T.nforce[k] - dfn * fabs(T.nforce[k]) * m;
      }
    } else {
      for (int k = 0; k < 3; k++) nfd[k] = T.nforce[k];
    }
  }
  // shear force (:639-664)
  for (int k = 0; k < 3; k++) {  // without the shear law ft stays as stored
    T.tfd[k] = 0.0;
    T.ftp[k] = T.ft0[k];
  }
  if (fl & kBondShear) {
    T.sc = -P.t[kBondKft] * T.A * dt;
    double pr[3];
    ab_project(T.ft0, en, pr);
    for (int k = 0; k < 3; k++) T.ftp[k] = (T.ft0[k] - pr[k]) + T.sc * T.vtr[k];
    if (damping) {
      const double dft = P.t[kBondDampFt];
      for (int k = 0; k < 3; k++) {
        double m;
        if (smooth) {
          const double e = 0.01 * T.ftp[k] * dt;
          T.tden_minvel[k] = !(e > T.minvel);
          T.tden[k] = T.tden_minvel[k] ? T.minvel : e;
          const double q = T.vtr[k] / T.tden[k];
          T.tclamp[k] = !(q > -1.0 && q < 1.0);
          m = fmin(1.0, fmax(-1.0, T.vtr[k] / fmax(T.minvel, e)));
        } else {
          T.tclamp[k] = true;
          m = ab_sgn(T.vtr[k]);
        }
        T.tm[k] = m;
        T.tfd[k] = T.ftp[k] - dft * fabs(T.ftp[k]) * m;
      }
    } else {
      for (int k = 0; k < 3; k++) T.tfd[k] = T.ftp[k];
    }
  }
  // twisting torque (:666-771)
  double ntd[3] = {0., 0., 0.};
  for (int c = 0; c < 3; c++) T.tn[c] = 0.0;
  if (fl & kBondNormalTorque) {
    const double k = P.t[kBondKtn], ku = P.t[kBondKutn], kc = P.t[kBondKctn];
    for (int c = 0; c < 3; c++) {
      T.thn1[c] = T.thn1[c] + dt * T.wn[c];
      double hmax = hout[15 + c], hmin = hout[21 + c];
      T.tn[c] = ab_hyst(T.thn1[c], hmax, hmin, k, ku, kc, T.J, T.hmaxn[c], T.hminn[c], T.brn[c]);
      hout[15 + c] = hmax;
      hout[21 + c] = hmin;
    }
    const double dtn = damping ? P.t[kBondDampTn] : 0.0;
    for (int c = 0; c < 3; c++) ntd[c] = damping ? T.tn[c] - dtn * fabs(T.tn[c]) * ab_sgn(T.wn[c]) : T.tn[c];
  }
  // bending torque (:774-873)
  double ttd[3] = {0., 0., 0.};
  for (int c = 0; c < 3; c++) T.tt[c] = 0.0;
  if (fl & kBondShearTorque) {
    const double k = P.t[kBondKtt], ku = P.t[kBondKutt], kc = P.t[kBondKctt];
    for (int c = 0; c < 3; c++) {
      T.tht1[c] = T.tht1[c] + dt * T.wt[c];
      double hmax = hout[18 + c], hmin = hout[24 + c];
      T.tt[c] = ab_hyst(T.tht1[c], hmax, hmin, k, ku, kc, T.I, T.hmaxt[c], T.hmint[c], T.brt[c]);
      hout[18 + c] = hmax;
      hout[24 + c] = hmin;
    }
    const double dtt = damping ? P.t[kBondDampTt] : 0.0;
    for (int c = 0; c < 3; c++) ttd[c] = damping ? T.tt[c] - dtt * fabs(T.tt[c]) * ab_sgn(T.wt[c]) : T.tt[c];
  }
  // stress breakage on undamped values (:876-891)
  if (fl & kBondStressBreak) {
    const double nfm = sqrt(dot3(T.nforce, T.nforce)), tfm = sqrt(dot3(T.ftp, T.ftp));
    const double ntm = sqrt(dot3(T.tn, T.tn)), ttm = sqrt(dot3(T.tt, T.tt));
    const double maxSigma =
        P.t[kBondMaxSigma] * (((fl & kBondUseRatioTC) && disp < -1.e-15) ? P.t[kBondRatioTC] : 1.0);
    const bool nstress = maxSigma < (nfm / T.A + ttm * T.rb / T.I);
    const bool tstress = P.t[kBondMaxTau] < (tfm / T.A + ntm * T.rb / T.J);
    if ((nstress || tstress) && a.upd) {
      hout[0] = 0.0;
      hout[1] = 0.0;
      T.status = kBondBroken;
      return kBondBroken;
    }
  }
  if (a.upd) {
    for (int k = 0; k < 3; k++) {
      hout[5 + k] = T.ftp[k];
      hout[8 + k] = T.thn1[k];
      hout[11 + k] = T.tht1[k];
    }
  }
  cross3(T.tfd, en, T.tor);
  for (int k = 0; k < 3; k++) {
    F[k] = nfd[k] + T.tfd[k];
    Ti[k] = T.cri * T.tor[k] + ntd[k] + ttd[k];
    Tj[k] = T.crj * T.tor[k] - ntd[k] - ttd[k];
  }
  T.status = kBondActive;
  return kBondActive;
}

// adjoint of one hysteresis component: tb = d(loss)/d(torque), hmaxb/hminb
// in: adjoints of the new extremes, out: of the stored ones; returns the
// adjoint of th and adds that of JI
__device__ __forceinline__ double ab_hyst_vjp(double th, double h1max, double h1min, int br, double k, double ku,
                                              double kc, double JI, double tb, double &hmaxb, double &hminb,
                                              double &JIb) {
  double thb = 0.0, h1maxb = 0.0, h1minb = 0.0;
  // new extremes
  if (th > h1max) thb += hmaxb;
  else h1maxb += hmaxb;
  if (th < h1min) thb += hminb;
  else h1minb += hminb;
  switch (br) {
    case 0: thb += -k * JI * tb; JIb += -k * th * tb; break;
    case 1:
      thb += -ku * JI * tb;
      h1maxb += (ku - k) * JI * tb;
      JIb += (-ku * th + (ku - k) * h1max) * tb;
      break;
    case 2: thb += kc * JI * tb; JIb += kc * th * tb; break;
    default:
      thb += -ku * JI * tb;
      h1minb += (ku - k) * JI * tb;
      JIb += (-ku * th + (ku - k) * h1min) * tb;
      break;
  }
  // sign reset
  hmaxb = (th < 0.0) ? 0.0 : h1maxb;
  hminb = (th > 0.0) ? 0.0 : h1minb;
  return thb;
}

// adjoint of the smooth or sign damping  out = x - c|x| m(v, x):
// xb/vb/minvelb receive the adjoints of x, v and minvel
__device__ __forceinline__ void ab_damp_vjp(double x, double v, double c, double m, bool clamp, double den,
                                            bool den_minvel, double dt, double outb, double &xb, double &vb,
                                            double &minvelb) {
  xb += outb * (1.0 - c * ab_sgn(x) * m);
  if (clamp) return;
  const double mb = -c * fabs(x) * outb;
  vb += mb / den;
  const double denb = -mb * v / (den * den);
  if (den_minvel) minvelb += denb;
  else xb += 0.01 * dt * denb;
}

// VJP: Fb/Tib/Tjb the adjoints of the bond's force and torques, houtb those of
// the history after the evaluation; fills ab (input adjoints, overwritten)
// and hinb (history adjoints before the evaluation, overwritten); returns the
// forward's result (kBond*)
__device__ int bond_vjp(const BondArgs &a, const BondPar &P, const double hin[kBondValues], const double Fb[3],
                         const double Tib[3], const double Tjb[3], const double houtb[kBondValues],
                         BondArgsBar &ab, double hinb[kBondValues]) {
  BondTape T;
  double hout[kBondValues], F[3], Ti[3], Tj[3];
  const int st = bond_fwd(a, P, hin, hout, F, Ti, Tj, T);
  for (int k = 0; k < 3; k++) ab.d[k] = ab.vr[k] = ab.wi[k] = ab.wj[k] = 0.0;
  ab.ri = ab.rj = 0.0;
  for (int k = 0; k < kBondValues; k++) hinb[k] = 0.0;
  if (st == kBondNone) {
    for (int k = 0; k < kBondValues; k++) hinb[k] = houtb[k];
    hinb[2] = hinb[3] = hinb[4] = 0.0;
    return st;
  }
  if (!T.evaluated) {  // broken on distance: bondFlag and initial_dist reset
    for (int k = T.created ? 14 : 5; k < kBondValues; k++) hinb[k] = houtb[k];
    return st;
  }
  const int fl = P.flags;
  const double dt = a.dt;
  const double *en = T.en;
  const bool active = st == kBondActive;
  const bool damping = (fl & kBondDamping) != 0, smooth = (fl & kBondDampingSmooth) != 0;
  double enb[3] = {0., 0., 0.}, rbar = 0.0, crib = 0.0, crjb = 0.0, Ab = 0.0, Jb = 0.0, Ib = 0.0;
  double minvelb = 0.0, vnb[3] = {0., 0., 0.}, vtrb[3] = {0., 0., 0.}, wnb[3] = {0., 0., 0.};
  double wtb[3] = {0., 0., 0.}, nfdb[3] = {0., 0., 0.}, tfdb[3] = {0., 0., 0.}, ntdb[3] = {0., 0., 0.};
  double ttdb[3] = {0., 0., 0.};
  // stored ft/thetan/thetat (only when the bond stays and history updates)
  double ftpb[3] = {0., 0., 0.}, thn1b[3] = {0., 0., 0.}, tht1b[3] = {0., 0., 0.};
  if (active && a.upd)
    for (int k = 0; k < 3; k++) {
      ftpb[k] = houtb[5 + k];
      thn1b[k] = houtb[8 + k];
      tht1b[k] = houtb[11 + k];
    }
  else
    for (int k = 5; k < 14; k++) hinb[k] = T.created ? 0.0 : houtb[k];  // passed through unchanged
  if (active) {
    // F = nfd + tfd, Ti = cri tor + ntd + ttd, Tj = crj tor - ntd - ttd, tor = tfd x en
    double torb[3];
    for (int k = 0; k < 3; k++) {
      torb[k] = T.cri * Tib[k] + T.crj * Tjb[k];
      nfdb[k] = Fb[k];
      tfdb[k] = Fb[k];
      ntdb[k] = Tib[k] - Tjb[k];
      ttdb[k] = Tib[k] - Tjb[k];
    }
    crib = dot3(T.tor, Tib);
    crjb = dot3(T.tor, Tjb);
    double c[3];
    cross3(en, torb, c);
    for (int k = 0; k < 3; k++) tfdb[k] += c[k];
    cross3(torb, T.tfd, c);
    for (int k = 0; k < 3; k++) enb[k] += c[k];
  }
  // bending
  if (fl & kBondShearTorque) {
    const double k = P.t[kBondKtt], ku = P.t[kBondKutt], kc = P.t[kBondKctt];
    const double dtt = damping ? P.t[kBondDampTt] : 0.0;
    for (int c = 0; c < 3; c++) {
      const double ttb = damping ? ttdb[c] * (1.0 - dtt * ab_sgn(T.tt[c]) * ab_sgn(T.wt[c])) : ttdb[c];
      double hmaxb = houtb[18 + c], hminb = houtb[24 + c];
      const double thb = ab_hyst_vjp(T.tht1[c], T.hmaxt[c], T.hmint[c], T.brt[c], k, ku, kc, T.I, ttb, hmaxb,
                                     hminb, Ib) + tht1b[c];
      hinb[18 + c] = hmaxb;
      hinb[24 + c] = hminb;
      if (active && a.upd) hinb[11 + c] = thb;
      else if (!T.created) hinb[11 + c] += thb;
      wtb[c] += dt * thb;
    }
  } else {
    for (int c = 0; c < 3; c++) {
      hinb[18 + c] = houtb[18 + c];
      hinb[24 + c] = houtb[24 + c];
      if (active && a.upd && !T.created) hinb[11 + c] = tht1b[c];  // tht' = tht
    }
  }
  // twisting
  if (fl & kBondNormalTorque) {
    const double k = P.t[kBondKtn], ku = P.t[kBondKutn], kc = P.t[kBondKctn];
    const double dtn = damping ? P.t[kBondDampTn] : 0.0;
    for (int c = 0; c < 3; c++) {
      const double tnb = damping ? ntdb[c] * (1.0 - dtn * ab_sgn(T.tn[c]) * ab_sgn(T.wn[c])) : ntdb[c];
      double hmaxb = houtb[15 + c], hminb = houtb[21 + c];
      const double thb = ab_hyst_vjp(T.thn1[c], T.hmaxn[c], T.hminn[c], T.brn[c], k, ku, kc, T.J, tnb, hmaxb,
                                     hminb, Jb) + thn1b[c];
      hinb[15 + c] = hmaxb;
      hinb[21 + c] = hminb;
      if (active && a.upd) hinb[8 + c] = thb;
      else if (!T.created) hinb[8 + c] += thb;
      wnb[c] += dt * thb;
    }
  } else {
    for (int c = 0; c < 3; c++) {
      hinb[15 + c] = houtb[15 + c];
      hinb[21 + c] = houtb[21 + c];
      if (active && a.upd && !T.created) hinb[8 + c] = thn1b[c];
    }
  }
  if (T.created)
    for (int k = 8; k < 14; k++) hinb[k] = 0.0;  // reset at creation: no dependence on hin
  // shear force: ftp = (ft0 - (ft0.en) en) + sc vtr, damped into tfd
  {
    double ft0b[3] = {0., 0., 0.};
    if (fl & kBondShear) {
      double fb[3];
      for (int k = 0; k < 3; k++) fb[k] = ftpb[k];
      if (damping) {
        const double dft = P.t[kBondDampFt];
        for (int k = 0; k < 3; k++)
          ab_damp_vjp(T.ftp[k], T.vtr[k], dft, T.tm[k], T.tclamp[k] || !smooth, T.tden[k], T.tden_minvel[k], dt,
                      tfdb[k], fb[k], vtrb[k], minvelb);
      } else {
        for (int k = 0; k < 3; k++) fb[k] += tfdb[k];
      }
      const double fe = dot3(fb, en), f0e = dot3(T.ft0, en);
      for (int k = 0; k < 3; k++) {
        ft0b[k] = fb[k] - fe * en[k];
        enb[k] += -(f0e * fb[k] + fe * T.ft0[k]);
        vtrb[k] += T.sc * fb[k];
      }
      Ab += -P.t[kBondKft] * dt * dot3(fb, T.vtr);
    } else {
      for (int k = 0; k < 3; k++) ft0b[k] = ftpb[k];  // ft stored unchanged
    }
    if (active && a.upd)
      for (int k = 0; k < 3; k++) hinb[5 + k] = T.created ? 0.0 : ft0b[k];
    else if (!T.created)
      for (int k = 0; k < 3; k++) hinb[5 + k] += ft0b[k];
  }
  // normal force
  double dispb = 0.0, dmaxb = 0.0, dminb = 0.0;
  if (T.ncomp) {
    double nfb[3];
    for (int k = 0; k < 3; k++) nfb[k] = 0.0;
    if (damping) {
      const double dfn = P.t[kBondDampFn];
      for (int k = 0; k < 3; k++) {
        double vdummy = 0.0;
        ab_damp_vjp(T.nforce[k], T.vn[k], dfn, T.nm[k], T.nclamp[k] || !smooth, T.nden[k], T.nden_minvel[k], dt,
                    nfdb[k], nfb[k], vdummy, minvelb);
        vnb[k] += vdummy;
      }
    } else {
      for (int k = 0; k < 3; k++) nfb[k] = nfdb[k];
    }
    const double fb = dot3(nfb, en);
    for (int k = 0; k < 3; k++) enb[k] += T.f * nfb[k];
    const double k1 = P.t[kBondKfn1], ku1 = P.t[kBondKufn1], kc1 = P.t[kBondKcfn1];
    const double k2 = P.t[kBondKfn2], ku2 = P.t[kBondKufn2], kc2 = P.t[kBondKcfn2];
    const double A = T.A, disp = T.disp;
    const double dsq = T.nbr >= 3 ? sqrt(fabs(disp)) : 0.0;
    switch (T.nbr) {
      case 0: dispb += k2 * A * fb; Ab += k2 * disp * fb; break;
      case 1:
        dispb += ku2 * A * fb;
        dminb += (k2 - ku2) * A * fb;
        Ab += (ku2 * disp + (k2 - ku2) * T.dmin) * fb;
        break;
      case 2: dispb += -kc2 * A * fb; Ab += -kc2 * disp * fb; break;
      case 3: dispb += -kc1 * ab_sgn(disp) / (2.0 * dsq) * fb; break;
      case 4:
        dispb += ku1 * ab_sgn(disp) / (2.0 * dsq) * fb;
        dmaxb += (k1 - ku1) * ab_sgn(T.dmax) / (2.0 * sqrt(fabs(T.dmax))) * fb;
        break;
      default: dispb += k1 * ab_sgn(disp) / (2.0 * dsq) * fb; break;
    }
  }
  // extremes of the normal displacement
  dmaxb += (T.disp < 0.0) ? 0.0 : houtb[14];
  dminb += (T.disp > 0.0) ? 0.0 : houtb[27];
  if (T.dmax_new) dispb += dmaxb;
  else hinb[14] = dmaxb;
  if (T.dmin_new) dispb += dminb;
  else hinb[27] = dminb;
  // disp = r0 - r; r0 = r at creation, else initial_dist; stored while bonded
  double r0b = dispb + (active ? houtb[1] : 0.0);
  rbar += -dispb;
  if (T.created) rbar += r0b;
  else hinb[1] = r0b;
  // kinematics
  const double rsi = T.rsi;
  {
    // minvel = 1e-5 rmin / dt
    double rminb = 1e-5 / dt * minvelb;
    // wt = wrel - wn, wn = (wrel.en) en
    double wnt[3], wrelb[3];
    for (int k = 0; k < 3; k++) {
      wnt[k] = wnb[k] - wtb[k];
      wrelb[k] = wtb[k];
    }
    const double we = dot3(T.wrel, en), wbe = dot3(wnt, en);
    for (int k = 0; k < 3; k++) {
      wrelb[k] += wbe * en[k];
      enb[k] += we * wnt[k] + wbe * T.wrel[k];
      ab.wi[k] += wrelb[k];
      ab.wj[k] -= wrelb[k];
    }
    // vtr = (vr - vn) + d x wr
    double vnt[3], c[3], wrb[3];
    for (int k = 0; k < 3; k++) {
      ab.vr[k] += vtrb[k];
      vnt[k] = vnb[k] - vtrb[k];
    }
    cross3(T.wr, vtrb, c);
    for (int k = 0; k < 3; k++) ab.d[k] += c[k];
    cross3(vtrb, a.d, wrb);
    // wr = fi wi + fj wj
    for (int k = 0; k < 3; k++) {
      ab.wi[k] += T.fi * wrb[k];
      ab.wj[k] += T.fj * wrb[k];
    }
    const double fib = dot3(a.wi, wrb), fjb = dot3(a.wj, wrb);
    // vn = (vr.en) en
    const double ve = dot3(a.vr, en), vbe = dot3(vnt, en);
    for (int k = 0; k < 3; k++) {
      ab.vr[k] += vbe * en[k];
      enb[k] += ve * vnt[k] + vbe * a.vr[k];
    }
    // cri = r ri rsi, crj = r rj rsi, fi = ri rsi, fj = rj rsi
    rbar += crib * a.ri * rsi + crjb * a.rj * rsi;
    ab.ri += crib * T.r * rsi + fib * rsi;
    ab.rj += crjb * T.r * rsi + fjb * rsi;
    const double rsib = crib * T.r * a.ri + crjb * T.r * a.rj + fib * a.ri + fjb * a.rj;
    ab.ri += -rsib * rsi * rsi;
    ab.rj += -rsib * rsi * rsi;
    // I = J/2, J = A rb^2/2, A = pi rb^2, rb = lambda rmin
    Jb += 0.5 * Ib;
    Ab += 0.5 * T.rb * T.rb * Jb;
    const double rbb = T.A * T.rb * Jb + 2.0 * 3.14159265358979323846 * T.rb * Ab;
    rminb += P.t[kBondLambda] * rbb;
    if (a.ri < a.rj) ab.ri += rminb;
    else ab.rj += rminb;
    // en = d / r, r = |d|
    const double rinvb = dot3(a.d, enb);
    rbar += -rinvb * T.rinv * T.rinv;
    for (int k = 0; k < 3; k++) ab.d[k] += T.rinv * enb[k] + rbar * a.d[k] * T.rinv;
  }
  return st;
}

}  // namespace gb300
