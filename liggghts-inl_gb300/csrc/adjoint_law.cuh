// Reverse mode (vector-Jacobian product) of the Hertz + tangential-history
// contact law for one pair or one primitive-wall contact, as device code.
//
// Forward law: the same equations as contact_law.cuh (NormalModel<HERTZ>,
// TangentialModel<TANGENTIAL_HISTORY>, SurfaceModel<SURFACE_DEFAULT>;
// src/normal_model_hertz.h:205-408, src/tangential_model_history.h:135-439,
// src/surface_model_default.h:146-211), written out in the form the
// adjoint needs:
//   en = d/|d|, deltan = radsum - |d|, vn = vr.en, vt = vr - vn en,
//   cri = ri - deltan/2, crj = rj - deltan/2,
//   wr = (cri wi + crj wj)/|d|, vtr = vt + d x wr,
//   sv = sqrt(reff deltan), q = sqrt(sv), kn = 4/3 Y sv, kt = 8 G sv,
//   gamma_n = K beta sqrt(2 Y meff) q, gamma_t = K beta sqrt(8 G meff) q,
//   Fn = kn deltan - gamma_n vn,
//   s1 = shear + dt vtr, s2 = s1 - (s1.en) en          (update_history)
//   sliding (kt^2 |s2|^2 > (mu|Fn|)^2): Ft = -mu|Fn| s2/|s2|, s3 = (mu|Fn|/kt) s2/|s2|
//   else: Ft = -kt s2 - gamma_t vtr, s3 = s2
//   F = Fn en + Ft, Ti = -cri (en x Ft), Tj = -crj (en x Ft)
// With CDT rolling friction (RollingModel<ROLLING_CDT>, src/rolling_model_cdt.h:
// 89-167): w = wi - wj (walls: wr), rt = mur kn deltan reff w/|w| projected
// off en, Ti -= rt, Tj += rt (w = 0: none).
// For a bonded pair the bond's force replaces Fn en (src/contact_models.h:
// 228-238): F = Ft here, Fn still caps the friction.
// Walls: radsum = reff = ri, meff = mi, no j terms.  Without
// update_history (the setup force pass) s2 = shear.
// The adjoint is exact for this piecewise-smooth law away from its switch
// points (touching/sliding transitions).
#pragma once

namespace gb300 {

struct VjpIn {
  double d[3], vr[3], wi[3], wj[3], sh[3];
  double ri, rj, mi, mj;
  double Y, G, beta, mu, dt;
  bool upd;     // update_history
  bool wall;
  bool bonded;  // a bond (cohesion bond/nonlinear) replaces the normal force
  bool rolling;  // CDT rolling friction with coefficient mur
  double mur;
};

struct VjpBar {  // adjoints of the outputs (in) and of the inputs (out)
  double F[3], Ti[3], Tj[3], s3[3];
  double d[3], vr[3], wi[3], wj[3], sh[3];
  double ri, rj, mi, mj, Y, G, beta, mu, mur;
};

__device__ __forceinline__ void cross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// Forward values of the law (also used by the forward kernels of the
// adjoint engine so that both sides share one formulation).
struct LawState {
  double r, rinv, en[3], radsum, deltan, vn, vt[3], cri, crj, wsum[3], wr[3], vtr[3];
  double reff, meff, sv, q, kn, kt, c0, c1, gn, gt, Fn, s1[3], rsht, s2[3], ss, Ffr, u, shat[3];
  double Ft[3], tor[3];
  bool slide;
  double rw[3], rwsq, rfac;  // rolling: relative spin, |w|^2, mur kn deltan reff / |w|
};

// ROLL = false compiles the rolling part out (kernels of systems without it)
template <bool ROLL = true>
__device__ __forceinline__ void law_forward(const VjpIn &a, LawState &S, double F[3], double Ti[3],
                                            double Tj[3], double s3[3]) {
  const double K = -2.0 * 0.91287092917527685576161630466800355658790782499663875;
  const double rsq = dot3(a.d, a.d);
  S.r = sqrt(rsq);
  S.rinv = 1.0 / S.r;
  for (int k = 0; k < 3; k++) S.en[k] = a.d[k] * S.rinv;
  S.radsum = a.wall ? a.ri : a.ri + a.rj;
  S.deltan = S.radsum - S.r;
  S.vn = dot3(a.vr, S.en);
  for (int k = 0; k < 3; k++) S.vt[k] = a.vr[k] - S.vn * S.en[k];
  S.cri = a.ri - 0.5 * S.deltan;
  S.crj = a.wall ? 0.0 : a.rj - 0.5 * S.deltan;
  for (int k = 0; k < 3; k++) {
    S.wsum[k] = S.cri * a.wi[k] + (a.wall ? 0.0 : S.crj * a.wj[k]);
    S.wr[k] = S.wsum[k] * S.rinv;
  }
  double c[3];
  cross3(a.d, S.wr, c);
  for (int k = 0; k < 3; k++) S.vtr[k] = S.vt[k] + c[k];
  S.reff = a.wall ? a.ri : a.ri * a.rj / (a.ri + a.rj);
  S.meff = a.wall ? a.mi : a.mi * a.mj / (a.mi + a.mj);
  S.sv = sqrt(S.reff * S.deltan);
  S.q = sqrt(S.sv);
  S.kn = 4.0 / 3.0 * a.Y * S.sv;
  S.kt = 8.0 * a.G * S.sv;
  S.c0 = K * a.beta * sqrt(2.0 * a.Y * S.meff);
  S.c1 = K * a.beta * sqrt(8.0 * a.G * S.meff);
  S.gn = S.c0 * S.q;
  S.gt = S.c1 * S.q;
  S.Fn = S.kn * S.deltan - S.gn * S.vn;
  if (a.upd) {
    for (int k = 0; k < 3; k++) S.s1[k] = a.sh[k] + S.vtr[k] * a.dt;
    S.rsht = dot3(S.s1, S.en);
    for (int k = 0; k < 3; k++) S.s2[k] = S.s1[k] - S.rsht * S.en[k];
  } else {
    for (int k = 0; k < 3; k++) S.s1[k] = S.s2[k] = a.sh[k];
    S.rsht = 0.0;
  }
  S.ss = dot3(S.s2, S.s2);
  S.Ffr = a.mu * fabs(S.Fn);
  S.slide = S.kt * S.kt * S.ss > S.Ffr * S.Ffr;
  if (S.slide) {
    S.u = sqrt(S.ss);
    for (int k = 0; k < 3; k++) {
      S.shat[k] = S.s2[k] / S.u;
      S.Ft[k] = -S.Ffr * S.shat[k];
      s3[k] = a.upd ? S.Ffr / S.kt * S.shat[k] : a.sh[k];
    }
  } else {
    S.u = 0.0;
    for (int k = 0; k < 3; k++) {
      S.shat[k] = 0.0;
      S.Ft[k] = -S.kt * S.s2[k] - S.gt * S.vtr[k];
      s3[k] = S.s2[k];
    }
  }
  cross3(S.en, S.Ft, S.tor);
  for (int k = 0; k < 3; k++) {
    F[k] = (a.bonded ? 0.0 : S.Fn * S.en[k]) + S.Ft[k];
    Ti[k] = -S.cri * S.tor[k];
    Tj[k] = -S.crj * S.tor[k];
  }
  S.rwsq = 0.0;
  if (ROLL && a.rolling) {
    for (int k = 0; k < 3; k++) S.rw[k] = a.wall ? S.wr[k] : a.wi[k] - a.wj[k];
    S.rwsq = dot3(S.rw, S.rw);
    if (S.rwsq > 0.) {
      S.rfac = a.mur * S.kn * S.deltan * S.reff / sqrt(S.rwsq);
      const double we = dot3(S.rw, S.en);
      for (int k = 0; k < 3; k++) {
        const double rt = S.rfac * (S.rw[k] - we * S.en[k]);
        Ti[k] -= rt;
        Tj[k] += rt;
      }
    }
  }
}

// b.F/Ti/Tj/s3 hold the output adjoints; fills the input adjoints of b.
template <bool ROLL = true>
__device__ void law_vjp(const VjpIn &a, VjpBar &b) {
  const double K = -2.0 * 0.91287092917527685576161630466800355658790782499663875;
  LawState S;
  double F[3], Ti[3], Tj[3], s3[3];
  law_forward<ROLL>(a, S, F, Ti, Tj, s3);
  double torb[3], enb[3], Ftb[3], tmp[3];
  // rolling friction (the last forward operation): rt = rfac (w - (w.en) en)
  double rwb[3] = {0., 0., 0.}, renb[3] = {0., 0., 0.};
  double knb_r = 0.0, deltanb_r = 0.0, reffb_r = 0.0, murb = 0.0;
  if (ROLL && a.rolling && S.rwsq > 0.) {
    double rtb[3], pw[3];
    const double we = dot3(S.rw, S.en);
    for (int k = 0; k < 3; k++) {
      rtb[k] = b.Tj[k] - b.Ti[k];
      pw[k] = S.rw[k] - we * S.en[k];
    }
    const double facb = dot3(rtb, pw), rte = dot3(rtb, S.en);
    const double iw = 1.0 / sqrt(S.rwsq);
    for (int k = 0; k < 3; k++) {
      rwb[k] = S.rfac * (rtb[k] - rte * S.en[k]) - facb * S.rfac * S.rw[k] / S.rwsq;
      renb[k] = -S.rfac * (rte * S.rw[k] + we * rtb[k]);
    }
    murb = facb * S.kn * S.deltan * S.reff * iw;
    knb_r = facb * a.mur * S.deltan * S.reff * iw;
    deltanb_r = facb * a.mur * S.kn * S.reff * iw;
    reffb_r = facb * a.mur * S.kn * S.deltan * iw;
  }
  for (int k = 0; k < 3; k++) torb[k] = -S.cri * b.Ti[k] - S.crj * b.Tj[k];
  double crib = -dot3(S.tor, b.Ti), crjb = -dot3(S.tor, b.Tj);
  cross3(S.Ft, torb, enb);
  for (int k = 0; k < 3; k++) enb[k] += renb[k];
  cross3(torb, S.en, Ftb);
  double Fnb = a.bonded ? 0.0 : dot3(b.F, S.en);
  for (int k = 0; k < 3; k++) {
    enb[k] += a.bonded ? 0.0 : S.Fn * b.F[k];
    Ftb[k] += b.F[k];
  }
  double s2b[3] = {0., 0., 0.}, vtrb[3] = {0., 0., 0.};
  double ktb = 0.0, gtb = 0.0, mub = 0.0, shb_direct[3] = {0., 0., 0.};
  if (S.slide) {
    const double s3dot = a.upd ? dot3(b.s3, S.shat) : 0.0;
    const double Ffrb = -dot3(Ftb, S.shat) + s3dot / S.kt;
    ktb += -(S.Ffr / (S.kt * S.kt)) * s3dot;
    double shatb[3];
    for (int k = 0; k < 3; k++) shatb[k] = -S.Ffr * Ftb[k] + (a.upd ? (S.Ffr / S.kt) * b.s3[k] : 0.0);
    const double sd = dot3(shatb, S.shat);
    for (int k = 0; k < 3; k++) s2b[k] += (shatb[k] - sd * S.shat[k]) / S.u;
    mub += fabs(S.Fn) * Ffrb;
    Fnb += a.mu * (S.Fn > 0 ? 1.0 : (S.Fn < 0 ? -1.0 : 0.0)) * Ffrb;
    if (!a.upd)
      for (int k = 0; k < 3; k++) shb_direct[k] = b.s3[k];
  } else {
    for (int k = 0; k < 3; k++) {
      s2b[k] += -S.kt * Ftb[k] + b.s3[k];
      vtrb[k] += -S.gt * Ftb[k];
    }
    ktb += -dot3(S.s2, Ftb);
    gtb += -dot3(S.vtr, Ftb);
  }
  if (a.upd) {
    const double s2e = dot3(s2b, S.en);
    double s1b[3];
    for (int k = 0; k < 3; k++) {
      s1b[k] = s2b[k] - s2e * S.en[k];
      enb[k] += -S.rsht * s2b[k] - s2e * S.s1[k];
      b.sh[k] = s1b[k];
      vtrb[k] += a.dt * s1b[k];
    }
  } else {
    for (int k = 0; k < 3; k++) b.sh[k] = s2b[k] + shb_direct[k];
  }
  const double knb = Fnb * S.deltan + knb_r;
  double deltanb = Fnb * S.kn + deltanb_r;
  const double gnb = -Fnb * S.vn;
  double vnb = -Fnb * S.gn;
  const double c0b = gnb * S.q, c1b = gtb * S.q, qb = gnb * S.c0 + gtb * S.c1;
  double Yb = 4.0 / 3.0 * S.sv * knb, Gb = 8.0 * S.sv * ktb;
  double svb = 4.0 / 3.0 * a.Y * knb + 8.0 * a.G * ktb;
  svb += qb / (2.0 * S.q);
  const double wb = svb / (2.0 * S.sv);
  const double reffb = wb * S.deltan + reffb_r;
  deltanb += wb * S.reff;
  const double betab = c0b * K * sqrt(2.0 * a.Y * S.meff) + c1b * K * sqrt(8.0 * a.G * S.meff);
  Yb += c0b * S.c0 / (2.0 * a.Y);
  Gb += c1b * S.c1 / (2.0 * a.G);
  const double meffb = (c0b * S.c0 + c1b * S.c1) / (2.0 * S.meff);
  double db[3], wrb[3];
  cross3(S.wr, vtrb, db);
  cross3(vtrb, a.d, wrb);
  if (a.wall)  // rolling of a wall contact spins with wr
    for (int k = 0; k < 3; k++) wrb[k] += rwb[k];
  for (int k = 0; k < 3; k++) {
    b.wi[k] = S.cri * S.rinv * wrb[k] + (a.wall ? 0.0 : rwb[k]);
    b.wj[k] = a.wall ? 0.0 : S.crj * S.rinv * wrb[k] - rwb[k];
  }
  crib += S.rinv * dot3(a.wi, wrb);
  if (!a.wall) crjb += S.rinv * dot3(a.wj, wrb);
  double rinvb = dot3(S.wsum, wrb);
  double rib = crib, rjb = a.wall ? 0.0 : crjb;
  deltanb += -0.5 * (crib + (a.wall ? 0.0 : crjb));
  const double vte = dot3(S.en, vtrb);  // vt adjoint is vtrb
  for (int k = 0; k < 3; k++) {
    b.vr[k] = vtrb[k];
    enb[k] += -S.vn * vtrb[k];
  }
  vnb += -vte;
  for (int k = 0; k < 3; k++) {
    b.vr[k] += vnb * S.en[k];
    enb[k] += vnb * a.vr[k];
  }
  double rb = -deltanb;
  rib += deltanb;
  if (!a.wall) rjb += deltanb;
  double mib, mjb;
  if (a.wall) {
    rib += reffb;
    mib = meffb;
    mjb = 0.0;
  } else {
    const double rs = a.ri + a.rj, ms = a.mi + a.mj;
    rib += reffb * a.rj * a.rj / (rs * rs);
    rjb += reffb * a.ri * a.ri / (rs * rs);
    mib = meffb * a.mj * a.mj / (ms * ms);
    mjb = meffb * a.mi * a.mi / (ms * ms);
  }
  for (int k = 0; k < 3; k++) db[k] += S.rinv * enb[k];
  rinvb += dot3(a.d, enb);
  rb += -rinvb * S.rinv * S.rinv;
  for (int k = 0; k < 3; k++) {
    db[k] += rb * a.d[k] * S.rinv;
    b.d[k] = db[k];
  }
  b.ri = rib;
  b.rj = rjb;
  b.mi = mib;
  b.mj = mjb;
  b.Y = Yb;
  b.G = Gb;
  b.beta = betab;
  b.mu = mub;
  b.mur = murb;
  (void)tmp;
}

}  // namespace gb300
