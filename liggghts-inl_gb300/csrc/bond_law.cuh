// cohesion bond/nonlinear of LIGGGHTS-INL for one particle pair, as device code.
//
//   CohesionModel<COHESION_BOND_NONLINEAR>::surfacesClose
//       src/cohesion_model_bond_nonlinear.h:394-940
//   createBondnonlinear / breakBondnonlinear                :961-992
//
// The model bonds a pair at step tsCreateBondnonlinear (or always) when the
// centres are closer than createDistanceBondnonlinear, then applies a
// piecewise elastoplastic normal force (sqrt law in compression, linear in
// tension, with loading/unloading/reverse stiffnesses K/Ku/Kc), an
// incremental shear force, and hysteretic twisting and bending torques, all
// with optional sign damping.  It breaks on distance or on stress.  A bonded
// pair's force REPLACES the normal model's; the tangential and rolling models
// then add theirs.
//
// The decisions that change the pair's state (creation distance, simple
// breakage distance, bondFlag) use r = sqrt(rsq), with rsq formed exactly, so
// bond topology is decided as in the reference.  The projection of the
// elastic twisting/bending torque that the reference forms before the
// component-wise hysteresis law overwrites it (:673-674, :788-789) has no
// effect and is not computed.
#pragma once
#include "contact_law.cuh"
#include "dem_device.cuh"

namespace gb300 {

struct BondIn {
  double d[3];          // x_i - x_j (image)
  double rsq;
  double radi, radj;
  double vi[3], vj[3], wi[3], wj[3];
  double xi[3];
  int tp;               // type-pair index it*(nt+1)+jt
};

__device__ __forceinline__ double bond_tab(const Sys &s, int table, int tp) {
  return __ldg(s.bondp + (size_t)table * (s.ntypes + 1) * (s.ntypes + 1) + tp);
}

__device__ __forceinline__ double sgn_d(double v) { return (double)((0.0 < v) - (v < 0.0)); }

// vectorProject3D (src/vector_liggghts.h:437-442) onto `on`, given `on`
// normalised as that function normalises it (n = on/|on|, 0 for on = 0);
// the model projects three vectors onto the same en, so the normalisation
// is formed once (same operations, same bits)
__device__ __forceinline__ void project3_n(const double v[3], const double n[3], double out[3]) {
  const double dot = v[0] * n[0] + v[1] * n[1] + v[2] * n[2];
  out[0] = dot * n[0];
  out[1] = dot * n[1];
  out[2] = dot * n[2];
}

// one component of the hysteretic twisting/bending law (:677-761, :792-866);
// ratio = (ku - k)/(ku + kc), precomputed per type pair
__device__ __forceinline__ double bond_hyst(double th, double &hmax, double &hmin, double k, double ku,
                                            double kc, double ratio, double JI) {
  if (th > 0.0) hmin = 0.0;
  else if (th < 0.0) hmax = 0.0;
  const double c1 = ratio * hmax, c2 = ratio * hmin;
  double t;
  if ((th >= hmax) || (th <= hmin)) t = -k * JI * th;
  else if (th > c1) t = -ku * JI * th + (ku - k) * JI * hmax;
  else if (th >= c2) t = kc * JI * th;
  else t = -ku * JI * th + (ku - k) * JI * hmin;
  if (th > hmax) hmax = th;
  if (th < hmin) hmin = th;
  return t;
}

// h points at the pair's bond value 0 (device history d = 3); hs is the
// stride between values.  Returns true when the pair is bonded and its
// forces (o) replace the normal model's.
__device__ bool bond_nonlinear(const Sys &s, const BondIn &b, double *h, size_t hs, int *flag,
                               bool update_history, long long ntimestep, ContactOut &o) {
  const int tp = b.tp;
  const double lambda = bond_tab(s, kBondLambda, tp);
  if (lambda < 1.e-15) return false;
  const int fl = s.bond_flags;
  const double r = sqrt(b.rsq);
  if (update_history) {
    if (h[0] < 1.e-15) {
      const bool create = ((fl & kBondCreateAlways) || ntimestep == s.bond_ts_create) &&
                          (r < bond_tab(s, kBondCreateDist, tp));
      if (!create) return false;
      *flag |= kContactCohesion;  // createBondnonlinear
      h[0] = 1.0;
      h[hs] = r;
      for (int k = 0; k < 3; k++) h[(2 + k) * hs] = __dadd_rn(b.xi[k], -b.d[k]);
      for (int k = 5; k < 14; k++) h[k * hs] = 0.0;
    }
  } else if (h[0] < 1.e-15) {
    return false;
  }
  if (!(fl & kBondStressBreak) && r > bond_tab(s, kBondMaxDist, tp) && update_history) {
    *flag &= ~kContactCohesion;  // breakBondnonlinear
    h[0] = 0.;
    h[hs] = 0.;
    return false;
  }
  *flag |= kContactCohesion;
  double ft[3] = {h[5 * hs], h[6 * hs], h[7 * hs]};
  double thn[3] = {h[8 * hs], h[9 * hs], h[10 * hs]};
  double tht[3] = {h[11 * hs], h[12 * hs], h[13 * hs]};
  const double rinv = 1. / r;
  const double en[3] = {rinv * b.d[0], rinv * b.d[1], rinv * b.d[2]};
  double enn[3];
  {
    const double norm = sqrt(en[0] * en[0] + en[1] * en[1] + en[2] * en[2]);
    const double inv = (norm == 0.) ? 0. : 1. / norm;
    enn[0] = en[0] * inv;
    enn[1] = en[1] * inv;
    enn[2] = en[2] * inv;
  }
  const double radi = b.radi, radj = b.radj;
  const double rmin = radi < radj ? radi : radj;
  const double rb = lambda * rmin;
  const double A = 3.14159265358979323846 * rb * rb;
  const double J = 0.5 * A * rb * rb;
  const double I = 0.5 * J;
  const double dt = s.dt;
  const double radsuminv = 1. / (radi + radj);
  const double cri = r * radi * radsuminv;
  const double crj = r * radj * radsuminv;
  // relative velocities (:518-545)
  const double vr[3] = {b.vi[0] - b.vj[0], b.vi[1] - b.vj[1], b.vi[2] - b.vj[2]};
  double vn[3];
  project3_n(vr, enn, vn);
  const double fi_ = radi * radsuminv, fj_ = radj * radsuminv;
  const double wr[3] = {fi_ * b.wi[0] + fj_ * b.wj[0], fi_ * b.wi[1] + fj_ * b.wj[1],
                        fi_ * b.wi[2] + fj_ * b.wj[2]};
  const double vtr[3] = {(vr[0] - vn[0]) + (b.d[1] * wr[2] - b.d[2] * wr[1]),
                         (vr[1] - vn[1]) + (b.d[2] * wr[0] - b.d[0] * wr[2]),
                         (vr[2] - vn[2]) + (b.d[0] * wr[1] - b.d[1] * wr[0])};
  const double wrel[3] = {b.wi[0] - b.wj[0], b.wi[1] - b.wj[1], b.wi[2] - b.wj[2]};
  double wn[3];
  project3_n(wrel, enn, wn);
  const double wt[3] = {wrel[0] - wn[0], wrel[1] - wn[1], wrel[2] - wn[2]};
  const double minvel = 1e-5 * rmin / dt;
  const bool damping = (fl & kBondDamping) != 0, smooth = (fl & kBondDampingSmooth) != 0;

  // normal force (:582-636)
  double nforce[3] = {0., 0., 0.}, nfd[3] = {0., 0., 0.};
  const double disp = h[hs] - r;
  double dmax, dmin;
  if (disp > h[14 * hs]) { h[14 * hs] = disp; dmax = disp; }
  else dmax = h[14 * hs];
  if (disp < h[27 * hs]) { h[27 * hs] = disp; dmin = disp; }
  else dmin = h[27 * hs];
  if (disp < 0.0) h[14 * hs] = 0.0;
  if (disp > 0.0) h[27 * hs] = 0.0;
  if (((fl & kBondTension) && disp < -1.e-15) || ((fl & kBondCompression) && disp > 1.e-15)) {
    const double k1 = bond_tab(s, kBondKfn1, tp), ku1 = bond_tab(s, kBondKufn1, tp);
    const double kc1 = bond_tab(s, kBondKcfn1, tp), k2 = bond_tab(s, kBondKfn2, tp);
    const double ku2 = bond_tab(s, kBondKufn2, tp), kc2 = bond_tab(s, kBondKcfn2, tp);
    const double q1 = bond_tab(s, kBondRatioFn1, tp);
    const double dc1 = q1 * q1 * dmax;
    const double dc2 = bond_tab(s, kBondRatioFn2, tp) * dmin;
    double f;
    if (disp < dmin) f = k2 * A * disp;
    else if (disp < dc2) f = ku2 * A * disp + (k2 - ku2) * A * dmin;
    else if (disp < 0.0) f = -kc2 * A * disp;
    else if (disp < dc1) f = -kc1 * sqrt(fabs(disp));
    else if (disp < dmax) f = ku1 * sqrt(fabs(disp)) + (k1 - ku1) * sqrt(fabs(dmax));
    else f = k1 * sqrt(fabs(disp));
    for (int k = 0; k < 3; k++) nforce[k] = f * en[k];
    if (damping) {
      const double dfn = bond_tab(s, kBondDampFn, tp);
      for (int k = 0; k < 3; k++) {
        const double m = smooth ? fmin(1.0, fmax(-1.0, vn[k] / fmax(minvel, 0.01 * nforce[k] * dt))) : sgn_d(vn[k]);
        nfd[k] = nforce[k] - dfn * fabs(nforce[k]) * m;
      }
    } else {
      for (int k = 0; k < 3; k++) nfd[k] = nforce[k];
    }
  }
  // shear force (:639-664)
  double tfd[3] = {0., 0., 0.};
  if (fl & kBondShear) {
    const double sc = -bond_tab(s, kBondKft, tp) * A * dt;
    double pr[3];
    project3_n(ft, enn, pr);
    for (int k = 0; k < 3; k++) ft[k] = (ft[k] - pr[k]) + sc * vtr[k];
    if (damping) {
      const double dft = bond_tab(s, kBondDampFt, tp);
      for (int k = 0; k < 3; k++) {
        const double m = smooth ? fmin(1.0, fmax(-1.0, vtr[k] / fmax(minvel, 0.01 * ft[k] * dt))) : sgn_d(vtr[k]);
        tfd[k] = ft[k] - dft * fabs(ft[k]) * m;
      }
    } else {
      for (int k = 0; k < 3; k++) tfd[k] = ft[k];
    }
  }
  // twisting torque (:666-771)
  double tn[3] = {0., 0., 0.}, ntd[3] = {0., 0., 0.};
  if (fl & kBondNormalTorque) {
    const double k = bond_tab(s, kBondKtn, tp), ku = bond_tab(s, kBondKutn, tp), kc = bond_tab(s, kBondKctn, tp);
    const double ratio = bond_tab(s, kBondRatioTn, tp);
    for (int c = 0; c < 3; c++) {
      thn[c] = thn[c] + dt * wn[c];
      double hmax = h[(15 + c) * hs], hmin = h[(21 + c) * hs];
      tn[c] = bond_hyst(thn[c], hmax, hmin, k, ku, kc, ratio, J);
      h[(15 + c) * hs] = hmax;
      h[(21 + c) * hs] = hmin;
    }
    const double dtn = damping ? bond_tab(s, kBondDampTn, tp) : 0.0;
    for (int c = 0; c < 3; c++) ntd[c] = damping ? tn[c] - dtn * fabs(tn[c]) * sgn_d(wn[c]) : tn[c];
  }
  // bending torque (:774-873)
  double tt[3] = {0., 0., 0.}, ttd[3] = {0., 0., 0.};
  if (fl & kBondShearTorque) {
    const double k = bond_tab(s, kBondKtt, tp), ku = bond_tab(s, kBondKutt, tp), kc = bond_tab(s, kBondKctt, tp);
    const double ratio = bond_tab(s, kBondRatioTt, tp);
    for (int c = 0; c < 3; c++) {
      tht[c] = tht[c] + dt * wt[c];
      double hmax = h[(18 + c) * hs], hmin = h[(24 + c) * hs];
      tt[c] = bond_hyst(tht[c], hmax, hmin, k, ku, kc, ratio, I);
      h[(18 + c) * hs] = hmax;
      h[(24 + c) * hs] = hmin;
    }
    const double dtt = damping ? bond_tab(s, kBondDampTt, tp) : 0.0;
    for (int c = 0; c < 3; c++) ttd[c] = damping ? tt[c] - dtt * fabs(tt[c]) * sgn_d(wt[c]) : tt[c];
  }
  // stress breakage on undamped values (:876-891)
  if (fl & kBondStressBreak) {
    const double nfm = sqrt(nforce[0] * nforce[0] + nforce[1] * nforce[1] + nforce[2] * nforce[2]);
    const double tfm = sqrt(ft[0] * ft[0] + ft[1] * ft[1] + ft[2] * ft[2]);
    const double ntm = sqrt(tn[0] * tn[0] + tn[1] * tn[1] + tn[2] * tn[2]);
    const double ttm = sqrt(tt[0] * tt[0] + tt[1] * tt[1] + tt[2] * tt[2]);
    const double maxSigma = bond_tab(s, kBondMaxSigma, tp) *
                            (((fl & kBondUseRatioTC) && disp < -1.e-15) ? bond_tab(s, kBondRatioTC, tp) : 1.0);
    const bool nstress = maxSigma < (nfm / A + ttm * rb / I);
    const bool tstress = bond_tab(s, kBondMaxTau, tp) < (tfm / A + ntm * rb / J);
    if ((nstress || tstress) && update_history) {
      *flag &= ~kContactCohesion;
      h[0] = 0.;
      h[hs] = 0.;
      return false;
    }
  }
  if (update_history) {
    for (int k = 0; k < 3; k++) {
      h[(5 + k) * hs] = ft[k];
      h[(8 + k) * hs] = thn[k];
      h[(11 + k) * hs] = tht[k];
    }
  }
  const double tor[3] = {tfd[1] * en[2] - tfd[2] * en[1], tfd[2] * en[0] - tfd[0] * en[2],
                         tfd[0] * en[1] - tfd[1] * en[0]};
  for (int k = 0; k < 3; k++) {
    o.F[k] = nfd[k] + tfd[k];
    o.Ti[k] = cri * tor[k] + ntd[k] + ttd[k];
    o.Tj[k] = crj * tor[k] - ntd[k] - ttd[k];
  }
  return true;
}

}  // namespace gb300
