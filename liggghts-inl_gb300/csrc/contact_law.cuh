// FP64 sphere contact law of LIGGGHTS-INL, as device code.
//
//   SurfaceModel<SURFACE_DEFAULT>::surfacesIntersect  src/surface_model_default.h:146-211
//   NormalModel<HERTZ>::surfacesIntersect             src/normal_model_hertz.h:205-408
//   NormalModel<HOOKE>::surfacesIntersect             src/normal_model_hooke.h:230-400
//   TangentialModel<TANGENTIAL_HISTORY>               src/tangential_model_history.h:135-439
//   RollingModel<ROLLING_CDT>                         src/rolling_model_cdt.h:89-167
//
// GB300 has ~1.25 TFLOP/s of FP64, so the law is restated with fewer FP64
// instructions; every change is an algebraic identity and moves results only
// at the rounding level:
//   * Hertz damping: gamma_n = -2 sqrt(5/6) beta sqrt(Sn meff) with
//     Sn = 2 Y sqrt(reff deltan) equals Kn * (reff deltan)^(1/4) with the
//     per-pair constant Kn = -2 sqrt(5/6) beta sqrt(2 Y meff) (likewise Kt
//     with 8 G): one sqrt per contact-step instead of three;
//   * Hooke: kn and gamma_n depend only on the pair (reff, meff, types), so
//     the pow() of the reference is evaluated once per neighbour build;
//   * Coulomb test kt|s| > mu|Fn| on squares; sqrt and division only when
//     the contact slides; shear = -Ft/kt as shear*ratio;
//   * 1/r and 1/|w_roll| as rsqrt;
//   * 4/3 Yeff and 8 Geff from the type table; (cri, crj)/r formed once;
//     the rolling torque folded into the torque products (one rounding
//     fewer).
// The quantities that decide the contact set (rsq, radsum) and the overlap
// deltan = radsum - sqrt(rsq) are formed exactly as in the reference.
#pragma once
#include "dem_device.cuh"

namespace gb300 {

enum { kHertz = 0, kHooke = 1 };

// Per type pair: Yeff, Geff, betaeff, coeffFrict, coeffRollFrict,
// coeffRestLog, and the Hertz stiffness prefactors 4/3 Yeff and 8 Geff
// (formed on the host as the reference forms them inside its law, so kn and
// kt keep their bits).  The table stacks kTypeTables matrices of (nt+1)^2.
constexpr int kTypeTables = 8;

struct TypePair {
  double Y, G, beta, mu, mur, restlog;
  double Y43, G8;
};

__device__ __forceinline__ TypePair load_typepair(const double *__restrict__ params, int nt,
                                                  int it, int jt) {
  const int m = (nt + 1) * (nt + 1);
  const int k = it * (nt + 1) + jt;
  TypePair t;
  t.Y = __ldg(params + k);
  t.G = __ldg(params + m + k);
  t.beta = __ldg(params + 2 * m + k);
  t.mu = __ldg(params + 3 * m + k);
  t.mur = __ldg(params + 4 * m + k);
  t.restlog = __ldg(params + 5 * m + k);
  t.Y43 = __ldg(params + 6 * m + k);
  t.G8 = __ldg(params + 7 * m + k);
  return t;
}

// host side: the two derived matrices from Yeff and Geff
inline void derive_type_tables(int m, double *tab) {
  for (int q = 0; q < m; q++) {
    tab[6 * m + q] = 4. / 3. * tab[q];
    tab[7 * m + q] = 8. * tab[m + q];
  }
}

// Per-pair constants of the normal law.  Hertz: (Kn, Kt) damping prefactors;
// Hooke: (kn, gamma_n) of src/normal_model_hooke.h:272-279.
template <int NORMAL>
__device__ __forceinline__ void contact_consts(const TypePair &tp, double meff, double reff,
                                               double charVel, bool tdamp, double &c0,
                                               double &c1) {
  if (NORMAL == kHertz) {
    const double sqrtFiveOverSix = 0.91287092917527685576161630466800355658790782499663875;
    const double k = -2. * sqrtFiveOverSix * tp.beta;
    c0 = k * sqrt(2. * tp.Y * meff);
    c1 = tdamp ? k * sqrt(8. * tp.G * meff) : 0.0;
  } else {
    const double sqrtval = sqrt(reff);
    const double kn = 16. / 15. * sqrtval * (tp.Y) *
                      pow(15. * meff * charVel * charVel / (16. * sqrtval * tp.Y), 0.2);
    const double lsq = tp.restlog * tp.restlog;
    c0 = kn;
    c1 = sqrt(4. * meff * kn * lsq / (lsq + 9.86960440108935861883 /* M_PI*M_PI */));
  }
}

struct ContactIn {
  double radi, radj, radsum, r, rinv;
  double reff, c0, c1;
  double en[3], d[3];
  double vr[3];          // v_i - v_j
  double wi[3], wj[3];
  double deltan_wall;    // wall: sidata.deltan as passed in (overlap)
};

struct ContactOut {
  double F[3];           // i_forces.delta_F
  double Ti[3];          // i_forces.delta_torque
  double Tj[3];          // j_forces.delta_torque
};

// shear[3] is the tangential history, updated in place when update_history.
// base: forces and torques of a bonded pair (cohesion bond/nonlinear), which
// replace the normal model's force before the tangential and rolling models
// add theirs (src/contact_models.h:228-238); nullptr otherwise.
template <int NORMAL, bool WALL>
__device__ __forceinline__ void contact_law(const ContactIn &c, const TypePair &tp, double dt,
                                            bool tdamp, bool limitf, bool rolling,
                                            bool update_history, double shear[3], ContactOut &o,
                                            const ContactOut *base = nullptr) {
  const double enx = c.en[0], eny = c.en[1], enz = c.en[2];
  // ---- surface model (sphere kinematics)
  const double vr1 = c.vr[0], vr2 = c.vr[1], vr3 = c.vr[2];
  const double vn = vr1 * enx + vr2 * eny + vr3 * enz;
  const double vt1 = vr1 - vn * enx;
  const double vt2 = vr2 - vn * eny;
  const double vt3 = vr3 - vn * enz;
  const double deltan = __dadd_rn(c.radsum, -c.r);
  const double dx = c.d[0], dy = c.d[1], dz = c.d[2];
  double wr1, wr2, wr3, cri, crj = 0.0;
  if (WALL) {
    cri = c.radi - 0.5 * c.deltan_wall;
    const double cr = cri * c.rinv;
    wr1 = cr * c.wi[0];
    wr2 = cr * c.wi[1];
    wr3 = cr * c.wi[2];
  } else {
    cri = c.radi - 0.5 * deltan;
    crj = c.radj - 0.5 * deltan;
    const double ai = cri * c.rinv, aj = crj * c.rinv;
    wr1 = ai * c.wi[0] + aj * c.wj[0];
    wr2 = ai * c.wi[1] + aj * c.wj[1];
    wr3 = ai * c.wi[2] + aj * c.wj[2];
  }
  const double vtr1 = vt1 - (dz * wr2 - dy * wr3);
  const double vtr2 = vt2 - (dx * wr3 - dz * wr1);
  const double vtr3 = vt3 - (dy * wr1 - dx * wr2);

  // ---- normal model
  double kn, kt, gamman, gammat;
  if (NORMAL == kHertz) {
    // sqrt(reff*deltan) and its square root from two reciprocal square
    // roots (x^-1/2, then (x^-1/2)^-1/2 = x^1/4): within an ulp or two of
    // the correctly rounded sqrt, with fewer FP64 instructions and no divide
    // (zero for a contact at zero overlap, as sqrt(0) gives)
    const double xr = c.reff * deltan;
    const bool pos = xr > 0.0;
    const double rs = rsqrt(pos ? xr : 1.0);
    const double sqrtval = pos ? xr * rs : 0.0;
    const double q = pos ? rsqrt(rs) : 0.0;
    kn = tp.Y43 * sqrtval;
    kt = tp.G8 * sqrtval;
    gamman = c.c0 * q;
    gammat = c.c1 * q;
  } else {
    kn = c.c0;
    kt = kn;
    gamman = c.c1;
    gammat = tdamp ? gamman : 0.0;
  }
  double Fn = kn * deltan - gamman * vn;
  if (limitf && Fn < 0.0) Fn = 0.0;

  // ---- tangential history
  double s0 = shear[0], s1 = shear[1], s2 = shear[2];
  if (update_history) {
    s0 += vtr1 * dt;
    s1 += vtr2 * dt;
    s2 += vtr3 * dt;
    const double rsht = s0 * enx + s1 * eny + s2 * enz;
    s0 -= rsht * enx;
    s1 -= rsht * eny;
    s2 -= rsht * enz;
  }
  double Ft1, Ft2, Ft3;
  const double ss = s0 * s0 + s1 * s1 + s2 * s2;
  const double Ft_friction = tp.mu * fabs(Fn);
  const double kt2ss = kt * kt * ss;
  if (kt2ss > Ft_friction * Ft_friction) {
    // sliding (ss > 0 here): cap the spring force at mu|Fn|;
    // mu|Fn| / (kt |shear|) with one reciprocal square root, no divide
    const double ratio = Ft_friction * rsqrt(kt2ss);
    Ft1 = -(kt * s0) * ratio;
    Ft2 = -(kt * s1) * ratio;
    Ft3 = -(kt * s2) * ratio;
    if (update_history) {
      s0 *= ratio;
      s1 *= ratio;
      s2 *= ratio;
    }
  } else {
    Ft1 = -(kt * s0) - gammat * vtr1;
    Ft2 = -(kt * s1) - gammat * vtr2;
    Ft3 = -(kt * s2) - gammat * vtr3;
  }
  if (update_history) {
    shear[0] = s0;
    shear[1] = s1;
    shear[2] = s2;
  }
  const double tor1 = eny * Ft3 - enz * Ft2;
  const double tor2 = enz * Ft1 - enx * Ft3;
  const double tor3 = enx * Ft2 - eny * Ft1;
  // rolling friction, constant directional torque: rt, taken from Ti and
  // given to Tj (folded into their products below)
  double rt1 = 0., rt2 = 0., rt3 = 0.;
  if (rolling) {
    double w1, w2, w3;
    if (WALL) {
      w1 = wr1;
      w2 = wr2;
      w3 = wr3;
    } else {
      w1 = c.wi[0] - c.wj[0];
      w2 = c.wi[1] - c.wj[1];
      w3 = c.wi[2] - c.wj[2];
    }
    const double wsq = w1 * w1 + w2 * w2 + w3 * w3;
    if (__double_as_longlong(wsq) != 0) {  // wsq > 0 (a sum of squares: +0 or positive)
      const double fac = tp.mur * kn * deltan * c.reff * rsqrt(wsq);
      rt1 = fac * w1;
      rt2 = fac * w2;
      rt3 = fac * w3;
      const double rtd = rt1 * enx + rt2 * eny + rt3 * enz;
      rt1 -= enx * rtd;
      rt2 -= eny * rtd;
      rt3 -= enz * rtd;
    }
  }
  if (base) {
    o.F[0] = base->F[0] + Ft1;
    o.F[1] = base->F[1] + Ft2;
    o.F[2] = base->F[2] + Ft3;
    o.Ti[0] = base->Ti[0] + (-cri * tor1 - rt1);
    o.Ti[1] = base->Ti[1] + (-cri * tor2 - rt2);
    o.Ti[2] = base->Ti[2] + (-cri * tor3 - rt3);
    o.Tj[0] = base->Tj[0] + (-crj * tor1 + rt1);
    o.Tj[1] = base->Tj[1] + (-crj * tor2 + rt2);
    o.Tj[2] = base->Tj[2] + (-crj * tor3 + rt3);
  } else {
    o.F[0] = Fn * enx + Ft1;
    o.F[1] = Fn * eny + Ft2;
    o.F[2] = Fn * enz + Ft3;
    o.Ti[0] = -cri * tor1 - rt1;
    o.Ti[1] = -cri * tor2 - rt2;
    o.Ti[2] = -cri * tor3 - rt3;
    o.Tj[0] = -crj * tor1 + rt1;
    o.Tj[1] = -crj * tor2 + rt2;
    o.Tj[2] = -crj * tor3 + rt3;
  }
}

}  // namespace gb300
