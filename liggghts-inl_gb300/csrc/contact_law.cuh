// FP64 sphere contact law of LIGGGHTS-INL, as device code.
//
//   SurfaceModel<SURFACE_DEFAULT>::surfacesIntersect  src/surface_model_default.h:146-211
//   NormalModel<HERTZ>::surfacesIntersect             src/normal_model_hertz.h:205-408
//   NormalModel<HOOKE>::surfacesIntersect             src/normal_model_hooke.h:230-400
//   TangentialModel<TANGENTIAL_HISTORY>               src/tangential_model_history.h:135-439
//   RollingModel<ROLLING_CDT>                         src/rolling_model_cdt.h:89-167
//
// The expressions keep the reference's operand order; FMA contraction is left
// to the compiler here (it changes results at the rounding level only).  The
// inputs that decide the contact set (rsq, radsum) are formed by the callers
// with explicit round-to-nearest intrinsics, bit-identical to the reference.
#pragma once
#include "dem_device.cuh"

namespace gb300 {

enum { kHertz = 0, kHooke = 1 };

struct TypePair {
  double Y, G, beta, mu, mur, restlog;
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
  return t;
}

struct ContactIn {
  double radi, radj, radsum, r, rinv, meff, reff;
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
template <int NORMAL, bool WALL>
__device__ __forceinline__ void contact_law(const ContactIn &c, const TypePair &tp, double dt,
                                            double charVel, bool tdamp, bool limitf, bool rolling,
                                            bool update_history, double shear[3], ContactOut &o) {
  const double enx = c.en[0], eny = c.en[1], enz = c.en[2];
  // ---- surface model (sphere kinematics)
  const double vr1 = c.vr[0], vr2 = c.vr[1], vr3 = c.vr[2];
  const double vn = vr1 * enx + vr2 * eny + vr3 * enz;
  const double vt1 = vr1 - vn * enx;
  const double vt2 = vr2 - vn * eny;
  const double vt3 = vr3 - vn * enz;
  const double deltan = c.radsum - c.r;
  const double dx = c.d[0], dy = c.d[1], dz = c.d[2];
  double wr1, wr2, wr3, cri, crj = 0.0;
  if (WALL) {
    cri = c.radi - 0.5 * c.deltan_wall;
    wr1 = cri * c.wi[0] * c.rinv;
    wr2 = cri * c.wi[1] * c.rinv;
    wr3 = cri * c.wi[2] * c.rinv;
  } else {
    cri = c.radi - 0.5 * deltan;
    crj = c.radj - 0.5 * deltan;
    wr1 = (cri * c.wi[0] + crj * c.wj[0]) * c.rinv;
    wr2 = (cri * c.wi[1] + crj * c.wj[1]) * c.rinv;
    wr3 = (cri * c.wi[2] + crj * c.wj[2]) * c.rinv;
  }
  const double vtr1 = vt1 - (dz * wr2 - dy * wr3);
  const double vtr2 = vt2 - (dx * wr3 - dz * wr1);
  const double vtr3 = vt3 - (dy * wr1 - dx * wr2);

  // ---- normal model
  const double reff = c.reff;
  const double meff = c.meff;
  double kn, kt, gamman, gammat;
  if (NORMAL == kHertz) {
    const double sqrtval = sqrt(reff * deltan);
    const double Sn = 2. * tp.Y * sqrtval;
    const double St = 8. * tp.G * sqrtval;
    kn = 4. / 3. * tp.Y * sqrtval;
    kt = St;
    const double sqrtFiveOverSix = 0.91287092917527685576161630466800355658790782499663875;
    gamman = -2. * sqrtFiveOverSix * tp.beta * sqrt(Sn * meff);
    gammat = tdamp ? -2. * sqrtFiveOverSix * tp.beta * sqrt(St * meff) : 0.0;
  } else {
    const double sqrtval = sqrt(reff);
    kn = 16. / 15. * sqrtval * (tp.Y) *
         pow(15. * meff * charVel * charVel / (16. * sqrtval * tp.Y), 0.2);
    kt = kn;
    const double lsq = tp.restlog * tp.restlog;
    gamman = sqrt(4. * meff * kn * lsq / (lsq + 9.86960440108935861883 /* M_PI*M_PI */));
    gammat = tdamp ? gamman : 0.0;
  }
  const double Fn_damping = -gamman * vn;
  const double Fn_contact = kn * deltan;
  double Fn = Fn_damping + Fn_contact;
  if (limitf && Fn < 0.0) Fn = 0.0;
  double F1 = Fn * enx, F2 = Fn * eny, F3 = Fn * enz;

  // ---- tangential history
  if (update_history) {
    shear[0] += vtr1 * dt;
    shear[1] += vtr2 * dt;
    shear[2] += vtr3 * dt;
    const double rsht = shear[0] * enx + shear[1] * eny + shear[2] * enz;
    shear[0] -= rsht * enx;
    shear[1] -= rsht * eny;
    shear[2] -= rsht * enz;
  }
  const double shrmag = sqrt(shear[0] * shear[0] + shear[1] * shear[1] + shear[2] * shear[2]);
  double Ft1 = -(kt * shear[0]);
  double Ft2 = -(kt * shear[1]);
  double Ft3 = -(kt * shear[2]);
  const double Ft_shear = kt * shrmag;
  const double Ft_friction = tp.mu * fabs(Fn);
  if (Ft_shear > Ft_friction) {
    if (shrmag != 0.0) {
      const double ratio = Ft_friction / Ft_shear;
      Ft1 *= ratio;
      Ft2 *= ratio;
      Ft3 *= ratio;
      if (update_history) {
        shear[0] = -Ft1 / kt;
        shear[1] = -Ft2 / kt;
        shear[2] = -Ft3 / kt;
      }
    } else {
      Ft1 = Ft2 = Ft3 = 0.0;
    }
  } else {
    Ft1 -= gammat * vtr1;
    Ft2 -= gammat * vtr2;
    Ft3 -= gammat * vtr3;
  }
  const double tor1 = eny * Ft3 - enz * Ft2;
  const double tor2 = enz * Ft1 - enx * Ft3;
  const double tor3 = enx * Ft2 - eny * Ft1;
  o.F[0] = F1 + Ft1;
  o.F[1] = F2 + Ft2;
  o.F[2] = F3 + Ft3;
  o.Ti[0] = -cri * tor1;
  o.Ti[1] = -cri * tor2;
  o.Ti[2] = -cri * tor3;
  o.Tj[0] = -crj * tor1;
  o.Tj[1] = -crj * tor2;
  o.Tj[2] = -crj * tor3;

  // ---- rolling friction, constant directional torque
  if (rolling) {
    double rt1 = 0., rt2 = 0., rt3 = 0.;
    if (WALL) {
      const double wrmag = sqrt(wr1 * wr1 + wr2 * wr2 + wr3 * wr3);
      if (wrmag > 0.) {
        const double Fnr = deltan * kn;
        rt1 = tp.mur * Fnr * wr1 / wrmag * reff;
        rt2 = tp.mur * Fnr * wr2 / wrmag * reff;
        rt3 = tp.mur * Fnr * wr3 / wrmag * reff;
        const double rtd = rt1 * enx + rt2 * eny + rt3 * enz;
        rt1 -= enx * rtd;
        rt2 -= eny * rtd;
        rt3 -= enz * rtd;
      }
    } else {
      const double w1 = c.wi[0] - c.wj[0], w2 = c.wi[1] - c.wj[1], w3 = c.wi[2] - c.wj[2];
      const double wmag = sqrt(w1 * w1 + w2 * w2 + w3 * w3);
      if (wmag > 0.) {
        const double fac = tp.mur * kn * deltan * reff / wmag;
        rt1 = fac * w1;
        rt2 = fac * w2;
        rt3 = fac * w3;
        const double rtd = rt1 * enx + rt2 * eny + rt3 * enz;
        rt1 -= enx * rtd;
        rt2 -= eny * rtd;
        rt3 -= enz * rtd;
      }
    }
    o.Ti[0] -= rt1;
    o.Ti[1] -= rt2;
    o.Ti[2] -= rt3;
    o.Tj[0] += rt1;
    o.Tj[1] += rt2;
    o.Tj[2] += rt3;
  }
}

}  // namespace gb300
