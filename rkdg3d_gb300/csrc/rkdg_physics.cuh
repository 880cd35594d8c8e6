// Device-side Euler physics and approximate Riemann solvers (sm_103a).
//
// Pointwise restatement of src/physics/physics.cpp and src/riemannsolvers/
// for compile-time dimension DIM and arithmetic type R: double for the plain
// FP64 path, float for the FP32-bulk path, Dual<N> (rkdg_dual.cuh) for the
// discrete adjoint.  In the FP32 path the pressure is recovered in FP64
// whenever internal energy loses more than three digits to cancellation (near
// vacuum / strong shocks), and divisions / square roots use the hardware
// reciprocal and reciprocal-square-root approximations (about 2 ulp) instead
// of the multi-instruction IEEE sequences; double and Dual keep IEEE
// division and square root.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

namespace rkdg {

template <typename R>
__device__ __forceinline__ R fdv(R a, R b) {
  return a / b;
}
template <>
__device__ __forceinline__ float fdv<float>(float a, float b) {
  return __fdividef(a, b);
}
template <typename R>
__device__ __forceinline__ R fsq(R x) {
  return sqrt(x);
}
template <>
__device__ __forceinline__ float fsq<float>(float x) {
  return x > 0.0f ? x * rsqrtf(x) : 0.0f;
}

// ComputePressure (physics.cpp:101-112), covolume EoS.
template <int DIM, typename R>
__device__ __forceinline__ R pressure(const R* s, R gamma, R b) {
  const R den = s[0];
  R v2 = R(0);
#pragma unroll
  for (int d = 0; d < DIM; d++) v2 += s[1 + d] * s[1 + d];
  v2 = fdv(v2, den);
  const R ie = s[1 + DIM] - R(0.5) * v2;
  if constexpr (std::is_same<R, float>::value) {
    if (fabsf(ie) < 1e-3f * fabsf(s[1 + DIM])) {
      double v2d = 0.0;
#pragma unroll
      for (int d = 0; d < DIM; d++) v2d += (double)s[1 + d] * (double)s[1 + d];
      v2d /= (double)den;
      return (float)(((double)gamma - 1.0) * ((double)s[1 + DIM] - 0.5 * v2d) /
                     (1.0 - (double)den * (double)b));
    }
  }
  return fdv((gamma - R(1)) * ie, R(1) - den * b);
}

// ComputeSoundSpeed (physics.cpp:134-140)
template <int DIM, typename R>
__device__ __forceinline__ R sound_speed_p(const R* s, R p, R gamma, R b) {
  const R den = s[0];
  return fsq(fdv(fdv(gamma * p, den), R(1) - den * b));
}

// StateIsPhysical (physics.cpp:6-50): covolume-aware pressure.
template <int DIM, typename R>
__device__ __forceinline__ bool state_is_physical(const R* s, R gamma, R b) {
  const R den = s[0];
  const R e = s[1 + DIM];
  if (den < R(0) || den != den) return false;
  if (e <= R(0) || e != e) return false;
  const R p = pressure<DIM>(s, gamma, b);
  if (p <= R(0) || p != p) return false;
  return true;
}

// StateIsPhysicalSay (physics.cpp:53-97): perfect-gas pressure (quirk Q10).
template <int DIM, typename R>
__device__ __forceinline__ bool state_is_physical_say(const R* s, R gamma) {
  const R den = s[0];
  const R e = s[1 + DIM];
  if (den < R(0) || den != den) return false;
  if (e <= R(0) || e != e) return false;
  R v2 = R(0);
#pragma unroll
  for (int i = 0; i < DIM; i++) v2 += s[1 + i] * s[1 + i];
  v2 = fdv(v2, den);
  const R p = (gamma - R(1)) * (e - R(0.5) * v2);
  if (p <= R(0) || p != p) return false;
  return true;
}

// ComputeMaxCharSpeed (physics.cpp:252-266)
template <int DIM, typename R>
__device__ __forceinline__ R max_char_speed(const R* s, R gamma, R b) {
  const R den = s[0];
  R v2 = R(0);
#pragma unroll
  for (int d = 0; d < DIM; d++) v2 += s[1 + d] * s[1 + d];
  v2 = fdv(v2, den);
  const R p = pressure<DIM>(s, gamma, b);
  const R c = sound_speed_p<DIM>(s, p, gamma, b);
  return fsq(fdv(v2, den)) + c;
}

// FP32 pointwise state quantities with one reciprocal of the density and one
// of the covolume factor: r = 1/rho, q = 1/(1 - rho b), the pressure (FP64
// where E - |m|^2/(2 rho) cancels, as pressure() does) and |u| + c.  Returns
// false where StateIsPhysicalSay fails (rho < 0, E <= 0, perfect-gas p <= 0,
// NaN).  Same quantities as the double path, rounded in a different order.
template <int DIM>
__device__ __forceinline__ bool state_f32(const float* s, float gamma, float b, float& r, float& q,
                                          float& p, float& speed) {
  const float den = s[0], E = s[1 + DIM];
  if (!(den >= 0.0f) || !(E > 0.0f)) return false;
  r = __fdividef(1.0f, den);
  float m2 = 0.0f;
#pragma unroll
  for (int d = 0; d < DIM; d++) m2 = fmaf(s[1 + d], s[1 + d], m2);
  const float v2 = m2 * r;  // |m|^2 / rho
  const float ie = E - 0.5f * v2;
  if (!((gamma - 1.0f) * ie > 0.0f)) return false;
  q = __fdividef(1.0f, 1.0f - den * b);
  if (fabsf(ie) < 1e-3f * fabsf(E)) {
    double m2d = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; d++) m2d += (double)s[1 + d] * (double)s[1 + d];
    p = (float)(((double)gamma - 1.0) * ((double)E - 0.5 * m2d / (double)den) /
                (1.0 - (double)den * (double)b));
  } else {
    p = (gamma - 1.0f) * ie * q;
  }
  speed = fsq(v2 * r) + fsq(gamma * p * r * q);
  return true;
}

// FP32 Rusanov flux (rs_rusanov.cpp:6-40) on unrotated states, built on
// state_f32.  Returns the wave speed, or -1 for a non-physical state.
template <int DIM>
__device__ __forceinline__ float rusanov_f32(const float* s1, const float* s2, const float* n,
                                             float* flux, float gamma, float b) {
  constexpr int NEQ = DIM + 2;
  float r1, q1, p1, e1, r2, q2, p2, e2;
  if (!state_f32<DIM>(s1, gamma, b, r1, q1, p1, e1)) return -1.0f;
  if (!state_f32<DIM>(s2, gamma, b, r2, q2, p2, e2)) return -1.0f;
  const float maxE = e1 > e2 ? e1 : e2;
  float d1 = 0.0f, d2 = 0.0f, nn = 0.0f;
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    d1 = fmaf(s1[1 + d], n[d], d1);
    d2 = fmaf(s2[1 + d], n[d], d2);
    nn = fmaf(n[d], n[d], nn);
  }
  const float h = 0.5f * rsqrtf(nn), a = 0.5f * maxE;
  const float u1 = d1 * r1, u2 = d2 * r2;
  flux[0] = h * (d1 + d2) - a * (s2[0] - s1[0]);
#pragma unroll
  for (int d = 0; d < DIM; d++)
    flux[1 + d] = h * (fmaf(u1, s1[1 + d], p1 * n[d]) + fmaf(u2, s2[1 + d], p2 * n[d])) -
                  a * (s2[1 + d] - s1[1 + d]);
  flux[NEQ - 1] = h * (u1 * (s1[NEQ - 1] + p1) + u2 * (s2[NEQ - 1] + p2)) -
                  a * (s2[NEQ - 1] - s1[NEQ - 1]);
  return maxE;
}

// ComputeFlux (physics.cpp:143-168): F[k][d]; also returns |u|+c at the node
// (FE_Evolution::GetFlux, fe_evolution.cpp:219-245).
template <int DIM, typename R>
__device__ __forceinline__ R flux_and_speed(const R* s, R F[DIM + 2][DIM], R gamma, R b) {
  if constexpr (std::is_same<R, float>::value) {
    float r, q, p, speed;
    if (!state_f32<DIM>(s, gamma, b, r, q, p, speed)) {
      // non-physical node: same arithmetic as the double path
      r = __fdividef(1.0f, s[0]);
      p = pressure<DIM>(s, gamma, b);
      float m2 = 0.0f;
#pragma unroll
      for (int d = 0; d < DIM; d++) m2 += s[1 + d] * s[1 + d];
      speed = fsq(m2 * r * r) + fsq(fdv(gamma * p * r, 1.0f - s[0] * b));
    }
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const float ud = s[1 + d] * r;
      F[0][d] = s[1 + d];
#pragma unroll
      for (int i = 0; i < DIM; i++) F[1 + i][d] = s[1 + i] * ud;
      F[1 + d][d] += p;
      F[1 + DIM][d] = (s[1 + DIM] + p) * ud;
    }
    return speed;
  }
  const R den = s[0];
  const R inv = fdv(R(1), den);
  R v2 = R(0);
#pragma unroll
  for (int d = 0; d < DIM; d++) v2 += s[1 + d] * s[1 + d];
  const R pres = pressure<DIM>(s, gamma, b);
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    F[0][d] = s[1 + d];
#pragma unroll
    for (int i = 0; i < DIM; i++) F[1 + i][d] = s[1 + i] * s[1 + d] * inv;
    F[1 + d][d] += pres;
  }
  const R H = (s[1 + DIM] + pres) * inv;
#pragma unroll
  for (int d = 0; d < DIM; d++) F[1 + DIM][d] = s[1 + d] * H;
  const R c = fsq(fdv(gamma * pres * inv, R(1) - den * b));
  return fsq(v2 * inv * inv) + c;
}

// ComputeFluxDotN (physics.cpp:171-195)
template <int DIM, typename R>
__device__ __forceinline__ void flux_dot_n(const R* s, const R* n, R* fn, R p) {
  const R den = s[0];
  R dvn = R(0);
#pragma unroll
  for (int d = 0; d < DIM; d++) dvn += s[1 + d] * n[d];
  fn[0] = dvn;
#pragma unroll
  for (int d = 0; d < DIM; d++) fn[1 + d] = fdv(dvn * s[1 + d], den) + p * n[d];
  const R H = fdv(s[1 + DIM] + p, den);
  fn[1 + DIM] = dvn * H;
}

// ComputeFluxF (physics.cpp:198-231): x-flux of a rotated state.
template <int DIM, typename R>
__device__ __forceinline__ void flux_F(const R* s, R* f, R p) {
  f[0] = s[1];
  f[1] = fdv(s[1] * s[1], s[0]) + p;
#pragma unroll
  for (int d = 1; d < DIM; d++) f[d + 1] = fdv(s[1] * s[d + 1], s[0]);
  const R H = fdv(s[1 + DIM] + p, s[0]);
  f[1 + DIM] = s[1] * H;
}

// RiemannSolver::Rotate / InverseRotate (rs_basic.cpp:11-67), including the
// degenerate branch at |cos psi| <= 1e-6 (quirk Q14).
template <int DIM, typename R>
__device__ __forceinline__ void rotate(R* s, const R* n) {
  R* m = s + 1;
  if constexpr (DIM == 2) {
    const R mx = n[0] * m[0] + n[1] * m[1];
    const R my = -n[1] * m[0] + n[0] * m[1];
    m[0] = mx;
    m[1] = my;
  } else {
    const R sp = n[2];
    const R cp = fsq(R(1) - sp * sp);
    const bool ok = fabs(cp) > R(1e-6);
    const R st = ok ? fdv(n[1], cp) : R(1);
    const R ct = ok ? fdv(n[0], cp) : R(0);
    const R mx = cp * ct * m[0] + cp * st * m[1] + sp * m[2];
    const R my = -st * m[0] + ct * m[1];
    const R mz = -sp * ct * m[0] - sp * st * m[1] + cp * m[2];
    m[0] = mx;
    m[1] = my;
    m[2] = mz;
  }
}
template <int DIM, typename R>
__device__ __forceinline__ void inverse_rotate(R* s, const R* n) {
  R* m = s + 1;
  if constexpr (DIM == 2) {
    const R mx = n[0] * m[0] - n[1] * m[1];
    const R my = n[1] * m[0] + n[0] * m[1];
    m[0] = mx;
    m[1] = my;
  } else {
    const R sp = n[2];
    const R cp = fsq(R(1) - sp * sp);
    const bool ok = fabs(cp) > R(1e-6);
    const R st = ok ? fdv(n[1], cp) : R(1);
    const R ct = ok ? fdv(n[0], cp) : R(0);
    const R mx = cp * ct * m[0] - st * m[1] - sp * ct * m[2];
    const R my = cp * st * m[0] + ct * m[1] - sp * st * m[2];
    const R mz = sp * m[0] + cp * m[2];
    m[0] = mx;
    m[1] = my;
    m[2] = mz;
  }
}

// a^e for a > 0 (the TRRS pressures).  double and float go through the
// base-2 logarithm and exponential: within a few ulp of pow() at a fraction of
// its FP64 cost (the TRRS speeds are the most expensive pointwise piece of the
// FP64 path); dual numbers keep pow().
template <typename R>
__device__ __forceinline__ R powr(R a, R e) {
  return pow(a, e);
}
template <>
__device__ __forceinline__ double powr<double>(double a, double e) {
  return exp2(e * log2(a));
}
template <>
__device__ __forceinline__ float powr<float>(float a, float e) {
  return exp2f(e * log2f(a));
}

// Wave-speed estimates on rotated states: TRRS ComputeToroCharSpeeds
// (physics.cpp:309-350) or Einfeldt ComputeEinfeldtCharSpeeds (269-296).
// Only lambda[0] and lambda[dim+1] are used by the solvers.
template <int DIM, typename R>
__device__ __forceinline__ void wave_speeds(const R* s1, const R* s2, R p1, R p2, R gamma, R b,
                                            int avg, R& SL, R& SR) {
  const R cL = sound_speed_p<DIM>(s1, p1, gamma, b);
  const R cR = sound_speed_p<DIM>(s2, p2, gamma, b);
  if (avg == 1) {
    const R ruL = s1[1], ruR = s2[1];
    const R uL = fdv(ruL, s1[0]), uR = fdv(ruR, s2[0]);
    const R sL = fsq(s1[0]), sR = fsq(s2[0]);
    const R sum = sL + sR;
    const R eta2 = fdv(R(0.5) * sL * sR, (sL + sR) * (sL + sR));
    const R uav = fdv(fdv(ruL, sL) + fdv(ruR, sR), sum);
    const R cav = fsq(fdv(sL * cL * cL + sR * cR * cR, sum) + eta2 * (uR - uL) * (uR - uL));
    SL = uav - cav;
    SR = uav + cav;
    return;
  }
  const R uL = fdv(s1[1], s1[0]), uR = fdv(s2[1], s2[0]);
  const R z = fdv(R(0.5) * (gamma - R(1)), gamma);
  const R pStar = powr(fdv(cL + cR - R(0.5) * (gamma - R(1)) * (uR - uL),
                           fdv(cL, powr(p1, z)) + fdv(cR, powr(p2, z))),
                       fdv(R(1), z));
  const R qL = pStar > p1 ? fsq(R(1) + fdv(R(0.5) * (gamma + R(1)) * (fdv(pStar, p1) - R(1)), gamma))
                          : R(1);
  const R qR = pStar > p2 ? fsq(R(1) + fdv(R(0.5) * (gamma + R(1)) * (fdv(pStar, p2) - R(1)), gamma))
                          : R(1);
  SL = uL - qL * cL;
  SR = uR + qR * cR;
}

// RiemannSolver*::Eval (rs_rusanov.cpp:6-40, rs_llf.cpp:6-37, rs_hll.cpp:6-50,
// rs_hllc.cpp:71-161).  s1, s2 are working copies (rotated in place, as the
// reference does through const_cast); n is the unit normal from side 1 to
// side 2.  Returns the solver's wave speed, or -1 for a non-physical state.
template <int DIM, typename R>
__device__ __forceinline__ R riemann(R* s1, R* s2, const R* n, R* flux, R gamma, R b, int rs,
                                     int avg) {
  constexpr int NEQ = DIM + 2;
  if constexpr (std::is_same<R, float>::value) {
    if (rs == 0) return rusanov_f32<DIM>(s1, s2, n, flux, gamma, b);
  }
  if (!state_is_physical_say<DIM>(s1, gamma)) return R(-1);
  if (!state_is_physical_say<DIM>(s2, gamma)) return R(-1);
  if (rs == 0) {
    const R p1 = pressure<DIM>(s1, gamma, b);
    const R p2 = pressure<DIM>(s2, gamma, b);
    R v1 = R(0), v2 = R(0);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      v1 += s1[1 + d] * s1[1 + d];
      v2 += s2[1 + d] * s2[1 + d];
    }
    const R e1 = fsq(fdv(fdv(v1, s1[0]), s1[0])) + sound_speed_p<DIM>(s1, p1, gamma, b);
    const R e2 = fsq(fdv(fdv(v2, s2[0]), s2[0])) + sound_speed_p<DIM>(s2, p2, gamma, b);
    const R maxE = e1 > e2 ? e1 : e2;
    R f1[NEQ], f2[NEQ];
    flux_dot_n<DIM>(s1, n, f1, p1);
    flux_dot_n<DIM>(s2, n, f2, p2);
    R nm = R(0);
#pragma unroll
    for (int i = 0; i < DIM; i++) nm += n[i] * n[i];
    nm = fsq(nm);
#pragma unroll
    for (int i = 0; i < NEQ; i++)
      flux[i] = fdv(R(0.5) * (f1[i] + f2[i]), nm) - R(0.5) * maxE * (s2[i] - s1[i]);
    return maxE;
  }
  rotate<DIM>(s1, n);
  rotate<DIM>(s2, n);
  const R p1 = pressure<DIM>(s1, gamma, b);
  const R p2 = pressure<DIM>(s2, gamma, b);
  R f1[NEQ], f2[NEQ];
  flux_F<DIM>(s1, f1, p1);
  flux_F<DIM>(s2, f2, p2);
  R SL, SR;
  wave_speeds<DIM>(s1, s2, p1, p2, gamma, b, avg, SL, SR);
  R ret;
  if (rs == 1) {
    const R maxE = fmax(fabs(SL), fabs(SR));
#pragma unroll
    for (int i = 0; i < NEQ; ++i) flux[i] = R(0.5) * (f1[i] + f2[i]) - R(0.5) * maxE * (s2[i] - s1[i]);
    ret = maxE;
  } else if (rs == 2) {
    const R maxE = fmax(fabs(SL), fabs(SR));
    if (SL >= R(0)) {
#pragma unroll
      for (int i = 0; i < NEQ; ++i) flux[i] = f1[i];
    } else if (SR <= R(0)) {
#pragma unroll
      for (int i = 0; i < NEQ; ++i) flux[i] = f2[i];
    } else {
      const R inv = fdv(R(1), SR - SL);
#pragma unroll
      for (int i = 0; i < NEQ; ++i) {
        if constexpr (std::is_same<R, float>::value)
          flux[i] = (SR * f1[i] - SL * f2[i] + SL * SR * (s2[i] - s1[i])) * inv;
        else
          flux[i] = (SR * f1[i] - SL * f2[i] + SL * SR * (s2[i] - s1[i])) / (SR - SL);
      }
    }
    ret = maxE;
  } else {
    const R maxE = SL > SR ? SL : SR;
    if (SL >= R(0)) {
#pragma unroll
      for (int i = 0; i < NEQ; ++i) flux[i] = f1[i];
    } else if (SR <= R(0)) {
#pragma unroll
      for (int i = 0; i < NEQ; ++i) flux[i] = f2[i];
    } else {
      const R cL = SL - fdv(s1[1], s1[0]);
      const R cR = SR - fdv(s2[1], s2[0]);
      const R sStar = fdv(p2 - p1 + s1[1] * cL - s2[1] * cR, s1[0] * cL - s2[0] * cR);
      const bool left = sStar > R(0);
      const R* st = left ? s1 : s2;
      const R* fK = left ? f1 : f2;
      const R pK = left ? p1 : p2;
      const R SK = left ? SL : SR;
      const R cK = left ? cL : cR;
      const R rhoL = st[0];
      const R extra = SK * (pK + rhoL * cK * (sStar - fdv(st[1], st[0])));
      const R inv = fdv(R(1), SK - sStar);
#pragma unroll
      for (int i = 0; i < NEQ; ++i) {
        const R Di = (i == 1) ? R(1) : ((i == DIM + 1) ? sStar : R(0));
        flux[i] = (sStar * (st[i] * SK - fK[i]) + Di * extra) * inv;
      }
    }
    ret = maxE;
  }
  inverse_rotate<DIM>(flux, n);
  return ret;
}

// computeRightState of the boundary integrators.
template <int DIM, typename R>
__device__ __forceinline__ void right_state(int type, const double* st, const R* s1, R* s2,
                                            const R* n, R gamma, R b, R rg) {
  constexpr int NEQ = DIM + 2;
#pragma unroll
  for (int i = 0; i < NEQ; ++i) s2[i] = s1[i];
  if (type == 0 || type == 4) {  // slip / wall
    rotate<DIM>(s2, n);
    s2[1] = -s2[1];
    inverse_rotate<DIM>(s2, n);
  } else if (type == 2) {  // fixed state in the rotated frame (quirk Q12)
#pragma unroll
    for (int i = 0; i < NEQ; ++i) s2[i] = (R)st[i];
    inverse_rotate<DIM>(s2, n);
  } else if (type == 3) {  // supersonic inlet, global frame
#pragma unroll
    for (int i = 0; i < NEQ; ++i) s2[i] = (R)st[i];
  } else if (type == 5) {  // subsonic inlet: 2 * fixed - own, rotated frame
    rotate<DIM>(s2, n);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) s2[i] = R(2) * (R)st[i] - s2[i];
    inverse_rotate<DIM>(s2, n);
  } else if (type == 6 || type == 7) {
    // subsonicInletTotalPressure / subsonicInletFixedPressure
    // (boundary_integrator_subsonic_inlet_{total,fixed}_pressure.cpp:10-40):
    // perfect-gas ghost state at the inlet's total temperature
    const R TTot = (R)st[1];
    R rhoU2 = R(0);
#pragma unroll
    for (int d = 0; d < DIM; d++) rhoU2 += s1[1 + d] * s1[1 + d];
    rhoU2 = fdv(rhoU2, s1[0]);
    const R MTTotSq = fdv(fdv(fdv(fdv(rhoU2, s1[0]), gamma), rg), TTot);
    const R MSq = fdv(MTTotSq, R(1) - R(0.5) * (gamma - R(1)) * MTTotSq);
    const R base = R(1) + R(0.5) * (gamma - R(1)) * MSq;
    const R p = type == 6 ? (R)st[0] * powr(base, -fdv(gamma, gamma - R(1))) : (R)st[0];
    const R T = fdv(TTot, base);
    const R rho = fdv(fdv(p, rg), T);
    s2[NEQ - 1] = fdv(p, gamma - R(1)) + R(0.5) * fdv(rhoU2, s1[0]) * rho;
#pragma unroll
    for (int d = 0; d < DIM; d++) s2[1 + d] = fdv(s1[1 + d], s1[0]) * rho;
    s2[0] = rho;
  } else if (type == 8) {
    // fixedPressureOutlet (boundary_integrator_open_fixed_pressure.cpp:10-30);
    // epsIn subtracts 0.5 |m|^2 (not 0.5 |m|^2 / rho), as the reference does
    const R pFix = (R)st[0];
    R rhoU2 = R(0);
#pragma unroll
    for (int d = 0; d < DIM; d++) rhoU2 += s1[1 + d] * s1[1 + d];
    const R U2 = fdv(fdv(rhoU2, s1[0]), s1[0]);
    const R epsIn = fdv(s1[NEQ - 1] - R(0.5) * rhoU2, s1[0]);
    const R rho = fdv(fdv(pFix, gamma - R(1)), epsIn);
    s2[NEQ - 1] = fdv(pFix, gamma - R(1)) + R(0.5) * rho * U2;
#pragma unroll
    for (int d = 0; d < DIM; d++) s2[1 + d] = fdv(s1[1 + d], s1[0]) * rho;
    s2[0] = rho;
  } else if (type == 9) {
    // totalPressureFixedTemperatureOutlet (boundary_integrator_open_total_
    // pressure.cpp:10-40); m.n from the normal's own components (the
    // reference indexes one past them)
    const R pTot = (R)st[0], TFix = (R)st[1];
    R rho2U2 = R(0), rhoN = R(0);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      rho2U2 += s1[1 + d] * s1[1 + d];
      rhoN += s1[1 + d] * n[d];
    }
    const R U2 = fdv(fdv(rho2U2, s1[0]), s1[0]);
    const R epsIn = rhoN > R(0) ? fdv(s1[NEQ - 1] - R(0.5) * rho2U2, s1[0])
                                : fdv(rg, gamma - R(1)) * TFix;
    const R M = fdv(fsq(U2), sound_speed_p<DIM>(s1, pressure<DIM>(s1, gamma, b), gamma, b));
    const bool sup = M > R(1);
    R p = sup ? pTot * powr(R(1) + R(0.5) * (gamma - R(1)) * M * M, -fdv(gamma, gamma - R(1)))
              : pTot;
    const R rho = sup ? fdv(fdv(p, gamma - R(1)), epsIn)
                      : fdv(p, R(0.5) * U2 + (gamma - R(1)) * epsIn);
    if (!sup) p = p - R(0.5) * U2 * rho;
    s2[NEQ - 1] = fdv(p, gamma - R(1)) + R(0.5) * rho * U2;
#pragma unroll
    for (int d = 0; d < DIM; d++) s2[1 + d] = s1[1 + d] * fdv(rho, s1[0]);
    s2[0] = rho;
  } else if (type == 10) {
    // charOutlet (boundary_integrator_char_outlet.cpp:14-57) with the ghost
    // vector entering as the interior state (the reference reads the previous
    // boundary point's ghost state there); st is the outer state
    R fx[NEQ];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) fx[i] = (R)st[i];
    const R cOut = sound_speed_p<DIM>(fx, pressure<DIM>(fx, gamma, b), gamma, b);
    const R UOut = fdv(fx[1], fx[0]);
    const R cIn = sound_speed_p<DIM>(s1, pressure<DIM>(s1, gamma, b), gamma, b);
    rotate<DIM>(s2, n);
    const R UIn = fdv(s2[1], s2[0]);
    const R UB = R(0.5) * (UIn + UOut) - fdv(cOut - cIn, gamma - R(1));
    const R cB = R(-0.25) * (gamma - R(1)) * (UOut - UIn) + R(0.5) * (cOut + cIn);
    const R sB = s2[1] < R(0) ? fdv(fdv(cOut * cOut, powr(fx[0], gamma - R(1))), gamma)
                              : fdv(fdv(cIn * cIn, powr(s2[0], gamma - R(1))), gamma);
    const R rhoB = powr(fdv(fdv(cB * cB, sB), gamma), fdv(R(1), gamma - R(1)));
    const R pB = fdv(rhoB * cB * cB, gamma);
    s2[0] = rhoB;
    s2[1] = UB;  // a velocity in the momentum slot, as the reference stores it
    const R v = fdv(s2[2], s2[0]);
    const R w = DIM == 3 ? fdv(s2[DIM == 3 ? 3 : 2], s2[0]) : R(0);
    s2[NEQ - 1] = fdv(pB, gamma - R(1)) * (R(1) - rhoB * b) + R(0.5) * rhoB * (UB * UB + v * v + w * w);
    inverse_rotate<DIM>(s2, n);
  }
}

}  // namespace rkdg
