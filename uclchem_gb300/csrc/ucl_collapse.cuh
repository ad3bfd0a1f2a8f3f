// Parameterised prestellar-core collapse on the device: the physics module
// of collapse.f90 (Priestley et al. 2018, AJ 156, 51), selected per model by
// ucl_model_params::collapse:
//   1 'BE1.1'     Bonnor-Ebert sphere, overdensity 1.1 (Aikawa et al. 2005)
//   2 'BE4'       Bonnor-Ebert sphere, overdensity 4
//   3 'filament'  magnetised filament (Nakamura et al. 1995)
//   4 'ambipolar' magnetised cloud collapsing by ambipolar diffusion (Fiedler
//                 et al. 1993)
// Each mode is a fit of the hydrodynamic models: central density rho0(t),
// radius parameter r0(t) and slope a(t) of the density profile
// rho(r) = rho0 / (1 + (r/r0)^a) (collapse.f90:177-261), and for modes 3-4 a
// radial-velocity fit (:264-381).  The parcel is at rout; modes 1-2 move it
// inward so that the mass inside it stays constant (:117-154), modes 3-4
// move it by v*dt with dt = targetTime - currentTime, which is zero when the
// physics update runs (the chemistry has reached targetTime), so the parcel
// stays at rout as in the reference.  After each interval the column
// density to the cloud edge is the trapezoid integral of the profile
// (:157-175) and Av = baseAv + N/1.6e21 (:82).
//
// Literal constants follow the reference's kinds: default-REAL literals are
// single precision promoted to double ((double)x.f below), 'd' literals are
// double.  Integer powers are taken by ipow-style multiplication.
#pragma once
#include "ucl_chem.cuh"

namespace ucl {

constexpr double COL_MH = 1.67262164e-24;  // constants.f90:7
constexpr double COL_AU = 2.063e5;         // constants.f90:12

// x**k for a constant integer k >= 0, by the right-to-left binary method
__device__ __forceinline__ double col_ipow(double x, int k) {
  unsigned e = (unsigned)k;
  double r = (e & 1u) ? x : 1.0;
  while (e >>= 1) {
    x = x * x;
    if (e & 1u) r = r * x;
  }
  return r;
}

// sound speed at 10 K (cm/s), the filament's velocity unit
__device__ __forceinline__ double col_cs10() { return sqrt(1.38e-16 * 10 / 2 / COL_MH); }
// (2 pi G rho_u)^-1/2 for rho_u = 2.2e4 mH: the filament's time unit (s)
__device__ __forceinline__ double col_tff() { return pow(2 * cK.PI * 6.67e-8 * 2.2e4 * COL_MH, -0.5); }
// filament distance unit (pc), collapse.f90:190-191
__device__ __forceinline__ double col_unitr() { return col_cs10() * col_tff() / cK.PC; }
// filament time unit (yr), collapse.f90:209-210
__device__ __forceinline__ double col_unitt() { return col_tff() / cK.SECONDS_PER_YEAR; }

// density profile, collapse.f90:178-196
__device__ double col_rhofit(int mode, double r, double rho0, double r0, double a) {
  if (mode == 1 || mode == 2) {
    const double rau = r * COL_AU;
    return rho0 / (1 + pow(rau / r0, a));
  }
  if (mode == 3) {
    const double unitrho = 2.2e4;
    const double x = r / col_unitr() / r0;
    return unitrho * rho0 / pow(1 + x * x, a);
  }
  const double r75 = r / 7.5e-1;
  return rho0 / (1 + pow(r75 / r0, a));
}

// central density, collapse.f90:199-222
__device__ double col_rho0fit(int mode, double t, double tmax) {
  double l;
  if (mode == 1) l = (double)61.8f * pow(tmax - t, (double)-0.01f) - (double)49.4f;
  else if (mode == 2) l = (double)68.4f * pow(tmax - t, (double)-0.01f) - (double)55.7f;
  else if (mode == 3) l = (double)3.54f * pow((double)5.47f - t / col_unitt(), (double)-0.15f) - (double)2.73f;
  else {
    if (t <= 6.0) return 2.0e3 + 1.7e3 * (t / 6.0 - 1.0);
    l = (double)5.3f * pow((double)16.138f - 1e-6 * t, (double)-0.1f) - 1.0;
  }
  return pow(10.0, l);
}

// radius parameter, collapse.f90:225-245
__device__ double col_r0fit(int mode, double t, double tmax) {
  double l;
  if (mode == 1) l = -((double)28.5f * pow(tmax - t, (double)-0.01f)) + (double)28.93f;
  else if (mode == 2) l = -((double)39.0f * pow(tmax - t, (double)-0.01f)) + (double)38.7f;
  else if (mode == 3) l = -((double)1.34f * pow((double)5.47f - t / col_unitt(), (double)-0.15f)) + (double)1.47f;
  else l = -((double)2.57f * pow((double)16.138f - 1e-6 * t, (double)-0.1f)) + (double)1.85f;
  return pow(10.0, l);
}

// slope, collapse.f90:248-261
__device__ double col_afit(int mode, double t) {
  if (mode == 1) return 2.4;
  if (mode == 2) return (double)1.9f + 0.5 * exp(-t / (double)1e5f);
  if (mode == 3) return 2.0 - 0.5 * col_ipow(t / col_unitt() / (double)5.47f, 9);
  return (double)2.4f - (double)0.2f * col_ipow(1e-6 * t / (double)16.138f, 40);
}

// radial velocity (cm/s), collapse.f90:264-290
__device__ double col_vrfit(int mode, double r, double rmin, double vmin, double a) {
  if (mode == 3) {
    const double nr = r / col_unitr() - rmin;
    double v;
    if (nr < 0.0) v = vmin * ((nr / rmin) * (nr / rmin) - 1);
    else v = vmin * (exp(-2.0 * a * nr) - 2 * exp(-a * nr));
    return col_cs10() * v;
  }
  if (mode == 4) {
    const double rmid = 0.5;
    const double r75 = r / 7.5e-1;
    const double nr = r75 - rmin;
    double v;
    if (r75 < rmin) v = vmin * ((nr / rmin) * (nr / rmin) - 1);
    else if (r75 <= rmid) v = (vmin - a) * pow(nr / (rmid - rmin), (double)0.3f) - vmin;
    else v = a / (1.0 - rmid) * (r75 - rmid) - a;
    return 1e3 * v;
  }
  return 0.0;
}

// radius of minimum velocity, collapse.f90:293-321
__device__ double col_rminfit(int mode, double t) {
  if (mode == 3) {
    const double tn = t / col_unitt();
    if (tn == 0.0) return 7.2;
    const double lg = log(tn);
    if (lg < 1.6) return -((double)1.149f * tn) + (double)7.2f;
    if (lg < 1.674) return -((double)9.2f * lg) + (double)16.25f;
    return -((double)22.0f * lg) + (double)37.65f;
  }
  const double t6 = 1e-6 * t;
  if (t6 <= (double)10.2f) return -((double)0.0039f * t6) + (double)0.49f;
  if (t6 <= (double)15.1f) return -((double)0.0306f * (t6 - (double)10.2f)) + (double)0.45f;
  return -((double)0.282f * (t6 - (double)15.1f)) + (double)0.3f;
}

// minimum velocity, collapse.f90:324-346
__device__ double col_vminfit(int mode, double t) {
  if (mode == 3) {
    const double tn = t / col_unitt();
    if (tn == 0.0) return 0.0;
    const double lg = log(tn);
    if (lg < 1.6) return (double)0.0891f * tn;
    if (lg < 1.674) return (double)5.5f * lg - (double)8.37f;
    return (double)18.9f * lg - (double)30.8f;
  }
  const double t6 = 1e-6 * t;
  return (double)3.44f * pow((double)16.138f - t6, (double)-0.35f) - (double)0.7f;
}

// velocity a-parameter, collapse.f90:349-378
__device__ double col_avfit(int mode, double t) {
  if (mode == 3) {
    const double tn = t / col_unitt();
    if (tn == 0.0) return 0.4;
    const double lg = log(tn);
    if (lg < 1.6) return (double)0.0101f * tn + (double)0.4f;
    if (lg < 1.674) return (double)0.695f * lg - (double)0.663f;
    return (double)2.69f * lg - (double)4.0f;
  }
  const double t6 = 1e-6 * t;
  if (t6 <= (double)10.2f) return (double)0.143f * t6;
  return (double)0.217f * (t6 - (double)10.2f) + (double)1.46f;
}

// Trapezoid sum over i = 1..np of 0.5 (rho(x_i) + rho(x_{i-1})) * w(i), all
// threads: kind 0 = column density (x_i = rin + i dr, w = dr*pc,
// collapse.f90:157-175), kind 1 = enclosed mass (x_i = i dr, w = dr*(i dr)^2,
// :117-134).  The terms are summed across the CTA (a block reduction, not
// the reference's left-to-right order: the sum differs in the last bits).
__device__ __noinline__ double col_trapezoid(int kind, int mode, int np, double x0, double dr, double rho0,
                                             double r0, double a, double* red) {
  double s = 0.0;
  for (int i = 1 + (int)threadIdx.x; i <= np; i += NT) {
    const double x1 = kind == 0 ? x0 + (i - 1) * dr : (i - 1) * dr;
    const double x2 = kind == 0 ? x0 + i * dr : i * dr;
    const double drho = 0.5 * (col_rhofit(mode, x2, rho0, r0, a) + col_rhofit(mode, x1, rho0, r0, a));
    if (kind == 0) s += drho * dr * cK.PC;
    else {
      const double ri = i * dr;
      s += drho * dr * (ri * ri);
    }
  }
  return block_sum<NT>(s, red);
}

// findNewRadius (collapse.f90:137-154): the first i with
// sum_{k<=i} 0.5 (rho(k dr) + rho((k-1) dr)) dr (k dr)^2 >= mass, dr = r/1e4,
// summed left to right as the reference does.  The profile values are
// evaluated by the whole CTA into `f` (CH + 1 doubles of shared scratch: the
// LU area, idle between intervals), a
// chunk at a time, and thread 0 accumulates.  Returns i*dr, or -1 if the
// mass is not reached within 2^24 steps (the reference would loop on).
// All threads call.
__device__ __noinline__ double col_new_radius(int mode, double mass, double r, double rho0, double r0,
                                              double a, double* f, int* flag) {
  constexpr int CH = 1024;
  const double dr = r / 1.0e4;
  __shared__ double s_m1, s_rad;
  __shared__ int s_done;
  if (threadIdx.x == 0) { s_m1 = 0.0; s_rad = -1.0; s_done = !(0.0 < mass); }
  __syncthreads();
  for (int base = 0; base < (1 << 24); base += CH) {
    if (s_done) break;
    for (int k = threadIdx.x; k <= CH; k += NT) f[k] = col_rhofit(mode, (base + k) * dr, rho0, r0, a);
    __syncthreads();
    if (threadIdx.x == 0) {
      double m1 = s_m1;
      for (int k = 1; k <= CH; ++k) {
        const int i = base + k;
        const double drho = 0.5 * (f[k] + f[k - 1]);
        const double ri = i * dr;
        m1 = m1 + drho * dr * (ri * ri);
        s_rad = i * dr;
        if (!(m1 < mass)) { s_done = 1; break; }
      }
      s_m1 = m1;
    }
    __syncthreads();
  }
  const double rad = s_done ? s_rad : -1.0;
  if (threadIdx.x == 0 && !s_done) *flag = 1;
  __syncthreads();
  return rad;
}

// updateTargetTime of the collapse module (collapse.f90:60-72), seconds
__device__ __forceinline__ double col_target_time(double ty, double spy) {
  if (ty > 10000) return (ty + 1000.0) * spy;
  if (ty > 1000) return (ty + 100.0) * spy;
  if (ty > 0.0) return (ty * 10) * spy;
  return 3.16e7 * 10.e-8;
}

}  // namespace ucl
