// Device chemistry of one system per CTA: rate coefficients, self-shielded
// photo rates, the flux-form right-hand side and its analytic Jacobian.
//
// Reference semantics followed (paths in the UCLCHEM project):
//   rates      src/fortran_src/rates.f90:21-378, surfacereactions.f90:63-211
//   photo      src/fortran_src/photoreactions.f90:46-304
//   RHS        src/fortran_src/chemistry.f90:294-352 + odes.f90:6-5181
#pragma once
#include "ucl_common.cuh"
#include "../../include/uclchem_gb300.h"

namespace ucl {

__constant__ Consts cK;

// Per-system physical state read by the chemistry (shared memory).
struct SysPhys {
  double T, Td, av, dens, phi, cs;  // gas/dust T, Av, density(dstep), CR-desorption yield, cloudSize/points
  double sm, sb, blr;               // safeMantle, safeBulk, bulkLayersReciprocal at interval start
  double h2col, cocol, ccol;        // column densities at interval start
  double avt, rf, scat1000;         // Av/1.086, radfield/1.7, dust scattering at 1000 A
  double h2crp;                     // h2CRPRate of the interval (improvedH2CRPDissociation)
};

// per-interval constants of the photo rates (Av and radfield are fixed over
// an output interval)


// ---------------------------------------------------------------------------
// splines and photo rates (scalar, one thread)
__device__ double spline_eval(const double* xa, const double* ya, const double* y2a, int n, double x) {
  int jlo = 0, jhi = n + 1;
  while (jhi - jlo != 1) {
    int jm = (jhi + jlo) >> 1;
    if (x > xa[jm - 1]) jlo = jm; else jhi = jm;
  }
  if (jlo == 0) { jlo = 1; jhi = 2; }
  if (jlo == n) { jlo = n - 1; jhi = n; }
  const double h = xa[jhi - 1] - xa[jlo - 1];
  const double a = (xa[jhi - 1] - x) / h, b = (x - xa[jlo - 1]) / h;
  return a * ya[jlo - 1] + b * ya[jhi - 1] + ((a * a * a - a) * y2a[jlo - 1] + (b * b * b - b) * y2a[jhi - 1]) * (h * h) / 6.0;
}

// second derivatives of the natural cubic spline through (x, y)
__device__ void spline_natural(const double* x, const double* y, int n, double* y2) {
  double u[8];
  y2[0] = 0.0;
  u[0] = 0.0;
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) / (x[i + 1] - x[i - 1]) -
            sig * u[i - 1]) / p;
  }
  y2[n - 1] = 0.0;
  for (int k = n - 2; k >= 0; k--) y2[k] = y2[k] * y2[k + 1] + u[k];
}

__device__ double xlambda(double lam) {
  double v = lam;
  if (lam < cK.lam[0]) v = cK.lam[0];
  if (lam > cK.lam[29]) v = cK.lam[29];
  double r = spline_eval(cK.lam, cK.xlam, cK.xlam_y2, 30, v);
  return r < 0.0 ? 0.0 : r;
}

__device__ double scatter_fn(double x1, double av) {
  const double c[6] = {1.0, 2.006, -1.438, 7.364e-01, -5.076e-01, -5.920e-02};
  const double k1[6] = {7.514e-01, 8.490e-01, 1.013, 1.282, 2.005, 5.832};
  double tl = (av / 1.086) * xlambda(x1);
  double s = 0.0;
  if (tl < 1.0) {
    double e = k1[0] * tl;
    if (e < 100.0) s = c[0] * exp(-e);
  } else {
    for (int i = 1; i < 6; i++) {
      double e = k1[i] * tl;
      if (e < 100.0) s = s + c[i] * exp(-e);
    }
  }
  return s;
}

__device__ double scatter_tl(double tl) {
  const double c[6] = {1.0, 2.006, -1.438, 7.364e-01, -5.076e-01, -5.920e-02};
  const double k1[6] = {7.514e-01, 8.490e-01, 1.013, 1.282, 2.005, 5.832};
  double s = 0.0;
  if (tl < 1.0) {
    double e = k1[0] * tl;
    if (e < 100.0) s = c[0] * exp(-e);
  } else {
    for (int i = 1; i < 6; i++) {
      double e = k1[i] * tl;
      if (e < 100.0) s = s + c[i] * exp(-e);
    }
  }
  return s;
}

__device__ void photo_setup(SysPhys& S, double radfield) {
  S.avt = S.av / 1.086;
  S.rf = radfield / (double)1.7f;
  S.scat1000 = scatter_tl(S.avt * cK.xl1000);
}

// H2 photodissociation with line self-shielding (photoreactions.f90:46-127)
__device__ double h2_photo_s(double nh2, const SysPhys& S) {
  const double taud = 0.5 * nh2 * (double)1.5e-2f * 1.0e-2 / cK.h2_dw;
  double sj;
  if (taud == 0.0) sj = 1.0;
  else if (taud < 2.0) sj = exp(-0.6666667 * taud);
  else if (taud < 10.0) sj = 0.638 * pow(taud, -1.25);
  else if (taud < 100.0) sj = 0.505 * pow(taud, -1.15);
  else sj = 0.344 * pow(taud, -1.0667);
  const double r = cK.h2_r, t = cK.h2_t;
  const double u = sqrt(taud * r) / t;
  const double sr = r / (t * sqrt(0.78539816 + u * u));
  return 5.18e-11 * S.rf * S.scat1000 * (sj + sr);
}

// CO photodissociation (photoreactions.f90:57-72, 251-304), evaluated by a
// whole warp: the seven row splines of the shielding table run in parallel
// lanes.  All 32 lanes must call; the result is returned in every lane.
__device__ double co_photo_w(double nh2, double nco, const SysPhys& S) {
  const int lane = threadIdx.x & 31;
  // the four logarithms in four lanes of one warp-wide evaluation (FP64
  // issue is per warp instruction, so this costs one log10, not four)
  const double larg = lane == 0 ? fabs(nco) + 1.0 : lane == 1 ? fabs(nh2) + 1.0 : lane == 2 ? nco + 1.0 : nh2 + 1.0;
  const double lg = log10(larg);
  const double lu = __shfl_sync(0xffffffffu, lg, 0), lw = __shfl_sync(0xffffffffu, lg, 1);
  double lognco = __shfl_sync(0xffffffffu, lg, 2), lognh2 = __shfl_sync(0xffffffffu, lg, 3);
  if (lognco < cK.nco_grid[0]) lognco = cK.nco_grid[0];
  if (lognh2 < cK.nh2_grid[0]) lognh2 = cK.nh2_grid[0];
  if (lognco > cK.nco_grid[6]) lognco = cK.nco_grid[6];
  if (lognh2 > cK.nh2_grid[5]) lognh2 = cK.nh2_grid[5];
  double yy = 0.0;
  if (lane < 7) yy = spline_eval(cK.nh2_grid, cK.sco[lane], cK.sco_y2[lane], 6, lognh2);
  double v[7];
#pragma unroll
  for (int j = 0; j < 7; j++) v[j] = __shfl_sync(0xffffffffu, yy, j);
  double y2 = 0.0;
  if (lane < 7) {
#pragma unroll
    for (int k = 0; k < 7; k++) y2 += cK.sco_m[lane][k] * v[k];
  }
  double w2[7];
#pragma unroll
  for (int j = 0; j < 7; j++) w2[j] = __shfl_sync(0xffffffffu, y2, j);
  // evaluate the column spline at log N(CO) (unit grid spacing)
  int jlo = (int)floor(lognco - cK.nco_grid[0]);
  if (jlo < 0) jlo = 0;
  if (jlo > 5) jlo = 5;
  double ya = v[0], yb = v[1], ya2 = w2[0], yb2 = w2[1];
#pragma unroll
  for (int j = 1; j < 6; j++)
    if (jlo == j) { ya = v[j]; yb = v[j + 1]; ya2 = w2[j]; yb2 = w2[j + 1]; }
  const double a = (cK.nco_grid[jlo + 1] - lognco), b = (lognco - cK.nco_grid[jlo]);
  const double val = a * ya + b * yb + ((a * a * a - a) * ya2 + (b * b * b - b) * yb2) / 6.0;
  double lb = (5675.0 - 200.6 * lw) - (571.6 - 24.09 * lw) * lu + (18.22 - 0.7664 * lw) * (lu * lu);
  if (lb > 1076.1) lb = 1076.1;
  if (lb < 913.6) lb = 913.6;
  const double tl = S.avt * xlambda(lb);
  // all exponentials in one warp-wide evaluation: lanes 1..5 the scattering
  // terms (lane 0 when tl < 1), lane 7 the shielding factor 10^val
  const double c[6] = {1.0, 2.006, -1.438, 7.364e-01, -5.076e-01, -5.920e-02};
  const double k1[6] = {7.514e-01, 8.490e-01, 1.013, 1.282, 2.005, 5.832};
  const int sl = lane < 6 ? lane : 0;
  const double e = k1[sl] * tl;
  const bool use = (tl < 1.0) ? (lane == 0) : (lane >= 1 && lane < 6);
  const double x = exp(lane == 7 ? val * 2.302585092994045684 : -e);
  const double term = (use && e < 100.0) ? c[sl] * x : 0.0;
  const double ssf = __shfl_sync(0xffffffffu, x, 7);
  double sca = 0.0;
#pragma unroll
  for (int j = 0; j < 6; j++) sca += __shfl_sync(0xffffffffu, term, j);
  return (2.e-10) * S.rf * ssf * sca;
}

// scalar versions used once per interval by calculateReactionRates
__device__ double h2_photo(double nh2, double radfield, double av) {
  SysPhys S;
  S.av = av;
  photo_setup(S, radfield);
  return h2_photo_s(nh2, S);
}

__device__ double co_photo(double nh2, double nco, double radfield, double av) {
  double lognco = log10(nco + 1.0), lognh2 = log10(nh2 + 1.0);
  if (lognco < cK.nco_grid[0]) lognco = cK.nco_grid[0];
  if (lognh2 < cK.nh2_grid[0]) lognh2 = cK.nh2_grid[0];
  if (lognco > cK.nco_grid[6]) lognco = cK.nco_grid[6];
  if (lognh2 > cK.nh2_grid[5]) lognh2 = cK.nh2_grid[5];
  double yy[7], y2[7];
  for (int j = 0; j < 7; j++) yy[j] = spline_eval(cK.nh2_grid, cK.sco[j], cK.sco_y2[j], 6, lognh2);
  spline_natural(cK.nco_grid, yy, 7, y2);
  double ssf = pow(10.0, spline_eval(cK.nco_grid, yy, y2, 7, lognco));
  double lu = log10(fabs(nco) + 1.0), lw = log10(fabs(nh2) + 1.0);
  double lb = (5675.0 - 200.6 * lw) - (571.6 - 24.09 * lw) * lu + (18.22 - 0.7664 * lw) * (lu * lu);
  if (lb > 1076.1) lb = 1076.1;
  if (lb < 913.6) lb = 913.6;
  return (2.e-10) * (radfield / (double)1.7f) * ssf * scatter_fn(lb, av);
}

__device__ double c_ionization(double alpha, double gamma, double T, double ncol, double nh2, double av, double radfield) {
  double tauc = gamma * av + 1.1e-17 * ncol + (0.9 * pow(T, 0.27) * pow(nh2 / 1.59e21, 0.45));
  return alpha * (radfield / (double)1.7f) * exp(-tauc);
}

__device__ double h2_form_eff(double gasT, double dustT) {  // surfacereactions.f90:63-107
  const double HFLUX = 1.0e-10;
  double tv = 1.45e5 * sqrt(gasT / 1.0e2);
  double g2 = gasT / 1.0e2;
  double stick = 1.0 / (1.0 + 0.04 * sqrt(gasT + dustT) + 0.2 * (gasT / 1.0e2) + 0.08 * (g2 * g2));
  double q = 1.0 + sqrt((3.0e4 - 110.0) / (450.0 - 110.0));
  double f1 = 0.005 * HFLUX / (2 * 3.0e12 * exp(-320.0 / dustT));
  double f2 = 1.0 * (q * q) / 4.0 * exp(-110.0 / dustT);
  double eps = 1.0 / (1.0 + 1.3e13 / (2 * HFLUX) * exp(-1.5 * 3.0e4 / dustT) * (q * q));
  double sil = 1.0 / (1.0 + f1 + f2) * eps;
  q = 1.0 + sqrt((3.0e4 - 260.0) / (800.0 - 260.0));
  f1 = 0.005 * HFLUX / (2 * 3.0e12 * exp(-520.0 / dustT));
  f2 = 1.0 * (q * q) / 4.0 * exp(-260.0 / dustT);
  eps = 1.0 / (1.0 + 1.3e13 / (2 * HFLUX) * exp(-1.5 * 3.0e4 / dustT) * (q * q));
  double gra = 1.0 / (1.0 + f1 + f2) * eps;
  return 0.5 * tv * (8.473e-22 * sil + 7.908e-22 * gra) * stick;
}

__device__ __forceinline__ double sticking(double s0, double tc, double T) {
  double tr = T / tc;
  return s0 * (1.0 + 2.5 * tr) / pow(1.0 + tr, 2.5);
}

__device__ __forceinline__ double densdot_fn(const ucl_model_params& P, double d) {  // physics-core.f90:90-103
  if (d < P.finalDens && P.freefall)
    return P.freefallFactor * pow(pow(d, 4.) / P.initialDens, (double)0.33f) *
           pow(8.4e-30 * P.initialDens * (pow(d / P.initialDens, (double)0.33f) - 1.), 0.5);
  return 0.0;
}

// ---------------------------------------------------------------------------
// Rate coefficients of one system (calculateReactionRates).  All threads.
// rate [nreac] out (any memory); aux [nreac] shared scratch.
// S.phi is updated to the grain-assisted recombination value (quirk Q1).
__device__ void dev_rates(const DevNet& N, const ucl_model_params& P, SysPhys& S, const double* abund,
                          double* rate, double* aux) {
  const double T = S.T, Td = S.Td, av = S.av, sm = S.sm;
  const double MINS = cK.MIN_SURFACE_ABUND;
  const double ICE = (double)0.3f;
  const double icefac_b = ICE * pow((double)(1.0f - 0.007f), 1.0 + 0.5 / S.blr);
  const bool swap_off = (Td > cK.MAX_GRAIN_TEMP) || (sm < MINS);
  const bool lh_on = (Td < cK.MAX_GRAIN_TEMP) && (sm > MINS);
  for (int j = threadIdx.x; j < N.nreac; j += NT) {
    const uint8_t t = N.rtype[j];
    const double a = N.alpha[j], b = N.beta[j], g = N.gama[j];
    double r = 0.0;
    switch (t) {
      case RT_CRP:
        r = a * P.zeta;
        // improvedH2CRPDissociation overwrites the H2 CR dissociation right
        // after the CRP block (rates.f90:38-41)
        if (P.improvedH2CRPDissociation && j == N.rx_h2crp) r = S.h2crp;
        break;
      case RT_PHOTON:
        r = a * exp(-g * av) * P.radfield / (double)1.7f;
        if (N.iceflag[j] == 2) r = r * icefac_b;
        else if (N.iceflag[j] == 1) r = r * ICE;
        break;
      case RT_CRPHOT:
        r = a * g * 1.0 / (1.0 - P.omega) * P.zeta * pow(T / 300, b);
        if (N.iceflag[j] == 2) r = r * icefac_b;
        else if (N.iceflag[j] == 1) r = r * ICE;
        break;
      case RT_FREEZE:
      case RT_EFREEZE: {
        const int jj = (t == RT_EFREEZE) ? N.partner[j] : j;  // E- freezes at the H rate
        double fr = 1.0 + N.beta[jj] * 16.71e-4 / (cK.GRAIN_RADIUS * T);
        if (P.freezeFactor == 0.0 || Td > cK.MAX_GRAIN_TEMP) fr = 0.0;
        else fr = fr * P.freezeFactor * N.alpha[jj] * cK.THERMAL_VEL * sqrt(T / N.mass_re1[jj]) * cK.GRAIN_CROSSSECTION_PER_H;
        if (t == RT_FREEZE) {
          if (N.stick[j] == 1) fr = sticking(0.87, 87.0, T) * fr;
          else if (N.stick[j] == 2) fr = sticking(1.0, 52.0, T) * fr;
        }
        r = fr;
        break;
      }
      case RT_DESOH2:
        r = (P.desorb && P.h2desorb && sm > MINS) ? ((g > P.ebmaxh2) ? 0.0 : P.epsilon * h2_form_eff(T, Td)) : 0.0;
        break;
      case RT_DESCR:
        r = (P.desorb && P.crdesorb && sm > MINS)
                ? ((g > P.ebmaxcr) ? 0.0 : 4.0 * cK.PI * P.zeta * 1.64e-4 * (cK.GRAIN_SURFACEAREA_PER_H) * S.phi)
                : 0.0;
        break;
      case RT_DEUVCR:
        if (P.desorb && P.uvdesorb && sm > MINS && P.zeta > 0) {
          double v = cK.GRAIN_CROSSSECTION_PER_H * P.uv_yield * 4.875e3 * P.zeta;
          v = v * (1 + (P.radfield / P.uvcreff) * (1.0 / P.zeta) * exp((double)(-1.8f) * av));
          r = (g > P.ebmaxuvcr) ? 0.0 : v;
        }
        break;
      case RT_CRS: r = a * (b * (g / 100) * ((double)8.6f * P.zeta * (double)1.3f)); break;
      case RT_EXRELAX: r = N.c0[j]; break;
      case RT_EXSOLID: r = a * ((N.c1[j] + N.c0[j]) / (cK.SURFACE_SITE_DENSITY * 1.8e-8)); break;
      case RT_THERM:
        if (P.thermdesorb) {
          r = N.c0[j] * exp(-g / Td);
          if (!N.three_phase) r = r * 2.0 * cK.SURFACE_SITE_DENSITY * cK.GRAIN_SURFACEAREA_PER_H;
        }
        break;
      case RT_LH:
      case RT_LHDES: {
        if (lh_on) {
          const int jl = (t == RT_LH) ? j : N.partner[j];
          // diffusionReactionRate (surfacereactions.f90:158-211); c0/c1 vdiff, c2/c3 binding energies, c4 tunnel
          const double v1 = N.c0[jl], v2 = N.c1[jl], e1 = N.c2[jl], e2 = N.c3[jl];
          double diffuse = v1 * exp(-0.5 * e1 / Td);
          diffuse = diffuse + (v2 * exp(-0.5 * e2 / Td));
          double desorb = v1 * exp(-e1 / Td);
          desorb = desorb + v2 * exp(-e2 / Td);
          double reac = N.gama[jl] / Td;
          if (reac > N.c4[jl]) reac = N.c4[jl];
          reac = (v1 > v2 ? v1 : v2) * exp(-reac);
          reac = reac / (reac + desorb + diffuse);
          const double d = N.alpha[jl] * reac * diffuse * cK.GAS_DUST_DENSITY_RATIO / cK.NUM_SITES_PER_GRAIN;
          const int jd = (t == RT_LH) ? N.partner[j] : j;
          const double des = (jd >= 0 && N.iceflag[jd] != 1) ? N.c0[jd < 0 ? 0 : jd] * d : 0.0;
          r = (t == RT_LH) ? (d - des) : des;
        }
        break;
      }
      case RT_ER:
      case RT_ERDES: {
        const int je = (t == RT_ER) ? j : N.partner[j];
        double fr = 1.0 + N.beta[je] * 16.71e-4 / (cK.GRAIN_RADIUS * T);
        if (P.freezeFactor == 0.0 || Td > cK.MAX_GRAIN_TEMP) fr = 0.0;
        else fr = fr * P.freezeFactor * N.alpha[je] * cK.THERMAL_VEL * sqrt(T / N.mass_re1[je]) * cK.GRAIN_CROSSSECTION_PER_H;
        const double d = fr * exp(-N.gama[je] / Td);
        const int jd = (t == RT_ER) ? N.partner[j] : j;
        const double des = (jd >= 0 && N.iceflag[jd] != 1) ? N.c0[jd < 0 ? 0 : jd] * d : 0.0;
        r = (t == RT_ER) ? (d - des) : des;
        break;
      }
      case RT_H2FORM: r = h2_form_eff(Td, Td); break;
      case RT_ZERO: r = 0.0; break;
      case RT_BULKSWAP: r = swap_off ? 0.0 : N.c0[j] * exp(-N.c1[j] / Td); break;
      case RT_SURFSWAP: r = swap_off ? 0.0 : 1.0; break;
      case RT_TWOBODY: r = a * pow(T / 300., b) * exp(-g / T); break;
      case RT_IONOPOL1: r = a * b * (0.62 + 0.4767 * g * sqrt(300.0 / T)); break;
      case RT_IONOPOL2: r = a * b * (1.0 + 0.0967 * g * sqrt(300.0 / T) + g * g * 300.0 / ((double)10.526f * T)); break;
      default: break;
    }
    aux[j] = r;  // value before the freeze-out shut-off / masks
  }
  __syncthreads();
  // grain-assisted recombination parameter (computed on every call; overwrites phi)
  double ph = P.radfield * exp(-2.5 * av) * sqrt(T) / (abund[N.neq - 1] * abund[N.nelec]);
  ph = fmin(fmax(ph, 1e2), 1e6);
  // freeze-out shut-off where a desorption route is much faster
  for (int k = threadIdx.x; k < N.n_fp; k += NT) {
    const int fpk = N.fp[k];
    const double l0 = aux[fpk] * abund[N.fp_re1[k]];
    const double lD = l0 * S.dens;
    bool off = false;
    if (N.desoh2_1 >= 0 && l0 < MINS * aux[N.desoh2_1 + k]) off = true;
    if (N.descr_1 >= 0 && lD < MINS * aux[N.descr_1 + k]) off = true;
    if (N.deuvcr_1 >= 0 && lD < MINS * aux[N.deuvcr_1 + k]) off = true;
    if (N.therm_1 >= 0 && P.thermdesorb && lD < MINS * aux[N.therm_1 + k]) off = true;
    if (off) aux[fpk] = 0.0;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < N.nreac; j += NT) {
    const uint8_t t = N.rtype[j];
    double r = aux[j];
    if (t == RT_THERM && sm < MINS) r = 0.0;
    if (t == RT_GAR) {
      const double* gp = N.gar + 7 * (size_t)N.partner[j];
      r = 0.6 * N.alpha[j] * gp[0] / (1. + gp[1] * pow(ph, gp[2]) * (1. + gp[3] * pow(T, gp[4]) * pow(ph, -gp[5] - gp[6] * log(T))));
    }
    if (!N.extrap[j] && T < N.tmin[j]) r = 0.0;
    if (!N.extrap[j] && T > N.tmax[j]) r = 0.0;
    if (j == N.rx_h2hv) r = h2_photo(S.h2col, P.radfield, av);
    if (j == N.rx_cohv) r = co_photo(S.h2col, S.cocol, P.radfield, av);
    if (j == N.rx_chv) r = c_ionization(N.alpha[j], N.gama[j], T, S.ccol, S.h2col, av, P.radfield);
    // (rx_* are -1 in a network without these reactions: never matched)
    rate[j] = r;
  }
  __syncthreads();
  if (threadIdx.x == 0) S.phi = ph;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Scalars shared by the RHS and the Jacobian of one evaluation
struct RhsScal {
  double D, sm, sb, ism, isb, blr, ts, y335, sc, kh2, kco;
  double dkh2_dn, dkco_dnh2, dkco_dnco;  // d rate / d column density
  int sm_on, blr_on, neg;
};

// A small integer coefficient (|c| < 2^20) as a double, built from its bits
// on the integer pipe: the same value as (double)c, without the FP64
// conversion (on this GPU the FP64 pipe issues a warp instruction in many
// cycles, and the RHS gather has one coefficient per term).
__device__ __forceinline__ double coef_to_double(int c) {
  const unsigned a = c < 0 ? (unsigned)(-c) : (unsigned)c;
  const int e = 31 - __clz(a);  // floor(log2 a) for a > 0
  unsigned hi = ((unsigned)(1023 + e) << 20) | ((a << (20 - e)) & 0xFFFFFu);
  hi = a ? (hi | (c < 0 ? 0x80000000u : 0u)) : 0u;
  return __hiloint2double((int)hi, 0);
}

// barrier of the `count` threads (a multiple of 32) that use named barrier `id`
__device__ __forceinline__ void bar_sync_named(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// flux of reaction r for the current scalars (shape-8 needs R.ts)
__device__ __forceinline__ double flux_of(int sh, double k, double D, double ya, double yb, const RhsScal& R) {
  switch (sh) {
    case SH_DYY: return k * D * ya * yb;
    case SH_Y: return k * ya;
    case SH_DY: return k * D * ya;
    case SH_Y_SM: return k * ya * R.ism;
    case SH_YY: return k * ya * yb;
    case SH_YY_BLR: return k * ya * yb * R.blr;
    case SH_Y_BLR: return k * ya * R.blr;
    case SH_DY_SM_Y: return k * D * ya * R.ism * yb;
    case SH_Y_TS_SM: return k * ya * R.ts * R.ism;
    default: return k * D * ya * yb * R.ism;
  }
}

// Right-hand side F(y) of one system.  All threads.  y, ydot, flux, part in
// shared memory; rate [nreac] anywhere.  With jac_scalars the photo-rate
// derivatives needed by the Jacobian are also formed.
//   warp 0: CO photodissociation (lane-parallel shielding splines)
//   warp 1: H2 photodissociation
//   warps 2..: the other reaction fluxes
__device__ __noinline__ void dev_rhs(const DevNet& N, const ucl_model_params& P, const SysPhys& S, const double* y,
                        const double* rate, double* ydot, double* flux, double* part, RhsScal& R,
                        bool jac_scalars = false) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    R.D = y[N.neq - 1];
    R.sm = fmax(1e-30, y[N.nsurf]);
    R.sb = fmax(1e-30, y[N.nbulk]);
    R.ism = 1.0 / R.sm;
    R.isb = 1.0 / R.sb;
    const double q = cK.NUM_SITES_PER_GRAIN / (cK.GAS_DUST_DENSITY_RATIO * R.sb);
    R.blr = q < 1.0 ? q : 1.0;
    R.sm_on = y[N.nsurf] > 1e-30;
    R.blr_on = (q < 1.0) && (y[N.nbulk] > 1e-30);
    R.ts = 0.0;
  }
  __syncthreads();
  const double D = R.D;
  const double h2col = 0.5 * y[N.nh2] * D * S.cs;
  if (warp == 0) {
    if (N.rx_cohv >= 0) {  // warp-uniform
    const double cocol = 0.5 * y[N.nco] * D * S.cs;
    const double k = co_photo_w(h2col, cocol, S);
    double d1 = 0.0, d2 = 0.0;
    if (jac_scalars) {
      const double e = 1e-6;
      const double dh = h2col * e + 1e-30, dc = cocol * e + 1e-30;
      d1 = (co_photo_w(h2col + dh, cocol, S) - k) / dh;
      d2 = (co_photo_w(h2col, cocol + dc, S) - k) / dc;
    }
    if (lane == 0) { R.kco = k; R.dkco_dnh2 = d1; R.dkco_dnco = d2; }
    }
  } else if (warp == 1) {
    if (lane == 0 && N.rx_h2hv >= 0) {
      R.kh2 = h2_photo_s(h2col, S);
      if (jac_scalars) {
        const double dh = h2col * 1e-6 + 1e-30;
        R.dkh2_dn = (h2_photo_s(h2col + dh, S) - R.kh2) / dh;
      }
    }
  } else {
    // warps 2..: the reaction fluxes, the surface-swap fluxes, the CSR
    // gather and the row sums, while warps 0 and 1 evaluate the
    // self-shielded photo rates.  The two photo reactions' terms are left
    // out here and added to their rows once the rates are known, so the
    // photo evaluation is off this critical path.  The warps synchronise on
    // named barrier 1 (NTF threads).
    constexpr int NTF = NT - 64;
    const int t = tid - 64;
    const int rh = N.rx_h2hv, rc = N.rx_cohv;
    // U reactions per thread per round, all table and rate loads first
    constexpr int U = 9;
    for (int r0 = t; r0 < N.nreac; r0 += U * NTF) {
      unsigned pk[U];
      double kk[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int r = r0 + u * NTF;
        pk[u] = r < N.nreac ? N.fpack[r] : 0u;
        kk[u] = r < N.nreac ? rate[r] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int r = r0 + u * NTF;
        const int sh = (int)(pk[u] >> 28);
        if (r < N.nreac && sh != SH_Y_TS_SM && r != rh && r != rc) {
          const int ya = (int)(pk[u] & 0x3FFFu), yb = (int)((pk[u] >> 14) & 0x3FFFu) - 1;
          flux[r] = flux_of(sh, kk[u], D, y[ya], yb >= 0 ? y[yb] : 0.0, R);
        }
      }
    }
    bar_sync_named(1, NTF);
    // totalSwap and the surface-swap fluxes (warp 2)
    if (warp == 2) {
      double sw = 0.0;
      for (int r = N.swap_lo + lane; r < N.swap_hi; r += 32) sw += flux[r];
      sw = warp_sum(sw);
      if (lane == 0) R.ts = sw;
      for (int k = lane; k < N.n_ts; k += 32) {
        const int r = N.ts_rx[k];
        flux[r] = rate[r] * y[N.fya[r]] * sw * R.ism;  // RATE*Y*totalSwap/safeMantle
      }
    }
    bar_sync_named(1, NTF);
    // chunked CSR gather: two chunks per thread per round, the <= 2 x 12
    // entry words loaded before any flux is read (photo terms skipped)
    constexpr int CHMAX = 12;
    for (int c0 = t; c0 < N.nchunk; c0 += 2 * NTF) {
      unsigned cp[2], e[2][CHMAX];
#pragma unroll
      for (int u = 0; u < 2; ++u) cp[u] = c0 + u * NTF < N.nchunk ? N.chpack[c0 + u * NTF] : 0u;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int beg = (int)(cp[u] & 0xFFFFu), len = (int)((cp[u] >> 16) & 0xFu);
#pragma unroll
        for (int j = 0; j < CHMAX; ++j) e[u][j] = j < len ? N.stpack[beg + j] : 0u;
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int len = (int)((cp[u] >> 16) & 0xFu);
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < CHMAX; ++j) {
          const int r = (int)(e[u][j] & 0xFFFFu);
          if (j < len && r != rh && r != rc) s += coef_to_double((signed char)(e[u][j] >> 16)) * flux[r];
        }
        if (c0 + u * NTF < N.nchunk) part[c0 + u * NTF] = s;
      }
    }
    bar_sync_named(1, NTF);
    // row sums of the chunk partials, in chunk order (rows without terms: 0)
    for (int i = t; i < N.neq; i += NTF) {
      const unsigned rw = N.rowch[i];
      const int c = (int)(rw & 0xFFFFu), cnt = (int)(rw >> 16);
      double s = 0.0;
      for (int k = 0; k < cnt; ++k) s = k == 0 ? part[c] : s + part[c + k];
      ydot[i] = s;
    }
  }
  // the photo fluxes (RATE*Y, checked when the tables are built), from the
  // warps that evaluated the rates
  if (tid == 0 && N.rx_cohv >= 0) flux[N.rx_cohv] = R.kco * y[N.fya[N.rx_cohv]];
  if (tid == 32 && N.rx_h2hv >= 0) flux[N.rx_h2hv] = R.kh2 * y[N.fya[N.rx_h2hv]];
  __syncthreads();
  // their terms in the rows of the species they touch
  if (tid < N.n_ph) {
    const double fh = N.rx_h2hv >= 0 ? flux[N.rx_h2hv] : 0.0, fc = N.rx_cohv >= 0 ? flux[N.rx_cohv] : 0.0;
    ydot[N.ph_row[tid]] += (double)N.ph_c1[tid] * fh + (double)N.ph_c2[tid] * fc;
  }
  __syncthreads();
  // surface <-> bulk transfer (odes.f90:4815-5180)
  if (warp == 0) {
    double s = 0.0;
    for (int k = lane; k < N.n_surface; k += 32) s += ydot[N.surface_list[k]];
    s = warp_sum(s);
    const bool neg = s < 0;
    const double sc = neg ? fmin(1.0, R.sb * R.ism) : 0.5 * cK.GAS_DUST_DENSITY_RATIO / cK.NUM_SITES_PER_GRAIN;
    const double f = neg ? s * sc * R.isb : s * sc;
    for (int k = lane; k < N.n_surface; k += 32) {
      const int si = N.surface_list[k], bi = N.bulk_list[k];
      const double t = f * (neg ? y[bi] : y[si]);
      ydot[si] = ydot[si] - t;
      ydot[bi] = ydot[bi] + t;
    }
    __syncwarp();
    double ss = 0.0, sb = 0.0;
    for (int k = lane; k < N.n_surface; k += 32) { ss += ydot[N.surface_list[k]]; sb += ydot[N.bulk_list[k]]; }
    ss = warp_sum(ss);
    sb = warp_sum(sb);
    if (lane == 0) {
      ydot[N.nsurf] = ss;
      ydot[N.nbulk] = sb;
      ydot[N.neq - 1] = densdot_fn(P, D);
      R.y335 = s;
      R.neg = neg;
      R.sc = sc;
    }
  } else if (warp == 1 && P.enforceChargeConservation && N.n_ion > 0) {
    // enforceChargeConservation: the electron derivative is the sum of the
    // positive ions' (chemistry.f90:333-335); ions are gas-phase species, so
    // this is independent of warp 0's ice transfer
    double s = 0.0;
    for (int k = lane; k < N.n_ion; k += 32) s += ydot[N.ion_list[k]];
    s = warp_sum(s);
    if (lane == 0) ydot[N.nelec] = s;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Analytic Jacobian of one system, dense row-major NEQ x NEQ in J (global):
// J[i*NEQ + j] = dF_i / dy_j.
// SCALED: J~ = W J W^-1 stored as float with W = diag(w) (error weights).
// Otherwise J stored as double.  Must follow a dev_rhs(..., jac_scalars=true)
// on the same y (uses R, flux).  dfa/dfb: [nreac] shared scratch.
template <bool SCALED, typename T>
__device__ __noinline__ void dev_jac(const DevNet& N, const ucl_model_params& P, const SysPhys& S, const double* y,
                        const double* rate, const double* w, const double* wi, T* J, const double* flux,
                        double* dfa, double* dfb, double* vec, double* jpart, const RhsScal& R) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = N.neq;
  const size_t nn = (size_t)n * n;
  const double D = R.D, ism = R.ism;
  {
    // zero J with 16-byte stores (n*n is a multiple of the vector width)
    using V = typename Vec2<T>::type;
    constexpr int W = Vec2<T>::W;
    V z;
    T* ze = reinterpret_cast<T*>(&z);
#pragma unroll
    for (int q = 0; q < W; ++q) ze[q] = (T)0;
    V* Jv = reinterpret_cast<V*>(J);
    const size_t nv = ((uintptr_t)J & 15) == 0 ? nn / W : 0;
    for (size_t i = tid; i < nv; i += NT) Jv[i] = z;
    for (size_t i = nv * W + tid; i < nn; i += NT) J[i] = (T)0;
  }
  for (int r = tid; r < N.nreac; r += NT) {
    const int sh = N.fshape[r];
    const double k = (r == N.rx_h2hv) ? R.kh2 : (r == N.rx_cohv) ? R.kco : rate[r];
    const double ya = y[N.fya[r]];
    const double yb = N.fyb[r] >= 0 ? y[N.fyb[r]] : 0.0;
    double a = 0.0, b = 0.0;
    switch (sh) {
      case SH_DYY: a = k * D * yb; b = k * D * ya; break;
      case SH_Y: a = k; break;
      case SH_DY: a = k * D; break;
      case SH_Y_SM: a = k * ism; break;
      case SH_YY: a = k * yb; b = k * ya; break;
      case SH_YY_BLR: a = k * yb * R.blr; b = k * ya * R.blr; break;
      case SH_Y_BLR: a = k * R.blr; break;
      case SH_DY_SM_Y: a = k * D * ism * yb; b = k * D * ya * ism; break;
      case SH_Y_TS_SM: a = k * R.ts * ism; break;
      default: a = k * D * yb * ism; b = k * D * ya * ism; break;
    }
    dfa[r] = a;
    dfb[r] = b;
  }
  __syncthreads();
  const double invD = 1.0 / D;
  const double dsm = R.sm_on ? -ism : 0.0;
  const double dblr = R.blr_on ? -R.isb : 0.0;
  // structural entries: partial sums per chunk of <= 8 contributions (two
  // chunks per thread per round, every table word loaded before use) ...
  constexpr int JCH = 8;
  for (int c0 = tid; c0 < N.njch; c0 += 2 * NT) {
    unsigned cw[2], e[2][JCH];
#pragma unroll
    for (int u = 0; u < 2; ++u) cw[u] = c0 + u * NT < N.njch ? N.jchunk[c0 + u * NT] : 0u;
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int beg = (int)(cw[u] & 0xFFFFu), len = (int)(cw[u] >> 16);
#pragma unroll
      for (int j = 0; j < JCH; ++j) e[u][j] = j < len ? N.jcpack[beg + j] : 0u;
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int len = (int)(cw[u] >> 16);
      double v = 0.0;
#pragma unroll
      for (int j = 0; j < JCH; ++j) {
        if (j < len) {
          const int key = (int)(e[u][j] & 0xFFFFu);
          const int r = key >> 3, slot = key & 7;
          double d;
          switch (slot) {
            case 0: d = dfa[r]; break;
            case 1: d = dfb[r]; break;
            case 2: d = flux[r] * invD; break;
            case 3: d = flux[r] * dsm; break;
            default: d = flux[r] * dblr; break;
          }
          v += coef_to_double((signed char)(e[u][j] >> 16)) * d;
        }
      }
      if (c0 + u * NT < N.njch) jpart[c0 + u * NT] = v;
    }
  }
  __syncthreads();
  // ... then one thread per entry sums its chunks and stores the entry
  for (int e = tid; e < N.n_jent; e += NT) {
    const unsigned ew = N.jent[e];
    const int i = N.je_row[e], j = N.je_col[e];
    const int c = (int)(ew & 0xFFFFu), cnt = (int)(ew >> 16);
    double v = 0.0;
    for (int k = 0; k < cnt; ++k) v = k == 0 ? jpart[c] : v + jpart[c + k];
    if (SCALED) J[(size_t)(i) * n + j] = (T)(v * w[i] * wi[j]);
    else J[(size_t)(i) * n + j] = (T)v;
  }
  __syncthreads();
  // surface-swap rank-1: J[i, bulk_k] += A_i * (k_k * blr)
  double* A = vec;  // [n_arow]
  for (int a = tid; a < N.n_arow; a += NT) {
    double s = 0.0;
    for (int c = N.ar_beg[a]; c < N.ar_end[a]; ++c) {
      const int r = N.ar_rx[c];
      s += (double)N.ar_coef[c] * rate[r] * y[N.fya[r]] * ism;
    }
    A[a] = s;
  }
  __syncthreads();
  const int nsw = N.swap_hi - N.swap_lo;
  for (int idx = tid; idx < N.n_arow * nsw; idx += NT) {
    const int a = idx % N.n_arow, kk = idx / N.n_arow;
    const int r = N.swap_lo + kk;
    const int i = N.ar_row[a], j = N.fya[r];
    const double v = A[a] * rate[r] * R.blr;
    if (SCALED) J[(size_t)(i) * n + j] += (T)(v * w[i] * wi[j]);
    else J[(size_t)(i) * n + j] += (T)v;
  }
  __syncthreads();
  // photo-rate dependence on the H2 / CO columns (and through them on D)
  if (tid < N.n_ph) {
    const int i = N.ph_row[tid];
    const double c1 = (double)N.ph_c1[tid], c2 = (double)N.ph_c2[tid];
    const double y1 = y[N.fya[N.rx_h2hv]], y2 = y[N.fya[N.rx_cohv]];
    const double half = 0.5 * S.cs;
    // d flux / d column: photo fluxes are rate * Y(reactant)
    const double dnh2 = (c1 * y1 * R.dkh2_dn + c2 * y2 * R.dkco_dnh2) * half * D;
    const double dnco = c2 * y2 * R.dkco_dnco * half * D;
    const double dD = (c1 * y1 * R.dkh2_dn + c2 * y2 * R.dkco_dnh2) * half * y[N.nh2] +
                      c2 * y2 * R.dkco_dnco * half * y[N.nco];
    if (SCALED) {
      J[(size_t)i * n + N.nh2] += (T)(dnh2 * w[i] * wi[N.nh2]);
      J[(size_t)i * n + N.nco] += (T)(dnco * w[i] * wi[N.nco]);
      J[(size_t)i * n + (n - 1)] += (T)(dD * w[i] * wi[n - 1]);
    } else {
      J[(size_t)i * n + N.nh2] += (T)dnh2;
      J[(size_t)i * n + N.nco] += (T)dnco;
      J[(size_t)i * n + (n - 1)] += (T)dD;
    }
  }
  __syncthreads();
  // surface <-> bulk transfer: rank-1 in the pre-transfer SURFACE row plus
  // the derivative of the transfer coefficients.
  T* g = (T*)(vec + 512);  // pre-transfer SURFACE row (scaled as stored)
  for (int j = tid; j < n; j += NT) g[j] = J[(size_t)(N.nsurf) * n + j];
  __syncthreads();
  const int ns = N.n_surface;
  const double y335 = R.y335;
  double* ck = vec;  // [ns] transfer coefficients c_k
  for (int k = tid; k < ns; k += NT)
    ck[k] = R.neg ? R.sc * y[N.bulk_list[k]] * R.isb : R.sc * y[N.surface_list[k]];
  __syncthreads();
  // ice rows: J[s_k,:] -= c_k g ; J[b_k,:] += c_k g  (row-major: threads over columns)
  T* uk = (T*)(vec + 256);  // [2*ns] scaled coefficients
  for (int k = tid; k < 2 * ns; k += NT) {
    const int kk = k < ns ? k : k - ns;
    const int row = k < ns ? N.surface_list[kk] : N.bulk_list[kk];
    const double u = SCALED ? ck[kk] * w[row] * wi[N.nsurf] : ck[kk];
    uk[k] = (T)(k < ns ? -u : u);
  }
  __syncthreads();
  // a warp per ice row, lanes over columns; two rows in flight per warp
  for (int k = warp; k < 2 * ns; k += 2 * NWARP) {
    T* Jr[2];
    T u[2];
    bool on[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int kq = k + h * NWARP;
      on[h] = kq < 2 * ns;
      const int kk = kq < ns ? kq : kq - ns;
      const int row = on[h] ? (kq < ns ? N.surface_list[kk] : N.bulk_list[kk]) : 0;
      u[h] = on[h] ? uk[kq] : (T)0;
      Jr[h] = J + (size_t)row * n;
    }
    for (int j = lane; j < n; j += 32) {
      const T gj = g[j];
      T a0 = on[0] ? Jr[0][j] : (T)0;
      T a1 = on[1] ? Jr[1][j] : (T)0;
      if (on[0]) Jr[0][j] = a0 + u[0] * gj;
      if (on[1]) Jr[1][j] = a1 + u[1] * gj;
    }
  }
  __syncthreads();
  {
    // derivative of the coefficients: sparse entries, one ice pair per
    // thread (rows differ between pairs)
    const bool use_sm = R.neg && (R.sb * R.ism < 1.0);
    const int colx = use_sm ? N.nsurf : N.nbulk;
    for (int k = tid; k < ns; k += NT) {
      const int si = N.surface_list[k], bi = N.bulk_list[k];
      double dself, dx = 0.0;
      int jself;
      if (R.neg) {
        jself = bi;
        if (use_sm) { dself = R.ism; if (R.sm_on) dx = -y[bi] * R.ism * R.ism; }
        else { dself = R.isb; if (y[N.nbulk] > 1e-30) dx = -y[bi] * R.isb * R.isb; }
      } else {
        jself = si;
        dself = R.sc;
      }
      const double v1 = y335 * dself, v2 = y335 * dx;
      if (SCALED) {
        J[(size_t)(si) * n + jself] -= (T)(v1 * w[si] * wi[jself]);
        J[(size_t)(bi) * n + jself] += (T)(v1 * w[bi] * wi[jself]);
        J[(size_t)(si) * n + colx] -= (T)(v2 * w[si] * wi[colx]);
        J[(size_t)(bi) * n + colx] += (T)(v2 * w[bi] * wi[colx]);
      } else {
        J[(size_t)(si) * n + jself] -= (T)v1;
        J[(size_t)(bi) * n + jself] += (T)v1;
        J[(size_t)(si) * n + colx] -= (T)v2;
        J[(size_t)(bi) * n + colx] += (T)v2;
      }
    }
  }
  __syncthreads();
  // SURFACE / BULK rows after transfer: sums of the ice rows
  for (int j = tid; j < n; j += NT) {
    double ssum = 0.0, bsum = 0.0;
#pragma unroll 8
    for (int k = 0; k < ns; ++k) {
      ssum += (double)J[(size_t)N.surface_list[k] * n + j] * (SCALED ? w[N.nsurf] * wi[N.surface_list[k]] : 1.0);
      bsum += (double)J[(size_t)N.bulk_list[k] * n + j] * (SCALED ? w[N.nbulk] * wi[N.bulk_list[k]] : 1.0);
    }
    J[(size_t)(N.nsurf) * n + j] = (T)ssum;
    J[(size_t)(N.nbulk) * n + j] = (T)bsum;
  }
  __syncthreads();
  if (P.enforceChargeConservation && N.n_ion > 0) {
    // electron row = sum of the ion rows (F sets ydot(nelec) to the ions' sum)
    for (int j = tid; j < n; j += NT) {
      double s = 0.0;
      for (int k = 0; k < N.n_ion; ++k) {
        const int r = N.ion_list[k];
        s += (double)J[(size_t)r * n + j] * (SCALED ? wi[r] : 1.0);
      }
      J[(size_t)(N.nelec) * n + j] = (T)(SCALED ? s * w[N.nelec] : s);
    }
    __syncthreads();
  }
  if (tid == 0) {
    double dd = 0.0;
    if (P.freefall && D < P.finalDens) {
      const double h = D * 1e-7;
      dd = (densdot_fn(P, D + h) - densdot_fn(P, D)) / h;
    }
    J[(size_t)((n - 1)) * n + (n - 1)] = (T)dd;
  }
  __syncthreads();
}

}  // namespace ucl
